// Layout and loads of the sliced node-block copies (SELL-32) that the
// single-vector products (bcsr.cu), the block products (block_pcg.cu) and
// the partitioned product read.
//
// A slice is kSliceRows consecutive block rows; slot group g of a slice
// holds block g - sell_ptr[slice] of each of its rows (slot t: block row
// kSliceRows * slice + t), padded with zero blocks past a row's end.  A
// group's values are 16-byte chunks of V = 16 / sizeof(T) entries: entries
// 0 .. V-1 of every slot (slot t at V t), then the next V, and the remaining
// B^2 mod V entries one per slot -- so a warp's load of one chunk over 32
// consecutive slots is one 512-byte run.
#pragma once

#include "elx_internal.h"
#include "elx_ptx.cuh"

namespace elx {

// Position of entry e of slot t inside a slot group.
template <class T, int B>
__host__ __device__ constexpr int sell_pos(int e, int t) {
  constexpr int R = kSliceRows, V = 16 / sizeof(T), Q = B * B / V;
  return e < V * Q ? (e / V) * V * R + V * t + e % V : V * Q * R + (e - V * Q) * R + t;
}

// Loads of a sliced copy: streaming (not kept in L1; for a matrix larger
// than L2, read from HBM once per product) or ordinary read-only loads (for
// a matrix that stays in L2 between products, where they measured faster).
template <bool STREAM, class T>
__device__ __forceinline__ T sell_ld(const T *p) {
  if constexpr (STREAM)
    return ptx::ld_stream(p);
  else
    return __ldg(p);
}

// One block of a sliced copy into registers (slot t of the group at grp).
template <class T, int B, bool LD>
__device__ __forceinline__ void sell_load(const T *grp, int t, T (&bv)[B * B]) {
  constexpr int BB = B * B, R = kSliceRows, V = 16 / sizeof(T), Q = BB / V;
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const T *p = grp + q * V * R + V * t;
    if constexpr (sizeof(T) == 4) {
      const float4 c = LD ? ptx::ld_stream4(p) : __ldg(reinterpret_cast<const float4 *>(p));
      bv[4 * q] = c.x;
      bv[4 * q + 1] = c.y;
      bv[4 * q + 2] = c.z;
      bv[4 * q + 3] = c.w;
    } else {
      const double2 c = LD ? ptx::ld_stream2(p) : __ldg(reinterpret_cast<const double2 *>(p));
      bv[2 * q] = c.x;
      bv[2 * q + 1] = c.y;
    }
  }
#pragma unroll
  for (int e = V * Q; e < BB; e++) bv[e] = sell_ld<LD>(grp + V * Q * R + (e - V * Q) * R + t);
}

// Block column of slot (g, t) of slice sl: its block row plus a 16-bit
// offset (col16) or the 32-bit column (sell_col).
template <bool D16, bool LD>
__device__ __forceinline__ int sell_column(const int32_t *sell_col, const int16_t *col16, int sl,
                                           int g, int t) {
  if constexpr (D16)
    return sl * kSliceRows + t + (int)sell_ld<LD>(col16 + (size_t)g * kSliceRows + t);
  else
    return sell_ld<LD>(sell_col + (size_t)g * kSliceRows + t);
}

}  // namespace elx
