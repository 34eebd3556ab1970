// CSRC matrix-vector product y = (D + L + L^T) x on the GPU
// (matvec_csrcsym1, mef/src/Matvec.f:528-621).
//
// The reference makes one row-ordered pass: row i's lower product
// t = ad(i) x(i) + sum al(k) x(ja(k)) and, for the same entries, the scatter of
// the mirrored upper part y(ja(k)) += al(k) x(i).  Each al(k) is read once.
// A GPU cannot scatter without atomics (nondeterministic in FP64), and
// gathering the upper part through a global transposed copy reads every value
// twice.  This kernel keeps the single read:
//
//   * Rows are cut into tiles of R consecutive rows; one CTA per tile.
//   * Row phase: LANES threads per row stream the row's entries (al, ja) once
//     from HBM (loads unrolled so that several are in flight), form the row
//     sum with x gathered from L2 as an FMA chain, and park each value and its
//     tile-local row number in shared memory.
//   * Column phase: the tile's transposed index (built once on the host,
//     structure.cpp:build_tiles) lists, per distinct column j of the tile,
//     the tile-local positions of its entries.  One thread per column sums
//     al(k) x(row(k)) from shared memory in that fixed order.  Columns inside
//     the tile are added to the tile's own rows in shared memory; columns left
//     of the tile (rows of earlier tiles) go to a halo slot in HBM.
//   * A second, row-parallel launch (krylov.cu) adds to every row its halo
//     slots in tile order.
//
// Every y(i) is therefore summed in the same order on every call
// (deterministic), and HBM traffic per call is al + ja + the 16-bit
// transposed positions + small per-column metadata, against 12 bytes per
// entry of algorithmic traffic.  The FP64 version does exactly 2 DFMA per
// entry, the minimum for the symmetric product; since GB300's FP64 pipe
// (2 DFMA/clock/SM) charges a whole warp instruction however few lanes are
// active, the arithmetic is arranged so that warps run loops of nearly equal
// length: two threads per row (one shuffle-add per row), consecutive rows of a
// tile have similar lengths, and the host orders each tile's columns by
// decreasing length.
#include "elx_internal.h"

namespace elx {
namespace {

constexpr int kTileThreads = 256;

template <class T, int LANES>
__global__ void __launch_bounds__(kTileThreads)
tile_spmv_kernel(int neq, const int32_t *__restrict__ ia, const int32_t *__restrict__ ja,
                 const T *__restrict__ al, const T *__restrict__ ad, TileDev td,
                 const T *__restrict__ x, T *__restrict__ ytile, T *__restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int R = td.rows;
  T *s_a = reinterpret_cast<T *>(smem);                 // [max_nnz] values
  T *s_x = s_a + td.max_nnz;                            // [R] x of the tile's rows
  T *s_y = s_x + R;                                     // [R]
  uint16_t *s_pos = reinterpret_cast<uint16_t *>(s_y + R);  // [max_nnz]
  uint8_t *s_row = reinterpret_cast<uint8_t *>(s_pos + td.max_nnz);  // [max_nnz]

  const int tile = blockIdx.x;
  const int r0 = tile * R;
  const int nr = min(R, neq - r0);
  const int base = ia[r0];
  const int nnz = ia[r0 + nr] - base;
  const int tid = threadIdx.x;

  for (int i = tid; i < nr; i += kTileThreads) s_x[i] = x[r0 + i];
  for (int q = tid; q < nnz; q += kTileThreads) s_pos[q] = td.tpos[base + q];
  __syncthreads();

  // ---- row phase: LANES threads per row
  const int lane = tid % LANES;
  constexpr int kSubs = kTileThreads / LANES;
  constexpr int U = 4;  // entries in flight per thread
  for (int i0 = 0; i0 < nr; i0 += kSubs) {
    const int i = i0 + tid / LANES;
    T s = 0;
    if (i < nr) {
      const int kb = ia[r0 + i], ke = ia[r0 + i + 1];
      for (int k0 = kb + lane; k0 < ke; k0 += U * LANES) {
        T a[U], xv[U];
        int j[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int k = k0 + u * LANES;
          a[u] = k < ke ? al[k] : T(0);
          j[u] = k < ke ? ja[k] : r0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) xv[u] = x[j[u]];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int k = k0 + u * LANES;
          if (k < ke) {
            s += a[u] * xv[u];
            s_a[k - base] = a[u];
            s_row[k - base] = (uint8_t)i;
          }
        }
      }
    }
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off, LANES);
    if (i < nr && lane == 0) s_y[i] = ad[r0 + i] * s_x[i] + s;
  }
  __syncthreads();

  // ---- column phase: one thread per distinct column of the tile
  const int g0 = td.tile_tgt[tile], g1 = td.tile_tgt[tile + 1];
  const int o0 = td.tile_out[tile], nout = td.tile_out[tile + 1] - o0;
  for (int g = g0 + tid; g < g1; g += kTileThreads) {
    T acc = 0;
    const int qb = td.tgt_start[g] - base, qe = td.tgt_start[g + 1] - base;
    for (int q = qb; q < qe; q++) {
      const int pos = s_pos[q];
      acc += s_a[pos] * s_x[s_row[pos]];
    }
    const int t = g - g0;
    if (t < nout) part[o0 + t] = acc;
    else s_y[td.tgt_col[g] - r0] += acc;
  }
  __syncthreads();
  for (int i = tid; i < nr; i += kTileThreads) ytile[r0 + i] = s_y[i];
}

__global__ void demote_kernel(int64_t n, const double *__restrict__ src, float *__restrict__ dst) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = (float)src[q];
}

template <class T>
void launch_tile(const CsrcDev &k, const TileDev &t, const T *al, const T *ad, const T *x,
                 T *ytile, T *part, cudaStream_t st) {
  const size_t smem = tile_smem_bytes(t, sizeof(T) == 4);
  if (t.lanes == 1)
    tile_spmv_kernel<T, 1><<<t.ntiles, kTileThreads, smem, st>>>(k.neq, k.ia, k.ja, al, ad, t, x,
                                                                 ytile, part);
  else
    tile_spmv_kernel<T, 2><<<t.ntiles, kTileThreads, smem, st>>>(k.neq, k.ia, k.ja, al, ad, t, x,
                                                                 ytile, part);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace

// Opt in to the tile kernels' shared memory once per structure (outside any
// stream capture).
void prepare_tile_kernels(const TileDev &t) {
  const int s64 = (int)tile_smem_bytes(t, false), s32 = (int)tile_smem_bytes(t, true);
  ELX_REQUIRE(s64 <= 227 * 1024, ELX_ERR_ARG, "tile needs more shared memory than a CTA has");
  auto attr = [](auto kern, int bytes) {
    ELX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  };
  attr(tile_spmv_kernel<double, 1>, s64);
  attr(tile_spmv_kernel<double, 2>, s64);
  attr(tile_spmv_kernel<float, 1>, s32);
  attr(tile_spmv_kernel<float, 2>, s32);
}

size_t tile_smem_bytes(const TileDev &t, bool fp32) {
  const size_t vs = fp32 ? 4 : 8;
  return (size_t)t.max_nnz * vs + 2 * (size_t)t.rows * vs + (size_t)t.max_nnz * 3 + 16;
}

void launch_tile_spmv64(const CsrcDev &k, const TileDev &t, const double *x, double *ytile,
                        double *part, cudaStream_t st) {
  launch_tile<double>(k, t, k.al, k.ad, x, ytile, part, st);
}

void launch_tile_spmv32(const CsrcDev &k, const TileDev &t, const float *x, float *ytile,
                        float *part, cudaStream_t st) {
  launch_tile<float>(k, t, k.al32, k.ad32, x, ytile, part, st);
}

// FP32 copies of ad and al for the mixed-precision inner iteration.
void launch_demote_values(const CsrcDev &k, cudaStream_t st) {
  demote_kernel<<<608, 256, 0, st>>>(k.neq, k.ad, k.ad32);
  if (k.nad) demote_kernel<<<1216, 256, 0, st>>>(k.nad, k.al, k.al32);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace elx
