// Node-block (BCSR) form of the CSRC matrix and its product y = K x.
//
// The elasticity matrix is a matrix of B x B node blocks (B = ndf): when no
// node is only partly fixed, numeq's numbering (Numeq.f:139-192) puts the B
// dofs of a node on consecutive equations, so block row I is equations
// B I .. B I + B - 1.  The CSRC arrays (ad, al: the reference's layout, which
// the assembly fills and the C ABI returns) are expanded after each assembly
// into full block rows -- lower blocks, the diagonal block, upper blocks as
// transposed copies of the lower ones -- with one column index per block
// instead of one per entry:
//
//   * bytes per stored entry: B^2 values + 1 index per B^2 entries, so
//     4.4 B (FP32) / 8.4 B (FP64) per entry against 6 / 10 B for the
//     two-sided gather with 16-bit column deltas;
//   * one thread per matrix row walks its block row: per block one column
//     index and B values, B x values, B FMAs -- every FMA lane does useful
//     work (no partially filled lane groups), which is what bounds the FP64
//     product on this GPU (its FP64 pipe retires 2 FMAs per clock per SM);
//   * no reductions inside a row, so the FP64 pipe does nothing but the
//     product's own FMAs.
//
// The product is still the reference's y = D x + L x + L^T x (matvec_csrcsym1,
// Matvec.f:528-621) with the same values, summed in a different order.
#include <algorithm>

#include "elx_krylov.h"
#include "elx_ptx.cuh"
#include "elx_reduce.cuh"

namespace elx {
namespace {

// Lower and diagonal blocks from the CSRC arrays: lower block q of block row
// I holds, in row B I + a, the B consecutive entries al[ia[B I + a] + B q ..];
// the diagonal block's strict lower part is the last a entries of row B I + a.
template <int B>
__global__ void fill_lower_blocks_kernel(int64_t nnzb, const int32_t *__restrict__ bia,
                                         const int32_t *__restrict__ bt,
                                         const int32_t *__restrict__ ia,
                                         const double *__restrict__ ad,
                                         const double *__restrict__ al,
                                         double *__restrict__ bval) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnzb;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t t = bt[p];
    if (t >= 0) continue;
    const int I = -1 - t;
    const int r0 = B * I;
    const int nl = (ia[r0 + 1] - ia[r0]) / B;
    const int q = (int)(p - bia[I]);
    double *out = bval + p * (B * B);
    if (q < nl) {
#pragma unroll
      for (int a = 0; a < B; a++)
#pragma unroll
        for (int b = 0; b < B; b++) out[a * B + b] = al[ia[r0 + a] + B * q + b];
    } else {
#pragma unroll
      for (int a = 0; a < B; a++)
#pragma unroll
        for (int b = 0; b < B; b++)
          out[a * B + b] = a == b  ? ad[r0 + a]
                           : a > b ? al[ia[r0 + a] + B * nl + b]
                                   : al[ia[r0 + b] + B * nl + a];
    }
  }
}

// Upper blocks: the transpose of their mirror.
template <int B>
__global__ void fill_upper_blocks_kernel(int64_t nnzb, const int32_t *__restrict__ bt,
                                         double *__restrict__ bval) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnzb;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t t = bt[p];
    if (t < 0) continue;
    const double *src = bval + (int64_t)t * (B * B);
    double *out = bval + p * (B * B);
#pragma unroll
    for (int a = 0; a < B; a++)
#pragma unroll
      for (int b = 0; b < B; b++) out[a * B + b] = src[b * B + a];
  }
}

__global__ void demote_blocks_kernel(int64_t n, const double *__restrict__ src,
                                     float *__restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

// y = K x, one thread per row, U blocks in flight, then the GatherEpi
// epilogue (dot products reduced in a fixed order over a fixed grid).
template <class T, int B, int EPI, int U>
__global__ void __launch_bounds__(256)
bcsr_spmv_kernel(int neq, const int32_t *__restrict__ bia, const int32_t *__restrict__ bja,
                 const T *__restrict__ bval, const T *__restrict__ x, T *__restrict__ y,
                 const T *__restrict__ w, PcgScalars *sc, double *partials,
                 unsigned int *counter, const int32_t *gate) {
  constexpr bool DOT = EPI == kEpiPcg || EPI == kEpiBicgAlpha || EPI == kEpiBicgOmega;
  constexpr int NV = EPI == kEpiBicgOmega ? 2 : 1;
  constexpr int BB = B * B;
  if (DOT && sc->done) return;
  if (gate && *gate == 0) return;
  T v[NV];
#pragma unroll
  for (int c = 0; c < NV; c++) v[c] = T(0);
  for (int row = blockIdx.x * 256 + threadIdx.x; row < neq; row += gridDim.x * 256) {
    const int I = row / B, a = row - I * B;
    const int pb = bia[I], pe = bia[I + 1];
    const T *vr = bval + (size_t)pb * BB + a * B;
    T acc0 = 0, acc1 = 0;
    int p = pb;
    for (; p + U <= pe; p += U) {
      int J[U];
      T av[U][B], xv[U][B];
#pragma unroll
      for (int u = 0; u < U; u++) J[u] = bja[p + u];
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int b = 0; b < B; b++) av[u][b] = vr[(size_t)(p - pb + u) * BB + b];
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int b = 0; b < B; b++) xv[u][b] = x[J[u] * B + b];
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int b = 0; b < B; b++) {
          if (u & 1)
            acc1 += av[u][b] * xv[u][b];
          else
            acc0 += av[u][b] * xv[u][b];
        }
    }
    for (; p < pe; p++) {
      const int J = bja[p];
#pragma unroll
      for (int b = 0; b < B; b++) acc0 += vr[(size_t)(p - pb) * BB + b] * x[J * B + b];
    }
    T yi = acc0 + acc1;
    if (EPI == kEpiScale) yi = yi * w[row];
    y[row] = yi;
    if (EPI == kEpiPcg) v[0] += x[row] * yi;
    if (EPI == kEpiBicgAlpha) v[0] += yi * w[row];
    if (EPI == kEpiBicgOmega) {
      v[0] += yi * w[row];
      v[1] += yi * yi;
    }
  }
  if (!DOT) return;
  double vb[NV];
  block_sum_widen<NV>(v, vb);
  if (!publish_partials<NV>(vb, partials, counter)) return;
  double tot[NV];
  gather_partials<NV>(tot, partials, counter);
  if (threadIdx.x == 0) {
    if (EPI == kEpiPcg) {
      sc->pq = tot[0];
      sc->alpha = tot[0] != 0.0 ? sc->d / tot[0] : 0.0;  // p = 0: no step
    } else if (EPI == kEpiBicgAlpha) {
      sc->pq = tot[0];
      sc->alpha = sc->rho / tot[0];
      sc->iters += 1;
    } else if (EPI == kEpiBicgOmega) {
      sc->omega = tot[0] / tot[NV - 1];
    }
  }
}

// y = K x with L lanes per block row (FP32): lane l takes blocks l, l + L,
// .. of the row (a block's B^2 values are contiguous, so consecutive lanes
// read one contiguous stream), then a fixed shuffle tree adds the lanes' B
// row sums.  Each group works on R block rows at once, all loads of the R
// rows issued before their FMAs, so that more bytes are in flight per warp.
// The FP32 pipe has room for the shuffles; the FP64 product keeps one thread
// per row (bcsr_spmv_kernel) so that its FP64 pipe does FMAs only.
template <class T, int B, int L, int R, int EPI>
__global__ void __launch_bounds__(256)
bcsr_spmv_group_kernel(int nb, const int32_t *__restrict__ bia, const int32_t *__restrict__ bja,
                       const T *__restrict__ bval, const T *__restrict__ x, T *__restrict__ y,
                       const T *__restrict__ w, PcgScalars *sc, double *partials,
                       unsigned int *counter, const int32_t *gate) {
  constexpr bool DOT = EPI == kEpiPcg || EPI == kEpiBicgAlpha || EPI == kEpiBicgOmega;
  constexpr int NV = EPI == kEpiBicgOmega ? 2 : 1;
  constexpr int BB = B * B;
  if (DOT && sc->done) return;
  if (gate && *gate == 0) return;
  T v[NV];
#pragma unroll
  for (int c = 0; c < NV; c++) v[c] = T(0);
  const int lane = threadIdx.x % L;
  const int ngroups = gridDim.x * (256 / L);
  for (int I0 = (blockIdx.x * 256 + threadIdx.x) / L; I0 < nb; I0 += R * ngroups) {
    int pb[R], pe[R];
    T acc[R][B];
    int kmax = 0;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int I = I0 + r * ngroups;
      pb[r] = I < nb ? bia[I] : 0;
      pe[r] = I < nb ? bia[I + 1] : 0;
      kmax = max(kmax, pe[r] - pb[r]);
#pragma unroll
      for (int a = 0; a < B; a++) acc[r][a] = T(0);
    }
    for (int k = lane; k < kmax; k += L) {
      T xv[R][B], bv[R][BB];
      bool on[R];
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int p = pb[r] + k;
        on[r] = p < pe[r];
        const int J = on[r] ? bja[p] : 0;
        const T *blk = bval + (size_t)(on[r] ? p : 0) * BB;
#pragma unroll
        for (int e = 0; e < BB; e++) bv[r][e] = on[r] ? blk[e] : T(0);
#pragma unroll
        for (int b = 0; b < B; b++) xv[r][b] = on[r] ? x[J * B + b] : T(0);
      }
#pragma unroll
      for (int r = 0; r < R; r++)
#pragma unroll
        for (int a = 0; a < B; a++)
#pragma unroll
          for (int b = 0; b < B; b++) acc[r][a] += bv[r][a * B + b] * xv[r][b];
    }
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1)
#pragma unroll
      for (int r = 0; r < R; r++)
#pragma unroll
        for (int a = 0; a < B; a++)
          acc[r][a] += __shfl_down_sync(0xffffffffu, acc[r][a], off, L);
    if (lane == 0) {
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int I = I0 + r * ngroups;
        if (I >= nb) continue;
#pragma unroll
        for (int a = 0; a < B; a++) {
          const int row = I * B + a;
          T yi = acc[r][a];
          if (EPI == kEpiScale) yi = yi * w[row];
          y[row] = yi;
          if (EPI == kEpiPcg) v[0] += x[row] * yi;
          if (EPI == kEpiBicgAlpha) v[0] += yi * w[row];
          if (EPI == kEpiBicgOmega) {
            v[0] += yi * w[row];
            v[1] += yi * yi;
          }
        }
      }
    }
  }
  if (!DOT) return;
  double vb[NV];
  block_sum_widen<NV>(v, vb);
  if (!publish_partials<NV>(vb, partials, counter)) return;
  double tot[NV];
  gather_partials<NV>(tot, partials, counter);
  if (threadIdx.x == 0) {
    if (EPI == kEpiPcg) {
      sc->pq = tot[0];
      sc->alpha = tot[0] != 0.0 ? sc->d / tot[0] : 0.0;  // p = 0: no step
    } else if (EPI == kEpiBicgAlpha) {
      sc->pq = tot[0];
      sc->alpha = sc->rho / tot[0];
      sc->iters += 1;
    } else if (EPI == kEpiBicgOmega) {
      sc->omega = tot[0] / tot[NV - 1];
    }
  }
}

// Position of entry e of slot t in a slot group of a sliced copy.  A group
// holds kSliceRows blocks as 16-byte chunks of V = 16 / sizeof(T) entries:
// entries 0 .. V-1 of every slot (slot t at V t), then the next V, and the
// remaining B^2 mod V entries one per slot, so that a thread reads its block
// with B^2 / V vector loads (plus B^2 mod V scalars) and a warp's load of one
// chunk is 512 contiguous bytes.
template <class T, int B>
__host__ __device__ constexpr int sell_pos(int e, int t) {
  constexpr int R = kSliceRows, V = 16 / sizeof(T), Q = B * B / V;
  return e < V * Q ? (e / V) * V * R + V * t + e % V : V * Q * R + (e - V * Q) * R + t;
}

// Sliced copy of the block-major FP64 values (as T): one thread per block
// row of the slice (slot t).
template <class T, int B>
__global__ void demote_sell_kernel(int nb, int nslices, const int32_t *__restrict__ bia,
                                   const int32_t *__restrict__ sell_ptr,
                                   const double *__restrict__ bval, T *__restrict__ sval) {
  constexpr int BB = B * B, R = kSliceRows;
  const int64_t nthreads = (int64_t)nslices * R;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nthreads;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int sl = (int)(i / R), t = (int)(i % R), I = (int)i;
    const int g0 = sell_ptr[sl], g1 = sell_ptr[sl + 1];
    const int p0 = I < nb ? bia[I] : 0;
    const int n = I < nb ? bia[I + 1] - p0 : 0;
    for (int g = g0; g < g1; g++) {
      const int k = g - g0;
      T *grp = sval + (size_t)g * BB * R;
#pragma unroll
      for (int e = 0; e < BB; e++)
        grp[sell_pos<T, B>(e, t)] = k < n ? (T)bval[(size_t)(p0 + k) * BB + e] : T(0);
    }
  }
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

// One block of a sliced copy into registers.
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

// y = K x on a sliced copy: one warp per slice, one thread per block row.
// Slot group g of a slice is one 128-byte line of column indices and B^2 / V
// 512-byte runs (plus B^2 mod V lines) of values, so every load of the
// matrix is fully used; the U groups' matrix loads are issued (in order) before
// any of their x gathers and FMAs.  Every lane of a warp runs the same number
// of groups (the slice's width), so the FP64 form has no idle FMA lanes but
// the padding.  Padding slots (zero values, the row's own column) do no harm.
// With D16 the column of slot (g, t) is its block row plus a 16-bit offset
// (col16: half the index bytes), else sell_col's 32-bit column.
template <class T, int B, int U, bool LD, int EPI, bool D16 = false>
__global__ void __launch_bounds__(256)
sell_spmv_kernel(int nb, int nslices, const int32_t *__restrict__ sell_ptr,
                 const int32_t *__restrict__ sell_col, const T *__restrict__ sval,
                 const T *__restrict__ x, T *__restrict__ y, const T *__restrict__ w,
                 PcgScalars *sc, double *partials, unsigned int *counter, const int32_t *gate,
                 const int16_t *__restrict__ col16 = nullptr) {
  constexpr bool DOT = EPI == kEpiPcg || EPI == kEpiBicgAlpha || EPI == kEpiBicgOmega;
  constexpr int NV = EPI == kEpiBicgOmega ? 2 : 1;
  constexpr int BB = B * B, R = kSliceRows;
  if (DOT && sc->done) return;
  if (gate && *gate == 0) return;
  T v[NV];
#pragma unroll
  for (int c = 0; c < NV; c++) v[c] = T(0);
  const int t = threadIdx.x % R;
  const int nwarps = gridDim.x * (256 / R);
  for (int sl = (blockIdx.x * 256 + threadIdx.x) / R; sl < nslices; sl += nwarps) {
    const int g0 = sell_ptr[sl], g1 = sell_ptr[sl + 1];
    T acc[B];
#pragma unroll
    for (int a = 0; a < B; a++) acc[a] = T(0);
    for (int g = g0; g < g1; g += U) {
      const int nu = min(U, g1 - g);
      int J[U];
      T bv[U][BB], xv[U][B];
#pragma unroll
      for (int u = 0; u < U; u++)
        if (u < nu) {
          if constexpr (D16)
            J[u] = sl * R + t + (int)sell_ld<LD>(col16 + (size_t)(g + u) * R + t);
          else
            J[u] = sell_ld<LD>(sell_col + (size_t)(g + u) * R + t);
        }
#pragma unroll
      for (int u = 0; u < U; u++)
        if (u < nu) sell_load<T, B, LD>(sval + (size_t)(g + u) * BB * R, t, bv[u]);
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int b = 0; b < B; b++) xv[u][b] = u < nu ? x[J[u] * B + b] : T(0);
#pragma unroll
      for (int u = 0; u < U; u++)
        if (u < nu)
#pragma unroll
          for (int a = 0; a < B; a++)
#pragma unroll
            for (int b = 0; b < B; b++) acc[a] += bv[u][a * B + b] * xv[u][b];
    }
    const int I = sl * R + t;
    if (I < nb) {
#pragma unroll
      for (int a = 0; a < B; a++) {
        const int row = I * B + a;
        T yi = acc[a];
        if (EPI == kEpiScale) yi = yi * w[row];
        y[row] = yi;
        if (EPI == kEpiPcg) v[0] += x[row] * yi;
        if (EPI == kEpiBicgAlpha) v[0] += yi * w[row];
        if (EPI == kEpiBicgOmega) {
          v[0] += yi * w[row];
          v[1] += yi * yi;
        }
      }
    }
  }
  if (!DOT) return;
  double vb[NV];
  block_sum_widen<NV>(v, vb);
  if (!publish_partials<NV>(vb, partials, counter)) return;
  double tot[NV];
  gather_partials<NV>(tot, partials, counter);
  if (threadIdx.x == 0) {
    if (EPI == kEpiPcg) {
      sc->pq = tot[0];
      sc->alpha = tot[0] != 0.0 ? sc->d / tot[0] : 0.0;  // p = 0: no step
    } else if (EPI == kEpiBicgAlpha) {
      sc->pq = tot[0];
      sc->alpha = sc->rho / tot[0];
      sc->iters += 1;
    } else if (EPI == kEpiBicgOmega) {
      sc->omega = tot[0] / tot[NV - 1];
    }
  }
}

int fill_grid(int64_t n) {
  const int64_t g = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 16));
}

}  // namespace

void launch_fill_blocks(const CsrcDev &k, cudaStream_t st) {
  if (!k.bval || k.nnzb == 0) return;
  const int g = fill_grid(k.nnzb);
  if (k.bsize == 3) {
    fill_lower_blocks_kernel<3><<<g, 256, 0, st>>>(k.nnzb, k.bia, k.bt, k.ia, k.ad, k.al, k.bval);
    fill_upper_blocks_kernel<3><<<g, 256, 0, st>>>(k.nnzb, k.bt, k.bval);
  } else {
    fill_lower_blocks_kernel<2><<<g, 256, 0, st>>>(k.nnzb, k.bia, k.bt, k.ia, k.ad, k.al, k.bval);
    fill_upper_blocks_kernel<2><<<g, 256, 0, st>>>(k.nnzb, k.bt, k.bval);
  }
  ELX_CUDA(cudaGetLastError());
}

void launch_demote_blocks(const CsrcDev &k, cudaStream_t st) {
  if (!k.bval || !k.bval32 || k.nnzb == 0) return;
  const int64_t n = k.nnzb * k.bsize * k.bsize;
  demote_blocks_kernel<<<fill_grid(n), 256, 0, st>>>(n, k.bval, k.bval32);
  ELX_CUDA(cudaGetLastError());
}

void launch_demote_sell(const CsrcDev &k, cudaStream_t st) {
  if (!k.bval || !k.sell_val || k.nslices == 0) return;
  const int g = fill_grid((int64_t)k.nslices * kSliceRows);
  if (k.bsize == 3)
    demote_sell_kernel<float, 3><<<g, 256, 0, st>>>(k.nb, k.nslices, k.bia, k.sell_ptr, k.bval,
                                                    k.sell_val);
  else
    demote_sell_kernel<float, 2><<<g, 256, 0, st>>>(k.nb, k.nslices, k.bia, k.sell_ptr, k.bval,
                                                    k.sell_val);
  ELX_CUDA(cudaGetLastError());
}

void launch_copy_sell64(const CsrcDev &k, cudaStream_t st) {
  if (!k.bval || !k.sell_val64 || k.nslices == 0) return;
  const int g = fill_grid((int64_t)k.nslices * kSliceRows);
  if (k.bsize == 3)
    demote_sell_kernel<double, 3><<<g, 256, 0, st>>>(k.nb, k.nslices, k.bia, k.sell_ptr, k.bval,
                                                     k.sell_val64);
  else
    demote_sell_kernel<double, 2><<<g, 256, 0, st>>>(k.nb, k.nslices, k.bia, k.sell_ptr, k.bval,
                                                     k.sell_val64);
  ELX_CUDA(cudaGetLastError());
}

void launch_sell64_local(int nb, int nslices, int bsize, const int32_t *sell_ptr,
                         const int32_t *sell_col, const double *sval, const double *x,
                         double *y, cudaStream_t st) {
  if (nslices <= 0) return;
  const int grid = std::max(1, std::min((nslices + 7) / 8, 1216));
  if (bsize == 3)
    sell_spmv_kernel<double, 3, 1, true, kEpiNone><<<grid, 256, 0, st>>>(
        nb, nslices, sell_ptr, sell_col, sval, x, y, nullptr, nullptr, nullptr, nullptr, nullptr);
  else
    sell_spmv_kernel<double, 2, 2, true, kEpiNone><<<grid, 256, 0, st>>>(
        nb, nslices, sell_ptr, sell_col, sval, x, y, nullptr, nullptr, nullptr, nullptr, nullptr);
  ELX_CUDA(cudaGetLastError());
}

// The gather entry points route here when the matrix has node blocks.
template <class T, int EPI>
void launch_bcsr(const CsrcDev &k, const T *x, T *y, const T *w, PcgScalars *sc,
                 double *partials, unsigned int *counter, const int32_t *gate,
                 cudaStream_t st) {
  const int sgrid = std::max(1, std::min((k.nslices + 7) / 8, 1216));
#define ELX_SELL(T_, B_, U_, LD_, VAL_)                                                     \
  sell_spmv_kernel<T_, B_, U_, LD_, EPI><<<sgrid, 256, 0, st>>>(                             \
      k.nb, k.nslices, k.sell_ptr, k.sell_col, VAL_, x, y, w, sc, partials, counter, gate)
  if constexpr (sizeof(T) == 4) {
    if (k.group_lanes == 0) {
      ELX_REQUIRE(k.sell_val != nullptr, ELX_ERR_STATE, "sliced FP32 node blocks missing");
      // one CTA per 8 slices, at most 8 per SM; 3 groups per step for B = 3
      // (64 registers) and 4 for B = 2: 50.7 / 52.4 / 50.2 / 60.0 us for
      // 1 / 2 / 3 / 4 groups with streaming loads on the 64^3 HEXA8 cube
#define ELX_SELL16(B_, U_, LD_)                                                          \
  sell_spmv_kernel<float, B_, U_, LD_, EPI, true><<<sgrid, 256, 0, st>>>(                  \
      k.nb, k.nslices, k.sell_ptr, k.sell_col, k.sell_val, x, y, w, sc, partials, counter, \
      gate, k.sell_d16)
      if (k.bsize == 3 && k.sell_d16) {
        if (k.sell_stream)
          ELX_SELL16(3, 3, true);
        else
          ELX_SELL16(3, 3, false);
      } else if (k.bsize == 3) {
        if (k.sell_stream)
          ELX_SELL(float, 3, 3, true, k.sell_val);
        else
          ELX_SELL(float, 3, 3, false, k.sell_val);
      } else {
        if (k.sell_stream)
          ELX_SELL(float, 2, 4, true, k.sell_val);
        else
          ELX_SELL(float, 2, 4, false, k.sell_val);
      }
#undef ELX_SELL16
      ELX_CUDA(cudaGetLastError());
      return;
    }
  } else {
    if (k.sell_val64) {
      // FP64-pipe bound: one group per step (48 registers) measured as fast
      // as two and faster than three (126.1 / 125.9 / 131.2 us on the 64^3
      // HEXA8 cube), streaming loads faster than cached ones (128.8 us)
      if (k.bsize == 3)
        ELX_SELL(double, 3, 1, true, k.sell_val64);
      else
        ELX_SELL(double, 2, 2, true, k.sell_val64);
      ELX_CUDA(cudaGetLastError());
      return;
    }
  }
#undef ELX_SELL
  const T *val;
  if constexpr (sizeof(T) == 8)
    val = k.bval;
  else
    val = k.bval32;
  ELX_REQUIRE(val != nullptr, ELX_ERR_STATE, "node-block values missing");
  // one wave of 8 CTAs per SM (152 SMs): 134 us against 142 us for one CTA
  // per 256 rows on the 64^3 HEXA8 cube (FP64), 47.6 against 52.0 us on the
  // 48^3 TETRA4 mesh
  int grid = std::max(1, std::min((k.neq + 255) / 256, 1216));
  if (k.gather_blocks > 0) grid = std::min((k.neq + 255) / 256, k.gather_blocks);
  if (sizeof(T) == 4 && k.group_lanes > 0) {
    // lane groups per block row (FP32); two rows in flight per group measured
    // slower (register pressure): 78.6 against 68.8 us on the 64^3 HEXA8 cube
    if (k.bsize == 3 && k.group_lanes == 8)
      bcsr_spmv_group_kernel<T, 3, 8, 1, EPI><<<grid, 256, 0, st>>>(
          k.nb, k.bia, k.bja, val, x, y, w, sc, partials, counter, gate);
    else if (k.bsize == 3)
      bcsr_spmv_group_kernel<T, 3, 16, 1, EPI><<<grid, 256, 0, st>>>(
          k.nb, k.bia, k.bja, val, x, y, w, sc, partials, counter, gate);
    else
      bcsr_spmv_group_kernel<T, 2, 8, 1, EPI><<<grid, 256, 0, st>>>(
          k.nb, k.bia, k.bja, val, x, y, w, sc, partials, counter, gate);
  } else if (k.bsize == 3) {
    bcsr_spmv_kernel<T, 3, EPI, 3><<<grid, 256, 0, st>>>(k.neq, k.bia, k.bja, val, x, y, w, sc,
                                                         partials, counter, gate);
  } else {
    bcsr_spmv_kernel<T, 2, EPI, 4><<<grid, 256, 0, st>>>(k.neq, k.bia, k.bja, val, x, y, w, sc,
                                                         partials, counter, gate);
  }
  ELX_CUDA(cudaGetLastError());
}

template void launch_bcsr<double, kEpiNone>(const CsrcDev &, const double *, double *,
                                            const double *, PcgScalars *, double *,
                                            unsigned int *, const int32_t *, cudaStream_t);
template void launch_bcsr<double, kEpiPcg>(const CsrcDev &, const double *, double *,
                                           const double *, PcgScalars *, double *,
                                           unsigned int *, const int32_t *, cudaStream_t);
template void launch_bcsr<double, kEpiBicgAlpha>(const CsrcDev &, const double *, double *,
                                                 const double *, PcgScalars *, double *,
                                                 unsigned int *, const int32_t *, cudaStream_t);
template void launch_bcsr<double, kEpiBicgOmega>(const CsrcDev &, const double *, double *,
                                                 const double *, PcgScalars *, double *,
                                                 unsigned int *, const int32_t *, cudaStream_t);
template void launch_bcsr<double, kEpiScale>(const CsrcDev &, const double *, double *,
                                             const double *, PcgScalars *, double *,
                                             unsigned int *, const int32_t *, cudaStream_t);
template void launch_bcsr<float, kEpiNone>(const CsrcDev &, const float *, float *,
                                           const float *, PcgScalars *, double *,
                                           unsigned int *, const int32_t *, cudaStream_t);
template void launch_bcsr<float, kEpiPcg>(const CsrcDev &, const float *, float *, const float *,
                                          PcgScalars *, double *, unsigned int *,
                                          const int32_t *, cudaStream_t);

}  // namespace elx
