// Block PCG: W load cases solved together over one read of the matrix per
// iteration.  Each column runs the reference's Jacobi PCG (pcg,
// mef/src/Iters.f:252-524) with its own scalars -- so each column's iterates
// are those of a single-RHS solve -- while the product K [p_1 .. p_W] reads
// the node-block matrix once for all W columns (an SpMM: every block value
// loaded from HBM once, used by W lanes).
//
// Multi-vectors are row-interleaved: entry (row, c) at row * W + c, so the
// W lanes of a group read one row's W columns as one contiguous run.
//
// Two precisions:
//   * FP64: the FP64 PCG per column (spmm with the fused dots, update,
//     direction), stopping per column on sqrt|(r, M r)| < tol ||b||_M.
//   * mixed: FP32 CG per column with reliable updates, as in the single-RHS
//     mixed solver: FP32 SpMM and vectors carry the recurrence; when a
//     column's FP32 residual has dropped tenfold (checked every few
//     iterations), its FP32 solution piece is folded into the FP64 solution
//     and its residual replaced by b - K x from one FP64 SpMM (all columns,
//     launched only when some column asks); the stopping test is the
//     reference's, on that FP64 residual.
// Converged columns stop changing (masked), the others go on; every kernel
// returns at once when no column is active.
#include <algorithm>
#include <type_traits>

#include <cstdlib>

#include "elx_krylov.h"
#include "elx_ptx.cuh"
#include "elx_reduce.cuh"
#include "elx_sell.cuh"

namespace elx {
namespace {

// Last-block stage of the column reductions: the NC totals of NC rows of
// `nblocks` partials ([c][block]), all threads loading (NC rows spread over
// the block's threads, several loads in flight per thread), then a fixed
// order over the slices.  Thread c < NC returns total c (others: 0).
template <int NC>
__device__ __forceinline__ double gather_columns(const double *partials, int nblocks) {
  static_assert(kThreads % NC == 0, "column count must divide the block");
  constexpr int S = kThreads / NC;
  __shared__ double sh[kThreads];
  const int c = threadIdx.x % NC, sl = threadIdx.x / NC;
  double t = 0.0;
#pragma unroll 4
  for (int b = sl; b < nblocks; b += S) t += __ldcg(partials + (size_t)c * nblocks + b);
  sh[threadIdx.x] = t;
  __syncthreads();
  double u = 0.0;
  if (threadIdx.x < NC)
    for (int k = 0; k < S; k++) u += sh[k * NC + threadIdx.x];
  return u;
}

// Per-column reduction of one value per thread, with thread t holding column
// t % W: warp tree over the groups, per-warp sums in shared memory, per-block
// sums published, the last block adds the blocks in a fixed order.  Returns
// true in the last block, whose threads c < W then hold column c's total in
// `out`.
template <int W>
__device__ __forceinline__ bool column_reduce(double v, double *partials, unsigned int *counter,
                                              double &out) {
  __shared__ double sh[kThreads / 32][W];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off >= W; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if (lane < W) sh[warp][lane] = v;
  __syncthreads();
  if (threadIdx.x < W) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) t += sh[w][threadIdx.x];
    partials[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = t;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  out = gather_columns<W>(partials, gridDim.x);
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// The same for two values per thread.
template <int W>
__device__ __forceinline__ bool column_reduce2(double v0, double v1, double *partials,
                                               unsigned int *counter, double &o0, double &o1) {
  __shared__ double sh[2][kThreads / 32][W];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off >= W; off >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, off);
    v1 += __shfl_down_sync(0xffffffffu, v1, off);
  }
  if (lane < W) {
    sh[0][warp][lane] = v0;
    sh[1][warp][lane] = v1;
  }
  __syncthreads();
  if (threadIdx.x < W) {
    double t0 = 0.0, t1 = 0.0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) {
      t0 += sh[0][w][threadIdx.x];
      t1 += sh[1][w][threadIdx.x];
    }
    partials[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = t0;
    partials[(size_t)(W + threadIdx.x) * gridDim.x + blockIdx.x] = t1;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // rows 0..W-1 hold the first values, W..2W-1 the second
  const double t = gather_columns<2 * W>(partials, gridDim.x);
  __shared__ double tt[2 * W];
  if (threadIdx.x < 2 * W) tt[threadIdx.x] = t;
  __syncthreads();
  o0 = o1 = 0.0;
  if (threadIdx.x < W) {
    o0 = tt[threadIdx.x];
    o1 = tt[W + threadIdx.x];
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// Vector of VC consecutive columns of one row (16-byte loads at most).
template <class T, int VC>
struct ColVec {
  T v[VC];
};
template <class T, int VC>
__device__ __forceinline__ ColVec<T, VC> load_cols(const T *p) {
  ColVec<T, VC> r;
  if constexpr (VC * sizeof(T) == 16) {
    using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    const V t = *reinterpret_cast<const V *>(p);
    const T *e = reinterpret_cast<const T *>(&t);
#pragma unroll
    for (int j = 0; j < VC; j++) r.v[j] = e[j];
  } else if constexpr (VC * sizeof(T) == 8 && sizeof(T) == 4) {
    const float2 t = *reinterpret_cast<const float2 *>(p);
    r.v[0] = t.x;
    r.v[1] = t.y;
  } else {
#pragma unroll
    for (int j = 0; j < VC; j++) r.v[j] = p[j];
  }
  return r;
}

template <class T, int VC>
__device__ __forceinline__ void store_cols(T *p, const ColVec<T, VC> &x) {
  if constexpr (VC == 4 && sizeof(T) == 4) {
    *reinterpret_cast<float4 *>(p) = make_float4(x.v[0], x.v[1], x.v[2], x.v[3]);
  } else if constexpr (VC == 2 && sizeof(T) == 8) {
    *reinterpret_cast<double2 *>(p) = make_double2(x.v[0], x.v[1]);
  } else {
#pragma unroll
    for (int j = 0; j < VC; j++) p[j] = x.v[j];
  }
}

// Per-column reduction when thread t holds columns (t % G) VC .. + VC - 1
// (G = W / VC lanes per group): warp tree over the groups, per-warp sums in
// shared memory, per-block sums published, the last block adds the blocks in
// a fixed order; returns true in the last block, whose threads c < W hold
// column c's total in `out`.
template <int W, int VC>
__device__ __forceinline__ bool column_reduce_v(double (&v)[VC], double *partials,
                                                unsigned int *counter, double &out) {
  constexpr int G = W / VC;
  __shared__ double sh[kThreads / 32][W];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off >= G; off >>= 1)
#pragma unroll
    for (int j = 0; j < VC; j++) v[j] += __shfl_down_sync(0xffffffffu, v[j], off);
  if (lane < G)
#pragma unroll
    for (int j = 0; j < VC; j++) sh[warp][lane * VC + j] = v[j];
  __syncthreads();
  if (threadIdx.x < W) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) t += sh[w][threadIdx.x];
    partials[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = t;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  out = gather_columns<W>(partials, gridDim.x);
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// Y = K X for W columns on a sliced copy of the node blocks.  A group of
// G = W / VC lanes works on one block row, each lane on VC consecutive
// columns (one 16-byte x load per row of a block); G warps take one slice
// (kSliceRows block rows).  The G lanes of a row load its block with the same
// 16-byte chunk loads (a broadcast), so one warp's load of a chunk covers
// 32 / G consecutive slots: 512 / G contiguous bytes, where the block-major
// form read each block as B^2 scalar loads at a 36-byte stride.  Every lane
// of a slice walks the slice's width; U slot groups' matrix loads are issued
// together, then each group's x loads and FMAs, whose order per row is the
// block order (the sums do not depend on U).  Padding slots hold zero
// blocks and the row's own column.  With DOT, also pq_c = (x_c, y_c) and
// alpha_c = d_c / pq_c for the active columns; a launch with gate != nullptr
// runs only while *gate != 0; with MASK only the lanes whose columns asked
// for a residual replacement compute.
template <class T, int B, int W, bool DOT, bool MASK, int U, bool LD, bool D16>
__global__ void __launch_bounds__(kThreads, 3)
sell_spmm_kernel(int nb, int nslices, const int32_t *__restrict__ sell_ptr,
                 const int32_t *__restrict__ sell_col, const int16_t *__restrict__ col16,
                 const T *__restrict__ sval, const T *__restrict__ X, T *__restrict__ Y,
                 ColScalars *cols, BlockHeader *hdr, double *partials, unsigned int *counter,
                 const int32_t *gate) {
  constexpr int VC = (16 / (int)sizeof(T)) < W ? (16 / (int)sizeof(T)) : W;
  constexpr int G = W / VC;
  constexpr int BB = B * B, R = kSliceRows;
  constexpr int SPC = kThreads / (R * G);  // slices per CTA pass
  static_assert(SPC >= 1, "a CTA must hold a whole slice");
  if (hdr->active == 0) return;
  if (gate && *gate == 0) return;
  const int c0 = (threadIdx.x % G) * VC;
  const int t = (threadIdx.x / G) % R;
  if constexpr (MASK) {
    bool need = false;
#pragma unroll
    for (int j = 0; j < VC; j++) need = need || (!cols[c0 + j].done && cols[c0 + j].update);
    if (!need) return;
  }
  T v[VC];  // this thread's share of (x_c, y_c), in T (the FP64 pipe is narrow)
#pragma unroll
  for (int j = 0; j < VC; j++) v[j] = T(0);
  // passes of SPC slices, every gridDim.x-th for this CTA (contiguous runs
  // of passes per CTA measured slower: 265 against 247 us, W = 16 FP32 on the
  // 96x96x48 plate)
  for (int sl = blockIdx.x * SPC + (int)threadIdx.x / (R * G); sl < nslices;
       sl += gridDim.x * SPC) {
    const int g0 = sell_ptr[sl], g1 = sell_ptr[sl + 1];
    T acc[B][VC];
#pragma unroll
    for (int a = 0; a < B; a++)
#pragma unroll
      for (int j = 0; j < VC; j++) acc[a][j] = T(0);
    for (int g = g0; g < g1; g += U) {
      const int nu = min(U, g1 - g);
      int J[U];
      T bv[U][BB];
#pragma unroll
      for (int u = 0; u < U; u++)
        if (u < nu) J[u] = sell_column<D16, LD>(sell_col, col16, sl, g + u, t);
#pragma unroll
      for (int u = 0; u < U; u++)
        if (u < nu) sell_load<T, B, LD>(sval + (size_t)(g + u) * BB * R, t, bv[u]);
      // x of each group loaded just before its FMAs (mostly L1 hits): the
      // registers go to more groups of matrix loads in flight (244 against
      // 299.5 us for W = 16 FP32 on the 96x96x48 plate with all loads issued
      // first; 3 groups at 3 CTAs per SM measured best of 3 / 4 / 6 / 8
      // groups at 1-3 CTAs per SM, 244-301 us)
#pragma unroll
      for (int u = 0; u < U; u++)
        if (u < nu) {
          ColVec<T, VC> xw[B];
#pragma unroll
          for (int b = 0; b < B; b++)
            xw[b] = load_cols<T, VC>(X + (size_t)(J[u] * B + b) * W + c0);
#pragma unroll
          for (int a = 0; a < B; a++)
#pragma unroll
            for (int b = 0; b < B; b++)
#pragma unroll
              for (int j = 0; j < VC; j++) acc[a][j] += bv[u][a * B + b] * xw[b].v[j];
        }
    }
    const int I = sl * R + t;
    if (I < nb) {
#pragma unroll
      for (int a = 0; a < B; a++) {
        const size_t q = (size_t)(I * B + a) * W + c0;
        ColVec<T, VC> yv;
#pragma unroll
        for (int j = 0; j < VC; j++) yv.v[j] = acc[a][j];
        store_cols<T, VC>(Y + q, yv);
        if (DOT) {
          const ColVec<T, VC> xq = load_cols<T, VC>(X + q);
#pragma unroll
          for (int j = 0; j < VC; j++) v[j] += xq.v[j] * acc[a][j];
        }
      }
    }
  }
  if constexpr (DOT) {
    double vd[VC];
#pragma unroll
    for (int j = 0; j < VC; j++) vd[j] = (double)v[j];
    double tot;
    if (!column_reduce_v<W, VC>(vd, partials, counter, tot)) return;
    if (threadIdx.x < W) {
      ColScalars &s = cols[threadIdx.x];
      if (!s.done) {
        s.pq = tot;
        s.alpha = tot != 0.0 ? s.d / tot : 0.0;  // p = 0: no step
      }
    }
  }
}

// ------------------------------------------------------------ FP64 block PCG

// x = 0, r = b, p = M b, d = (b, M b), conv = tol sqrt|d| per column.
template <int W>
__global__ void __launch_bounds__(kThreads)
bpcg_start_kernel(int n, const double *__restrict__ b, const double *__restrict__ m,
                  double *__restrict__ x, double *__restrict__ r, double *__restrict__ p,
                  ColScalars *cols, BlockHeader *hdr, double *partials, unsigned int *counter) {
  double v = 0.0;
  const size_t nw = (size_t)n * W;
  for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nw;
       q += (size_t)gridDim.x * kThreads) {
    const double bi = b[q], zi = bi * m[q / W];
    x[q] = 0.0;
    r[q] = bi;
    p[q] = zi;
    v += bi * zi;
  }
  double tot;
  if (!column_reduce<W>(v, partials, counter, tot)) return;
  if (threadIdx.x < W) {
    ColScalars &s = cols[threadIdx.x];
    s = ColScalars{};
    s.d = tot;
    s.bmb = tot;
    s.conv = hdr->tol * sqrt(fabs(tot));
    s.rmax = sqrt(fabs(tot));
    if (tot == 0.0) s.done = 1;  // b_c = 0: x_c = 0
    if (hdr->maxit <= 0 && !s.done) {
      s.done = 1;
      s.status = ELX_ERR_NO_CONVERGENCE;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int act = 0;
    for (int c = 0; c < W; c++) act += cols[c].done ? 0 : 1;
    hdr->active = act;
    hdr->any_update = 0;
  }
}

// x += alpha p, r -= alpha q, d' = (r, M r), beta = d'/d; per-column stop.
template <int W>
__global__ void __launch_bounds__(kThreads)
bpcg_update_kernel(int n, const double *__restrict__ p, const double *__restrict__ qv,
                   const double *__restrict__ m, double *__restrict__ x, double *__restrict__ r,
                   ColScalars *cols, BlockHeader *hdr, double *partials, unsigned int *counter) {
  if (hdr->active == 0) return;
  const int c = threadIdx.x % W;
  const bool on = !cols[c].done;
  const double alpha = cols[c].alpha;
  double v = 0.0;
  const size_t nw = (size_t)n * W;
  if (on)
    for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nw;
         q += (size_t)gridDim.x * kThreads) {
      x[q] += alpha * p[q];
      const double ri = r[q] - alpha * qv[q];
      r[q] = ri;
      v += ri * (ri * m[q / W]);
    }
  double tot;
  if (!column_reduce<W>(v, partials, counter, tot)) return;
  if (threadIdx.x < W) {
    ColScalars &s = cols[threadIdx.x];
    if (!s.done) {
      s.iters += 1;
      s.beta = s.d != 0.0 ? tot / s.d : 0.0;
      s.d = tot;
      if (sqrt(fabs(tot)) < s.conv) {
        s.done = 1;
      } else if (s.iters >= hdr->maxit || !(tot == tot)) {
        s.done = 1;
        s.status = ELX_ERR_NO_CONVERGENCE;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int act = 0;
    for (int k = 0; k < W; k++) act += cols[k].done ? 0 : 1;
    hdr->active = act;
  }
}

// p = M r + beta p for the active columns.
template <class T, int W>
__global__ void __launch_bounds__(kThreads)
bpcg_direction_kernel(int n, const T *__restrict__ r, const T *__restrict__ m,
                      T *__restrict__ p, const ColScalars *cols, const BlockHeader *hdr) {
  if (hdr->active == 0) return;
  const int c = threadIdx.x % W;
  if (cols[c].done) return;
  const T beta = (T)cols[c].beta;
  const size_t nw = (size_t)n * W;
  for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nw;
       q += (size_t)gridDim.x * kThreads)
    p[q] = r[q] * m[q / W] + beta * p[q];
}

// ------------------------------------------------------------ mixed block PCG

// x_hi = 0, x_lo = 0, r = (float) b, p = M r, d = (r, M r) and
// (b, M b) in FP64, conv = tol sqrt|(b, M b)|.
template <int W>
__global__ void __launch_bounds__(kThreads)
brel_start_kernel(int n, const double *__restrict__ b, const double *__restrict__ m,
                  const float *__restrict__ m32, double *__restrict__ xhi,
                  float *__restrict__ xlo, float *__restrict__ r, float *__restrict__ p,
                  ColScalars *cols, BlockHeader *hdr, double *partials, unsigned int *counter) {
  double v0 = 0.0, v1 = 0.0;
  const size_t nw = (size_t)n * W;
  for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nw;
       q += (size_t)gridDim.x * kThreads) {
    const double bi = b[q];
    const float ri = (float)bi;
    xhi[q] = 0.0;
    xlo[q] = 0.0f;
    r[q] = ri;
    p[q] = ri * m32[q / W];
    v0 += bi * (bi * m[q / W]);
    v1 += (double)ri * (double)(ri * m32[q / W]);
  }
  double bmb, d;
  if (!column_reduce2<W>(v0, v1, partials, counter, bmb, d)) return;
  if (threadIdx.x < W) {
    ColScalars &s = cols[threadIdx.x];
    s = ColScalars{};
    s.bmb = bmb;
    s.d = d;
    s.conv = hdr->tol * sqrt(fabs(bmb));
    s.rmax = sqrt(fabs(d));
    s.best = sqrt(fabs(bmb));
    if (bmb == 0.0) s.done = 1;
    if (hdr->maxit <= 0 && !s.done) {
      s.done = 1;
      s.status = ELX_ERR_NO_CONVERGENCE;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int act = 0;
    for (int c = 0; c < W; c++) act += cols[c].done ? 0 : 1;
    hdr->active = act;
    hdr->any_update = 0;
  }
}

// FP32 step: x_lo += alpha p, r -= alpha q, d' = (r, M r); beta; flag a
// replacement when ||r||_M < delta rmax, < conv, or at maxit.  Each thread
// takes VC consecutive columns of a row (16-byte accesses).
template <int W>
__global__ void __launch_bounds__(kThreads)
brel_update_kernel(int n, const float *__restrict__ p, const float *__restrict__ qv,
                   const float *__restrict__ m32, float *__restrict__ xlo,
                   float *__restrict__ r, ColScalars *cols, BlockHeader *hdr,
                   double *partials, unsigned int *counter) {
  constexpr int VC = W < 4 ? W : 4;
  constexpr int G = W / VC;
  if (hdr->active == 0) return;
  const int c0 = (threadIdx.x % G) * VC;
  bool on[VC];
  float alpha[VC], v[VC];
#pragma unroll
  for (int j = 0; j < VC; j++) {
    on[j] = !cols[c0 + j].done;
    alpha[j] = on[j] ? (float)cols[c0 + j].alpha : 0.0f;
    v[j] = 0.0f;
  }
  bool any = false;
#pragma unroll
  for (int j = 0; j < VC; j++) any = any || on[j];
  const size_t ng = (size_t)n * G;
  if (any)
    for (size_t t = (size_t)blockIdx.x * kThreads + threadIdx.x; t < ng;
         t += (size_t)gridDim.x * kThreads) {
      const size_t row = t / G, q = row * W + c0;
      const float mi = m32[row];
      ColVec<float, VC> pv = load_cols<float, VC>(p + q), qq = load_cols<float, VC>(qv + q);
      ColVec<float, VC> xv = load_cols<float, VC>(xlo + q), rv = load_cols<float, VC>(r + q);
#pragma unroll
      for (int j = 0; j < VC; j++) {
        xv.v[j] += alpha[j] * pv.v[j];
        rv.v[j] -= alpha[j] * qq.v[j];
        v[j] += rv.v[j] * (rv.v[j] * mi);
      }
      store_cols<float, VC>(xlo + q, xv);
      store_cols<float, VC>(r + q, rv);
    }
  double vd[VC];
#pragma unroll
  for (int j = 0; j < VC; j++) vd[j] = (double)v[j];
  double tot;
  if (!column_reduce_v<W, VC>(vd, partials, counter, tot)) return;
  if (threadIdx.x < W) {
    ColScalars &s = cols[threadIdx.x];
    if (!s.done) {
      s.iters += 1;
      if (!(tot == tot) || isinf(tot)) {
        // the FP32 recurrence broke down: this column is solved in FP64
        s.done = 1;
        s.status = ELX_ERR_NO_CONVERGENCE;
        s.failed = 1;
      } else {
        const double rn = sqrt(fabs(tot));
        s.beta = s.d != 0.0 ? tot / s.d : 0.0;
        s.d = tot;
        if (rn < hdr->delta * s.rmax || rn < s.conv || s.iters >= hdr->maxit ||
            s.iters - s.last_rep >= kMixedCheckEvery || rn > kMixedDiverge * s.rmax) {
          s.update = 1;
          hdr->any_update = 1;
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int act = 0;
    for (int k = 0; k < W; k++) act += cols[k].done ? 0 : 1;
    hdr->active = act;
  }
}

// At a replacement point where some column asked for one, for every active
// column (one full-width FP64 product costs least per column, and replacing
// a column early does not hurt it): x_hi += x_lo, x_lo = 0.
template <int W>
__global__ void __launch_bounds__(kThreads)
brel_accumulate_kernel(int n, double *__restrict__ xhi, float *__restrict__ xlo,
                       const ColScalars *cols, const BlockHeader *hdr) {
  if (hdr->active == 0 || !hdr->any_update) return;
  const int c = threadIdx.x % W;
  if (cols[c].done) return;
  const size_t nw = (size_t)n * W;
  for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nw;
       q += (size_t)gridDim.x * kThreads) {
    xhi[q] += (double)xlo[q];
    xlo[q] = 0.0f;
  }
}

// For the active columns (z = K x_hi in FP64): r = (float)(b - z),
// rho = (b - z, M (b - z)) in FP64; stop on the reference's test, else go on
// from the replaced residual.
template <int W>
__global__ void __launch_bounds__(kThreads)
brel_residual_kernel(int n, const double *__restrict__ b, const double *__restrict__ z,
                     const double *__restrict__ m, float *__restrict__ r, ColScalars *cols,
                     BlockHeader *hdr, double *partials, unsigned int *counter) {
  if (hdr->active == 0 || !hdr->any_update) return;
  const int c = threadIdx.x % W;
  const bool on = !cols[c].done;
  double v = 0.0;
  const size_t nw = (size_t)n * W;
  if (on)
    for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nw;
         q += (size_t)gridDim.x * kThreads) {
      const double ri = b[q] - z[q];
      r[q] = (float)ri;
      v += ri * (ri * m[q / W]);
    }
  double tot;
  if (!column_reduce<W>(v, partials, counter, tot)) return;
  if (threadIdx.x < W) {
    ColScalars &s = cols[threadIdx.x];
    if (!s.done) {
      // a column replaced with the others (not by its own request) is not
      // held to the halving test, only to the divergence test
      const bool own = s.update != 0;
      const double rt = sqrt(fabs(tot));
      s.update = 0;
      s.nupdates += 1;
      if (own) s.last_rep = s.iters;
      if (rt < s.conv) {
        s.done = 1;
      } else if (!(tot == tot) || rt > kMixedDiverge * s.best) {
        s.done = 1;
        s.status = ELX_ERR_NO_CONVERGENCE;
        s.failed = 1;
      } else if (s.iters >= hdr->maxit) {
        s.done = 1;
        s.status = ELX_ERR_NO_CONVERGENCE;
      } else {
        if (own) s.stall = rt < 0.5 * s.best ? 0 : s.stall + 1;
        s.best = fmin(s.best, rt);
        if (s.stall >= kMixedStall) {
          s.done = 1;
          s.status = ELX_ERR_NO_CONVERGENCE;
          s.failed = 1;
        }
        s.d = tot;
        s.rmax = rt;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int act = 0;
    for (int k = 0; k < W; k++) act += cols[k].done ? 0 : 1;
    hdr->active = act;
    hdr->any_update = 0;
  }
}

// Post-solve diagnostics per column (Iters.f:433-458) from z = K x:
// xKx, ||x||^2, ||b - Kx||_M^2, ||b - Kx||^2 into out[4 c + 0..3] (two
// kernels, two sums each).
template <int W>
__global__ void __launch_bounds__(kThreads)
bdiag_kernel(int n, const double *__restrict__ x, const double *__restrict__ z, double *out,
             double *partials, unsigned int *counter) {
  double v0 = 0, v1 = 0;
  const size_t nw = (size_t)n * W;
  for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nw;
       q += (size_t)gridDim.x * kThreads) {
    const double xi = x[q];
    v0 += xi * z[q];
    v1 += xi * xi;
  }
  double t0, t1;
  if (!column_reduce2<W>(v0, v1, partials, counter, t0, t1)) return;
  if (threadIdx.x < W) {
    out[4 * threadIdx.x + 0] = t0;
    out[4 * threadIdx.x + 1] = t1;
  }
}

template <int W>
__global__ void __launch_bounds__(kThreads)
bdiag_res_kernel(int n, const double *__restrict__ z, const double *__restrict__ b,
                 const double *__restrict__ m, double *out, double *partials,
                 unsigned int *counter) {
  double v2 = 0, v3 = 0;
  const size_t nw = (size_t)n * W;
  for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nw;
       q += (size_t)gridDim.x * kThreads) {
    const double ri = b[q] - z[q];
    v2 += ri * (ri * m[q / W]);
    v3 += ri * ri;
  }
  double t2, t3;
  if (!column_reduce2<W>(v2, v3, partials, counter, t2, t3)) return;
  if (threadIdx.x < W) {
    out[4 * threadIdx.x + 2] = t2;
    out[4 * threadIdx.x + 3] = t3;
  }
}

// Column-major (caller) <-> row-interleaved (device) copies of W columns.
template <class T>
__global__ void interleave_kernel(int n, int w, const double *__restrict__ colmajor,
                                  T *__restrict__ inter) {
  const size_t nw = (size_t)n * w;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nw;
       q += (size_t)gridDim.x * blockDim.x) {
    const size_t row = q / w, c = q % w;
    inter[q] = (T)colmajor[c * n + row];
  }
}

__global__ void deinterleave_kernel(int n, int w, const double *__restrict__ inter,
                                    double *__restrict__ colmajor) {
  const size_t nw = (size_t)n * w;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nw;
       q += (size_t)gridDim.x * blockDim.x) {
    const size_t c = q / n, row = q % n;
    colmajor[q] = inter[row * w + c];
  }
}

int bgrid(size_t nw) {
  const size_t g = (nw + kThreads - 1) / kThreads;
  // multi-vectors of W columns keep eight blocks per SM busy (29.9 / 31.6 /
  // 37.6 ms per load case at 8 / 4 / 2 blocks per SM, 96x96x48 plate)
  return (int)std::max<size_t>(1, std::min<size_t>(g, (size_t)grid_cap(8)));
}

// Y = K X on the sliced copy of precision T: one CTA pass per SPC slices,
// at most the context's grid bound (the partial sums of the dots hold one
// row per CTA).
template <class T, int W>
void spmm_w(const CsrcDev &k, const T *X, T *Y, ColScalars *cols, BlockHeader *hdr,
            double *partials, unsigned int *counter, const int32_t *gate, bool dot,
            cudaStream_t st) {
  constexpr int VC = (16 / (int)sizeof(T)) < W ? (16 / (int)sizeof(T)) : W;
  constexpr int SPC = kThreads / (kSliceRows * (W / VC));
  const T *val;
  bool ld;
  if constexpr (sizeof(T) == 4) {
    val = k.sell_val;
    ld = k.sell_stream;
  } else {
    val = k.sell_val64;
    ld = k.sell64_stream;
  }
  ELX_REQUIRE(val != nullptr && k.sell_ptr != nullptr, ELX_ERR_STATE,
              "sliced node blocks missing for the block product");
  const bool d16 = k.sell_d16 != nullptr;
  const int grid = std::max(1, std::min((k.nslices + SPC - 1) / SPC, k.max_grid));
  // slot groups of matrix loads per step: ELX_SPMM_UNROLL, else the
  // autotuner's choice for this width, else three in FP32 and one in FP64
  // (FP64-pipe bound)
  constexpr int wi = W == 1 ? 0 : W == 2 ? 1 : W == 4 ? 2 : W == 8 ? 3 : 4;
  const int tuned = sizeof(T) == 4 ? k.spmm_unroll_w32[wi] : k.spmm_unroll_w64[wi];
  const int u = k.spmm_unroll > 0 ? k.spmm_unroll : tuned > 0 ? tuned : (sizeof(T) == 4 ? 3 : 1);
#define ELX_SPMM(B_, DOT_, U_, LD_, D16_)                                                  \
  do {                                                                                      \
    sell_spmm_kernel<T, B_, W, DOT_, false, U_, LD_, D16_><<<grid, kThreads, 0, st>>>(      \
        k.nb, k.nslices, k.sell_ptr, k.sell_col, k.sell_d16, val, X, Y, cols, hdr, partials, \
        counter, gate);                                                                     \
  } while (0)
#define ELX_SPMM_LD(B_, DOT_, U_)           \
  if (ld && d16)                            \
    ELX_SPMM(B_, DOT_, U_, true, true);     \
  else if (ld)                              \
    ELX_SPMM(B_, DOT_, U_, true, false);    \
  else if (d16)                             \
    ELX_SPMM(B_, DOT_, U_, false, true);    \
  else                                      \
    ELX_SPMM(B_, DOT_, U_, false, false)
  if (k.bsize == 3) {
    if (dot) {
      if (u >= 3)
        ELX_SPMM_LD(3, true, 3);
      else if (u == 2)
        ELX_SPMM_LD(3, true, 2);
      else
        ELX_SPMM_LD(3, true, 1);
    } else {
      if (u >= 3)
        ELX_SPMM_LD(3, false, 3);
      else
        ELX_SPMM_LD(3, false, 1);
    }
  } else {
    if (dot)
      ELX_SPMM_LD(2, true, 2);
    else
      ELX_SPMM_LD(2, false, 2);
  }
#undef ELX_SPMM_LD
#undef ELX_SPMM
}

template <int W>
void iteration_w(const CsrcDev &k, const BlockVecs &v, bool mixed, bool replacement_point,
                 cudaStream_t st) {
  const int n = k.neq;
  const int g = bgrid((size_t)n * W);
  unsigned int *cnt = v.counters;
  if (!mixed) {
    spmm_w<double, W>(k, v.p, v.q, v.cols, v.hdr, v.partials, cnt + 0, nullptr, true, st);
    bpcg_update_kernel<W><<<g, kThreads, 0, st>>>(n, v.p, v.q, v.m, v.x, v.r, v.cols, v.hdr,
                                                  v.partials, cnt + 1);
    bpcg_direction_kernel<double, W><<<g, kThreads, 0, st>>>(n, v.r, v.m, v.p, v.cols, v.hdr);
  } else {
    spmm_w<float, W>(k, v.p32, v.q32, v.cols, v.hdr, v.partials, cnt + 0, nullptr, true,
                     st);
    brel_update_kernel<W><<<g, kThreads, 0, st>>>(n, v.p32, v.q32, v.m32, v.xlo, v.r32, v.cols,
                                                  v.hdr, v.partials, cnt + 1);
    bpcg_direction_kernel<float, W><<<g, kThreads, 0, st>>>(n, v.r32, v.m32, v.p32, v.cols,
                                                            v.hdr);
    if (replacement_point) {
      brel_accumulate_kernel<W><<<g, kThreads, 0, st>>>(n, v.x, v.xlo, v.cols, v.hdr);
      spmm_w<double, W>(k, v.x, v.z, v.cols, v.hdr, v.partials, cnt + 2,
                        &v.hdr->any_update, false, st);
      brel_residual_kernel<W><<<g, kThreads, 0, st>>>(n, v.b, v.z, v.m, v.r32, v.cols, v.hdr,
                                                      v.partials, cnt + 3);
    }
  }
  ELX_CUDA(cudaGetLastError());
}

template <int W>
void start_w(const CsrcDev &k, const BlockVecs &v, bool mixed, cudaStream_t st) {
  const int n = k.neq;
  const int g = bgrid((size_t)n * W);
  if (mixed)
    brel_start_kernel<W><<<g, kThreads, 0, st>>>(n, v.b, v.m, v.m32, v.x, v.xlo, v.r32, v.p32,
                                                 v.cols, v.hdr, v.partials, v.counters + 4);
  else
    bpcg_start_kernel<W><<<g, kThreads, 0, st>>>(n, v.b, v.m, v.x, v.r, v.p, v.cols, v.hdr,
                                                 v.partials, v.counters + 4);
  ELX_CUDA(cudaGetLastError());
}

template <int W>
void diag_w(const CsrcDev &k, const BlockVecs &v, double *out, cudaStream_t st) {
  const int n = k.neq;
  const int g = bgrid((size_t)n * W);
  // z = K x with the gate open (active may be 0 after the solve)
  spmm_w<double, W>(k, v.x, v.z, v.cols, v.hdr_on, v.partials, v.counters + 5, nullptr,
                    false, st);
  bdiag_kernel<W><<<g, kThreads, 0, st>>>(n, v.x, v.z, out, v.partials, v.counters + 5);
  bdiag_res_kernel<W><<<g, kThreads, 0, st>>>(n, v.z, v.b, v.m, out, v.partials,
                                              v.counters + 5);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace

bool block_width_supported(int w) { return w == 1 || w == 2 || w == 4 || w == 8 || w == 16; }

#define ELX_W_DISPATCH(w, call) \
  switch (w) {                  \
    case 1: call(1); break;     \
    case 2: call(2); break;     \
    case 4: call(4); break;     \
    case 8: call(8); break;     \
    case 16: call(16); break;   \
    default: throw Error{ELX_ERR_ARG, "unsupported block width"}; \
  }

void launch_block_start(const CsrcDev &k, const BlockVecs &v, bool mixed, cudaStream_t st) {
#define CALL(W) start_w<W>(k, v, mixed, st)
  ELX_W_DISPATCH(v.w, CALL)
#undef CALL
}

void launch_block_iteration(const CsrcDev &k, const BlockVecs &v, bool mixed,
                            bool replacement_point, cudaStream_t st) {
#define CALL(W) iteration_w<W>(k, v, mixed, replacement_point, st)
  ELX_W_DISPATCH(v.w, CALL)
#undef CALL
}

void launch_block_diagnostics(const CsrcDev &k, const BlockVecs &v, double *out,
                              cudaStream_t st) {
#define CALL(W) diag_w<W>(k, v, out, st)
  ELX_W_DISPATCH(v.w, CALL)
#undef CALL
}

// The autotuner's products: the solver's own form (with the fused (p, q)
// dots), on the block vectors before the solve initialises its scalars.
void launch_spmm32(const CsrcDev &k, const BlockVecs &v, cudaStream_t st) {
#define CALL(W)                                                                                \
  spmm_w<float, W>(k, v.p32, v.q32, v.cols, v.hdr_on, v.partials, v.counters + 6, \
                   nullptr, true, st)
  ELX_W_DISPATCH(v.w, CALL)
#undef CALL
  ELX_CUDA(cudaGetLastError());
}

void launch_spmm64(const CsrcDev &k, const BlockVecs &v, cudaStream_t st) {
#define CALL(W)                                                                            \
  spmm_w<double, W>(k, v.p, v.q, v.cols, v.hdr_on, v.partials, v.counters + 6, \
                    nullptr, true, st)
  ELX_W_DISPATCH(v.w, CALL)
#undef CALL
  ELX_CUDA(cudaGetLastError());
}

void launch_interleave(int n, int w, const double *colmajor, double *inter, cudaStream_t st) {
  interleave_kernel<double><<<bgrid((size_t)n * w), kThreads, 0, st>>>(n, w, colmajor, inter);
  ELX_CUDA(cudaGetLastError());
}

void launch_deinterleave(int n, int w, const double *inter, double *colmajor, cudaStream_t st) {
  deinterleave_kernel<<<bgrid((size_t)n * w), kThreads, 0, st>>>(n, w, inter, colmajor);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace elx
