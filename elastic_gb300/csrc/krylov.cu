// Jacobi-preconditioned CG on the GPU (pcg, mef/src/Iters.f:252-524, with
// the diagonal preconditioner of Solv.f:65-69 / Precond.f:22-45), and its
// mixed-precision form: FP32 inner PCG inside FP64 iterative refinement.
//
// One PCG iteration is three kernels that keep every scalar on the device,
// so the host never waits inside the loop:
//   1. q = K p (spmv.cu) fused with the dot (p, q); the last block to finish
//      computes alpha = d / (p, q)                            (Iters.f:366-372)
//   2. x += alpha p, r -= alpha q, z = M r (not stored) fused with (r, z);
//      the last block computes beta, d and the stopping test
//      sqrt|d| < tol * ||b||_M                                (Iters.f:377-419)
//   3. p = M r + beta p                                       (Iters.f:411-414)
// Every kernel returns at once when the stopping flag is set, so the host can
// enqueue iterations in batches (captured once as a CUDA graph) and read the
// flag between batches.  Vectors are T = double or float; scalars and dot
// products are always accumulated in double.  Reductions are two-level with a
// fixed grid (elx_reduce.cuh), so results are deterministic.
//
// Mixed precision (rel_* kernels below): FP32 CG with reliable updates.  The
// FP32 iteration (FP32 SpMV, update, direction) carries the recurrence; the
// solution is accumulated in FP64 (x_hi += x_lo at each replacement), and
// whenever the FP32 residual has dropped tenfold since the last replacement
// (checked every few iterations) it is replaced by the FP64 residual
// b - K x_hi; the stopping test is the reference's ||r||_M < tol ||b||_M on
// that FP64 residual.
#include <atomic>
#include <cstdlib>

#include "elx_krylov.h"
#include "elx_reduce.cuh"

namespace elx {
namespace {

// 16-byte vector of T: the vector kernels stream 16 bytes per load.
template <class T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int W = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int W = 2;
};

// ------------------------------------------------------------ kernels
__global__ void __launch_bounds__(kThreads)
diag_inverse_kernel(int n, const double *__restrict__ ad, double *__restrict__ m,
                    float *__restrict__ m32, int32_t *zero_row) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double a = ad[i];
    if (a == 0.0) atomicMin(zero_row, i + 1);
    const double mi = 1.0 / a;
    m[i] = mi;
    if (m32) m32[i] = (float)mi;
  }
}

// x = 0, r = b, p = M b and d = (b, M b); conv = tol * sqrt|d| (Iters.f:343-360
// with x0 = 0, for which K x0 = 0 and r0 = b exactly).
template <class T>
__global__ void __launch_bounds__(kThreads)
pcg_start_kernel(int n, const T *__restrict__ b, const T *__restrict__ m, T *__restrict__ x,
                 T *__restrict__ r, T *__restrict__ p, PcgScalars *sc, double *partials,
                 unsigned int *counter) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const T bi = b[i], zi = bi * m[i];
    x[i] = T(0);
    r[i] = bi;
    p[i] = zi;
    v[0] += (double)bi * (double)zi;
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    sc->d = tot[0];
    sc->bmb = tot[0];
    sc->conv = sc->tol * sqrt(fabs(tot[0]));
    sc->iters = 0;
    sc->status = 0;
    // b = 0: x = 0 is exact; the reference would divide 0 by 0 here.
    sc->done = (tot[0] == 0.0 || sc->maxit <= 0) ? 1 : 0;
    if (sc->maxit <= 0 && tot[0] != 0.0) sc->status = ELX_ERR_NO_CONVERGENCE;
  }
}

// Second launch of the tiled SpMV (spmv.cu): y(i) = ytile(i) + its halo slots
// in tile order, in place.  With sc != nullptr it also forms (p, y) and
// alpha = d / (p, y) for the PCG (Iters.f:366-372).
__global__ void __launch_bounds__(kThreads)
halo_dot_kernel(int neq, const int32_t *__restrict__ halo_ptr,
                const int32_t *__restrict__ halo_slot, const double *__restrict__ part,
                const double *__restrict__ p, double *__restrict__ y, PcgScalars *sc,
                double *partials, unsigned int *counter) {
  if (sc && sc->done) return;
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < neq; i += gridDim.x * kThreads) {
    double yi = y[i];
    for (int h = halo_ptr[i]; h < halo_ptr[i + 1]; h++) yi += part[halo_slot[h]];
    y[i] = yi;
    if (sc) v[0] += p[i] * yi;
  }
  if (!sc) return;
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    sc->pq = tot[0];
    sc->alpha = tot[0] != 0.0 ? sc->d / tot[0] : 0.0;  // p = 0: no step
  }
}

// x += alpha p; r -= alpha q; (r, M r); beta, d, stopping test.
// 16-byte vector loads; the tail of n % W elements is done element-wise.
template <class T>
__global__ void __launch_bounds__(kThreads)
pcg_update_kernel(int n, const T *__restrict__ p, const T *__restrict__ q,
                  const T *__restrict__ m, T *__restrict__ x, T *__restrict__ r,
                  PcgScalars *sc, double *partials, unsigned int *counter) {
  if (sc->done) return;
  using VT = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::W;
  const T alpha = (T)sc->alpha;
  double v[1] = {0.0};
  const int stride = gridDim.x * kThreads, t0 = blockIdx.x * kThreads + threadIdx.x;
  const int nv = n / W;
  for (int iv = t0; iv < nv; iv += stride) {
    VT pv = reinterpret_cast<const VT *>(p)[iv], qv = reinterpret_cast<const VT *>(q)[iv];
    VT mv = reinterpret_cast<const VT *>(m)[iv], xv = reinterpret_cast<VT *>(x)[iv];
    VT rv = reinterpret_cast<VT *>(r)[iv];
    const T *pe = reinterpret_cast<const T *>(&pv), *qe = reinterpret_cast<const T *>(&qv);
    const T *me = reinterpret_cast<const T *>(&mv);
    T *xe = reinterpret_cast<T *>(&xv), *re = reinterpret_cast<T *>(&rv);
#pragma unroll
    for (int c = 0; c < W; c++) {
      xe[c] += alpha * pe[c];
      re[c] = re[c] - alpha * qe[c];
      v[0] += (double)re[c] * (double)(re[c] * me[c]);
    }
    reinterpret_cast<VT *>(x)[iv] = xv;
    reinterpret_cast<VT *>(r)[iv] = rv;
  }
  for (int i = nv * W + t0; i < n; i += stride) {
    x[i] += alpha * p[i];
    const T ri = r[i] - alpha * q[i];
    r[i] = ri;
    v[0] += (double)ri * (double)(ri * m[i]);
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    const double di = tot[0];
    sc->beta = di / sc->d;
    sc->d = di;
    const int it = sc->iters + 1;
    sc->iters = it;
    if (sqrt(fabs(di)) < sc->conv) {
      sc->done = 1;
    } else if (it >= sc->maxit || !(di == di)) {
      sc->done = 1;
      sc->status = ELX_ERR_NO_CONVERGENCE;
    }
  }
}

// p = M r + beta p (16-byte vector loads).
template <class T>
__global__ void __launch_bounds__(kThreads)
pcg_direction_kernel(int n, const T *__restrict__ r, const T *__restrict__ m, T *__restrict__ p,
                     const PcgScalars *sc) {
  if (sc->done) return;
  using VT = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::W;
  const T beta = (T)sc->beta;
  const int stride = gridDim.x * kThreads, t0 = blockIdx.x * kThreads + threadIdx.x;
  const int nv = n / W;
  for (int iv = t0; iv < nv; iv += stride) {
    VT rv = reinterpret_cast<const VT *>(r)[iv], mv = reinterpret_cast<const VT *>(m)[iv];
    VT pv = reinterpret_cast<VT *>(p)[iv];
    const T *re = reinterpret_cast<const T *>(&rv), *me = reinterpret_cast<const T *>(&mv);
    T *pe = reinterpret_cast<T *>(&pv);
#pragma unroll
    for (int c = 0; c < W; c++) pe[c] = re[c] * me[c] + beta * pe[c];
    reinterpret_cast<VT *>(p)[iv] = pv;
  }
  for (int i = nv * W + t0; i < n; i += stride) p[i] = r[i] * m[i] + beta * p[i];
}

// Post-solve diagnostics (Iters.f:433-458): z = K x is given; r = b - z;
// xKx = (x, z), ||x||^2, (r, M r), (r, r).
__global__ void __launch_bounds__(kThreads)
diagnostics_kernel(int n, const double *__restrict__ x, const double *__restrict__ z,
                   const double *__restrict__ b, const double *__restrict__ m,
                   double *out, double *partials, unsigned int *counter) {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double xi = x[i], zi = z[i], ri = b[i] - zi;
    v[0] += xi * zi;
    v[1] += xi * xi;
    v[2] += ri * (ri * m[i]);
    v[3] += ri * ri;
  }
  block_sum<4>(v);
  if (!publish_partials<4>(v, partials, counter)) return;
  double tot[4];
  gather_partials<4>(tot, partials, counter);
  if (threadIdx.x == 0)
    for (int i = 0; i < 4; i++) out[i] = tot[i];
}

// Refinement residual: r = b - z (z = K x in FP64), r32 = (float) r, and
// (r, M r) into out[0].  With z == nullptr (x = 0) r = b.
__global__ void __launch_bounds__(kThreads)
refine_residual_kernel(int n, const double *__restrict__ b, const double *__restrict__ z,
                       const double *__restrict__ m, double *__restrict__ r,
                       float *__restrict__ r32, double *out, double *partials,
                       unsigned int *counter) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double ri = z ? b[i] - z[i] : b[i];
    r[i] = ri;
    r32[i] = (float)ri;
    v[0] += ri * (ri * m[i]);
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) out[0] = tot[0];
}

__global__ void __launch_bounds__(kThreads)
convert_kernel(int n, const double *__restrict__ src, float *__restrict__ dst) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    dst[i] = (float)src[i];
}

__global__ void __launch_bounds__(kThreads)
widen_kernel(int n, const float *__restrict__ src, double *__restrict__ dst) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    dst[i] = (double)src[i];
}

// x += d (the FP32 correction), in FP64.
__global__ void __launch_bounds__(kThreads)
refine_accumulate_kernel(int n, double *__restrict__ x, const float *__restrict__ d, int first) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    x[i] = first ? (double)d[i] : x[i] + (double)d[i];
}

// ---------------------------------------------------- reliable updates
// Mixed-precision CG with reliable updates (residual replacement): one FP32
// CG whose search direction is never restarted; the FP32 solution piece xlo
// is folded into the FP64 solution and the FP32 residual replaced by the
// true FP64 residual b - K xhi whenever ||r||_M has dropped by delta since
// the last replacement, or looks converged.  The stopping test is the
// reference's, on the FP64 residual.

// x_lo = 0, p = M r, rho = (r, M r), rmax = sqrt(rho).  conv is set by the host
// from the FP64 (b, M b).
__global__ void __launch_bounds__(kThreads)
rel_start_kernel(int n, const float *__restrict__ r, const float *__restrict__ m,
                 float *__restrict__ xlo, float *__restrict__ p, PcgScalars *sc,
                 double *partials, unsigned int *counter) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const float ri = r[i], zi = ri * m[i];
    xlo[i] = 0.0f;
    p[i] = zi;
    v[0] += (double)ri * (double)zi;
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    sc->d = tot[0];
    sc->rmax = sqrt(fabs(tot[0]));
    sc->iters = 0;
    sc->status = 0;
    sc->update = 0;
    sc->nupdates = 0;
    sc->done = (sc->bmb == 0.0 || sc->maxit <= 0) ? 1 : 0;
    if (sc->maxit <= 0 && sc->bmb != 0.0) sc->status = ELX_ERR_NO_CONVERGENCE;
  }
}

// x_lo += alpha p; r -= alpha q; rho = (r, M r); beta; and the replacement
// flag when ||r||_M has dropped by delta since the last replacement, looks
// converged, or maxit is reached (rel_residual_kernel then decides, from the
// FP64 residual, at the next replacement point).
__global__ void __launch_bounds__(kThreads)
rel_update_kernel(int n, const float *__restrict__ p, const float *__restrict__ q,
                  const float *__restrict__ m, float *__restrict__ xlo, float *__restrict__ r,
                  PcgScalars *sc, double *partials, unsigned int *counter) {
  if (sc->done) return;
  const float alpha = (float)sc->alpha;
  float v[1] = {0.0f};  // widened to double per warp
  const int stride = gridDim.x * kThreads, t0 = blockIdx.x * kThreads + threadIdx.x;
  const int nv = n / 4;
  for (int iv = t0; iv < nv; iv += stride) {
    const float4 pv = reinterpret_cast<const float4 *>(p)[iv];
    const float4 qv = reinterpret_cast<const float4 *>(q)[iv];
    const float4 mv = reinterpret_cast<const float4 *>(m)[iv];
    float4 xv = reinterpret_cast<float4 *>(xlo)[iv];
    float4 rv = reinterpret_cast<float4 *>(r)[iv];
    xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
    rv.x -= alpha * qv.x; rv.y -= alpha * qv.y; rv.z -= alpha * qv.z; rv.w -= alpha * qv.w;
    v[0] += rv.x * (rv.x * mv.x) + rv.y * (rv.y * mv.y) + rv.z * (rv.z * mv.z) +
            rv.w * (rv.w * mv.w);
    reinterpret_cast<float4 *>(xlo)[iv] = xv;
    reinterpret_cast<float4 *>(r)[iv] = rv;
  }
  for (int i = nv * 4 + t0; i < n; i += stride) {
    xlo[i] += alpha * p[i];
    const float ri = r[i] - alpha * q[i];
    r[i] = ri;
    v[0] += ri * (ri * m[i]);
  }
  double vb[1];
  block_sum_widen<1>(v, vb);
  if (!publish_partials<1>(vb, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    const double di = tot[0];
    const int it = sc->iters + 1;
    sc->iters = it;
    const double rn = sqrt(fabs(di));
    if (!(di == di) || isinf(di)) {
      // the FP32 recurrence broke down (overflow): solve in FP64 instead
      sc->done = 1;
      sc->status = ELX_ERR_NO_CONVERGENCE;
      sc->failed = 1;
      return;
    }
    // an FP32 residual of exactly zero (a small system solved in FP32):
    // beta = 0, and the next replacement point takes over
    sc->beta = sc->d != 0.0 ? di / sc->d : 0.0;
    sc->d = di;
    // a residual growing past kMixedDiverge x the last replaced one asks for
    // a replacement too (whose progress watch then weighs it)
    if (rn < sc->delta * sc->rmax || rn < sc->conv || it >= sc->maxit ||
        it - sc->last_rep >= kMixedCheckEvery || rn > kMixedDiverge * sc->rmax)
      sc->update = 1;
  }
}

// When a replacement is due: x_hi += x_lo, x_lo = 0.
__global__ void __launch_bounds__(kThreads)
rel_accumulate_kernel(int n, double *__restrict__ xhi, float *__restrict__ xlo,
                      const PcgScalars *sc) {
  if (sc->done || !sc->update) return;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    xhi[i] += (double)xlo[i];
    xlo[i] = 0.0f;
  }
}

// When a replacement is due (z = K x_hi in FP64): r_hi = b - z, r = (float)
// r_hi, rho = (r_hi, M r_hi); stop on the reference's test, else continue
// (the search direction is kept; the next alpha uses the replaced rho).
__global__ void __launch_bounds__(kThreads)
rel_residual_kernel(int n, const double *__restrict__ b, const double *__restrict__ z,
                    const double *__restrict__ m, double *__restrict__ rhi,
                    float *__restrict__ r, PcgScalars *sc, double *partials,
                    unsigned int *counter) {
  if (sc->done || !sc->update) return;
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double ri = b[i] - z[i];
    rhi[i] = ri;
    r[i] = (float)ri;
    v[0] += ri * (ri * m[i]);
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    const double di = tot[0], rt = sqrt(fabs(di));
    sc->update = 0;
    sc->nupdates += 1;
    sc->last_rep = sc->iters;
    if (rt < sc->conv) {
      sc->done = 1;
    } else if (!(di == di) || rt > kMixedDiverge * sc->best) {
      sc->done = 1;
      sc->status = ELX_ERR_NO_CONVERGENCE;
      sc->failed = 1;
    } else if (sc->iters >= sc->maxit) {
      sc->done = 1;
      sc->status = ELX_ERR_NO_CONVERGENCE;
    } else {
      sc->stall = rt < 0.5 * sc->best ? 0 : sc->stall + 1;
      sc->best = fmin(sc->best, rt);
      if (sc->stall >= kMixedStall) {
        sc->done = 1;
        sc->status = ELX_ERR_NO_CONVERGENCE;
        sc->failed = 1;
      }
      sc->d = di;
      sc->rmax = rt;
    }
  }
}

}  // namespace

void launch_rel_start(int n, const float *r, const float *m, float *xlo, float *p,
                      PcgScalars *sc, double *partials, unsigned int *counter, cudaStream_t st) {
  rel_start_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, r, m, xlo, p, sc, partials, counter);
  ELX_CUDA(cudaGetLastError());
}

// One reliable-update iteration: the FP32 CG step (3 kernels), and at
// replacement points (every few iterations) three more kernels that run only
// when the replacement flag is set.
void launch_rel_iteration(const CsrcDev &k, const double *b, const double *m, double *xhi,
                          double *rhi, double *z, float *xlo, float *r, float *p, float *q,
                          const float *m32, PcgScalars *sc, double *partials,
                          unsigned int *counters, bool replacement_point, cudaStream_t st) {
  const int n = k.neq;
  launch_gather_spmv32(k, p, q, sc, partials, counters + 0, st);
  rel_update_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, p, q, m32, xlo, r, sc, partials,
                                                         counters + 1);
  pcg_direction_kernel<float><<<vector_grid(n), kThreads, 0, st>>>(n, r, m32, p, sc);
  if (replacement_point) {
    rel_accumulate_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, xhi, xlo, sc);
    launch_gather_spmv64(k, xhi, z, nullptr, nullptr, nullptr, st, &sc->update);
    rel_residual_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, b, z, m, rhi, r, sc, partials,
                                                             counters + 5);
  }
  ELX_CUDA(cudaGetLastError());
}

int sm_count() {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices];
  int dev = 0;
  ELX_CUDA(cudaGetDevice(&dev));
  const bool cached = dev >= 0 && dev < kMaxDevices;
  if (cached) {
    const int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
  }
  int n = 0;
  ELX_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  if (cached) cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

int vector_grid(int n) {
  // a fixed multiple of the SM count keeps the partial count small and fixed;
  // two blocks per SM beat eight: the last block's sum of the
  // partials is shorter and the streams stay full with grid-stride loops
  // (FP64 PCG 57.6 against 58.9 ms on the 64^3 HEXA8 cube, 121.5 against
  // 128.9 ms on the 48^3 TETRA4 mesh; one, 1.5, 3, 4 and 16 per SM no better)
  const int cap = grid_cap(2);
  int g = (n + kThreads - 1) / kThreads;
  return g < cap ? (g < 1 ? 1 : g) : cap;
}

void launch_diag_inverse(int n, const double *ad, double *m, float *m32, int32_t *zero_row,
                         cudaStream_t st) {
  diag_inverse_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, ad, m, m32, zero_row);
  ELX_CUDA(cudaGetLastError());
}

template <class T>
void launch_pcg_start(int n, const T *b, const T *m, T *x, T *r, T *p, PcgScalars *sc,
                      double *partials, unsigned int *counter, cudaStream_t st) {
  pcg_start_kernel<T><<<vector_grid(n), kThreads, 0, st>>>(n, b, m, x, r, p, sc, partials,
                                                           counter);
  ELX_CUDA(cudaGetLastError());
}
template void launch_pcg_start<double>(int, const double *, const double *, double *, double *,
                                       double *, PcgScalars *, double *, unsigned int *,
                                       cudaStream_t);
template void launch_pcg_start<float>(int, const float *, const float *, float *, float *,
                                      float *, PcgScalars *, double *, unsigned int *,
                                      cudaStream_t);

void launch_pcg_iteration(const CsrcDev &k, const TileDev &td, int spmv_kind, double *x,
                          double *r, double *p, double *q, double *part, const double *m,
                          PcgScalars *sc, double *partials, unsigned int *counters,
                          int32_t *err, cudaStream_t st) {
  const int n = k.neq;
  if (spmv_kind == kSpmvTiled) {
    launch_tile_spmv64(k, td, p, q, part, err, st, sc);
    halo_dot_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, td.halo_ptr, td.halo_slot, part, p,
                                                         q, sc, partials, counters + 0);
  } else {
    launch_gather_spmv64(k, p, q, sc, partials, counters + 0, st);
  }
  pcg_update_kernel<double><<<vector_grid(n), kThreads, 0, st>>>(n, p, q, m, x, r, sc, partials,
                                                                 counters + 1);
  pcg_direction_kernel<double><<<vector_grid(n), kThreads, 0, st>>>(n, r, m, p, sc);
  ELX_CUDA(cudaGetLastError());
}

void launch_pcg_iteration32(const CsrcDev &k, float *x, float *r, float *p, float *q,
                            const float *m, PcgScalars *sc, double *partials,
                            unsigned int *counters, cudaStream_t st) {
  const int n = k.neq;
  launch_gather_spmv32(k, p, q, sc, partials, counters + 0, st);
  pcg_update_kernel<float><<<vector_grid(n), kThreads, 0, st>>>(n, p, q, m, x, r, sc, partials,
                                                                counters + 1);
  pcg_direction_kernel<float><<<vector_grid(n), kThreads, 0, st>>>(n, r, m, p, sc);
  ELX_CUDA(cudaGetLastError());
}

// y = K x with the PCG's own SpMV launches (no dot).
void launch_spmv64(const CsrcDev &k, const TileDev &td, int spmv_kind, const double *x, double *y,
                   double *part, int32_t *err, cudaStream_t st) {
  if (spmv_kind == kSpmvTiled) {
    launch_tile_spmv64(k, td, x, y, part, err, st);
    halo_dot_kernel<<<vector_grid(k.neq), kThreads, 0, st>>>(k.neq, td.halo_ptr, td.halo_slot,
                                                              part, nullptr, y, nullptr, nullptr,
                                                              nullptr);
  } else {
    launch_gather_spmv64(k, x, y, nullptr, nullptr, nullptr, st);
  }
  ELX_CUDA(cudaGetLastError());
}

void launch_diagnostics(int n, const double *x, const double *z, const double *b,
                        const double *m, double *out, double *partials, unsigned int *counter,
                        cudaStream_t st) {
  diagnostics_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, x, z, b, m, out, partials, counter);
  ELX_CUDA(cudaGetLastError());
}

void launch_refine_residual(int n, const double *b, const double *z, const double *m, double *r,
                            float *r32, double *out, double *partials, unsigned int *counter,
                            cudaStream_t st) {
  refine_residual_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, b, z, m, r, r32, out, partials,
                                                              counter);
  ELX_CUDA(cudaGetLastError());
}

void launch_convert(int n, const double *src, float *dst, cudaStream_t st) {
  convert_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, src, dst);
  ELX_CUDA(cudaGetLastError());
}

void launch_widen(int n, const float *src, double *dst, cudaStream_t st) {
  widen_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, src, dst);
  ELX_CUDA(cudaGetLastError());
}

void launch_refine_accumulate(int n, double *x, const float *d, bool first, cudaStream_t st) {
  refine_accumulate_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, x, d, first ? 1 : 0);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace elx
