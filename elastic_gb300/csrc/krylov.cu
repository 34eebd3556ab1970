// Jacobi-preconditioned CG on the GPU (pcg, mef/src/Iters.f:252-524, with
// the diagonal preconditioner of Solv.f:65-69 / Precond.f:22-45).
//
// One iteration is four kernels that keep every scalar on the device, so the
// host never waits inside the loop:
//   1. q = K p: the pipelined single-read SpMV (spmv.cu), then its halo launch
//      fused with the dot (p, q); the last block to finish computes
//      alpha = d / (p, q)                                   (Iters.f:366-372)
//   2. x += alpha p, r -= alpha q, z = M r (not stored) fused with (r, z);
//      the last block computes beta, d and the stopping test
//      sqrt|d| < tol * ||b||_M                              (Iters.f:377-419)
//   3. p = M r + beta p                                     (Iters.f:411-414)
// Every kernel returns at once when the stopping flag is set, so the host can
// enqueue iterations in batches (captured once as a CUDA graph) and read the
// flag between batches.  Reductions are two-level with a fixed grid: each
// block reduces its threads in a fixed tree and the last block to arrive
// sums the block partials in a fixed order, so results are deterministic.
#include "elx_krylov.h"
#include "elx_reduce.cuh"

namespace elx {
namespace {

// ------------------------------------------------------------ kernels
__global__ void __launch_bounds__(kThreads)
diag_inverse_kernel(int n, const double *__restrict__ ad, double *__restrict__ m,
                    int32_t *zero_row) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double a = ad[i];
    if (a == 0.0) atomicMin(zero_row, i + 1);
    m[i] = 1.0 / a;
  }
}

// x = 0, r = b, p = M b and d = (b, M b); conv = tol * sqrt|d| (Iters.f:343-360
// with x0 = 0, for which K x0 = 0 and r0 = b exactly).
__global__ void __launch_bounds__(kThreads)
pcg_start_kernel(int n, const double *__restrict__ b, const double *__restrict__ m,
                 double *__restrict__ x, double *__restrict__ r, double *__restrict__ p,
                 PcgScalars *sc, double *partials, unsigned int *counter) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double bi = b[i], zi = bi * m[i];
    x[i] = 0.0;
    r[i] = bi;
    p[i] = zi;
    v[0] += bi * zi;
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

// Second launch of the SpMV (spmv.cu): y(i) = ytile(i) + its halo slots in
// tile order, in place.  With sc != nullptr it also forms (p, y) and
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
    sc->alpha = sc->d / tot[0];
  }
}

// x += alpha p; r -= alpha q; (r, M r); beta, d, stopping test.
__global__ void __launch_bounds__(kThreads)
pcg_update_kernel(int n, const double *__restrict__ p, const double *__restrict__ q,
                  const double *__restrict__ m, double *__restrict__ x,
                  double *__restrict__ r, PcgScalars *sc, double *partials,
                  unsigned int *counter) {
  if (sc->done) return;
  const double alpha = sc->alpha;
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    v[0] += ri * (ri * m[i]);
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

// p = M r + beta p.
__global__ void __launch_bounds__(kThreads)
pcg_direction_kernel(int n, const double *__restrict__ r, const double *__restrict__ m,
                     double *__restrict__ p, const PcgScalars *sc) {
  if (sc->done) return;
  const double beta = sc->beta;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    p[i] = r[i] * m[i] + beta * p[i];
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

}  // namespace

int vector_grid(int n) {
  // a fixed multiple of the SM count keeps the partial count small and fixed
  int g = (n + kThreads - 1) / kThreads;
  return g < 1216 ? (g < 1 ? 1 : g) : 1216;
}

void launch_diag_inverse(int n, const double *ad, double *m, int32_t *zero_row, cudaStream_t st) {
  diag_inverse_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, ad, m, zero_row);
  ELX_CUDA(cudaGetLastError());
}

void launch_pcg_start(int n, const double *b, const double *m, double *x, double *r, double *p,
                      PcgScalars *sc, double *partials, unsigned int *counter, cudaStream_t st) {
  pcg_start_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, b, m, x, r, p, sc, partials, counter);
  ELX_CUDA(cudaGetLastError());
}

void launch_pcg_iteration(const CsrcDev &k, const TileDev &td, int spmv_kind, double *x,
                          double *r, double *p, double *q, double *part, const double *m,
                          PcgScalars *sc, double *partials, unsigned int *counters,
                          int32_t *err, cudaStream_t st) {
  const int n = k.neq;
  if (spmv_kind == kSpmvTiled) {
    launch_tile_spmv64(k, td, p, q, part, err, st);
    halo_dot_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, td.halo_ptr, td.halo_slot, part, p,
                                                         q, sc, partials, counters + 0);
  } else {
    launch_gather_spmv64(k, p, q, sc, partials, counters + 0, st);
  }
  pcg_update_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, p, q, m, x, r, sc, partials,
                                                         counters + 1);
  pcg_direction_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, r, m, p, sc);
  ELX_CUDA(cudaGetLastError());
}

// y = K x with the PCG's own two SpMV launches (no dot).
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

}  // namespace elx
