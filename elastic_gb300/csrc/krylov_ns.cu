// The reference's two other Krylov solvers on the GPU primitives of the PCG:
//
//   * pbicgstab (mef/src/Iters.f:1079-1349): BiCGSTAB with right Jacobi
//     preconditioning (z = M p), stopping on the 2-norm ||r|| < tol ||b||,
//     tested after each half step.  Five kernels per iteration (two SpMVs
//     with fused dot epilogues, two update passes with fused reductions, one
//     direction pass), device-resident scalars, captured in batches.
//   * gmres (mef/src/Iters.f:528-808): GMRES(k) with left Jacobi
//     preconditioning, modified Gram-Schmidt, Givens rotations and a
//     back-substitution per restart cycle.  One restart cycle is one captured
//     graph: per Arnoldi step the SpMV (with the M scaling fused), one kernel
//     per Gram-Schmidt projection (each applies the previous projection and
//     forms the next dot, in the reference's order), one kernel for the last
//     projection + norm + rotations, one normalisation; then the
//     back-substitution (one thread: k is small) and x += sum y_j g_j.
//
// Every kernel returns at once when the solve (or, inside a GMRES cycle, the
// Arnoldi loop) has stopped, so a captured graph runs to its end harmlessly.
// All reductions are the deterministic two-level ones of elx_reduce.cuh.
#include <cmath>

#include "elx_krylov.h"
#include "elx_reduce.cuh"

namespace elx {
namespace {

// ---------------------------------------------------------------- BiCGSTAB

// Iters.f:1171-1197 with x0 = 0: r0 = r = p = b - K 0 = b, z = M p,
// d = (b, b), conv = tol sqrt|d|; the first (r, r0) is the same sum.
__global__ void __launch_bounds__(kThreads)
bicg_start_kernel(int n, const double *__restrict__ b, const double *__restrict__ m,
                  double *__restrict__ x, double *__restrict__ r, double *__restrict__ r0,
                  double *__restrict__ p, double *__restrict__ z, PcgScalars *sc,
                  double *partials, unsigned int *counter) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double bi = b[i];
    x[i] = 0.0;
    r[i] = bi;
    r0[i] = bi;
    p[i] = bi;
    z[i] = bi * m[i];
    v[0] += bi * bi;
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    sc->d = tot[0];
    sc->conv = sc->tol * sqrt(fabs(tot[0]));
    sc->rho = tot[0];
    sc->iters = 0;
    sc->status = ELX_OK;
    sc->done = 0;
    if (tot[0] == 0.0) {
      sc->done = 1;  // b = 0: x = 0 is the solution
    } else if (sc->maxit <= 0) {
      sc->done = 1;
      sc->status = ELX_ERR_NO_CONVERGENCE;
    }
  }
}

// First half step (Iters.f:1204-1228): x += alpha z, r -= alpha v, z = M r,
// d = (r, r); stop when sqrt|d| < conv.
__global__ void __launch_bounds__(kThreads)
bicg_half_kernel(int n, const double *__restrict__ v, const double *__restrict__ m,
                 double *__restrict__ x, double *__restrict__ r, double *__restrict__ z,
                 PcgScalars *sc, double *partials, unsigned int *counter) {
  if (sc->done) return;
  const double alpha = sc->alpha;
  double s[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    x[i] += alpha * z[i];
    const double ri = r[i] - alpha * v[i];
    r[i] = ri;
    z[i] = ri * m[i];
    s[0] += ri * ri;
  }
  block_sum<1>(s);
  if (!publish_partials<1>(s, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    sc->d = tot[0];
    if (sqrt(fabs(tot[0])) < sc->conv) {
      sc->done = 1;
    } else if (!(tot[0] == tot[0])) {
      sc->done = 1;
      sc->status = ELX_ERR_NO_CONVERGENCE;
    }
  }
}

// Second half step (Iters.f:1232-1257): x += omega z, r -= omega t,
// d = (r, r) and (r, r0); stop when sqrt|d| < conv, else
// beta = ((r, r0) / rho) (alpha / omega) and rho = (r, r0).
__global__ void __launch_bounds__(kThreads)
bicg_full_kernel(int n, const double *__restrict__ z, const double *__restrict__ t,
                 const double *__restrict__ r0, double *__restrict__ x, double *__restrict__ r,
                 PcgScalars *sc, double *partials, unsigned int *counter) {
  if (sc->done) return;
  const double omega = sc->omega;
  double s[2] = {0.0, 0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    x[i] += omega * z[i];
    const double ri = r[i] - omega * t[i];
    r[i] = ri;
    s[0] += ri * ri;
    s[1] += ri * r0[i];
  }
  block_sum<2>(s);
  if (!publish_partials<2>(s, partials, counter)) return;
  double tot[2];
  gather_partials<2>(tot, partials, counter);
  if (threadIdx.x == 0) {
    sc->d = tot[0];
    if (sqrt(fabs(tot[0])) < sc->conv) {
      sc->done = 1;
    } else if (sc->iters >= sc->maxit || !(tot[0] == tot[0])) {
      sc->done = 1;
      sc->status = ELX_ERR_NO_CONVERGENCE;
    } else {
      sc->beta = (tot[1] / sc->rho) * (sc->alpha / omega);
      sc->rho = tot[1];
    }
  }
}

// p = r + beta (p - omega v), z = M p (Iters.f:1261-1266).
__global__ void __launch_bounds__(kThreads)
bicg_direction_kernel(int n, const double *__restrict__ r, const double *__restrict__ v,
                      const double *__restrict__ m, double *__restrict__ p,
                      double *__restrict__ z, const PcgScalars *sc) {
  if (sc->done) return;
  const double beta = sc->beta, omega = sc->omega;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double pi = r[i] + beta * (p[i] - omega * v[i]);
    p[i] = pi;
    z[i] = pi * m[i];
  }
}

// ------------------------------------------------------------------ GMRES

// Small dense arrays of one GMRES(k) solve, 1-based like the reference:
// e(1..k+1), c(1..k), s(1..k), y(1..k), nrm(1..k+1) (the norms that
// normalise g_{i+1}) and the (k+1) x k Hessenberg matrix, column-major.
struct GmresArrays {
  double *e, *c, *s, *y, *nrm, *h;
  int k;
  __device__ double &H(int i, int j) const { return h[(size_t)(j - 1) * (k + 1) + (i - 1)]; }
};

__host__ __device__ inline GmresArrays gmres_arrays(double *base, int k) {
  GmresArrays a;
  a.k = k;
  a.e = base;                   // k + 2
  a.c = a.e + (k + 2);          // k + 1
  a.s = a.c + (k + 1);          // k + 1
  a.y = a.s + (k + 1);          // k + 1
  a.nrm = a.y + (k + 1);        // k + 2
  a.h = a.nrm + (k + 2);        // (k + 1) k
  return a;
}

// x = 0, g_1 = M b, econv = tol ||M b|| (Iters.f:606-616).
__global__ void __launch_bounds__(kThreads)
gmres_init_kernel(int n, const double *__restrict__ b, const double *__restrict__ m,
                  double *__restrict__ x, double *__restrict__ g1, GmresState *gs,
                  double *partials, unsigned int *counter) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    x[i] = 0.0;
    const double gi = b[i] * m[i];
    g1[i] = gi;
    v[0] += gi * gi;
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    gs->econv = gs->tol * sqrt(tot[0]);
    gs->nit = 0;
    gs->cycles = 0;
    gs->ni = 0;
    gs->run = 0;
    gs->conv_flag = 0;
    gs->status = ELX_OK;
    gs->live = 1;
    gs->done = 0;
    if (tot[0] == 0.0) {
      gs->live = 0;  // b = 0: x = 0 is the solution
      gs->done = 1;
    } else if (gs->maxit <= 0) {
      gs->live = 0;
      gs->done = 1;
      gs->status = ELX_ERR_NO_CONVERGENCE;
    }
  }
}

// Restart (Iters.f:627-646): g_1 = M (b - K x) (K x already in g_1),
// e(1) = ||g_1||; opens the Arnoldi loop.
__global__ void __launch_bounds__(kThreads)
gmres_residual_kernel(int n, const double *__restrict__ b, const double *__restrict__ m,
                      double *__restrict__ g1, GmresState *gs, double *arrays, int k,
                      double *partials, unsigned int *counter) {
  if (!gs->live) return;
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double gi = (b[i] - g1[i]) * m[i];
    g1[i] = gi;
    v[0] += gi * gi;
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    const GmresArrays a = gmres_arrays(arrays, k);
    a.e[1] = sqrt(tot[0]);
    a.nrm[1] = a.e[1];
    gs->ni = 0;
    gs->run = 1;
  }
}

// g = g / *den while the Arnoldi loop runs.
__global__ void __launch_bounds__(kThreads)
gmres_scale_kernel(int n, double *__restrict__ g, const double *den, const GmresState *gs) {
  if (!gs->run) return;
  const double d = *den;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    g[i] = g[i] / d;
}

// Gram-Schmidt projection jj of Arnoldi step i (Iters.f:671-677): first the
// update of projection jj-1, w -= H(jj-1, i) g_{jj-1}, then
// H(jj, i) = (w, g_jj).
__global__ void __launch_bounds__(kThreads)
gmres_mgs_kernel(int n, int i, int jj, double *__restrict__ w, const double *__restrict__ gprev,
                 const double *__restrict__ gj, GmresState *gs, double *arrays, int k,
                 double *partials, unsigned int *counter) {
  if (!gs->run) return;
  const GmresArrays a = gmres_arrays(arrays, k);
  const double hp = jj > 1 ? a.H(jj - 1, i) : 0.0;
  double v[1] = {0.0};
  for (int q = blockIdx.x * kThreads + threadIdx.x; q < n; q += gridDim.x * kThreads) {
    double wq = w[q];
    if (jj > 1) {
      wq = wq - hp * gprev[q];
      w[q] = wq;
    }
    v[0] += wq * gj[q];
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) a.H(jj, i) = tot[0];
}

// End of Arnoldi step i (Iters.f:681-704): the last projection update,
// H(i+1, i) = ||w||, the stored rotations applied to column i, a new
// rotation, the residual estimate e(i+1); closes the loop when
// |e(i+1)| <= econv or i = k.
__global__ void __launch_bounds__(kThreads)
gmres_step_end_kernel(int n, int i, double *__restrict__ w, const double *__restrict__ gi,
                      GmresState *gs, double *arrays, int k, double *partials,
                      unsigned int *counter) {
  if (!gs->run) return;
  const GmresArrays a = gmres_arrays(arrays, k);
  const double hp = a.H(i, i);
  double v[1] = {0.0};
  for (int q = blockIdx.x * kThreads + threadIdx.x; q < n; q += gridDim.x * kThreads) {
    const double wq = w[q] - hp * gi[q];
    w[q] = wq;
    v[0] += wq * wq;
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x != 0) return;
  const double norm = sqrt(tot[0]);
  a.nrm[i + 1] = norm;
  a.H(i + 1, i) = norm;
  for (int j = 1; j <= i - 1; j++) {
    const double aux1 = a.c[j] * a.H(j, i) + a.s[j] * a.H(j + 1, i);
    const double aux2 = -a.s[j] * a.H(j, i) + a.c[j] * a.H(j + 1, i);
    a.H(j, i) = aux1;
    a.H(j + 1, i) = aux2;
  }
  const double rr = sqrt(a.H(i, i) * a.H(i, i) + a.H(i + 1, i) * a.H(i + 1, i));
  a.c[i] = a.H(i, i) / rr;
  a.s[i] = a.H(i + 1, i) / rr;
  a.H(i, i) = rr;
  a.H(i + 1, i) = 0.0;
  a.e[i + 1] = -a.s[i] * a.e[i];
  a.e[i] = a.c[i] * a.e[i];
  gs->nit += 1;
  gs->ni = i;
  if (fabs(a.e[i + 1]) <= gs->econv || i == k) gs->run = 0;
}

// Back-substitution H y = e (Iters.f:710-717); one thread, k is small.
__global__ void gmres_backsolve_kernel(GmresState *gs, double *arrays, int k) {
  if (!gs->live || threadIdx.x != 0) return;
  const GmresArrays a = gmres_arrays(arrays, k);
  const int ni = gs->ni;
  gs->run = 0;
  a.y[ni] = a.e[ni] / a.H(ni, ni);
  for (int i = ni - 1; i >= 1; i--) {
    double yi = 0.0;
    for (int j = i + 1; j <= ni; j++) yi = yi - a.H(i, j) * a.y[j];
    a.y[i] = (yi + a.e[i]) / a.H(i, i);
  }
  gs->conv_flag = fabs(a.e[ni + 1]) <= gs->econv;
}

// x += sum_j y(j) g_j, j = 1..ni in order (Iters.f:721-725).
__global__ void __launch_bounds__(kThreads)
gmres_update_x_kernel(int n, double *__restrict__ x, const double *__restrict__ g,
                      const GmresState *gs, const double *arrays, int k) {
  if (!gs->live) return;
  const int ni = gs->ni;
  const double *y = gmres_arrays(const_cast<double *>(arrays), k).y;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    double xi = x[i];
    for (int j = 1; j <= ni; j++) xi = xi + y[j] * g[(size_t)(j - 1) * n + i];
    x[i] = xi;
  }
}

// End of a restart cycle (Iters.f:739): stop on |e(ni+1)| <= econv or
// after maxit cycles.
__global__ void gmres_cycle_end_kernel(GmresState *gs) {
  if (!gs->live || threadIdx.x != 0) return;
  gs->cycles += 1;
  if (gs->conv_flag) {
    gs->live = 0;
    gs->done = 1;
  } else if (gs->cycles >= gs->maxit) {
    gs->live = 0;
    gs->done = 1;
    gs->status = ELX_ERR_NO_CONVERGENCE;
  }
}

}  // namespace

size_t gmres_array_doubles(int k) {
  return (size_t)(k + 2) * 2 + (size_t)(k + 1) * 3 + (size_t)(k + 1) * k;
}

void launch_bicg_start(int n, const double *b, const double *m, double *x, double *r,
                       double *r0, double *p, double *z, PcgScalars *sc, double *partials,
                       unsigned int *counter, cudaStream_t st) {
  bicg_start_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, b, m, x, r, r0, p, z, sc, partials,
                                                         counter);
  ELX_CUDA(cudaGetLastError());
}

// One BiCGSTAB iteration: v = K z (alpha), half step, t = K z (omega), full
// step, direction.  Five launches.
void launch_bicg_iteration(const CsrcDev &k, const double *m, double *x, double *r,
                           const double *r0, double *p, double *z, double *v, double *t,
                           PcgScalars *sc, double *partials, unsigned int *counters,
                           cudaStream_t st) {
  const int n = k.neq;
  launch_gather_epi64(k, kEpiBicgAlpha, z, v, r0, sc, partials, counters + 0, nullptr, st);
  bicg_half_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, v, m, x, r, z, sc, partials,
                                                        counters + 1);
  launch_gather_epi64(k, kEpiBicgOmega, z, t, r, sc, partials, counters + 2, nullptr, st);
  bicg_full_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, z, t, r0, x, r, sc, partials,
                                                        counters + 3);
  bicg_direction_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, r, v, m, p, z, sc);
  ELX_CUDA(cudaGetLastError());
}

void launch_gmres_init(int n, const double *b, const double *m, double *x, double *g1,
                       GmresState *gs, double *partials, unsigned int *counter,
                       cudaStream_t st) {
  gmres_init_kernel<<<vector_grid(n), kThreads, 0, st>>>(n, b, m, x, g1, gs, partials, counter);
  ELX_CUDA(cudaGetLastError());
}

// One restart cycle of GMRES(kdim) on the basis g (kdim + 1 columns of n).
// Returns the number of kernels enqueued.
int launch_gmres_cycle(const CsrcDev &k, int kdim, const double *b, const double *m, double *x,
                       double *g, GmresState *gs, double *arrays, double *partials,
                       unsigned int *counter, cudaStream_t st) {
  const int n = k.neq;
  const int grid = vector_grid(n);
  auto col = [&](int j) { return g + (size_t)(j - 1) * n; };
  const GmresArrays a = gmres_arrays(arrays, kdim);
  int launches = 0;
  launch_gather_epi64(k, kEpiNone, x, col(1), nullptr, nullptr, nullptr, nullptr, &gs->live, st);
  gmres_residual_kernel<<<grid, kThreads, 0, st>>>(n, b, m, col(1), gs, arrays, kdim, partials,
                                                   counter);
  gmres_scale_kernel<<<grid, kThreads, 0, st>>>(n, col(1), a.nrm + 1, gs);
  launches += 3;
  for (int i = 1; i <= kdim; i++) {
    launch_gather_epi64(k, kEpiScale, col(i), col(i + 1), m, nullptr, nullptr, nullptr,
                        &gs->run, st);
    for (int jj = 1; jj <= i; jj++)
      gmres_mgs_kernel<<<grid, kThreads, 0, st>>>(n, i, jj, col(i + 1),
                                                  jj > 1 ? col(jj - 1) : nullptr, col(jj), gs,
                                                  arrays, kdim, partials, counter);
    gmres_step_end_kernel<<<grid, kThreads, 0, st>>>(n, i, col(i + 1), col(i), gs, arrays, kdim,
                                                     partials, counter);
    gmres_scale_kernel<<<grid, kThreads, 0, st>>>(n, col(i + 1), a.nrm + i + 1, gs);
    launches += i + 3;
  }
  gmres_backsolve_kernel<<<1, 32, 0, st>>>(gs, arrays, kdim);
  gmres_update_x_kernel<<<grid, kThreads, 0, st>>>(n, x, g, gs, arrays, kdim);
  gmres_cycle_end_kernel<<<1, 32, 0, st>>>(gs);
  launches += 3;
  ELX_CUDA(cudaGetLastError());
  return launches;
}

}  // namespace elx
