// Device-side scalar state and launch entry points of the Krylov solvers.
#pragma once

#include "elx_internal.h"

namespace elx {

// Scalars of one PCG solve, resident in device memory.
struct PcgScalars {
  double tol;     // relative tolerance (input)
  double d;       // (r, M r) of the current iterate
  double bmb;     // (b, M b)
  double conv;    // tol * sqrt|(b, M b)|
  double alpha, beta, pq;
  int32_t maxit;  // (input)
  int32_t iters;
  int32_t done;
  int32_t status;
};

int vector_grid(int n);

void launch_diag_inverse(int n, const double *ad, double *m, int32_t *zero_row, cudaStream_t st);
void launch_pcg_start(int n, const double *b, const double *m, double *x, double *r, double *p,
                      PcgScalars *sc, double *partials, unsigned int *counter, cudaStream_t st);
// SpMV kernel families (spmv.cu)
constexpr int kSpmvGather = 0;  // two-sided gather (lower + transposed upper)
constexpr int kSpmvTiled = 1;   // single-read tiles with a transposed index per tile

void launch_pcg_iteration(const CsrcDev &k, const TileDev &td, int spmv_kind, double *x,
                          double *r, double *p, double *q, double *part, const double *m,
                          PcgScalars *sc, double *partials, unsigned int *counters,
                          int32_t *err, cudaStream_t st);
void launch_spmv64(const CsrcDev &k, const TileDev &td, int spmv_kind, const double *x, double *y,
                   double *part, int32_t *err, cudaStream_t st);
void launch_diagnostics(int n, const double *x, const double *z, const double *b,
                        const double *m, double *out, double *partials, unsigned int *counter,
                        cudaStream_t st);

}  // namespace elx
