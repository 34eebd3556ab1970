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
  double rmax;    // mixed precision: ||r||_M at the last residual replacement
  double delta;   // mixed precision: replace when ||r||_M < delta * rmax (input)
  double rho;     // BiCGSTAB: (r, r0)
  double omega;   // BiCGSTAB: (t, r) / (t, t)
  int32_t maxit;  // (input)
  int32_t iters;
  int32_t done;
  int32_t status;
  int32_t update;    // mixed precision: a residual replacement is due
  int32_t nupdates;  // mixed precision: replacements so far
  // mixed precision: progress watch of the FP64 residual at replacements
  double best;       // smallest ||b - K x||_M seen so far
  int32_t last_rep;  // iteration of the last replacement
  int32_t stall;     // own replacements in a row that did not halve `best`
  int32_t failed;    // the FP32 iteration diverged or stalled: solve in FP64
  int32_t pad_;
};

// Progress watch of the mixed-precision solvers.  A matrix rounded to FP32
// can lose definiteness when K is ill-conditioned (cond(K) near 1/eps32, as
// in 2-D meshes of 10^6 dofs): the FP32 recurrence then stalls or diverges.
// At every replacement the FP64 residual is compared with the best so far;
// a residual kMixedDiverge times the best, or kMixedStall own replacements
// in a row that do not halve it, end the FP32 iteration (`failed`), and the
// host solves the case in FP64.  A replacement is forced every
// kMixedCheckEvery iterations so that a stall is seen.
constexpr int kMixedCheckEvery = 512;
constexpr double kMixedDiverge = 100.0;
constexpr int kMixedStall = 4;

// State of one GMRES(k) solve, resident in device memory (the small dense
// arrays live in a separate buffer of gmres_array_doubles(k) doubles).
struct GmresState {
  double tol;         // (input)
  double econv;       // tol ||M b||
  int32_t maxit;      // restart cycles (input)
  int32_t live;       // the solve is running
  int32_t run;        // the current cycle's Arnoldi loop is running
  int32_t ni;         // Arnoldi steps in the current cycle
  int32_t nit;        // Arnoldi steps in all cycles
  int32_t cycles;
  int32_t conv_flag;  // |e(ni+1)| <= econv after the current cycle
  int32_t done;
  int32_t status;
};

// Block PCG (block_pcg.cu): per-column scalars, a header shared by the
// columns, and the device arrays of one block of W columns (multi-vectors
// row-interleaved: entry (row, c) at row * W + c).
struct ColScalars {
  double d, alpha, beta, pq, rmax, conv, bmb;
  int32_t iters, done, status, update, nupdates, pad;
  double best;  // progress watch, as in PcgScalars
  int32_t last_rep, stall, failed, pad2;
};
struct BlockHeader {
  double tol;      // (input)
  double delta;    // mixed precision: replacement threshold (input)
  int32_t maxit;   // (input)
  int32_t active;  // columns still iterating
  int32_t any_update;
  int32_t pad;
};
struct BlockVecs {
  int w = 0;
  const double *b = nullptr, *m = nullptr;
  double *x = nullptr, *r = nullptr, *p = nullptr, *q = nullptr, *z = nullptr;
  const float *m32 = nullptr;
  float *xlo = nullptr, *r32 = nullptr, *p32 = nullptr, *q32 = nullptr;
  ColScalars *cols = nullptr;
  BlockHeader *hdr = nullptr;     // the solve's header
  BlockHeader *hdr_on = nullptr;  // a header with active = 1 (products outside a solve)
  double *partials = nullptr;     // 2 * 16 * (8 CTAs per SM) doubles
  unsigned int *counters = nullptr;  // 8
};
bool block_width_supported(int w);
void launch_block_start(const CsrcDev &k, const BlockVecs &v, bool mixed, cudaStream_t st);
void launch_block_iteration(const CsrcDev &k, const BlockVecs &v, bool mixed,
                            bool replacement_point, cudaStream_t st);
void launch_block_diagnostics(const CsrcDev &k, const BlockVecs &v, double *out,
                              cudaStream_t st);
void launch_spmm32(const CsrcDev &k, const BlockVecs &v, cudaStream_t st);  // q32 = K p32
void launch_spmm64(const CsrcDev &k, const BlockVecs &v, cudaStream_t st);  // q = K p
void launch_interleave(int n, int w, const double *colmajor, double *inter, cudaStream_t st);
void launch_deinterleave(int n, int w, const double *inter, double *colmajor, cudaStream_t st);

int vector_grid(int n);

// SpMV kernel families (spmv.cu)
constexpr int kSpmvGather = 0;  // two-sided gather (lower + transposed upper)
constexpr int kSpmvTiled = 1;   // single-read tiles with a transposed index per tile

void launch_diag_inverse(int n, const double *ad, double *m, float *m32, int32_t *zero_row,
                         cudaStream_t st);
template <class T>
void launch_pcg_start(int n, const T *b, const T *m, T *x, T *r, T *p, PcgScalars *sc,
                      double *partials, unsigned int *counter, cudaStream_t st);
void launch_pcg_iteration(const CsrcDev &k, const TileDev &td, int spmv_kind, double *x,
                          double *r, double *p, double *q, double *part, const double *m,
                          PcgScalars *sc, double *partials, unsigned int *counters,
                          int32_t *err, cudaStream_t st);
void launch_pcg_iteration32(const CsrcDev &k, float *x, float *r, float *p, float *q,
                            const float *m, PcgScalars *sc, double *partials,
                            unsigned int *counters, cudaStream_t st);
void launch_spmv64(const CsrcDev &k, const TileDev &td, int spmv_kind, const double *x, double *y,
                   double *part, int32_t *err, cudaStream_t st);
void launch_diagnostics(int n, const double *x, const double *z, const double *b,
                        const double *m, double *out, double *partials, unsigned int *counter,
                        cudaStream_t st);
void launch_refine_residual(int n, const double *b, const double *z, const double *m, double *r,
                            float *r32, double *out, double *partials, unsigned int *counter,
                            cudaStream_t st);
void launch_refine_accumulate(int n, double *x, const float *d, bool first, cudaStream_t st);
void launch_rel_start(int n, const float *r, const float *m, float *xlo, float *p,
                      PcgScalars *sc, double *partials, unsigned int *counter, cudaStream_t st);
void launch_rel_iteration(const CsrcDev &k, const double *b, const double *m, double *xhi,
                          double *rhi, double *z, float *xlo, float *r, float *p, float *q,
                          const float *m32, PcgScalars *sc, double *partials,
                          unsigned int *counters, bool replacement_point, cudaStream_t st);
void launch_convert(int n, const double *src, float *dst, cudaStream_t st);

// BiCGSTAB and GMRES (krylov_ns.cu)
void launch_bicg_start(int n, const double *b, const double *m, double *x, double *r,
                       double *r0, double *p, double *z, PcgScalars *sc, double *partials,
                       unsigned int *counter, cudaStream_t st);
void launch_bicg_iteration(const CsrcDev &k, const double *m, double *x, double *r,
                           const double *r0, double *p, double *z, double *v, double *t,
                           PcgScalars *sc, double *partials, unsigned int *counters,
                           cudaStream_t st);
size_t gmres_array_doubles(int k);
void launch_gmres_init(int n, const double *b, const double *m, double *x, double *g1,
                       GmresState *gs, double *partials, unsigned int *counter,
                       cudaStream_t st);
int launch_gmres_cycle(const CsrcDev &k, int kdim, const double *b, const double *m, double *x,
                       double *g, GmresState *gs, double *arrays, double *partials,
                       unsigned int *counter, cudaStream_t st);
void launch_widen(int n, const float *src, double *dst, cudaStream_t st);

}  // namespace elx
