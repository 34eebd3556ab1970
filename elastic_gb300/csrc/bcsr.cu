// Node-block (BCSR) form of the CSRC matrix and its product y = K x.
//
// The elasticity matrix is a matrix of B x B node blocks (B = ndf): when no
// node is only partly fixed, numeq's numbering (Numeq.f:139-192) puts the B
// dofs of a node on consecutive equations, so block row I is equations
// B I .. B I + B - 1.  The CSRC arrays (ad, al: the reference's layout, which
// the assembly fills and the C ABI returns) are expanded after each assembly
// into sliced copies of the full block rows (elx_sell.cuh) -- lower blocks,
// the diagonal block, upper blocks as transposed copies of the lower ones --
// with one column index per block instead of one per entry:
//
//   * bytes per stored entry: B^2 values + 1 index per B^2 entries, so
//     4.4 B (FP32) / 8.4 B (FP64) per entry against 6 / 10 B for the
//     two-sided gather with 16-bit column deltas;
//   * one thread per matrix block row walks its slots: per block one column
//     index and B^2 values, B x values, B^2 FMAs -- every FMA lane does
//     useful work (the rows of a slice are padded to the same width), which
//     is what bounds the FP64 product on this GPU (its FP64 pipe retires 2
//     FMAs per clock per SM);
//   * no reductions inside a row, so the FP64 pipe does nothing but the
//     product's own FMAs.
//
// The product is still the reference's y = D x + L x + L^T x (matvec_csrcsym1,
// Matvec.f:528-621) with the same values, summed in a different order.
#include <algorithm>

#include "elx_krylov.h"
#include "elx_ptx.cuh"
#include "elx_reduce.cuh"
#include "elx_sell.cuh"

namespace elx {
namespace {

// Sliced copy (as T) of the node blocks, straight from the CSRC arrays: one
// thread per block row of a slice (slot t).  Block k of row I is, in the
// order of the structure's block rows: a lower block (k < nl, the entries
// al[ia[B I + a] + B k + b]), the diagonal block (k = nl: ad on the
// diagonal, the last a entries of row B I + a below it, mirrored above), or
// an upper block (k > nl): the transpose of the lower block that mirrors it
// in block row J = its block column, at position bt[p] - bia[J] of that
// row.  Padding slots get zero blocks.
template <class T, int B>
__global__ void fill_sell_kernel(int nb, int nslices, const int32_t *__restrict__ bia,
                                 const int32_t *__restrict__ bt,
                                 const int32_t *__restrict__ sell_ptr,
                                 const int32_t *__restrict__ sell_col,
                                 const int32_t *__restrict__ ia, const double *__restrict__ ad,
                                 const double *__restrict__ al, T *__restrict__ sval) {
  constexpr int BB = B * B, R = kSliceRows;
  const int64_t nthreads = (int64_t)nslices * R;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nthreads;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int sl = (int)(i / R), t = (int)(i % R), I = (int)i;
    const int g0 = sell_ptr[sl], g1 = sell_ptr[sl + 1];
    const int p0 = I < nb ? bia[I] : 0;
    const int n = I < nb ? bia[I + 1] - p0 : 0;
    const int r0 = B * I;
    const int nl = I < nb ? (ia[r0 + 1] - ia[r0]) / B : 0;
    int row[B];
#pragma unroll
    for (int a = 0; a < B; a++) row[a] = I < nb ? ia[r0 + a] : 0;
    for (int g = g0; g < g1; g++) {
      const int k = g - g0;
      T *grp = sval + (size_t)g * BB * R;
      T v[BB];
      if (k < nl) {
#pragma unroll
        for (int a = 0; a < B; a++)
#pragma unroll
          for (int b = 0; b < B; b++) v[a * B + b] = (T)al[row[a] + B * k + b];
      } else if (k == nl && k < n) {
#pragma unroll
        for (int a = 0; a < B; a++)
#pragma unroll
          for (int b = 0; b < B; b++)
            v[a * B + b] = (T)(a == b  ? ad[r0 + a]
                               : a > b ? al[row[a] + B * nl + b]
                                       : al[row[b] + B * nl + a]);
      } else if (k < n) {
        const int J = sell_col[(size_t)g * R + t];
        const int q = bt[p0 + k] - bia[J];
        int rj[B];
#pragma unroll
        for (int b = 0; b < B; b++) rj[b] = ia[B * J + b];
#pragma unroll
        for (int a = 0; a < B; a++)
#pragma unroll
          for (int b = 0; b < B; b++) v[a * B + b] = (T)al[rj[b] + B * q + a];
      } else {
#pragma unroll
        for (int e = 0; e < BB; e++) v[e] = T(0);
      }
#pragma unroll
      for (int e = 0; e < BB; e++) grp[sell_pos<T, B>(e, t)] = v[e];
    }
  }
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
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, grid_cap(16)));
}

template <class T>
void fill_sell(const CsrcDev &k, T *out, cudaStream_t st) {
  if (!out || k.nslices == 0) return;
  const int g = fill_grid((int64_t)k.nslices * kSliceRows);
  if (k.bsize == 3)
    fill_sell_kernel<T, 3><<<g, 256, 0, st>>>(k.nb, k.nslices, k.bia, k.bt, k.sell_ptr,
                                              k.sell_col, k.ia, k.ad, k.al, out);
  else
    fill_sell_kernel<T, 2><<<g, 256, 0, st>>>(k.nb, k.nslices, k.bia, k.bt, k.sell_ptr,
                                              k.sell_col, k.ia, k.ad, k.al, out);
  ELX_CUDA(cudaGetLastError());
}

// The FP64 pipe's FMA rate: 8 independent register-resident DFMA chains
// per thread (enough to cover the FMA latency), `reps` steps each, no
// memory traffic but one store per thread.
__global__ void __launch_bounds__(256) fp64_fma_probe_kernel(int reps, double b, double c,
                                                             double *out) {
  double a[8];
#pragma unroll
  for (int i = 0; i < 8; i++) a[i] = (double)(threadIdx.x + i);
  for (int r = 0; r < reps; r++)
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = fma(a[i], b, c);
  double t = 0.0;
#pragma unroll
  for (int i = 0; i < 8; i++) t += a[i];
  out[blockIdx.x * 256 + threadIdx.x] = t;
}

}  // namespace

double measure_fp64_fma_rate(int device, double *per_clock_per_sm) {
  ELX_CUDA(cudaSetDevice(device));
  const int grid = grid_cap(8);
  const int reps = 8192;
  double *out = nullptr;
  cudaEvent_t e0, e1;
  ELX_CUDA(cudaMalloc(&out, sizeof(double) * (size_t)grid * 256));
  ELX_CUDA(cudaEventCreate(&e0));
  ELX_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 6; rep++) {
    ELX_CUDA(cudaEventRecord(e0));
    fp64_fma_probe_kernel<<<grid, 256>>>(reps, 0.999999, 1e-9, out);
    ELX_CUDA(cudaEventRecord(e1));
    ELX_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    ELX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0) best = std::min(best, ms);  // the first launch warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double fma = (double)grid * 256 * 8 * reps;
  const double rate = fma / (best * 1e-3);
  if (per_clock_per_sm) {
    int khz = 0;
    ELX_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, device));
    *per_clock_per_sm = rate / (sm_count() * (double)khz * 1e3);
  }
  return rate;
}

void launch_fill_sell64(const CsrcDev &k, cudaStream_t st) { fill_sell<double>(k, k.sell_val64, st); }
void launch_fill_sell32(const CsrcDev &k, cudaStream_t st) { fill_sell<float>(k, k.sell_val, st); }

void launch_sell64_local(int nb, int nslices, int bsize, const int32_t *sell_ptr,
                         const int32_t *sell_col, const double *sval, const double *x,
                         double *y, cudaStream_t st) {
  if (nslices <= 0) return;
  const int grid = std::max(1, std::min((nslices + 7) / 8, grid_cap(8)));
  if (bsize == 3)
    sell_spmv_kernel<double, 3, 1, true, kEpiNone><<<grid, 256, 0, st>>>(
        nb, nslices, sell_ptr, sell_col, sval, x, y, nullptr, nullptr, nullptr, nullptr, nullptr);
  else
    sell_spmv_kernel<double, 2, 2, true, kEpiNone><<<grid, 256, 0, st>>>(
        nb, nslices, sell_ptr, sell_col, sval, x, y, nullptr, nullptr, nullptr, nullptr, nullptr);
  ELX_CUDA(cudaGetLastError());
}

// The gather entry points route here when the matrix has node blocks: the
// sliced copy of precision T, one warp per slice, one CTA per 8 slices.
template <class T, int EPI>
void launch_bcsr(const CsrcDev &k, const T *x, T *y, const T *w, PcgScalars *sc,
                 double *partials, unsigned int *counter, const int32_t *gate,
                 cudaStream_t st) {
  const int sgrid = std::max(1, std::min((k.nslices + 7) / 8, k.max_grid));
#define ELX_SELL(T_, B_, U_, LD_, VAL_)                                                     \
  sell_spmv_kernel<T_, B_, U_, LD_, EPI><<<sgrid, 256, 0, st>>>(                             \
      k.nb, k.nslices, k.sell_ptr, k.sell_col, VAL_, x, y, w, sc, partials, counter, gate)
  if constexpr (sizeof(T) == 4) {
    ELX_REQUIRE(k.sell_val != nullptr, ELX_ERR_STATE, "sliced FP32 node blocks missing");
    // at most 8 CTAs per SM; 3 groups per step for B = 3 (64 registers) and
    // 4 for B = 2: 50.7 / 52.4 / 50.2 / 60.0 us for 1 / 2 / 3 / 4 groups with
    // streaming loads on the 64^3 HEXA8 cube
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
  } else {
    ELX_REQUIRE(k.sell_val64 != nullptr, ELX_ERR_STATE, "sliced FP64 node blocks missing");
    // FP64-pipe bound: one group per step (48 registers) measured as fast
    // as two and faster than three (126.1 / 125.9 / 131.2 us on the 64^3
    // HEXA8 cube), streaming loads faster than cached ones (128.8 us)
    if (k.bsize == 3)
      ELX_SELL(double, 3, 1, true, k.sell_val64);
    else
      ELX_SELL(double, 2, 2, true, k.sell_val64);
  }
#undef ELX_SELL
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
