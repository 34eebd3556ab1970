// CSRC matrix-vector product y = (D + L + L^T) x on the GPU
// (matvec_csrcsym1, mef/src/Matvec.f:528-621).
//
// The reference computes each row's lower product and scatters the mirrored
// upper contributions y(ja(k)) += al(k) x(i) in one row-ordered pass.  A GPU
// cannot scatter without atomics, so the upper part is gathered instead:
// row i reads the lower entries of its own row (ja, al) and the entries of
// column i of L through the transposed index (jat, alt), where alt is al
// permuted into column order once per assembly.  Each row is owned by a
// group of LANES threads that stride over its entries and reduce with warp
// shuffles in a fixed tree, so every y(i) is summed in the same order on
// every call (deterministic).
#include "elx_internal.h"

namespace elx {
namespace {

template <int LANES, class T>
__global__ void __launch_bounds__(256)
spmv_kernel(int neq, const int32_t *__restrict__ ia, const int32_t *__restrict__ ja,
            const T *__restrict__ al, const int32_t *__restrict__ iat,
            const int32_t *__restrict__ jat, const T *__restrict__ alt,
            const T *__restrict__ ad, const T *__restrict__ x, T *__restrict__ y) {
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int row = gtid / LANES, lane = gtid % LANES;
  T s = 0;
  if (row < neq) {
    for (int p = ia[row] + lane; p < ia[row + 1]; p += LANES) s += al[p] * x[ja[p]];
    for (int p = iat[row] + lane; p < iat[row + 1]; p += LANES) s += alt[p] * x[jat[p]];
  }
#pragma unroll
  for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off, LANES);
  if (row < neq && lane == 0) y[row] = ad[row] * x[row] + s;
}

template <class T>
__global__ void permute_kernel(int64_t n, const int32_t *__restrict__ pt,
                               const T *__restrict__ src, T *__restrict__ dst) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = src[pt[q]];
}

__global__ void demote_kernel(int64_t n, const double *__restrict__ src, float *__restrict__ dst) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = (float)src[q];
}

constexpr int kLanes = 8;

}  // namespace

void launch_spmv64(const CsrcDev &k, const double *x, double *y, cudaStream_t st) {
  const int64_t threads = (int64_t)k.neq * kLanes;
  const int blocks = (int)((threads + 255) / 256);
  spmv_kernel<kLanes, double><<<blocks, 256, 0, st>>>(k.neq, k.ia, k.ja, k.al, k.iat, k.jat,
                                                       k.alt, k.ad, x, y);
  ELX_CUDA(cudaGetLastError());
}

void launch_spmv32(const CsrcDev &k, const float *x, float *y, cudaStream_t st) {
  const int64_t threads = (int64_t)k.neq * kLanes;
  const int blocks = (int)((threads + 255) / 256);
  spmv_kernel<kLanes, float><<<blocks, 256, 0, st>>>(k.neq, k.ia, k.ja, k.al32, k.iat, k.jat,
                                                      k.alt32, k.ad32, x, y);
  ELX_CUDA(cudaGetLastError());
}

// alt = al permuted into column order (after every assembly).
void launch_transpose_values(const CsrcDev &k, cudaStream_t st) {
  if (k.nad == 0) return;
  permute_kernel<double><<<1216, 256, 0, st>>>(k.nad, k.pt, k.al, k.alt);
  ELX_CUDA(cudaGetLastError());
}

// FP32 copies of ad, al, alt for the mixed-precision inner iteration.
void launch_demote_values(const CsrcDev &k, cudaStream_t st) {
  demote_kernel<<<608, 256, 0, st>>>(k.neq, k.ad, k.ad32);
  if (k.nad) {
    demote_kernel<<<1216, 256, 0, st>>>(k.nad, k.al, k.al32);
    demote_kernel<<<1216, 256, 0, st>>>(k.nad, k.alt, k.alt32);
  }
  ELX_CUDA(cudaGetLastError());
}

}  // namespace elx
