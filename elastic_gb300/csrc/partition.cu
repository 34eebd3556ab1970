// The partitioned product on one GPU: the data path of a run with one
// row-block partition per GPU (the reference's overlapping MPI partitions,
// matvec_csrcrsym1, Matvec.f:1090-1191), here with every partition on the
// same device.
//
// A partition owns the block rows [I0, I1) of the RCM order, cut on
// multiples of the slice height so that its rows are whole slices of the
// sliced FP64 copy: its values are a contiguous range of that copy, used in
// place.  Its column indices are renumbered locally -- owned blocks 0..,
// then the halo blocks (columns of owned rows outside [I0, I1), ascending)
// -- and its x is gathered into [x_owned; x_halo] (the exchange that NCCL or
// peer copies do between GPUs; here a gather kernel), after which the
// sliced kernel forms y_owned = K_own x_own + K_rect x_halo.  Each row sums
// its blocks in the same order as the single-partition product, so the
// result is bitwise the same.
#include <algorithm>

#include "elx_context.h"

namespace elx {
namespace {

__global__ void partition_gather_kernel(int64_t nown, int64_t n, int B, int64_t first,
                                        const int32_t *__restrict__ halo_blocks,
                                        const double *__restrict__ x,
                                        double *__restrict__ xloc) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t h = k - nown;
    xloc[k] = h < 0 ? x[first + k] : x[(int64_t)halo_blocks[h / B] * B + h % B];
  }
}

}  // namespace
}  // namespace elx

namespace elx_api {

// Builds (once per partition count) the device arrays of every partition.
void ensure_partitions(elx_ctx *c, int nparts) {
  require(c->use_blocks, ELX_ERR_ARG,
          "the partitioned product needs node blocks (every node all free or all fixed)");
  if (c->parts_n == nparts) return;
  release_partitions(c);
  const elx::Structure &s = c->s;
  const int B = s.bsize, R = elx::kSliceRows;
  const std::vector<int32_t> b = elx::partition_bounds(s, B, nparts);
  require(!b.empty(), ELX_ERR_ARG, "more partitions than slices of 32 node rows");
  c->parts.resize(nparts);
  for (int p = 0; p < nparts; p++) {
    elx_ctx::DevPartition &d = c->parts[p];
    d.I0 = b[p] / B;
    d.I1 = b[p + 1] / B;
    d.s0 = d.I0 / R;
    d.s1 = (d.I1 + R - 1) / R;
    const int32_t g0 = s.sell_ptr[d.s0], g1 = s.sell_ptr[d.s1];
    std::vector<int32_t> hb;
    for (int sl = d.s0; sl < d.s1; sl++)
      for (int32_t g = s.sell_ptr[sl]; g < s.sell_ptr[sl + 1]; g++)
        for (int t = 0; t < R; t++) {
          const int32_t J = s.sell_col[(int64_t)g * R + t];
          if (sl * R + t < s.nb && (J < d.I0 || J >= d.I1)) hb.push_back(J);
        }
    std::sort(hb.begin(), hb.end());
    hb.erase(std::unique(hb.begin(), hb.end()), hb.end());
    std::vector<int32_t> col((size_t)(g1 - g0) * R), ptr(d.s1 - d.s0 + 1);
    for (int sl = d.s0; sl <= d.s1; sl++) ptr[sl - d.s0] = s.sell_ptr[sl] - g0;
    const int nown = d.I1 - d.I0;
    for (int sl = d.s0; sl < d.s1; sl++)
      for (int32_t g = s.sell_ptr[sl]; g < s.sell_ptr[sl + 1]; g++)
        for (int t = 0; t < R; t++) {
          const int64_t q = (int64_t)g * R + t;
          const int32_t J = s.sell_col[q];
          int32_t L = 0;  // rows past the matrix (last slice): any owned column
          if (sl * R + t < s.nb)
            L = J >= d.I0 && J < d.I1
                    ? J - d.I0
                    : nown + (int32_t)(std::lower_bound(hb.begin(), hb.end(), J) - hb.begin());
          col[(size_t)(g - g0) * R + t] = L;
        }
    d.nhb = (int32_t)hb.size();
    d.voff = (int64_t)g0 * R * B * B;
    c->upload(d.sptr, ptr.data(), ptr.size());
    c->upload(d.scol, col.data(), col.size());
    if (hb.empty())
      c->alloc(d.hb, 16);
    else
      c->upload(d.hb, hb.data(), hb.size());
    c->alloc(d.xloc, (size_t)(nown + d.nhb) * B * 8 + 64);
  }
  c->parts_n = nparts;
  c->sync();
}

void release_partitions(elx_ctx *c) {
  for (elx_ctx::DevPartition &d : c->parts)
    for (DBuf *v : {&d.sptr, &d.scol, &d.hb, &d.xloc}) c->release(*v);
  c->parts.clear();
  c->parts_n = 0;
}

// y = K x through the partitions (device vectors).
void partition_product(elx_ctx *c, int nparts, const double *x, double *y) {
  require(c->use_blocks, ELX_ERR_ARG,
          "the partitioned product needs node blocks (every node all free or all fixed)");
  require(c->sell_val64.p != nullptr, ELX_ERR_STATE, "sliced FP64 node blocks missing");
  ensure_partitions(c, nparts);
  const int B = c->s.bsize;
  for (const elx_ctx::DevPartition &d : c->parts) {
    const int64_t nown = (int64_t)(d.I1 - d.I0) * B, n = nown + (int64_t)d.nhb * B;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, elx::grid_cap(8)));
    elx::partition_gather_kernel<<<grid, 256, 0, c->stream>>>(
        nown, n, B, (int64_t)d.I0 * B, d.hb.as<int32_t>(), x, d.xloc.as<double>());
    ELX_CUDA(cudaGetLastError());
    elx::launch_sell64_local(d.I1 - d.I0, d.s1 - d.s0, B, d.sptr.as<int32_t>(),
                             d.scol.as<int32_t>(), c->sell_val64.as<double>() + d.voff,
                             d.xloc.as<double>(), y + (int64_t)d.I0 * B, c->stream);
    c->launches += 2;
  }
}

}  // namespace elx_api
