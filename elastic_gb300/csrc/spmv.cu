// CSRC matrix-vector product y = (D + L + L^T) x on the GPU
// (matvec_csrcsym1, mef/src/Matvec.f:528-621).
//
// The reference makes one row-ordered pass: row i's lower product
// t = ad(i) x(i) + sum al(k) x(ja(k)) and, for the same entries, the scatter of
// the mirrored upper part y(ja(k)) += al(k) x(i).  Each al(k) is read once.
// A GPU cannot scatter without atomics (nondeterministic in FP64), and
// gathering the upper part through a global transposed copy reads every value
// twice.  This kernel keeps the single read:
//
//   * Rows are cut into tiles of R consecutive rows.  Each tile has a
//     transposed index (built once on the host, structure.cpp:build_tiles):
//     per distinct column j of its entries, the tile-local positions of
//     those entries, columns ordered by decreasing length.
//   * A persistent CTA per SM walks its tiles through a 3-stage shared-memory
//     pipeline.  Two tiles ahead, one thread issues 1-D bulk copies (TMA,
//     cp.async.bulk + mbarrier) of the tile's al, ja, ia, transposed
//     positions and column list.  One tile ahead, all threads gather
//     x(ja(k)) and the tile's own x and ad into shared memory with per-thread
//     cp.async (the addresses come from the staged ja), and record each
//     entry's row.  So the arithmetic never waits on HBM or L2.
//   * Compute (FP64: exactly 2 DFMA per entry, the minimum for the symmetric
//     product), on two warp groups at once:
//       - row warps: two threads per row, ad(i) x(i) + sum al(k) x(ja(k));
//       - column warps: one thread per distinct column j, sum al(k) x(row(k))
//         over the column's entries in their fixed order.  Columns inside the
//         tile land on the tile's rows; columns left of it (rows of earlier
//         tiles) go to a halo slot in HBM.
//   * A second, row-parallel launch (krylov.cu) adds to every row its halo
//     slots in tile order.
//
// Every y(i) is therefore summed in the same order on every call
// (deterministic), and HBM traffic per call is al + ja + the 16-bit
// transposed positions + small per-tile metadata, against 12 bytes per entry
// of algorithmic traffic.  GB300's FP64 pipe (2 DFMA/clock/SM) charges a
// whole warp instruction however few lanes are active, so warps are given
// loops of nearly equal length: two threads per row (one shuffle-add per
// row), consecutive rows of a tile have similar lengths, and the columns are
// length-sorted.
#include "elx_krylov.h"
#include "elx_ptx.cuh"
#include "elx_reduce.cuh"

#include <algorithm>
#include <atomic>
#include <cstdlib>

namespace elx {
namespace {

constexpr int kPipeThreads = 256;  // warps 0-3 rows, warps 4-7 columns
constexpr int kStages = 3;

// Byte offsets of the regions of one pipeline stage (each 16-byte aligned).
struct PipeLayout {
  uint32_t al, ja, tpos, ia, tst, tcol, xj, row, xown, adown, bytes;
};

__host__ __device__ inline uint32_t up16(uint32_t v) { return (v + 15u) & ~15u; }

__host__ __device__ inline PipeLayout pipe_layout(int max_nnz, int max_tgt, int R, int vs) {
  const uint32_t pad_v = 16 / vs;
  PipeLayout L;
  uint32_t o = 0;
  L.al = o;    o = up16(o + (max_nnz + 2 * pad_v) * vs);
  L.ja = o;    o = up16(o + (max_nnz + 8) * 4);
  L.tpos = o;  o = up16(o + (max_nnz + 16) * 2);
  L.ia = o;    o = up16(o + (R + 1 + 8) * 4);
  L.tst = o;   o = up16(o + (max_tgt + 1 + 8) * 4);
  L.tcol = o;  o = up16(o + (max_tgt + 8) * 4);
  L.xj = o;    o = up16(o + max_nnz * vs);
  L.row = o;   o = up16(o + max_nnz);
  L.xown = o;  o = up16(o + R * vs);
  L.adown = o; o = up16(o + R * vs);
  L.bytes = o;
  return L;
}

// header: kStages barriers (64 B), kStages descriptors (128 B), s_y and s_yc
__host__ __device__ inline uint32_t pipe_header(int R, int vs) {
  return 192 + up16(2 * R * vs);
}

template <class T>
__global__ void __launch_bounds__(kPipeThreads, 2)
spmv_pipe_kernel(const T *__restrict__ al, const T *__restrict__ ad, const int32_t *__restrict__ ja,
                 const int32_t *__restrict__ ia, TileDev td, PipeLayout L,
                 const T *__restrict__ x, T *__restrict__ y, T *__restrict__ part, int32_t *err,
                 int stall, const PcgScalars *sc) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int PV = 16 / sizeof(T);  // elements per 16 bytes
  const int tid = threadIdx.x;
  const int R = td.rows;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
  int32_t *sdesc = reinterpret_cast<int32_t *>(smem + 64);
  T *s_y = reinterpret_cast<T *>(smem + 192);
  T *s_yc = s_y + R;
  unsigned char *stages = smem + pipe_header(R, sizeof(T));

  const int ntiles = td.ntiles;
  if ((int)blockIdx.x >= ntiles) return;
  if (sc && sc->done) return;  // an iteration past the solve's convergence
  const int my_n = (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1;

  if (tid == 0) {
    for (int s = 0; s < kStages; s++) ptx::mbar_init(&bar[s], 1);
    ptx::fence_barrier_init();
  }
  __syncthreads();

  // ---- producer helpers (thread 0)
  int nd[8];
  auto load_desc = [&](int i) {
    const int4 *p = reinterpret_cast<const int4 *>(td.desc + 8 * ((size_t)blockIdx.x + (size_t)i * gridDim.x));
    const int4 a = p[0], b = p[1];
    nd[0] = a.x; nd[1] = a.y; nd[2] = a.z; nd[3] = a.w;
    nd[4] = b.x; nd[5] = b.y; nd[6] = b.z; nd[7] = b.w;
  };
  auto issue = [&](int i) {
    const int s = i % kStages;
    unsigned char *st = stages + (size_t)s * L.bytes;
    int32_t *dd = sdesc + 8 * s;
#pragma unroll
    for (int k = 0; k < 8; k++) dd[k] = nd[k];
    const int base = nd[0], nnz = nd[1], g0 = nd[2], ng = nd[3], r0 = nd[6], nr = nd[7];
    const int a0 = base & ~(PV - 1), a1 = (base + nnz + PV - 1) & ~(PV - 1);
    const int j0 = base & ~3, j1 = (base + nnz + 3) & ~3;
    const int p0 = base & ~7, p1 = (base + nnz + 7) & ~7;
    const int i0 = r0 & ~3, i1 = (r0 + nr + 1 + 3) & ~3;
    const int s0 = g0 & ~3, s1 = (g0 + ng + 1 + 3) & ~3;
    const int c0 = g0 & ~3, c1 = (g0 + ng + 3) & ~3;
    const uint32_t bytes = (uint32_t)(a1 - a0) * sizeof(T) + (uint32_t)(j1 - j0) * 4 +
                           (uint32_t)(p1 - p0) * 2 + (uint32_t)(i1 - i0) * 4 +
                           (uint32_t)(s1 - s0) * 4 + (uint32_t)(c1 - c0) * 4;
    ptx::fence_proxy_async();
    ptx::mbar_arrive_expect_tx(&bar[s], bytes);
    if (a1 > a0) ptx::bulk_g2s(st + L.al, al + a0, (a1 - a0) * sizeof(T), &bar[s]);
    if (j1 > j0) ptx::bulk_g2s(st + L.ja, ja + j0, (j1 - j0) * 4, &bar[s]);
    if (p1 > p0) ptx::bulk_g2s(st + L.tpos, td.tpos + p0, (p1 - p0) * 2, &bar[s]);
    ptx::bulk_g2s(st + L.ia, ia + i0, (i1 - i0) * 4, &bar[s]);
    ptx::bulk_g2s(st + L.tst, td.tgt_start + s0, (s1 - s0) * 4, &bar[s]);
    if (c1 > c0) ptx::bulk_g2s(st + L.tcol, td.tgt_col + c0, (c1 - c0) * 4, &bar[s]);
  };

  // ---- one tile ahead: gathers of x(ja), own x and ad; entry -> row map.
  // False when the tile's copies did not arrive within the wait's limit
  // (err is set): nothing of the tile is read then.
  auto gather = [&](int i) -> bool {
    const int s = i % kStages;
    unsigned char *st = stages + (size_t)s * L.bytes;
    const int32_t *d = sdesc + 8 * s;
    if (!ptx::mbar_wait_bounded(&bar[s], (uint32_t)((i / kStages) & 1), err, 1)) return false;
    const int base = d[0], nnz = d[1], r0 = d[6], nr = d[7];
    const int32_t *s_ja = reinterpret_cast<const int32_t *>(st + L.ja) + (base & 3);
    const int32_t *s_ia = reinterpret_cast<const int32_t *>(st + L.ia) + (r0 & 3);
    T *s_xj = reinterpret_cast<T *>(st + L.xj);
    T *s_xown = reinterpret_cast<T *>(st + L.xown);
    T *s_adown = reinterpret_cast<T *>(st + L.adown);
    uint8_t *s_row = reinterpret_cast<uint8_t *>(st + L.row);
    for (int q = tid; q < nnz; q += kPipeThreads) ptx::cp_async<sizeof(T)>(&s_xj[q], x + s_ja[q]);
    for (int r = tid; r < nr; r += kPipeThreads) {
      ptx::cp_async<sizeof(T)>(&s_xown[r], x + r0 + r);
      ptx::cp_async<sizeof(T)>(&s_adown[r], ad + r0 + r);
      const int kb = s_ia[r] - base, ke = s_ia[r + 1] - base;
      for (int k = kb; k < ke; k++) s_row[k] = (uint8_t)r;
    }
    return true;
  };

  // stall != 0 (a test of the bounded waits): the producer issues nothing,
  // so that every wait runs out
  if (tid == 0 && !stall) {
    for (int i = 0; i < kStages - 1 && i < my_n; i++) {
      load_desc(i);
      issue(i);
    }
    if (kStages - 1 < my_n) load_desc(kStages - 1);
  }
  __syncthreads();
  bool ok = gather(0);
  ptx::cp_async_commit();

  for (int i = 0; i < my_n; i++) {
    if (tid == 0 && !stall && i + kStages - 1 < my_n) {
      issue(i + kStages - 1);
      if (i + kStages < my_n) load_desc(i + kStages);
    }
    if (ok && i + 1 < my_n) ok = gather(i + 1);
    ptx::cp_async_commit();
    ptx::cp_async_wait<1>();
    if (__syncthreads_or(!ok)) {
      // a wait ran out (err is set): no further tile is read or computed;
      // the gathers already issued land, and thread 0 gives the bulk copies
      // still in flight (tiles i .. i + kStages - 1) 10 ms each before the
      // CTA leaves
      ptx::cp_async_wait<0>();
      if (tid == 0)
        for (int j = i; j < my_n && j < i + kStages; j++)
          ptx::mbar_wait_bounded(&bar[j % kStages], (uint32_t)((j / kStages) & 1), err, 1,
                                 10000000ull);
      return;
    }

    // ---- compute tile i
    const int s = i % kStages;
    const unsigned char *st = stages + (size_t)s * L.bytes;
    const int32_t *d = sdesc + 8 * s;
    const int base = d[0], ng = d[3], o0 = d[4], nout = d[5], r0 = d[6], nr = d[7];
    const T *s_al = reinterpret_cast<const T *>(st + L.al) + (base & (PV - 1));
    const T *s_xj = reinterpret_cast<const T *>(st + L.xj);
    const T *s_xown = reinterpret_cast<const T *>(st + L.xown);
    const T *s_adown = reinterpret_cast<const T *>(st + L.adown);
    const int32_t *s_ia = reinterpret_cast<const int32_t *>(st + L.ia) + (r0 & 3);
    if (tid < kPipeThreads / 2) {
      // row warps: two threads per row, two accumulators per thread
      const int lane = tid & 1;
      for (int rr0 = 0; rr0 < nr; rr0 += kPipeThreads / 4) {
        const int r = rr0 + (tid >> 1);
        T acc0 = 0, acc1 = 0;
        if (r < nr) {
          const int kb = s_ia[r] - base, ke = s_ia[r + 1] - base;
          int k = kb + lane;
          for (; k + 2 < ke; k += 4) {
            acc0 += s_al[k] * s_xj[k];
            acc1 += s_al[k + 2] * s_xj[k + 2];
          }
          if (k < ke) acc0 += s_al[k] * s_xj[k];
        }
        T acc = acc0 + acc1;
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        if (r < nr && lane == 0) s_y[r] = s_adown[r] * s_xown[r] + acc;
      }
    } else {
      // column warps: one thread per distinct column, two accumulators
      const int c = tid - kPipeThreads / 2;
      const uint16_t *s_tpos = reinterpret_cast<const uint16_t *>(st + L.tpos) + (base & 7);
      const int32_t *s_tst = reinterpret_cast<const int32_t *>(st + L.tst) + (d[2] & 3);
      const int32_t *s_tcol = reinterpret_cast<const int32_t *>(st + L.tcol) + (d[2] & 3);
      const uint8_t *s_row = reinterpret_cast<const uint8_t *>(st + L.row);
      for (int r = c; r < nr; r += kPipeThreads / 2) s_yc[r] = T(0);
      ptx::named_barrier(1, kPipeThreads / 2);
      for (int g = c; g < ng; g += kPipeThreads / 2) {
        const int qb = s_tst[g] - base, qe = s_tst[g + 1] - base;
        T acc0 = 0, acc1 = 0;
        int q = qb;
        for (; q + 1 < qe; q += 2) {
          const int p0 = s_tpos[q], p1 = s_tpos[q + 1];
          const T a0 = s_al[p0], a1 = s_al[p1];
          const T x0 = s_xown[s_row[p0]], x1 = s_xown[s_row[p1]];
          acc0 += a0 * x0;
          acc1 += a1 * x1;
        }
        if (q < qe) {
          const int p0 = s_tpos[q];
          acc0 += s_al[p0] * s_xown[s_row[p0]];
        }
        const T acc = acc0 + acc1;
        if (g < nout) part[o0 + g] = acc;
        else s_yc[s_tcol[g] - r0] = acc;
      }
    }
    __syncthreads();
    for (int r = tid; r < nr; r += kPipeThreads) y[r0 + r] = s_y[r] + s_yc[r];
    __syncthreads();
  }
}

// Two-sided gather: LANES threads per row stride over the row's lower
// entries and over its upper entries (column i of L through the transposed
// copy), UNROLL entries in flight per thread, then a fixed shuffle tree.
// Rows are walked with a fixed grid so that the epilogue's dot products
// reduce in a fixed order.
// BASE is the index base of ia/ja/iat/jat contents (0 inside the library,
// 1 for arrays in the reference's 1-based convention).  With DELTA the
// columns come as 16-bit distances from the row (ja16: row - col below the
// diagonal, jat16: col - row above it): 2 bytes per stored entry instead of 4.
// EPI selects what happens besides y = K x (GatherEpi); w is the epilogue's
// second vector.  A launch with gate != nullptr runs only while *gate != 0.
template <class T, int LANES, int U, int EPI, int BASE = 0, bool DELTA = false>
__global__ void __launch_bounds__(256)
gather_spmv_kernel(int neq, const int32_t *__restrict__ ia, const int32_t *__restrict__ ja,
                   const T *__restrict__ al, const int32_t *__restrict__ iat,
                   const int32_t *__restrict__ jat, const T *__restrict__ alt,
                   const T *__restrict__ ad, const T *__restrict__ x, T *__restrict__ y,
                   const T *__restrict__ w, PcgScalars *sc, double *partials,
                   unsigned int *counter, const int32_t *gate,
                   const uint16_t *__restrict__ ja16 = nullptr,
                   const uint16_t *__restrict__ jat16 = nullptr) {
  constexpr bool DOT = EPI == kEpiPcg || EPI == kEpiBicgAlpha || EPI == kEpiBicgOmega;
  constexpr int NV = EPI == kEpiBicgOmega ? 2 : 1;
  if (DOT && sc->done) return;
  if (gate && *gate == 0) return;
  constexpr int RPB = 256 / LANES;  // rows per block pass
  const int lane = threadIdx.x % LANES, sub = threadIdx.x / LANES;
  T v[NV];  // this thread's share of the dot products, widened per warp
#pragma unroll
  for (int c = 0; c < NV; c++) v[c] = T(0);
  for (int row0 = blockIdx.x * RPB; row0 < neq; row0 += gridDim.x * RPB) {
    const int row = row0 + sub;
    T acc0 = 0, acc1 = 0;
    if (row < neq) {
#pragma unroll
      for (int part = 0; part < 2; part++) {
        const int32_t *cols = part ? jat : ja;
        const uint16_t *dels = part ? jat16 : ja16;
        const T *vals = part ? alt : al;
        const int kb = (part ? iat[row] : ia[row]) - BASE;
        const int ke = (part ? iat[row + 1] : ia[row + 1]) - BASE;
        for (int k0 = kb + lane; k0 < ke; k0 += U * LANES) {
          T a[U], xv[U];
          int j[U];
#pragma unroll
          for (int u = 0; u < U; u++) {
            const int k = k0 + u * LANES;
            a[u] = k < ke ? vals[k] : T(0);
            if (DELTA)
              j[u] = k < ke ? (part ? row + (int)dels[k] : row - (int)dels[k]) : row;
            else
              j[u] = k < ke ? cols[k] - BASE : row;
          }
#pragma unroll
          for (int u = 0; u < U; u++) xv[u] = x[j[u]];
#pragma unroll
          for (int u = 0; u < U; u += 2) {
            if (k0 + u * LANES < ke) acc0 += a[u] * xv[u];
            if (k0 + (u + 1) * LANES < ke) acc1 += a[u + 1] * xv[u + 1];
          }
        }
      }
    }
    T s = acc0 + acc1;
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off, LANES);
    if (row < neq && lane == 0) {
      const T xi = x[row];
      T yi = ad[row] * xi + s;
      if (EPI == kEpiScale) yi = yi * w[row];
      y[row] = yi;
      if (EPI == kEpiPcg) v[0] += xi * yi;
      if (EPI == kEpiBicgAlpha) v[0] += yi * w[row];
      if (EPI == kEpiBicgOmega) {
        v[0] += yi * w[row];
        v[1] += yi * yi;
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

template <class T>
__global__ void permute_kernel(int64_t n, const int32_t *__restrict__ pt,
                               const T *__restrict__ src, T *__restrict__ dst) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = src[pt[q]];
}

int gather_grid(int neq, int lanes) {
  const int rpb = 256 / lanes;
  const int g = (neq + rpb - 1) / rpb;
  const int cap = grid_cap(32);  // fixed upper bound: 32 CTAs per SM
  return g < cap ? (g < 1 ? 1 : g) : cap;
}

template <class T, int EPI>
void launch_gather(const CsrcDev &k, const T *al, const T *alt, const T *ad, const T *x, T *y,
                   const T *w, PcgScalars *sc, double *partials, unsigned int *counter,
                   cudaStream_t st, const int32_t *gate = nullptr) {
  if (k.bsize > 0) {  // node blocks
    launch_bcsr<T, EPI>(k, x, y, w, sc, partials, counter, gate, st);
    return;
  }
  // 4 threads per row and 4 entries in flight per thread measured fastest on
  // the 64^3 HEXA8 cube (lanes 2/4/8 x unroll 2/4 swept: 166.8 us vs >= 174 us)
  // a gated product (run only when *gate != 0) is launched with one wave of
  // CTAs, so that it costs little when the gate is closed
  int grid = gather_grid(k.neq, 4);
  if (k.gather_blocks > 0) grid = std::min(grid, k.gather_blocks);
  if (gate) grid = std::min(grid, k.max_grid);
  if (k.ja16)
    gather_spmv_kernel<T, 4, 4, EPI, 0, true><<<grid, 256, 0, st>>>(
        k.neq, k.ia, k.ja, al, k.iat, k.jat, alt, ad, x, y, w, sc, partials, counter, gate,
        k.ja16, k.jat16);
  else
    gather_spmv_kernel<T, 4, 4, EPI><<<grid, 256, 0, st>>>(k.neq, k.ia, k.ja, al, k.iat, k.jat,
                                                           alt, ad, x, y, w, sc, partials,
                                                           counter, gate);
  ELX_CUDA(cudaGetLastError());
}

__global__ void demote_kernel(int64_t n, const double *__restrict__ src, float *__restrict__ dst) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = (float)src[q];
}

int g_num_sms = 0;

template <class T>
void launch_tile(const CsrcDev &k, const TileDev &t, const T *al, const T *ad, const T *x,
                 T *ytile, T *part, int32_t *err, const PcgScalars *sc, cudaStream_t st) {
  const int vs = sizeof(T);
  const PipeLayout L = pipe_layout(t.max_nnz, t.max_tgt, t.rows, vs);
  const size_t smem = pipe_header(t.rows, vs) + (size_t)kStages * L.bytes;
  // two CTAs per SM, so that one CTA's barriers overlap the other's arithmetic
  const int grid = std::min(t.ntiles, 2 * (g_num_sms > 0 ? g_num_sms : 148));
  // ELX_PIPE_STALL_TEST=1: the waits run out on purpose (tests of the
  // timeout path; read at every launch)
  const char *env = getenv("ELX_PIPE_STALL_TEST");
  const int stall = env && atoi(env) == 1 ? 1 : 0;
  spmv_pipe_kernel<T><<<grid, kPipeThreads, smem, st>>>(al, ad, k.ja, k.ia, t, L, x, ytile, part,
                                                       err, stall, sc);
  ELX_CUDA(cudaGetLastError());
}

}  // namespace

size_t pipe_smem_bytes(int max_nnz, int max_tgt, int rows, bool fp32) {
  const int vs = fp32 ? 4 : 8;
  return pipe_header(rows, vs) + (size_t)kStages * pipe_layout(max_nnz, max_tgt, rows, vs).bytes;
}

size_t tile_smem_bytes(const TileDev &t, bool fp32) {
  return pipe_smem_bytes(t.max_nnz, t.max_tgt, t.rows, fp32);
}

// Opt in to the kernels' shared memory once per structure (outside any stream
// capture) and record the SM count for the persistent grid.
void prepare_tile_kernels(const TileDev &t) {
  const size_t s64 = tile_smem_bytes(t, false), s32 = tile_smem_bytes(t, true);
  ELX_REQUIRE(s64 <= 113 * 1024, ELX_ERR_ARG, "SpMV tile needs more shared memory than half an SM");
  ELX_CUDA(cudaFuncSetAttribute(spmv_pipe_kernel<double>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s64));
  ELX_CUDA(cudaFuncSetAttribute(spmv_pipe_kernel<float>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s32));
  int dev = 0;
  ELX_CUDA(cudaGetDevice(&dev));
  ELX_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
}

void launch_tile_spmv64(const CsrcDev &k, const TileDev &t, const double *x, double *ytile,
                        double *part, int32_t *err, cudaStream_t st, const PcgScalars *sc) {
  launch_tile<double>(k, t, k.al, k.ad, x, ytile, part, err, sc, st);
}

void launch_tile_spmv32(const CsrcDev &k, const TileDev &t, const float *x, float *ytile,
                        float *part, int32_t *err, cudaStream_t st) {
  launch_tile<float>(k, t, k.al32, k.ad32, x, ytile, part, err, nullptr, st);
}

// FP32 copies of ad, al and alt for the mixed-precision inner iteration.
void launch_demote_values(const CsrcDev &k, cudaStream_t st) {
  demote_kernel<<<grid_cap(4), 256, 0, st>>>(k.neq, k.ad, k.ad32);
  if (k.nad) {
    demote_kernel<<<grid_cap(8), 256, 0, st>>>(k.nad, k.al, k.al32);
    demote_kernel<<<grid_cap(8), 256, 0, st>>>(k.nad, k.alt, k.alt32);
  }
  ELX_CUDA(cudaGetLastError());
}

// alt = al permuted into column order (after every assembly or upload).
void launch_transpose_values(const CsrcDev &k, cudaStream_t st) {
  if (k.nad == 0) return;
  permute_kernel<double><<<grid_cap(8), 256, 0, st>>>(k.nad, k.pt, k.al, k.alt);
  ELX_CUDA(cudaGetLastError());
}

void launch_gather_spmv64(const CsrcDev &k, const double *x, double *y, PcgScalars *sc,
                          double *partials, unsigned int *counter, cudaStream_t st,
                          const int32_t *gate) {
  if (sc)
    launch_gather<double, kEpiPcg>(k, k.al, k.alt, k.ad, x, y, nullptr, sc, partials, counter,
                                   st, gate);
  else
    launch_gather<double, kEpiNone>(k, k.al, k.alt, k.ad, x, y, nullptr, nullptr, nullptr,
                                    nullptr, st, gate);
}

void launch_gather_spmv32(const CsrcDev &k, const float *x, float *y, PcgScalars *sc,
                          double *partials, unsigned int *counter, cudaStream_t st) {
  if (sc)
    launch_gather<float, kEpiPcg>(k, k.al32, k.alt32, k.ad32, x, y, nullptr, sc, partials,
                                  counter, st);
  else
    launch_gather<float, kEpiNone>(k, k.al32, k.alt32, k.ad32, x, y, nullptr, nullptr, nullptr,
                                   nullptr, st);
}

void launch_gather_epi64(const CsrcDev &k, int epi, const double *x, double *y, const double *w,
                         PcgScalars *sc, double *partials, unsigned int *counter,
                         const int32_t *gate, cudaStream_t st) {
  switch (epi) {
    case kEpiNone:
      launch_gather<double, kEpiNone>(k, k.al, k.alt, k.ad, x, y, w, sc, partials, counter, st,
                                      gate);
      break;
    case kEpiPcg:
      launch_gather<double, kEpiPcg>(k, k.al, k.alt, k.ad, x, y, w, sc, partials, counter, st,
                                     gate);
      break;
    case kEpiBicgAlpha:
      launch_gather<double, kEpiBicgAlpha>(k, k.al, k.alt, k.ad, x, y, w, sc, partials, counter,
                                           st, gate);
      break;
    case kEpiBicgOmega:
      launch_gather<double, kEpiBicgOmega>(k, k.al, k.alt, k.ad, x, y, w, sc, partials, counter,
                                           st, gate);
      break;
    case kEpiScale:
      launch_gather<double, kEpiScale>(k, k.al, k.alt, k.ad, x, y, w, sc, partials, counter, st,
                                       gate);
      break;
    default:
      throw Error{ELX_ERR_ARG, "unknown SpMV epilogue"};
  }
}

}  // namespace elx

// ---------------------------------------------------------------------------
// Allocation-free entry point.
//
// Some callers cannot let a library allocate device memory: a driver that,
// like the reference's own memory manager (one pool for everything), carves
// all device arrays out of a pool it allocated once; code that runs where
// cudaMalloc is not allowed or would synchronise the device in the middle of
// an asynchronous pipeline.  elx_spmv_dot_noalloc serves them: the caller
// passes every input and output as device pointers, and the only scratch the
// kernel needs -- one partial sum per block, the last-block ticket and the
// scalar slot of the fused dot product -- lives in the file-scope array
// below, which every GPU that loads this library holds until the process
// exits.
namespace elx {
namespace {

constexpr int kNoAllocMaxBlocks = 16384;          // partial sums in the scratch
constexpr int kNoAllocRowsPerBlock = 256 / 4;     // rows per block of the kernel
constexpr int64_t kNoAllocMaxRows = (int64_t)kNoAllocMaxBlocks * kNoAllocRowsPerBlock;

struct NoAllocScratch {
  double partials[kNoAllocMaxBlocks];
  PcgScalars scalars;
  unsigned int counter;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of the scratch per device (in the device's primary
// context), looked up once per device.  Two host threads making their first
// call on one device at once both look it up and store the same address.
constexpr int kMaxDevices = 64;
std::atomic<NoAllocScratch *> g_noalloc_addr[kMaxDevices];

}  // namespace
}  // namespace elx

extern "C" int elx_spmv_dot_noalloc(int32_t neq, const int32_t *ia, const int32_t *ja,
                                    const double *ad, const double *al, const int32_t *iat,
                                    const int32_t *jat, const double *alt, const double *x,
                                    double *y, double *xy, void *stream) {
  using namespace elx;
  if (neq <= 0 || (int64_t)neq > kNoAllocMaxRows) return ELX_ERR_ARG;
  if (!ia || !ja || !ad || !al || !iat || !jat || !alt || !x || !y || !xy) return ELX_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ELX_ERR_CUDA;
  NoAllocScratch *sc = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (!sc) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return ELX_ERR_CUDA;
    sc = static_cast<NoAllocScratch *>(p);
    g_noalloc_addr[dev].store(sc, std::memory_order_release);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the scalars and the ticket must start at zero (done = 0 lets the kernel
  // run; the ticket counts the blocks that have published their partials)
  if (cudaMemsetAsync(&sc->scalars, 0, sizeof(PcgScalars), st) != cudaSuccess ||
      cudaMemsetAsync(&sc->counter, 0, sizeof(unsigned int), st) != cudaSuccess)
    return ELX_ERR_CUDA;
  const int grid = (neq + kNoAllocRowsPerBlock - 1) / kNoAllocRowsPerBlock;
  gather_spmv_kernel<double, 4, 4, kEpiPcg, 1><<<grid, 256, 0, st>>>(
      neq, ia, ja, al, iat, jat, alt, ad, x, y, nullptr, &sc->scalars, sc->partials,
      &sc->counter, nullptr);
  if (cudaGetLastError() != cudaSuccess) return ELX_ERR_CUDA;
  if (cudaMemcpyAsync(xy, &sc->scalars.pq, sizeof(double), cudaMemcpyDeviceToDevice, st) !=
      cudaSuccess)
    return ELX_ERR_CUDA;
  return ELX_OK;
}
