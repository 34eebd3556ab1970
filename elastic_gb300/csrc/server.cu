// Solve server: a request loop over many meshes at once, with continuous
// batching of their PCG iterations.
//
// A request is a mesh, its boundary conditions and nrhs load cases (nodal
// forces), solved to a tolerance with the reference's Jacobi PCG (pcg,
// mef/src/Iters.f:252-524) in FP64; its answer is the nodal displacement of
// every load case (update_mec, Predict.f:183-209).  The server
//   * builds each request's structure on a pool of host threads (node graph,
//     RCM, numeq, CSRC pattern, element colouring, node blocks), while the
//     GPU works on earlier requests;
//   * admits a prepared request when its device memory fits the HBM budget
//     next to the requests already resident, gives it its own context
//     (matrix, preconditioner, Krylov vectors stay resident until it is
//     done) and assembles it on the context's stream, overlapping the
//     iterations of the others;
//   * runs one PCG iteration of every active (request, load case) slot as
//     three packed launches -- the SpMV with (p, q), the update with (r, M r)
//     and the direction -- over all slots at once, each slot with its own
//     scalars and its own stopping test (a converged slot's blocks return at
//     once and the slot leaves the pack at the next poll);
//   * lets new requests join the pack between polls (every few iterations),
//     so that slots and memory freed by finished requests are reused at once.
//
// A slot's blocks, rows per block and partial sums depend only on the slot,
// never on its neighbours in the pack, so a result is bitwise the same alone
// and in any mix.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "elx_context.h"
#include "elx_gate.h"
#include "elx_reduce.cuh"

namespace elx {

// One (request, load case) in the pack.
struct SlotScalars {
  double d, alpha, beta, pq, conv;
  int32_t iters, done, status, maxit;
  uint32_t ticket[4];
};

struct SlotDesc {
  const int32_t *sell_ptr, *sell_col;  // the request's sliced FP64 node blocks
  const double *sval, *m;
  double *x, *r, *p, *q;
  SlotScalars *sc;
  int32_t bsize, n, nb;
  int32_t cta0, ncta;    // this slot's blocks in the packed vector launches
  int32_t scta0, sncta;  // and in the packed product (8 slices per block)
};

namespace {

constexpr int kRowsPerCta = kThreads;  // one row per thread

// The slot of a block: cta0 (vector launches) or scta0 (the product).
template <bool PRODUCT>
__device__ __forceinline__ int find_slot(const SlotDesc *d, int nslots, int cta) {
  int lo = 0, hi = nslots - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((PRODUCT ? d[mid].scta0 : d[mid].cta0) <= cta) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The slot's last block to arrive adds the slot's block partials in order;
// returns true in that block (all threads), with the total in thread 0.
__device__ __forceinline__ bool slot_reduce(double v, const SlotDesc &D, int cta0, int ncta,
                                            int phase, double *partials, double &tot) {
  double vv[1] = {v};
  block_sum<1>(vv);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = vv[0];
    __threadfence();
    last = atomicAdd(&D.sc->ticket[phase], 1u) == (unsigned)ncta - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double t[1] = {0.0};
#pragma unroll 4
  for (int b = threadIdx.x; b < ncta; b += kThreads) t[0] += __ldcg(partials + cta0 + b);
  block_sum<1>(t);
  if (threadIdx.x == 0) {
    tot = t[0];
    D.sc->ticket[phase] = 0u;
  }
  return true;
}

// One block row of the slot's sliced FP64 copy (slot t of slice sl): the
// row sums of the single-solve product (sell_spmv_kernel), into y and (p, y).
template <int B>
__device__ __forceinline__ double slice_rows(const SlotDesc &D, int sl, int t) {
  constexpr int BB = B * B, R = kSliceRows, Q = BB / 2;
  const int g0 = D.sell_ptr[sl], g1 = D.sell_ptr[sl + 1];
  double acc[B];
#pragma unroll
  for (int a = 0; a < B; a++) acc[a] = 0.0;
  for (int g = g0; g < g1; g++) {
    const int J = D.sell_col[(size_t)g * R + t];
    const double *grp = D.sval + (size_t)g * BB * R;
    double bv[BB];
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const double2 c = __ldg(reinterpret_cast<const double2 *>(grp + q * 2 * R + 2 * t));
      bv[2 * q] = c.x;
      bv[2 * q + 1] = c.y;
    }
#pragma unroll
    for (int e = 2 * Q; e < BB; e++) bv[e] = __ldg(grp + 2 * Q * R + (e - 2 * Q) * R + t);
    double xv[B];
#pragma unroll
    for (int b = 0; b < B; b++) xv[b] = D.p[J * B + b];
#pragma unroll
    for (int a = 0; a < B; a++)
#pragma unroll
      for (int b = 0; b < B; b++) acc[a] += bv[a * B + b] * xv[b];
  }
  const int I = sl * R + t;
  double v = 0.0;
  if (I < D.nb) {
#pragma unroll
    for (int a = 0; a < B; a++) {
      const int row = I * B + a;
      D.q[row] = acc[a];
      v += D.p[row] * acc[a];
    }
  }
  return v;
}

// q = K p and (p, q) for every slot; alpha = d / (p, q)   (Iters.f:366-372)
// One warp per slice of the slot's sliced copy, 8 slices per block.
__global__ void __launch_bounds__(kThreads)
packed_spmv_kernel(const SlotDesc *desc, int nslots, double *partials) {
  const SlotDesc D = desc[find_slot<true>(desc, nslots, blockIdx.x)];
  if (D.sc->done) return;
  const int sl = (blockIdx.x - D.scta0) * (kThreads / kSliceRows) + threadIdx.x / kSliceRows;
  const int nsl = (D.nb + kSliceRows - 1) / kSliceRows;
  double v = 0.0;
  if (sl < nsl)
    v = D.bsize == 3 ? slice_rows<3>(D, sl, threadIdx.x % kSliceRows)
                     : slice_rows<2>(D, sl, threadIdx.x % kSliceRows);
  double tot;
  if (!slot_reduce(v, D, D.scta0, D.sncta, 0, partials, tot)) return;
  if (threadIdx.x == 0) {
    D.sc->pq = tot;
    D.sc->alpha = D.sc->d / tot;
  }
}

// x += alpha p, r -= alpha q, d' = (r, M r), beta = d'/d and the stopping
// test sqrt|d'| < tol ||b||_M                               (Iters.f:377-419)
__global__ void __launch_bounds__(kThreads)
packed_update_kernel(const SlotDesc *desc, int nslots, double *partials) {
  const SlotDesc D = desc[find_slot<false>(desc, nslots, blockIdx.x)];
  if (D.sc->done) return;
  const int row = (blockIdx.x - D.cta0) * kRowsPerCta + threadIdx.x;
  double v = 0.0;
  if (row < D.n) {
    const double alpha = D.sc->alpha;
    D.x[row] += alpha * D.p[row];
    const double ri = D.r[row] - alpha * D.q[row];
    D.r[row] = ri;
    v = ri * (ri * D.m[row]);
  }
  double tot;
  if (!slot_reduce(v, D, D.cta0, D.ncta, 1, partials, tot)) return;
  if (threadIdx.x == 0) {
    SlotScalars &S = *D.sc;
    S.iters += 1;
    S.beta = tot / S.d;
    S.d = tot;
    if (sqrt(fabs(tot)) < S.conv) {
      S.done = 1;
    } else if (S.iters >= S.maxit || !(tot == tot)) {
      S.done = 1;
      S.status = ELX_ERR_NO_CONVERGENCE;
    }
  }
}

// p = M r + beta p                                          (Iters.f:411-414)
__global__ void __launch_bounds__(kThreads)
packed_direction_kernel(const SlotDesc *desc, int nslots) {
  const SlotDesc D = desc[find_slot<false>(desc, nslots, blockIdx.x)];
  if (D.sc->done) return;
  const int row = (blockIdx.x - D.cta0) * kRowsPerCta + threadIdx.x;
  if (row < D.n) D.p[row] = D.r[row] * D.m[row] + D.sc->beta * D.p[row];
}

// x = 0, r = b, p = M b, d = (b, M b), conv = tol sqrt|d| for one slot
// (Iters.f:343-360), launched on its request's stream over a fixed grid.
__global__ void __launch_bounds__(kThreads)
slot_start_kernel(int n, const double *__restrict__ b, const double *__restrict__ m,
                  double *__restrict__ x, double *__restrict__ r, double *__restrict__ p,
                  SlotScalars *S, double tol, int maxit, double *partials,
                  unsigned int *counter) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const double bi = b[i];
    x[i] = 0.0;
    r[i] = bi;
    p[i] = bi * m[i];
    v[0] += bi * (bi * m[i]);
  }
  block_sum<1>(v);
  if (!publish_partials<1>(v, partials, counter)) return;
  double tot[1];
  gather_partials<1>(tot, partials, counter);
  if (threadIdx.x == 0) {
    SlotScalars z{};
    z.d = tot[0];
    z.conv = tol * sqrt(fabs(tot[0]));
    z.maxit = maxit;
    if (tot[0] == 0.0) z.done = 1;  // b = 0: x = 0
    if (maxit <= 0 && !z.done) {
      z.done = 1;
      z.status = ELX_ERR_NO_CONVERGENCE;
    }
    *S = z;
  }
}

}  // namespace
}  // namespace elx

using namespace elx_api;
using elx::SlotDesc;
using elx::SlotScalars;

// ------------------------------------------------------------------ host side

struct SrvRequest {
  int64_t ticket = 0;
  elx::Mesh mesh;
  std::vector<int32_t> bc;
  int nrhs = 0;
  std::vector<double> f;  // nrhs x (ndf x nnode)
  double tol = 1e-8;
  int maxit = 10000;
  // submitted, prepared (host structure built), admission started and done
  // (device memory, uploads, assembly), solve started (joined the pack or
  // the block solve began), done
  double t_submit = 0, t_prepared = 0, t_admit0 = 0, t_admitted = 0, t_start = 0, t_done = 0;
  // host preparation
  elx::Structure s;
  std::vector<double> b0;  // nrhs x neq
  int64_t need_bytes = 0;
  int64_t charged = 0;  // bytes counted against the budget while resident
  bool counted = false;
  bool large = false;   // solved whole on its own stream (block PCG), not packed
  bool small_counted = false;  // counted among the gate's small requests
  // device state
  elx_ctx *ctx = nullptr;
  DBuf vecs;  // b (nrhs x neq), then per load case x, r, p, q
  cudaEvent_t ready = nullptr;
  std::vector<int> slots;  // indices into the server's slot scalars
  // result
  std::vector<double> u;  // nrhs x (ndf x nnode)
  std::vector<elx_info> infos;
  int status = ELX_OK;
  std::string err;
  bool done = false;
};

struct elx_server {
  int device = 0;
  int64_t budget = 0;
  int poll_steps = 8;
  int max_slots = 4096;
  int large_dofs = 100000;  // requests with at least this many equations ...
  int large_mode = 0;       // ... 0: auto (mixed in 3-D, FP64 in 2-D), 1: FP64, 2: mixed,
                            // -1: packed like the others
  cudaStream_t stream = nullptr;

  std::mutex mu;
  std::condition_variable cv_prep, cv_admit, cv_done;
  std::deque<std::shared_ptr<SrvRequest>> to_prep, prepared;
  std::map<int64_t, std::shared_ptr<SrvRequest>> all;
  int64_t next_ticket = 1;
  bool stopping = false;
  std::vector<std::thread> prep_threads, large_threads;
  std::vector<std::thread> admit_threads;
  std::thread loop_thread;
  std::condition_variable cv_large;
  std::deque<std::shared_ptr<SrvRequest>> large_ready;
  std::string fatal;

  // shared under mu: admitted requests ready to join, free slot indices,
  // bytes held by admitted requests
  std::deque<std::shared_ptr<SrvRequest>> joinable;
  std::vector<int> slot_free;
  int64_t used = 0;
  int resident = 0;  // admitted, not yet retired

  // GPU loop state (loop thread only)
  std::vector<std::shared_ptr<SrvRequest>> active;
  void *d_desc = nullptr, *d_part = nullptr;
  size_t desc_bytes = 0, part_bytes = 0;
  SlotScalars *d_sc = nullptr;   // max_slots
  SlotScalars *h_sc = nullptr;   // pinned copy
  SlotDesc *h_desc = nullptr;    // pinned, max_slots
  cudaEvent_t ev_poll = nullptr;

  // statistics
  std::atomic<int64_t> submitted{0}, completed{0}, peak_used{0}, peak_slots{0}, iterations{0},
      large_solved{0};
  bool pool_user = false;     // holds the device pool's memory while it lives
  // stream priority of the pack and of the packed requests' admissions (the
  // device's greatest; the block solves keep the default, its least), or 0
  // when ELX_SERVER_PRIORITY=0
  int prio_hi = 0;
  // batch gate of the block solves: while small requests are being admitted
  // or iterate in the pack, one block solve runs its iteration batches at a
  // time; otherwise all large workers do (ELX_SERVER_GATE=0: no gate)
  bool gate_on = true;
  elx::BatchGate gate;
  double phase_s[2][5] = {};  // under mu: per-phase seconds of finished requests
  int64_t phase_n[2] = {};    // (packed, block) and their count
};

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Device bytes a request will hold (the allocations of upload_structure,
// the assembly and the per-load-case vectors), from its prepared structure.
int64_t estimate_bytes(const SrvRequest &q) {
  const elx::Mesh &m = q.mesh;
  const elx::Structure &s = q.s;
  const int64_t n = s.neq, nad = s.nad, nen = m.nen, numel = m.numel;
  int64_t b = 0;
  b += 4 * nen * numel + 8 * numel + 4 * (int64_t)s.slot.size() + 8 * (int64_t)m.x.size() +
       4 * (int64_t)s.id.size() + 8 * (int64_t)m.e.size();
  // ia, the node-block pattern (bia, bt), the sliced FP64 copy (values,
  // columns, 16-bit offsets, pointers), ad, al
  const int64_t slots = (int64_t)s.sell_ptr[s.nslices] * elx::kSliceRows;
  b += 4 * (n + 1) + 4 * (s.nb + 1) + 4 * s.nnzb;
  b += 8 * slots * s.bsize * s.bsize + 6 * slots + 4 * (s.nslices + 1) + 6 * 64;
  b += 8 * n + 8 * nad;
  b += 8 * (int64_t)(m.ndf * m.nnode) + 8 * 8 * n;     // u, b0, b, x, r, p, q, m, z
  if (q.large) {
    // block PCG of up to 16 columns: b, x in the request's buffer; block
    // multi-vectors (7 FP64, 4 FP32 per column), the sliced FP32 copy and
    // the FP32 vectors
    int w = 1;
    while (w < q.nrhs && w < 16) w *= 2;
    b += 2 * 8 * n * q.nrhs + 7 * 8 * n * w + 4 * 4 * n * w;
    b += 4 * slots * s.bsize * s.bsize + 5 * 4 * n;
    b += 8 * 2 * 16 * elx::grid_cap(8) + (64 << 10);
  } else {
    b += 5 * 8 * n * q.nrhs;                           // per load case
  }
  b += 160 << 10;                                      // scalars, partials, padding
  return b;
}

void prep_request(SrvRequest &q) {
  // graph -> RCM -> numeq -> CSRC pattern -> colouring, slot map, node blocks
  std::vector<int32_t> xadj, adj, perm0;
  elx::Structure &s = q.s;
  elx::node_graph(q.mesh, xadj, adj);
  elx::rcm_order(q.mesh.nnode, xadj, adj, perm0);
  s.perm.resize(q.mesh.nnode);
  for (int i = 0; i < q.mesh.nnode; i++) s.perm[i] = perm0[i] + 1;
  s.neq = elx::number_equations(q.mesh, perm0, q.bc.data(), s.id);
  if (s.neq <= 0) throw Error{ELX_ERR_ARG, "no free equations"};
  elx::csrc_pattern(q.mesh, s, xadj, adj, s.ia, s.ja);
  s.nad = (int64_t)s.ia[s.neq] - 1;
  if (s.nad >= INT32_MAX) throw Error{ELX_ERR_ARG, "nad exceeds 32-bit indexing"};
  elx::derive_structure(q.mesh, s);
  elx::build_blocks(s, q.mesh.ndf);
  if (!s.blocked)
    throw Error{ELX_ERR_ARG, "served meshes need whole-node boundary conditions (node blocks)"};
  // load vectors (pload_mec, Pload.f:2-58): b0(id) = f on the free dofs
  const size_t nd = (size_t)q.mesh.ndf * q.mesh.nnode;
  q.b0.assign((size_t)q.nrhs * s.neq, 0.0);
  for (int k = 0; k < q.nrhs; k++)
    for (size_t j = 0; j < nd; j++)
      if (s.id[j] > 0) q.b0[(size_t)k * s.neq + s.id[j] - 1] = q.f[k * nd + j];
  q.f.clear();
  q.f.shrink_to_fit();
}

void finish(elx_server *sv, const std::shared_ptr<SrvRequest> &q) {
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (q->t_done == 0) q->t_done = now_s();
    if (q->status == ELX_OK && q->t_start > 0) {
      const int k = q->large ? 1 : 0;
      const double t[6] = {q->t_submit, q->t_prepared, q->t_admit0, q->t_admitted, q->t_start,
                           q->t_done};
      for (int i = 0; i < 5; i++) sv->phase_s[k][i] += t[i + 1] - t[i];
      sv->phase_n[k]++;
    }
    q->done = true;
    q->mesh = elx::Mesh{};
    q->s = elx::Structure{};
    q->b0.clear();
    q->f.clear();
  }
  sv->completed++;
  sv->cv_done.notify_all();
}

void prep_worker(elx_server *sv) {
  for (;;) {
    std::shared_ptr<SrvRequest> q;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_prep.wait(lk, [&] { return sv->stopping || !sv->to_prep.empty(); });
      if (sv->stopping) return;
      q = sv->to_prep.front();
      sv->to_prep.pop_front();
    }
    try {
      prep_request(*q);
      q->large = sv->large_mode >= 0 && q->s.neq >= sv->large_dofs;
      q->need_bytes = estimate_bytes(*q);
      q->t_prepared = now_s();
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->prepared.push_back(q);
    } catch (const Error &e) {
      q->status = e.code;
      q->err = e.msg;
      finish(sv, q);
      continue;
    } catch (const std::bad_alloc &) {
      q->status = ELX_ERR_OOM;
      q->err = "host allocation failed";
      finish(sv, q);
      continue;
    }
    sv->cv_admit.notify_all();
  }
}

// The block solves' batch gate (elx_ctx::batch_gate of large requests).
void block_gate(void *user, int enter) {
  auto *sv = static_cast<elx_server *>(user);
  if (enter)
    sv->gate.enter();
  else
    sv->gate.leave();
}

// Frees a request's device state, slots and budget share.
void release_request(elx_server *sv, SrvRequest &q) {
  if (q.ready) cudaEventDestroy(q.ready);
  q.ready = nullptr;
  if (q.small_counted) sv->gate.small(-1);
  q.small_counted = false;
  if (q.ctx) {
    q.ctx->release(q.vecs);
    elx_destroy(q.ctx);
    q.ctx = nullptr;
  }
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    for (int i : q.slots) sv->slot_free.push_back(i);
    q.slots.clear();
    sv->used -= q.charged;
    q.charged = 0;
    if (q.counted) sv->resident--;
    q.counted = false;
  }
  sv->cv_admit.notify_all();
}

// Context, uploads, assembly, preconditioner and slot starts of an admitted
// request, all on the request's own stream; `ready` marks their end.
void admit(elx_server *sv, SrvRequest &q) {
  elx_opts o{};
  o.device = sv->device;
  int st = elx_create(&q.ctx, &o);
  if (st != ELX_OK) throw Error{st, "context creation failed"};
  elx_ctx *c = q.ctx;
  if (q.large && sv->gate_on) {
    c->batch_gate = block_gate;
    c->batch_gate_user = sv;
  }
  if (!q.large && sv->prio_hi != 0) {
    // a small request's uploads, assembly and slot starts ahead of the block
    // solves (nothing is queued on the context's stream yet)
    ELX_CUDA(cudaStreamDestroy(c->stream));
    c->stream = nullptr;
    ELX_CUDA(cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, sv->prio_hi));
  }
  c->mesh = std::move(q.mesh);
  c->s = std::move(q.s);
  c->have_mesh = true;
  upload_structure(c, true);
  require(c->use_blocks, ELX_ERR_ARG, "served meshes need node blocks");
  assemble_resident(c);  // u = 0, b0 = 0: K only (the loads are the slots' b)
  build_preconditioner(c);
  const size_t n = (size_t)c->s.neq;
  if (!q.large) {
    // the packed product reads the sliced FP64 copy
    require(c->sell_val64.p != nullptr, ELX_ERR_STATE, "sliced FP64 node blocks missing");
  }
  if (q.large) {
    // b and x of all load cases (column-major) for the request's block solve
    c->alloc(q.vecs, 2 * n * q.nrhs * 8);
    ELX_CUDA(cudaMemcpyAsync(q.vecs.p, q.b0.data(), n * q.nrhs * 8, cudaMemcpyHostToDevice,
                             c->stream));
    ELX_CUDA(cudaEventCreateWithFlags(&q.ready, cudaEventDisableTiming));
    ELX_CUDA(cudaEventRecord(q.ready, c->stream));
    ELX_CUDA(cudaEventSynchronize(q.ready));
    q.b0.clear();
    q.b0.shrink_to_fit();
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->peak_used = std::max<int64_t>(sv->peak_used.load(), sv->used);
    return;  // the estimate stays charged: the block buffers come with the solve
  }
  c->alloc(q.vecs, 5 * n * q.nrhs * 8);
  ELX_CUDA(cudaMemcpyAsync(q.vecs.p, q.b0.data(), n * q.nrhs * 8, cudaMemcpyHostToDevice,
                           c->stream));
  double *base = q.vecs.as<double>();
  for (int k = 0; k < q.nrhs; k++) {
    double *b = base + (size_t)k * n;
    double *x = base + n * q.nrhs + (size_t)k * 4 * n;
    elx::slot_start_kernel<<<elx::vector_grid((int)n), elx::kThreads, 0, c->stream>>>(
        (int)n, b, c->m.as<double>(), x, x + n, x + 2 * n, sv->d_sc + q.slots[k], q.tol,
        q.maxit, c->partials.as<double>(), c->counters.as<unsigned int>() + 7);
  }
  ELX_CUDA(cudaGetLastError());
  c->launches += q.nrhs;
  ELX_CUDA(cudaEventCreateWithFlags(&q.ready, cudaEventDisableTiming));
  ELX_CUDA(cudaEventRecord(q.ready, c->stream));
  ELX_CUDA(cudaEventSynchronize(q.ready));  // this thread only; the pack runs on
  q.b0.clear();
  q.b0.shrink_to_fit();
  // the budget counts what the context really holds
  std::lock_guard<std::mutex> lk(sv->mu);
  sv->used += c->used - q.charged;
  q.charged = c->used;
  sv->peak_used = std::max<int64_t>(sv->peak_used.load(), sv->used);
}

// Results of a finished request: x per load case -> nodal displacements
// (update_mec, Predict.f:183-209).
void collect(elx_server *sv, SrvRequest &q) {
  elx_ctx *c = q.ctx;
  const size_t n = (size_t)c->s.neq;
  const size_t nd = (size_t)c->mesh.ndf * c->mesh.nnode;
  std::vector<double> x(n * q.nrhs);
  const double *base = q.vecs.as<double>() + n * q.nrhs;
  for (int k = 0; k < q.nrhs; k++)
    ELX_CUDA(cudaMemcpyAsync(x.data() + (size_t)k * n, base + (size_t)k * 4 * n, n * 8,
                             cudaMemcpyDeviceToHost, c->stream));
  ELX_CUDA(cudaStreamSynchronize(c->stream));
  q.u.assign(nd * q.nrhs, 0.0);
  q.infos.assign(q.nrhs, elx_info{});
  for (int k = 0; k < q.nrhs; k++) {
    for (size_t j = 0; j < nd; j++) {
      const int e = c->s.id[j];
      q.u[k * nd + j] = e > 0 ? x[(size_t)k * n + e - 1] : 0.0;
    }
    const SlotScalars &S = sv->h_sc[q.slots[k]];
    elx_info &in = q.infos[k];
    in.iters = S.iters;
    in.status = S.done ? S.status : ELX_ERR_NO_CONVERGENCE;
    in.conv = S.conv;
    in.norm_m_r = std::sqrt(std::fabs(S.d));  // the recursive residual at the stop
    if (in.status != ELX_OK && q.status == ELX_OK) {
      q.status = in.status;
      q.err = "no convergence";
    }
  }
  q.t_done = now_s();
}

// Admission: prepared requests in arrival order, each once its estimated
// bytes fit the budget next to the resident ones (or the server is empty),
// built up on its own stream while the pack keeps running.
void admit_loop(elx_server *sv) {
  try {
    ELX_CUDA(cudaSetDevice(sv->device));
    for (;;) {
      std::shared_ptr<SrvRequest> q;
      bool reject = false;
      {
        std::unique_lock<std::mutex> lk(sv->mu);
        sv->cv_admit.wait(lk, [&] {
          if (sv->stopping) return true;
          if (sv->prepared.empty()) return false;
          const auto &h = sv->prepared.front();
          const bool fits_mem = sv->budget <= 0 || sv->used + h->need_bytes <= sv->budget;
          const bool fits_slots = h->large || (int)sv->slot_free.size() >= h->nrhs;
          const bool idle = sv->resident == 0;
          return (fits_mem && fits_slots) ||
                 (idle && (!fits_mem || (!h->large && h->nrhs > sv->max_slots)));
        });
        if (sv->stopping) return;
        q = sv->prepared.front();
        sv->prepared.pop_front();
        const bool fits_mem = sv->budget <= 0 || sv->used + q->need_bytes <= sv->budget;
        if (!fits_mem || (!q->large && q->nrhs > sv->max_slots)) {
          reject = true;
        } else {
          for (int k = 0; !q->large && k < q->nrhs; k++) {
            q->slots.push_back(sv->slot_free.back());
            sv->slot_free.pop_back();
          }
          // hold the estimate until the real footprint is known
          q->charged = q->need_bytes;
          sv->used += q->charged;
          sv->resident++;
          q->counted = true;
        }
      }
      if (reject) {
        q->status = ELX_ERR_OOM;
        q->err = "request needs more device memory or slots than the server has";
        finish(sv, q);
        continue;
      }
      try {
        q->t_admit0 = now_s();
        if (!q->large) {
          sv->gate.small(1);
          q->small_counted = true;
        }
        admit(sv, *q);
        q->t_admitted = now_s();
        {
          std::lock_guard<std::mutex> lk(sv->mu);
          (q->large ? sv->large_ready : sv->joinable).push_back(q);
        }
        sv->cv_admit.notify_all();
        sv->cv_large.notify_all();
      } catch (const Error &e) {
        q->status = e.code;
        q->err = e.msg;
        release_request(sv, *q);
        finish(sv, q);
      }
    }
  } catch (const Error &e) {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->fatal = e.msg;
    sv->stopping = true;
  }
  sv->cv_done.notify_all();
  sv->cv_admit.notify_all();
}

// Large requests: each solved whole on its context's stream by the block PCG
// (all its load cases over one matrix read per iteration; width fixed by the
// number of load cases, so the result does not depend on what else runs),
// several at once on different streams next to the pack.
void large_loop(elx_server *sv) {
  for (;;) {
    std::shared_ptr<SrvRequest> q;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_large.wait(lk, [&] { return sv->stopping || !sv->large_ready.empty(); });
      if (sv->stopping) return;
      q = sv->large_ready.front();
      sv->large_ready.pop_front();
    }
    try {
      q->t_start = now_s();
      ELX_CUDA(cudaSetDevice(sv->device));
      elx_ctx *c = q->ctx;
      const size_t n = (size_t)c->s.neq;
      int w = 1;
      while (w < q->nrhs && w < 16) w *= 2;
      const double *b = q->vecs.as<double>();
      double *x = q->vecs.as<double>() + n * q->nrhs;
      q->infos.assign(q->nrhs, elx_info{});
      try {
        // auto (0): mixed in 3-D; FP64 in 2-D, where the FP32 iteration needs
        // about twice the FP64 iterations and diverges above ~3e5 dofs (2-D
        // plane-stress strips of 58k / 141k / 361k dofs: 2.0x / 3.2x the
        // FP64 time, then an FP64 fallback)
        const bool mixed = sv->large_mode == 2 || (sv->large_mode == 0 && c->mesh.ndm == 3);
        solve_block(c, q->nrhs, mixed ? ELX_PREC_MIXED : ELX_PREC_FP64, q->tol, q->maxit, w, b, x,
                    q->infos.data(), true);
      } catch (const Error &e) {
        if (e.code != ELX_ERR_NO_CONVERGENCE) throw;
        q->status = e.code;
        q->err = e.msg;
      }
      std::vector<double> xh(n * q->nrhs);
      ELX_CUDA(cudaMemcpyAsync(xh.data(), x, n * q->nrhs * 8, cudaMemcpyDeviceToHost, c->stream));
      ELX_CUDA(cudaStreamSynchronize(c->stream));
      const size_t nd = (size_t)c->mesh.ndf * c->mesh.nnode;
      q->u.assign(nd * q->nrhs, 0.0);
      for (int k = 0; k < q->nrhs; k++)
        for (size_t j = 0; j < nd; j++) {
          const int e = c->s.id[j];
          q->u[k * nd + j] = e > 0 ? xh[(size_t)k * n + e - 1] : 0.0;
        }
      {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->peak_used = std::max<int64_t>(sv->peak_used.load(), sv->used);
      }
      sv->large_solved++;
    } catch (const Error &e) {
      q->status = e.code;
      q->err = e.msg;
    }
    q->t_done = now_s();
    release_request(sv, *q);
    finish(sv, q);
  }
}

// The pack: joins admitted requests, runs poll_steps packed PCG iterations
// of all active load cases, retires finished requests; repeats.
void gpu_loop(elx_server *sv) {
  try {
    ELX_CUDA(cudaSetDevice(sv->device));
    int nslots = 0, grid = 0, sgrid = 0;
    bool repack = false;
    for (;;) {
      // 1. admitted requests join the pack
      {
        std::unique_lock<std::mutex> lk(sv->mu);
        if (sv->active.empty())
          sv->cv_admit.wait(lk, [&] { return sv->stopping || !sv->joinable.empty(); });
        if (sv->stopping) return;
        while (!sv->joinable.empty()) {
          sv->joinable.front()->t_start = now_s();
          sv->active.push_back(sv->joinable.front());
          sv->joinable.pop_front();
          repack = true;
        }
      }
      // 2. (re)pack: one descriptor per slot, blocks assigned slot by slot
      if (repack) {
        nslots = 0;
        grid = 0;
        sgrid = 0;
        for (auto &q : sv->active) {
          elx_ctx *c = q->ctx;
          const size_t n = (size_t)c->s.neq;
          double *base = q->vecs.as<double>() + n * q->nrhs;
          const int per_cta = elx::kThreads / elx::kSliceRows;
          for (int k = 0; k < q->nrhs; k++) {
            SlotDesc &d = sv->h_desc[nslots++];
            d.sell_ptr = c->sell_ptr.as<int32_t>();
            d.sell_col = c->sell_col.as<int32_t>();
            d.sval = c->sell_val64.as<double>();
            d.nb = c->s.nb;
            d.scta0 = sgrid;
            d.sncta = (c->s.nslices + per_cta - 1) / per_cta;
            sgrid += d.sncta;
            d.m = c->m.as<double>();
            d.x = base + (size_t)k * 4 * n;
            d.r = d.x + n;
            d.p = d.x + 2 * n;
            d.q = d.x + 3 * n;
            d.sc = sv->d_sc + q->slots[k];
            d.bsize = c->s.bsize;
            d.n = (int)n;
            d.cta0 = grid;
            d.ncta = (int)((n + elx::kThreads - 1) / elx::kThreads);
            grid += d.ncta;
          }
        }
        sv->peak_slots = std::max<int64_t>(sv->peak_slots.load(), nslots);
        const int pgrid = std::max(grid, sgrid);
        if ((size_t)pgrid * 8 > sv->part_bytes) {
          if (sv->d_part) cudaFree(sv->d_part);
          sv->d_part = nullptr;
          sv->part_bytes = 0;
          ELX_CUDA(cudaMalloc(&sv->d_part, (size_t)pgrid * 8 * 2));
          sv->part_bytes = (size_t)pgrid * 8 * 2;
        }
        ELX_CUDA(cudaMemcpyAsync(sv->d_desc, sv->h_desc, nslots * sizeof(SlotDesc),
                                 cudaMemcpyHostToDevice, sv->stream));
        repack = false;
      }
      // 3. poll_steps packed PCG iterations of every active load case
      const SlotDesc *dd = static_cast<const SlotDesc *>(sv->d_desc);
      double *part = static_cast<double *>(sv->d_part);
      for (int it = 0; it < sv->poll_steps; it++) {
        elx::packed_spmv_kernel<<<sgrid, elx::kThreads, 0, sv->stream>>>(dd, nslots, part);
        elx::packed_update_kernel<<<grid, elx::kThreads, 0, sv->stream>>>(dd, nslots, part);
        elx::packed_direction_kernel<<<grid, elx::kThreads, 0, sv->stream>>>(dd, nslots);
      }
      ELX_CUDA(cudaGetLastError());
      sv->iterations += sv->poll_steps;
      ELX_CUDA(cudaMemcpyAsync(sv->h_sc, sv->d_sc, sizeof(SlotScalars) * sv->max_slots,
                               cudaMemcpyDeviceToHost, sv->stream));
      ELX_CUDA(cudaEventRecord(sv->ev_poll, sv->stream));
      ELX_CUDA(cudaEventSynchronize(sv->ev_poll));
      // 4. retire the requests whose load cases have all stopped
      for (size_t i = 0; i < sv->active.size();) {
        auto q = sv->active[i];
        bool all = true;
        for (int k : q->slots) all = all && sv->h_sc[k].done;
        if (!all) {
          i++;
          continue;
        }
        try {
          collect(sv, *q);
        } catch (const Error &e) {
          q->status = e.code;
          q->err = e.msg;
        }
        sv->active.erase(sv->active.begin() + i);
        repack = true;
        release_request(sv, *q);
        finish(sv, q);
      }
    }
  } catch (const Error &e) {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->fatal = e.msg;
    sv->stopping = true;
  }
  sv->cv_done.notify_all();
  sv->cv_admit.notify_all();
}

}  // namespace

extern "C" {

int elx_server_create(elx_server **out, const elx_server_opts *opts) {
  if (!out) return ELX_ERR_ARG;
  *out = nullptr;
  elx_server *sv = new (std::nothrow) elx_server();
  if (!sv) return ELX_ERR_OOM;
  int nthreads = 4, nlarge = 2;
  if (opts) {
    sv->device = opts->device;
    sv->budget = opts->hbm_budget;
    if (opts->poll_steps > 0) sv->poll_steps = opts->poll_steps;
    if (opts->max_slots > 0) sv->max_slots = opts->max_slots;
    if (opts->prep_threads > 0) nthreads = opts->prep_threads;
    if (opts->large_dofs > 0) sv->large_dofs = opts->large_dofs;
    sv->large_mode = opts->large_mode;
    if (opts->large_workers > 0) nlarge = opts->large_workers;
  }
  sv->gate.set_workers(nlarge);
  const char *gate_env = std::getenv("ELX_SERVER_GATE");
  sv->gate_on = !(gate_env && std::atoi(gate_env) == 0);
  const cudaError_t e1 = cudaSetDevice(sv->device);
  cudaError_t e = e1;
  if (e == cudaSuccess) {
    // the request contexts' memory stays in the device pool between requests
    elx::device_pool(sv->device);
    elx::pool_users(sv->device, 1);
    sv->pool_user = true;
  }
  int least = 0, greatest = 0;
  if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  const char *prio_env = std::getenv("ELX_SERVER_PRIORITY");
  sv->prio_hi = prio_env && std::atoi(prio_env) == 0 ? 0 : greatest;
  if (e == cudaSuccess)
    e = cudaStreamCreateWithPriority(&sv->stream, cudaStreamNonBlocking, sv->prio_hi);
  if (e == cudaSuccess) e = cudaMalloc(&sv->d_sc, sizeof(SlotScalars) * sv->max_slots);
  if (e == cudaSuccess) e = cudaMemset(sv->d_sc, 0, sizeof(SlotScalars) * sv->max_slots);
  if (e == cudaSuccess) e = cudaMalloc(&sv->d_desc, sizeof(SlotDesc) * sv->max_slots);
  if (e == cudaSuccess)
    e = cudaHostAlloc(&sv->h_sc, sizeof(SlotScalars) * sv->max_slots, cudaHostAllocDefault);
  if (e == cudaSuccess)
    e = cudaHostAlloc(&sv->h_desc, sizeof(SlotDesc) * sv->max_slots, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sv->ev_poll, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    elx_server_destroy(sv);
    return ELX_ERR_CUDA;
  }
  for (int i = sv->max_slots - 1; i >= 0; i--) sv->slot_free.push_back(i);
  for (int i = 0; i < nthreads; i++) sv->prep_threads.emplace_back(prep_worker, sv);
  // admissions (uploads, assembly) of several requests at once, each on its
  // own context's stream, taken from the prepared queue in arrival order
  const char *adm_env = std::getenv("ELX_SERVER_ADMIT_THREADS");
  const int nadmit = adm_env && std::atoi(adm_env) > 0 ? std::atoi(adm_env) : 2;
  for (int i = 0; i < nadmit; i++) sv->admit_threads.emplace_back(admit_loop, sv);
  for (int i = 0; i < nlarge; i++) sv->large_threads.emplace_back(large_loop, sv);
  sv->loop_thread = std::thread(gpu_loop, sv);
  *out = sv;
  return ELX_OK;
}

void elx_server_destroy(elx_server *sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stopping = true;
  }
  sv->cv_prep.notify_all();
  sv->cv_admit.notify_all();
  sv->cv_done.notify_all();
  sv->cv_large.notify_all();
  for (auto &t : sv->prep_threads)
    if (t.joinable()) t.join();
  for (auto &t : sv->large_threads)
    if (t.joinable()) t.join();
  for (auto &t : sv->admit_threads)
    if (t.joinable()) t.join();
  if (sv->loop_thread.joinable()) sv->loop_thread.join();
  cudaSetDevice(sv->device);
  // the pack's last launches (a loop that stopped on an error) end before
  // the requests' memory goes back: their frees are ordered on the request
  // streams only
  if (sv->stream) cudaStreamSynchronize(sv->stream);
  for (auto &q : sv->active) release_request(sv, *q);
  for (auto &q : sv->joinable) release_request(sv, *q);
  for (auto &q : sv->large_ready) release_request(sv, *q);
  if (sv->d_sc) cudaFree(sv->d_sc);
  if (sv->d_desc) cudaFree(sv->d_desc);
  if (sv->d_part) cudaFree(sv->d_part);
  if (sv->h_sc) cudaFreeHost(sv->h_sc);
  if (sv->h_desc) cudaFreeHost(sv->h_desc);
  if (sv->ev_poll) cudaEventDestroy(sv->ev_poll);
  if (sv->stream) cudaStreamDestroy(sv->stream);
  if (sv->pool_user) elx::pool_users(sv->device, -1);
  delete sv;
}

int elx_server_submit(elx_server *sv, int32_t ndm, int32_t ndf, int32_t nen, int32_t numel,
                      int32_t nnode, const int32_t *ix, const double *x, const int32_t *ie,
                      const double *e, int32_t prop, int32_t numat, const int32_t *bc,
                      int32_t nrhs, const double *f, double tol, int32_t maxit,
                      int64_t *ticket) {
  if (!sv || !ticket) return ELX_ERR_ARG;
  try {
    require(ix && x && ie && e && bc && f, ELX_ERR_ARG, "null request array");
    require(nrhs >= 1 && tol > 0 && maxit >= 0, ELX_ERR_ARG, "bad request arguments");
    check_mesh(ndm, ndf, nen, numel, nnode, ix, ie, numat, prop);
    auto q = std::make_shared<SrvRequest>();
    fill_mesh(q->mesh, ndm, ndf, nen, numel, nnode, ix, x, ie, e, prop, numat);
    const size_t nd = (size_t)ndf * nnode;
    q->bc.assign(bc, bc + nd);
    q->f.assign(f, f + nd * nrhs);
    q->nrhs = nrhs;
    q->tol = tol;
    q->maxit = maxit;
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      if (sv->stopping) return ELX_ERR_STATE;
      q->ticket = sv->next_ticket++;
      q->t_submit = now_s();
      sv->all[q->ticket] = q;
      sv->to_prep.push_back(q);
    }
    sv->submitted++;
    sv->cv_prep.notify_one();
    *ticket = q->ticket;
    return ELX_OK;
  } catch (const Error &er) {
    return er.code;
  } catch (const std::bad_alloc &) {
    return ELX_ERR_OOM;
  }
}

int elx_server_wait(elx_server *sv, int64_t ticket, double timeout_s, double *u,
                    elx_info *info, double *latency_s) {
  if (!sv) return ELX_ERR_ARG;
  std::shared_ptr<SrvRequest> q;
  {
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->all.find(ticket);
    if (it == sv->all.end()) return ELX_ERR_ARG;
    q = it->second;
    auto ready = [&] { return q->done || !sv->fatal.empty(); };
    if (timeout_s < 0) {
      sv->cv_done.wait(lk, ready);
    } else if (!sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
      return ELX_ERR_TIMEOUT;
    }
    if (!q->done) return ELX_ERR_CUDA;  // the GPU loop stopped on an error
    sv->all.erase(ticket);
  }
  if (u && !q->u.empty()) std::memcpy(u, q->u.data(), q->u.size() * sizeof(double));
  if (info)
    for (size_t k = 0; k < q->infos.size(); k++) info[k] = q->infos[k];
  if (latency_s) *latency_s = q->t_done - q->t_submit;
  return q->status;
}

int elx_server_get_stats(elx_server *sv, elx_server_stats *st) {
  if (!sv || !st) return ELX_ERR_ARG;
  st->submitted = sv->submitted;
  st->completed = sv->completed;
  st->peak_bytes = sv->peak_used;
  st->peak_slots = sv->peak_slots;
  st->iterations = sv->iterations;
  st->large_solved = sv->large_solved;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    st->resident_bytes = sv->used;
    for (int k = 0; k < 2; k++) {
      st->phase_n[k] = sv->phase_n[k];
      for (int i = 0; i < 5; i++) st->phase_s[k][i] = sv->phase_s[k][i];
    }
  }
  return sv->fatal.empty() ? ELX_OK : ELX_ERR_CUDA;
}

}  // extern "C"
