// C ABI of the library (include/elastic_gb300.h): the context, host<->device
// staging and the orchestration of the assembly and solver kernels.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "elx_context.h"


namespace elx_api {

template <class F>
int guarded(elx_ctx *ctx, F &&f) {
  if (!ctx) return ELX_ERR_ARG;
  try {
    ELX_CUDA(cudaSetDevice(ctx->device));
    f();
    ctx->err.clear();
    return ELX_OK;
  } catch (const Error &e) {
    ctx->err = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    ctx->err = "host allocation failed";
    return ELX_ERR_OOM;
  }
}

void require(bool c, int code, const char *what) {
  if (!c) throw Error{code, what};
}

void release_block(elx_ctx *c) {
  for (DBuf *v : {&c->bk_b, &c->bk_x, &c->bk_r, &c->bk_p, &c->bk_q, &c->bk_z, &c->bk_xlo,
                  &c->bk_r32, &c->bk_p32, &c->bk_q32, &c->bk_cols, &c->bk_hdr, &c->bk_part,
                  &c->bk_cnt, &c->bk_diag, &c->bk_colmajor})
    c->release(*v);
  c->blk_cap = 0;
}

// Rows per SpMV tile: the largest candidate whose three-stage FP64 pipeline
// lets two CTAs share an SM's shared memory; ELX_TILE_ROWS overrides (tuning).
void choose_tiles(elx::Structure &s) {
  if (const char *env = getenv("ELX_TILE_ROWS")) {
    const int r = atoi(env);
    if (r >= 8 && r <= 256) {
      elx::build_tiles(s, r);
      ELX_REQUIRE(elx::pipe_smem_bytes(s.max_tile_nnz, s.max_tile_tgt, r, false) <= 113 * 1024,
                  ELX_ERR_ARG, "ELX_TILE_ROWS too large for shared memory");
      return;
    }
  }
  const double mean = s.neq ? (double)s.nad / s.neq : 0.0;
  for (int r : {96, 80, 64, 56, 48, 40, 32, 28, 24, 20, 16, 12, 8}) {
    // estimate first (cheap), then build and check the exact size
    if (r > 8 && elx::pipe_smem_bytes((int)(1.1 * mean * r) + 16, (int)(0.5 * mean * r) + 16, r,
                                      false) > 110 * 1024)
      continue;
    elx::build_tiles(s, r);
    if (elx::pipe_smem_bytes(s.max_tile_nnz, s.max_tile_tgt, r, false) <= 110 * 1024) return;
  }
  throw Error{ELX_ERR_ARG, "rows too long for the SpMV tiles"};
}

// Uploads everything the kernels need once the structure is known.
void upload_structure(elx_ctx *c, bool prederived) {
  const elx::Mesh &m = c->mesh;
  elx::Structure &s = c->s;
  c->drop_graphs();
  if (!prederived) elx::derive_structure(m, s);
  const int nen1 = m.nen + 1;
  std::vector<int32_t> conn((size_t)m.nen * m.numel), mat(m.numel), elnum(m.numel);
  for (int t = 0; t < m.numel; t++) {
    const int el = s.elem_order[t];
    for (int a = 0; a < m.nen; a++) {
      int no = m.ix[(size_t)el * nen1 + a];
      conn[(size_t)a * m.numel + t] = no > 0 ? no - 1 : 0;
    }
    mat[t] = m.ix[(size_t)el * nen1 + m.nen] - 1;
    elnum[t] = el + 1;
  }
  std::vector<int32_t> eq(s.id.size());
  for (size_t q = 0; q < eq.size(); q++) eq[q] = s.id[q] - 1;
  std::vector<int32_t> ia0(s.ia.size());
  for (size_t i = 0; i < ia0.size(); i++) ia0[i] = s.ia[i] - 1;
  c->upload(c->conn, conn.data(), conn.size());
  c->upload(c->mat, mat.data(), mat.size());
  c->upload(c->elnum, elnum.data(), elnum.size());
  c->upload(c->slot, s.slot.data(), s.slot.size());
  c->upload(c->x, m.x.data(), m.x.size());
  c->upload(c->eq, eq.data(), eq.size());
  c->upload(c->e, m.e.data(), m.e.size());
  c->upload(c->ia, ia0.data(), ia0.size());
  if (const char *env = getenv("ELX_DELTA16")) c->use_delta = atoi(env) != 0;
  if (const char *env = getenv("ELX_GATHER_BLOCKS")) c->gather_blocks = atoi(env);
  if (const char *env = getenv("ELX_SPMM_UNROLL")) c->spmm_unroll = atoi(env);
  c->spmv_kind = elx::kSpmvGather;
  if (const char *env = getenv("ELX_SPMV"))
    c->spmv_kind = std::string(env) == "tile" ? elx::kSpmvTiled : elx::kSpmvGather;
  // node blocks unless disabled (ELX_BLOCKS=0) or the tiled kernel is asked for
  bool want_blocks = c->spmv_kind == elx::kSpmvGather;
  if (const char *env = getenv("ELX_BLOCKS")) want_blocks = want_blocks && atoi(env) != 0;
  if (want_blocks && !prederived) elx::build_blocks(s, m.ndf);
  c->use_blocks = want_blocks && s.blocked;
  for (DBuf *v : {&c->iat, &c->jat, &c->pt, &c->ja16, &c->jat16, &c->tile_tgt, &c->tile_out,
                  &c->tgt_col, &c->tgt_start, &c->tpos, &c->halo_ptr, &c->halo_slot,
                  &c->tile_desc, &c->part, &c->alt, &c->ja, &c->bia, &c->bt, &c->sell_ptr,
                  &c->sell_col, &c->sell_val, &c->sell_val64, &c->sell_d16})
    c->release(*v);
  if (c->use_blocks) {
    // the node-block product replaces both scalar kernel families: the
    // sliced FP64 copy is the only device copy of the full block rows (the
    // fill reads the CSRC arrays through bia / bt); ja stays on the host
    s.tile_rows = s.ntiles = 0;
    s.bw16 = false;
    c->upload(c->bia, s.bia.data(), s.bia.size());
    c->upload(c->bt, s.bt.data(), s.bt.size());
    c->upload(c->sell_ptr, s.sell_ptr.data(), s.sell_ptr.size());
    c->upload(c->sell_col, s.sell_col.data(), s.sell_col.size());
    const size_t slots = (size_t)s.sell_ptr[s.nslices] * elx::kSliceRows;
    const size_t bytes64 = slots * s.bsize * s.bsize * 8;
    c->alloc(c->sell_val64, bytes64 + 64);
    int l2 = 0;
    ELX_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->device));
    // streaming loads unless the copy fits in 60 % of L2 (ELX_SELL_STREAM=0/1
    // forces either: 49.7 against 54.5 us for the FP32 copy of the 64^3 HEXA8
    // cube, 277 MB; 17.2 against 12.6 us on the 48^3 TETRA4 mesh, 64 MB)
    const double colb = (double)slots * 4;
    c->sell_stream = (double)bytes64 / 2 + colb > 0.6 * l2;
    c->sell64_stream = (double)bytes64 + colb > 0.6 * l2;
    if (const char *env = getenv("ELX_SELL_STREAM"))
      c->sell_stream = c->sell64_stream = atoi(env) != 0;
    // 16-bit column offsets when every block column is within 32767 block
    // rows of its row (RCM keeps the bandwidth small): half the index bytes
    // of a copy streamed from HBM (48.8 against 50.5 us for the FP32 product
    // on the 64^3 HEXA8 cube; a copy resident in L2 gains nothing: 12.6 us
    // either way on the 48^3 TETRA4 mesh)
    if (c->sell_stream) {
      const int R = elx::kSliceRows;
      std::vector<int16_t> d16(s.sell_col.size());
      bool fits = std::getenv("ELX_SELL_D16") == nullptr || std::atoi(std::getenv("ELX_SELL_D16"));
      for (int sl = 0; sl < s.nslices && fits; sl++)
        for (int32_t g = s.sell_ptr[sl]; g < s.sell_ptr[sl + 1] && fits; g++)
          for (int t = 0; t < R; t++) {
            const int I = sl * R + t;
            // rows past the matrix (last slice) read the last row's x
            const int J = I < s.nb ? s.sell_col[(size_t)g * R + t] : s.nb - 1;
            const int d = J - I;
            if (d < -32768 || d > 32767) {
              fits = false;
              break;
            }
            d16[(size_t)g * R + t] = (int16_t)d;
          }
      if (fits) c->upload(c->sell_d16, d16.data(), d16.size());
    }
    c->alloc(c->part, 16);
  } else {
    {
      std::vector<int32_t> ja0(s.ja.size());
      for (size_t i = 0; i < ja0.size(); i++) ja0[i] = s.ja[i] - 1;
      c->upload(c->ja, ja0.data(), ja0.size());
    }
    choose_tiles(s);
    elx::build_transpose(s);
    c->upload(c->iat, s.iat.data(), s.iat.size());
    c->upload(c->jat, s.jat.data(), s.jat.size());
    c->upload(c->pt, s.pt.data(), s.pt.size());
    if (s.bw16) {
      c->upload(c->ja16, s.ja16.data(), s.ja16.size());
      c->upload(c->jat16, s.jat16.data(), s.jat16.size());
    }
    c->upload(c->tile_tgt, s.tile_tgt.data(), s.tile_tgt.size());
    c->upload(c->tile_out, s.tile_out.data(), s.tile_out.size());
    c->upload(c->tgt_col, s.tgt_col.data(), s.tgt_col.size());
    c->upload(c->tgt_start, s.tgt_start.data(), s.tgt_start.size());
    c->upload(c->tpos, s.tpos.data(), s.tpos.size());
    c->upload(c->halo_ptr, s.halo_ptr.data(), s.halo_ptr.size());
    c->upload(c->halo_slot, s.halo_slot.data(), s.halo_slot.size());
    c->upload(c->tile_desc, s.tile_desc.data(), s.tile_desc.size());
    c->alloc(c->part, (size_t)s.tile_out[s.ntiles] * 8);
    elx::prepare_tile_kernels(c->tile_dev());
    c->alloc(c->alt, (size_t)s.nad * 8 + 64);
  }
  const size_t n = (size_t)s.neq, nad = (size_t)s.nad;
  c->alloc(c->ad, n * 8 + 64);
  c->alloc(c->al, nad * 8 + 64);
  for (DBuf *v : {&c->ad32, &c->al32, &c->alt32, &c->m32, &c->p32, &c->q32, &c->r32, &c->x32,
                  &c->r0v, &c->tv, &c->unit, &c->gbasis, &c->garrays, &c->gstate})
    c->release(*v);
  release_block(c);
  c->tuned_width[0] = c->tuned_width[1] = 0;
  for (auto &row : c->tuned_unroll)
    for (int &u : row) u = 0;
  for (DBuf *v : {&c->node_count, &c->tstress, &c->tx0buf, &c->fbuf, &c->ld_node, &c->ld_ptr,
                  &c->ld_ent, &c->ld_vec, &c->vtkbuf})
    c->release(*v);
  c->have_stress = false;
  release_partitions(c);
  c->have_fp32 = false;
  c->alloc(c->u, (size_t)m.ndf * m.nnode * 8);
  ELX_CUDA(cudaMemsetAsync(c->u.p, 0, c->u.bytes, c->stream));
  c->alloc(c->b0, n * 8);
  ELX_CUDA(cudaMemsetAsync(c->b0.p, 0, c->b0.bytes, c->stream));
  for (DBuf *v : {&c->b, &c->xs, &c->r, &c->p, &c->q, &c->m, &c->z}) c->alloc(*v, n * 8);
  ELX_CUDA(cudaMemsetAsync(c->b.p, 0, c->b.bytes, c->stream));
  c->alloc(c->scal, sizeof(elx::PcgScalars) * 2);
  ELX_CUDA(cudaMemsetAsync(c->scal.p, 0, c->scal.bytes, c->stream));  // slot 1: done = 0
  c->alloc(c->partials, sizeof(double) * 4 * std::max(4096, elx::grid_cap(32)));
  c->alloc(c->counters, sizeof(unsigned int) * 16);
  ELX_CUDA(cudaMemsetAsync(c->counters.p, 0, c->counters.bytes, c->stream));
  c->alloc(c->flags, sizeof(int32_t) * 4);
  ELX_CUDA(cudaMemsetAsync(c->flags.p, 0, c->flags.bytes, c->stream));
  c->alloc(c->diag, sizeof(double) * 8);
  c->drop_graphs();
  c->sync();
  c->have_structure = true;
  c->have_matrix = false;
}

// FP32 copy of the matrix (after each assembly) and the FP32 inner-solver
// vectors (once per structure), allocated on first use.  With node blocks
// the single-vector and the block products both read the sliced FP32 copy,
// filled straight from ad / al.
void ensure_fp32(elx_ctx *c) {
  const size_t n = (size_t)c->s.neq, nad = (size_t)c->s.nad;
  if (!c->m32.p) {
    if (!c->use_blocks) {
      c->alloc(c->ad32, n * 4 + 64);
      c->alloc(c->al32, nad * 4 + 64);
      c->alloc(c->alt32, nad * 4 + 64);
    }
    for (DBuf *v : {&c->m32, &c->p32, &c->q32, &c->r32, &c->x32}) c->alloc(*v, n * 4 + 64);
    c->drop_graphs();
  }
  if (c->use_blocks && !c->sell_val.p) {
    c->alloc(c->sell_val, (size_t)c->s.sell_ptr[c->s.nslices] * elx::kSliceRows *
                                  c->s.bsize * c->s.bsize * 4 + 64);
    c->drop_graphs();
  }
  if (c->have_fp32) return;
  if (!c->use_blocks) {
    elx::launch_demote_values(c->csrc_dev(), c->stream);
    c->launches += c->s.nad ? 2 : 1;
  } else {
    elx::launch_fill_sell32(c->csrc_dev(), c->stream);
    c->launches += 1;
  }
  c->have_fp32 = true;
}

// The kernel-side copies of a new CSRC matrix: the sliced FP64 node blocks,
// or the transposed upper values of the gather.
void refresh_derived_values(elx_ctx *c) {
  const elx::CsrcDev k = c->csrc_dev();
  if (c->use_blocks) {
    elx::launch_fill_sell64(k, c->stream);
    c->launches += 1;
  } else if (c->s.nad) {
    elx::launch_transpose_values(k, c->stream);
    c->launches += 1;
  }
}

void assemble_resident(elx_ctx *c) {
  require(c->have_structure, ELX_ERR_STATE, "assemble before the structure is set");
  const elx::Structure &s = c->s;
  ELX_CUDA(cudaMemsetAsync(c->ad.p, 0, c->ad.bytes, c->stream));
  ELX_CUDA(cudaMemsetAsync(c->al.p, 0, c->al.bytes, c->stream));
  ELX_CUDA(cudaMemcpyAsync(c->b.p, c->b0.p, (size_t)s.neq * 8, cudaMemcpyDeviceToDevice,
                           c->stream));
  const int32_t big = INT_MAX;
  int32_t *bad = c->flags.as<int32_t>();
  ELX_CUDA(cudaMemcpyAsync(bad, &big, sizeof(big), cudaMemcpyHostToDevice, c->stream));
  const elx::MeshDev md = c->mesh_dev();
  const elx::CsrcDev k = c->csrc_dev();
  for (const elx::Segment &seg : s.segments)
    elx::launch_assembly(md, k, seg, c->u.as<double>(), c->b.as<double>(), bad, c->stream);
  refresh_derived_values(c);
  c->launches += (int64_t)s.segments.size();
  ELX_CUDA(cudaMemcpyAsync(c->h_flags, bad, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  c->sync();
  c->have_fp32 = false;
  if (c->h_flags[0] != INT_MAX) {
    c->have_matrix = false;
    throw Error{ELX_ERR_BAD_DET, "non-positive Jacobian determinant in element " +
                                     std::to_string(c->h_flags[0])};
  }
  c->have_matrix = true;
}

// Jacobi preconditioner m = 1/ad with the zero-diagonal check of Iters.f:337-342.
void build_preconditioner(elx_ctx *c) {
  const int32_t big = INT_MAX;
  int32_t *zero = c->flags.as<int32_t>() + 1;
  ELX_CUDA(cudaMemcpyAsync(zero, &big, sizeof(big), cudaMemcpyHostToDevice, c->stream));
  elx::launch_diag_inverse(c->s.neq, c->ad.as<double>(), c->m.as<double>(),
                           c->m32.p ? c->m32.as<float>() : nullptr, zero, c->stream);
  c->launches += 1;
  ELX_CUDA(cudaMemcpyAsync(c->h_flags + 1, zero, sizeof(int32_t), cudaMemcpyDeviceToHost,
                           c->stream));
  c->sync();
  if (c->h_flags[1] != INT_MAX)
    throw Error{ELX_ERR_ZERO_DIAG, "zero diagonal coefficient in equation " +
                                       std::to_string(c->h_flags[1])};
}

constexpr int kBatch = 16;        // PCG iterations per captured graph launch
constexpr int kMaxGmresK = 256;   // GMRES restart length: one graph node per projection
constexpr int kReplaceEvery = 4;  // mixed precision: replacement check interval
// mixed precision: replace the residual when the FP32 one has dropped to
// this fraction of the last replaced one.  0.1 / 0.15 / 0.2 / 0.3: 480 /
// 476 / 488 / 488 iterations on the 64^3 HEXA8 cube at 1e-8, 3208 / 2944 /
// 2924 / 2908 on the 48^3 TETRA4 mesh at 1e-10 (FP64: 404 and 2438)
constexpr double kReplaceDrop = 0.15;

// Captures kBatch iterations (FP64 or the FP32 inner iteration) as a graph.
cudaGraphExec_t capture_batch(elx_ctx *c, bool fp32) {
  cudaGraph_t g;
  ELX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  const elx::CsrcDev k = c->csrc_dev();
  try {
    const elx::TileDev td = c->tile_dev();
    for (int i = 0; i < kBatch; i++) {
      if (fp32)
        elx::launch_rel_iteration(k, c->b.as<double>(), c->m.as<double>(), c->xs.as<double>(),
                                  c->r.as<double>(), c->z.as<double>(), c->x32.as<float>(),
                                  c->r32.as<float>(), c->p32.as<float>(), c->q32.as<float>(),
                                  c->m32.as<float>(), c->scal.as<elx::PcgScalars>(),
                                  c->partials.as<double>(), c->counters.as<unsigned int>(),
                                  i % kReplaceEvery == kReplaceEvery - 1, c->stream);
      else
        elx::launch_pcg_iteration(k, td, c->spmv_kind, c->xs.as<double>(), c->r.as<double>(),
                                  c->p.as<double>(), c->q.as<double>(), c->part.as<double>(),
                                  c->m.as<double>(), c->scal.as<elx::PcgScalars>(),
                                  c->partials.as<double>(), c->counters.as<unsigned int>(),
                                  c->flags.as<int32_t>() + 2, c->stream);
    }
  } catch (...) {
    cudaStreamEndCapture(c->stream, &g);
    throw;
  }
  ELX_CUDA(cudaStreamEndCapture(c->stream, &g));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t inst = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  ELX_CUDA(inst);
  return exec;
}

void capture_pcg_graph(elx_ctx *c) {
  if (!c->pcg_graph) c->pcg_graph = capture_batch(c, false);
  c->pcg_graph_iters = kBatch;
}

// Launches batches of `graph` until the scalars' stopping flag is set (two
// batches in flight; the host reads the flag of the older one).
elx::PcgScalars run_batches(elx_ctx *c, cudaGraphExec_t graph, double kernels_per_iter,
                            int maxit) {
  elx::PcgScalars *d_sc = c->scal.as<elx::PcgScalars>();
  int launched = 0, checked = 0;
  auto launch_batch = [&](int slot) {
    ELX_CUDA(cudaGraphLaunch(graph, c->stream));
    c->launches += (int64_t)(kernels_per_iter * kBatch + 0.5);
    ELX_CUDA(cudaMemcpyAsync(&c->h_scal[slot], d_sc, sizeof(elx::PcgScalars),
                             cudaMemcpyDeviceToHost, c->stream));
    ELX_CUDA(cudaEventRecord(c->ev[slot], c->stream));
  };
  const int max_batches = maxit / kBatch + 2;
  launch_batch(0);
  launched = 1;
  if (max_batches > 1) {
    launch_batch(1);
    launched = 2;
  }
  for (;;) {
    const int slot = checked & 1;
    ELX_CUDA(cudaEventSynchronize(c->ev[slot]));
    checked++;
    if (c->h_scal[slot].done) break;
    if (launched >= max_batches) break;  // guard; the kernels stop at maxit themselves
    launch_batch(launched & 1);
    launched++;
  }
  c->sync();
  elx::PcgScalars last;
  ELX_CUDA(cudaMemcpy(&last, d_sc, sizeof(last), cudaMemcpyDeviceToHost));
  return last;
}

void fill_info(elx_ctx *c, elx_info *info, const elx::PcgScalars &sc, double secs) {
  if (!info) return;
  const double neq = c->s.neq, nad = (double)c->s.nad;
  info->iters = sc.iters;
  info->status = sc.status;
  info->xkx = c->h_diag[0];
  info->norm_x = std::sqrt(c->h_diag[1]);
  info->norm_m_r = std::sqrt(std::fabs(c->h_diag[2]));
  info->norm_r = std::sqrt(c->h_diag[3]);
  info->conv = sc.conv;
  info->seconds = secs;
  // flop_cg(neq, nad, it, 2) (Matvec.f:1499-1531)
  const double fl = ((neq + 4.0 * nad) + 2.0 * (2.0 * neq) + 7.0 * neq + 2.0) * sc.iters;
  info->mflops = secs > 0 ? fl * 1e-6 / secs : 0.0;
  info->refinements = 0;
  info->inner_iters = 0;
}

// y = K x for resident vectors (FP64), with the PCG's own SpMV launches.
void spmv64(elx_ctx *c, const double *x, double *y) {
  elx::launch_spmv64(c->csrc_dev(), c->tile_dev(), c->spmv_kind, x, y, c->part.as<double>(),
                     c->flags.as<int32_t>() + 2, c->stream);
  c->launches += c->spmv_kind == elx::kSpmvTiled ? 2 : 1;
}

// A bounded device wait of the pipelined (tiled) SpMV that gave up leaves
// its code in flags[2]; reported, and cleared, as ELX_ERR_TIMEOUT.
void check_pipe_waits(elx_ctx *c) {
  ELX_CUDA(cudaMemcpyAsync(c->h_flags + 2, c->flags.as<int32_t>() + 2, sizeof(int32_t),
                           cudaMemcpyDeviceToHost, c->stream));
  c->sync();
  if (c->h_flags[2] != 0) {
    ELX_CUDA(cudaMemsetAsync(c->flags.as<int32_t>() + 2, 0, sizeof(int32_t), c->stream));
    c->sync();
    throw Error{ELX_ERR_TIMEOUT, "a bounded device wait of the SpMV pipeline gave up"};
  }
}

// Post-solve diagnostics (Iters.f:433-458) of the resident x: z = K x,
// xKx, ||x||, ||b - Kx||_M, ||b - Kx|| into h_diag[0..3].
void post_diagnostics(elx_ctx *c) {
  spmv64(c, c->xs.as<double>(), c->z.as<double>());
  elx::launch_diagnostics(c->s.neq, c->xs.as<double>(), c->z.as<double>(), c->b.as<double>(),
                          c->m.as<double>(), c->diag.as<double>(), c->partials.as<double>(),
                          c->counters.as<unsigned int>() + 3, c->stream);
  c->launches += 1;
  ELX_CUDA(cudaMemcpyAsync(c->h_diag, c->diag.p, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                           c->stream));
  check_pipe_waits(c);
}

void set_scalars(elx_ctx *c, double tol, int maxit) {
  elx::PcgScalars init{};
  init.tol = tol;
  init.maxit = maxit;
  c->h_scal[0] = init;
  ELX_CUDA(cudaMemcpyAsync(c->scal.p, &c->h_scal[0], sizeof(init), cudaMemcpyHostToDevice,
                           c->stream));
}

void pcg64(elx_ctx *c, double tol, int maxit, elx_info *info) {
  auto t0 = std::chrono::steady_clock::now();
  build_preconditioner(c);
  set_scalars(c, tol, maxit);
  elx::launch_pcg_start<double>(c->s.neq, c->b.as<double>(), c->m.as<double>(),
                                c->xs.as<double>(), c->r.as<double>(), c->p.as<double>(),
                                c->scal.as<elx::PcgScalars>(), c->partials.as<double>(),
                                c->counters.as<unsigned int>() + 2, c->stream);
  c->launches += 1;
  capture_pcg_graph(c);
  elx::PcgScalars last =
      run_batches(c, c->pcg_graph, c->spmv_kind == elx::kSpmvTiled ? 4 : 3, maxit);
  post_diagnostics(c);
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (!last.done) last.status = ELX_ERR_NO_CONVERGENCE;
  fill_info(c, info, last, secs);
  if (last.status != ELX_OK)
    throw Error{last.status, "no convergence after " + std::to_string(last.iters) +
                                 " iterations"};
}

// Mixed precision: FP32 CG with reliable updates (krylov.cu): the FP32
// iteration carries the Krylov recurrence, the FP64 solution and the FP64
// residual are refreshed each time the FP32 residual has dropped tenfold,
// and the stopping test is the reference's, ||b - K x||_M < tol ||b||_M, on
// the FP64 residual.
void pcg_mixed(elx_ctx *c, double tol, int maxit, elx_info *info) {
  auto t0 = std::chrono::steady_clock::now();
  ensure_fp32(c);
  build_preconditioner(c);
  if (!c->pcg32_graph) c->pcg32_graph = capture_batch(c, true);
  const int n = c->s.neq;
  double *bmb_d = c->diag.as<double>() + 4;
  // r_hi = b (x = 0), r = (float) b, (b, M b) in FP64
  elx::launch_refine_residual(n, c->b.as<double>(), nullptr, c->m.as<double>(),
                              c->r.as<double>(), c->r32.as<float>(), bmb_d,
                              c->partials.as<double>(), c->counters.as<unsigned int>() + 5,
                              c->stream);
  ELX_CUDA(cudaMemsetAsync(c->xs.p, 0, (size_t)n * 8, c->stream));
  ELX_CUDA(cudaMemcpyAsync(c->h_diag + 4, bmb_d, sizeof(double), cudaMemcpyDeviceToHost,
                           c->stream));
  c->sync();
  const double bmb = c->h_diag[4];
  elx::PcgScalars init{};
  init.tol = tol;
  init.maxit = maxit;
  init.bmb = bmb;
  init.conv = tol * std::sqrt(std::fabs(bmb));
  init.delta = kReplaceDrop;
  init.best = std::sqrt(std::fabs(bmb));  // ||b - K 0||_M
  c->h_scal[0] = init;
  ELX_CUDA(cudaMemcpyAsync(c->scal.p, &c->h_scal[0], sizeof(init), cudaMemcpyHostToDevice,
                           c->stream));
  elx::launch_rel_start(n, c->r32.as<float>(), c->m32.as<float>(), c->x32.as<float>(),
                        c->p32.as<float>(), c->scal.as<elx::PcgScalars>(),
                        c->partials.as<double>(), c->counters.as<unsigned int>() + 2, c->stream);
  c->launches += 2;
  elx::PcgScalars last = run_batches(c, c->pcg32_graph, 3 + 3.0 / kReplaceEvery, maxit);
  // fold the last FP32 piece (zero unless maxit stopped the iteration)
  elx::launch_refine_accumulate(n, c->xs.as<double>(), c->x32.as<float>(), false, c->stream);
  c->launches += 1;
  post_diagnostics(c);
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (!last.done) last.status = ELX_ERR_NO_CONVERGENCE;
  if (last.failed) {
    // the FP32 iteration diverged or stalled (an FP32 matrix too
    // ill-conditioned for it): the case is solved in FP64 from scratch;
    // refinements = -1 marks the fallback, inner_iters the FP32 work spent
    pcg64(c, tol, maxit, info);
    if (info) {
      info->refinements = -1;
      info->inner_iters = last.iters;
    }
    return;
  }
  fill_info(c, info, last, secs);
  if (info) {
    info->refinements = last.nupdates;
    info->inner_iters = last.iters;
  }
  if (last.status != ELX_OK)
    throw Error{last.status, "mixed precision: no convergence after " +
                                 std::to_string(last.iters) + " iterations"};
}

// pbicgstab (Iters.f:1079-1349) on the device: right Jacobi, 2-norm test.
// With plain, bicgstab (Iters.f:812-1075): the same iteration with M = I (a
// vector of ones: z = 1 * p is p exactly), whose beta from (r, b) equals the
// (r, r0) of pbicgstab because x0 = 0 makes r0 = b exactly.
void bicgstab64(elx_ctx *c, double tol, int maxit, elx_info *info, bool plain) {
  auto t0 = std::chrono::steady_clock::now();
  const size_t n = (size_t)c->s.neq;
  if (!c->r0v.p) {
    c->alloc(c->r0v, n * 8);
    c->alloc(c->tv, n * 8);
    c->drop_graphs();
  }
  if (plain && !c->unit.p) {
    const std::vector<double> one(n, 1.0);
    c->upload(c->unit, one.data(), n);
    c->sync();
  }
  build_preconditioner(c);  // the zero-diagonal check of Iters.f:900-905 too
  const double *m = plain ? c->unit.as<double>() : c->m.as<double>();
  if (c->bicg_graph && c->bicg_plain != plain) {
    cudaGraphExecDestroy(c->bicg_graph);
    c->bicg_graph = nullptr;
  }
  c->bicg_plain = plain;
  set_scalars(c, tol, maxit);
  auto *sc = c->scal.as<elx::PcgScalars>();
  elx::launch_bicg_start(c->s.neq, c->b.as<double>(), m, c->xs.as<double>(),
                         c->r.as<double>(), c->r0v.as<double>(), c->p.as<double>(),
                         c->z.as<double>(), sc, c->partials.as<double>(),
                         c->counters.as<unsigned int>() + 2, c->stream);
  c->launches += 1;
  if (!c->bicg_graph) {
    cudaGraph_t g;
    ELX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    try {
      for (int i = 0; i < kBatch; i++)
        elx::launch_bicg_iteration(c->csrc_dev(), m, c->xs.as<double>(),
                                   c->r.as<double>(), c->r0v.as<double>(), c->p.as<double>(),
                                   c->z.as<double>(), c->q.as<double>(), c->tv.as<double>(), sc,
                                   c->partials.as<double>(), c->counters.as<unsigned int>() + 6,
                                   c->stream);
    } catch (...) {
      cudaStreamEndCapture(c->stream, &g);
      throw;
    }
    ELX_CUDA(cudaStreamEndCapture(c->stream, &g));
    const cudaError_t inst = cudaGraphInstantiate(&c->bicg_graph, g, 0);
    cudaGraphDestroy(g);
    ELX_CUDA(inst);
  }
  elx::PcgScalars last = run_batches(c, c->bicg_graph, 5, maxit);
  post_diagnostics(c);
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (!last.done) last.status = ELX_ERR_NO_CONVERGENCE;
  fill_info(c, info, last, secs);
  if (info) {
    info->mflops = 0.0;
    if (plain) info->norm_m_r = info->norm_r;  // no M: the 2-norm residual
  }
  if (last.status != ELX_OK)
    throw Error{last.status, "BiCGSTAB: no convergence after " + std::to_string(last.iters) +
                                 " iterations"};
}

// gmres (Iters.f:528-808) on the device: GMRES(k), left Jacobi, one captured
// graph per restart cycle; maxit counts cycles, iters the Arnoldi steps.
void gmres64(elx_ctx *c, int kdim, double tol, int maxit, elx_info *info) {
  auto t0 = std::chrono::steady_clock::now();
  require(kdim >= 1 && kdim <= kMaxGmresK, ELX_ERR_ARG, "GMRES restart length out of range");
  const size_t n = (size_t)c->s.neq;
  if (c->gmres_k != kdim || !c->gbasis.p) {
    if (c->gmres_graph) cudaGraphExecDestroy(c->gmres_graph);
    c->gmres_graph = nullptr;
    c->alloc(c->gbasis, n * 8 * (size_t)(kdim + 1));
    c->alloc(c->garrays, elx::gmres_array_doubles(kdim) * 8);
    if (!c->gstate.p) c->alloc(c->gstate, sizeof(elx::GmresState));
    c->gmres_k = kdim;
  }
  build_preconditioner(c);
  auto *gs = c->gstate.as<elx::GmresState>();
  elx::GmresState init{};
  init.tol = tol;
  init.maxit = maxit;
  ELX_CUDA(cudaMemcpyAsync(gs, &init, sizeof(init), cudaMemcpyHostToDevice, c->stream));
  ELX_CUDA(cudaMemsetAsync(c->garrays.p, 0, c->garrays.bytes, c->stream));
  elx::launch_gmres_init(c->s.neq, c->b.as<double>(), c->m.as<double>(), c->xs.as<double>(),
                         c->gbasis.as<double>(), gs, c->partials.as<double>(),
                         c->counters.as<unsigned int>() + 2, c->stream);
  c->launches += 1;
  if (!c->gmres_graph) {
    cudaGraph_t g;
    ELX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    try {
      c->gmres_launches = elx::launch_gmres_cycle(
          c->csrc_dev(), kdim, c->b.as<double>(), c->m.as<double>(), c->xs.as<double>(),
          c->gbasis.as<double>(), gs, c->garrays.as<double>(), c->partials.as<double>(),
          c->counters.as<unsigned int>() + 6, c->stream);
    } catch (...) {
      cudaStreamEndCapture(c->stream, &g);
      throw;
    }
    ELX_CUDA(cudaStreamEndCapture(c->stream, &g));
    const cudaError_t inst = cudaGraphInstantiate(&c->gmres_graph, g, 0);
    cudaGraphDestroy(g);
    ELX_CUDA(inst);
  }
  elx::GmresState st{};
  for (int cyc = 0; cyc <= maxit; cyc++) {
    ELX_CUDA(cudaMemcpyAsync(&st, gs, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
    c->sync();
    if (!st.live) break;
    ELX_CUDA(cudaGraphLaunch(c->gmres_graph, c->stream));
    c->launches += c->gmres_launches;
  }
  ELX_CUDA(cudaMemcpyAsync(&st, gs, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
  post_diagnostics(c);
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  elx::PcgScalars last{};
  last.iters = st.nit;
  last.status = st.done ? st.status : ELX_ERR_NO_CONVERGENCE;
  last.conv = st.econv;
  fill_info(c, info, last, secs);
  if (info) {
    info->mflops = 0.0;
    info->refinements = st.cycles;  // restart cycles
  }
  if (last.status != ELX_OK)
    throw Error{last.status, "GMRES: no convergence after " + std::to_string(st.cycles) +
                                 " cycles (" + std::to_string(st.nit) + " iterations)"};
}

// ---------------------------------------------------------------- block PCG

constexpr int kMaxBlockWidth = 16;

// Device arrays for blocks of up to `cap` columns (FP32 ones only for the
// mixed solver), allocated on first use.
void ensure_block(elx_ctx *c, int cap, bool mixed) {
  const size_t n = (size_t)c->s.neq;
  if (c->blk_cap < cap) {
    release_block(c);
    if (c->block_graph) cudaGraphExecDestroy(c->block_graph);
    c->block_graph = nullptr;
    c->block_graph_w = 0;
    for (DBuf *v : {&c->bk_b, &c->bk_x, &c->bk_r, &c->bk_p, &c->bk_q, &c->bk_z, &c->bk_colmajor})
      c->alloc(*v, n * cap * 8);
    c->alloc(c->bk_cols, sizeof(elx::ColScalars) * kMaxBlockWidth);
    c->alloc(c->bk_hdr, sizeof(elx::BlockHeader) * 2);
    c->alloc(c->bk_part, sizeof(double) * 2 * kMaxBlockWidth * elx::grid_cap(8));
    c->alloc(c->bk_cnt, sizeof(unsigned int) * 8);
    ELX_CUDA(cudaMemsetAsync(c->bk_cnt.p, 0, c->bk_cnt.bytes, c->stream));
    c->alloc(c->bk_diag, sizeof(double) * 4 * kMaxBlockWidth);
    elx::BlockHeader on{};
    on.active = 1;
    ELX_CUDA(cudaMemcpyAsync(c->bk_hdr.as<elx::BlockHeader>() + 1, &on, sizeof(on),
                             cudaMemcpyHostToDevice, c->stream));
    c->sync();
    c->blk_cap = cap;
  }
  if (mixed && !c->bk_xlo.p) {
    for (DBuf *v : {&c->bk_xlo, &c->bk_r32, &c->bk_p32, &c->bk_q32})
      c->alloc(*v, n * c->blk_cap * 4);
    if (c->block_graph) cudaGraphExecDestroy(c->block_graph);
    c->block_graph = nullptr;
    c->block_graph_w = 0;
  }
}

elx::BlockVecs block_vecs(elx_ctx *c, int w) {
  elx::BlockVecs v;
  v.w = w;
  v.b = c->bk_b.as<double>(); v.m = c->m.as<double>();
  v.x = c->bk_x.as<double>(); v.r = c->bk_r.as<double>(); v.p = c->bk_p.as<double>();
  v.q = c->bk_q.as<double>(); v.z = c->bk_z.as<double>();
  v.m32 = c->m32.as<float>();
  v.xlo = c->bk_xlo.as<float>(); v.r32 = c->bk_r32.as<float>(); v.p32 = c->bk_p32.as<float>();
  v.q32 = c->bk_q32.as<float>();
  v.cols = c->bk_cols.as<elx::ColScalars>();
  v.hdr = c->bk_hdr.as<elx::BlockHeader>();
  v.hdr_on = v.hdr + 1;
  v.partials = c->bk_part.as<double>();
  v.counters = c->bk_cnt.as<unsigned int>();
  return v;
}

// The block width whose product costs least per column, and per width the
// product's tiling: each supported width's product timed on the resident
// matrix (FP32 for the mixed solver, FP64 otherwise; the solver's own form,
// with the fused dots), best of three launches after one warm-up, for 1, 2
// and 3 slot groups of matrix loads in flight (3x3 node blocks; 2x2 blocks
// have one form), the fastest kept.  ELX_SPMM_UNROLL fixes the tiling.
int autotune_block_width(elx_ctx *c, bool mixed, double *times_us = nullptr) {
  const int slot = mixed ? 1 : 0;
  if (c->tuned_width[slot] && !times_us) return c->tuned_width[slot];
  ensure_block(c, kMaxBlockWidth, mixed);
  if (mixed) ensure_fp32(c);
  const size_t n = (size_t)c->s.neq;
  ELX_CUDA(cudaMemsetAsync(c->bk_p.p, 0, n * kMaxBlockWidth * 8, c->stream));
  if (mixed) ELX_CUDA(cudaMemsetAsync(c->bk_p32.p, 0, n * kMaxBlockWidth * 4, c->stream));
  const bool tile = c->s.bsize == 3 && c->spmm_unroll == 0;
  int best = 1;
  double best_cost = 1e300;
  int idx = 0;
  for (int w : {1, 2, 4, 8, 16}) {
    const elx::BlockVecs v = block_vecs(c, w);
    double t_w = 1e300;
    int u_w = 0;
    for (int u : {1, 2, 3}) {
      if (!tile && u > 1) break;
      c->tuned_unroll[slot][idx] = tile ? u : 0;
      const elx::CsrcDev k = c->csrc_dev();
      double t_best = 1e300;
      for (int rep = 0; rep < 4; rep++) {
        ELX_CUDA(cudaEventRecord(c->ev_t[0], c->stream));
        if (mixed)
          elx::launch_spmm32(k, v, c->stream);
        else
          elx::launch_spmm64(k, v, c->stream);
        ELX_CUDA(cudaEventRecord(c->ev_t[1], c->stream));
        ELX_CUDA(cudaEventSynchronize(c->ev_t[1]));
        float ms = 0.f;
        ELX_CUDA(cudaEventElapsedTime(&ms, c->ev_t[0], c->ev_t[1]));
        if (rep > 0) t_best = std::min(t_best, (double)ms);
      }
      c->launches += 4;
      if (t_best < t_w) {
        t_w = t_best;
        u_w = tile ? u : 0;
      }
    }
    c->tuned_unroll[slot][idx] = u_w;
    if (times_us) times_us[idx] = t_w * 1e3;
    idx++;
    const double cost = t_w / w;
    if (cost < best_cost * 0.97) {  // a wider block must win by 3 %
      best_cost = cost;
      best = w;
    }
  }
  c->tuned_width[slot] = best;
  c->drop_graphs();  // a captured block iteration holds the earlier tiling
  return best;
}

// Solves nrhs load cases (b column-major, neq x nrhs, on the host or the
// device) in blocks of `width` columns; x likewise; one elx_info per column.
void solve_block(elx_ctx *c, int nrhs, int precision, double tol, int maxit, int width,
                 const double *b, double *x, elx_info *infos, bool device_ptrs) {
  require(c->have_matrix, ELX_ERR_STATE, "solve before the matrix is assembled");
  require(nrhs >= 1 && tol > 0 && maxit >= 0, ELX_ERR_ARG, "bad block solve arguments");
  require(precision == ELX_PREC_FP64 || precision == ELX_PREC_MIXED, ELX_ERR_ARG,
          "unknown precision");
  require(width == 0 || elx::block_width_supported(width), ELX_ERR_ARG,
          "block width must be 0 (autotune), 1, 2, 4, 8 or 16");
  require(c->use_blocks, ELX_ERR_ARG,
          "block solves need node blocks (every node all free or all fixed)");
  const bool mixed = precision == ELX_PREC_MIXED;
  auto t0 = std::chrono::steady_clock::now();
  if (mixed) ensure_fp32(c);
  build_preconditioner(c);
  if (width == 0) width = autotune_block_width(c, mixed);
  int w = 1;
  while (w < width && w < nrhs) w *= 2;
  ensure_block(c, std::max(w, c->blk_cap), mixed);
  const size_t n = (size_t)c->s.neq;
  const elx::CsrcDev k = c->csrc_dev();
  const elx::BlockVecs v = block_vecs(c, w);
  if (!c->block_graph || c->block_graph_w != w || c->block_graph_mixed != mixed) {
    if (c->block_graph) cudaGraphExecDestroy(c->block_graph);
    c->block_graph = nullptr;
    cudaGraph_t g;
    ELX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    try {
      for (int i = 0; i < kBatch; i++)
        elx::launch_block_iteration(k, v, mixed, i % kReplaceEvery == kReplaceEvery - 1,
                                    c->stream);
    } catch (...) {
      cudaStreamEndCapture(c->stream, &g);
      throw;
    }
    ELX_CUDA(cudaStreamEndCapture(c->stream, &g));
    const cudaError_t inst = cudaGraphInstantiate(&c->block_graph, g, 0);
    cudaGraphDestroy(g);
    ELX_CUDA(inst);
    c->block_graph_w = w;
    c->block_graph_mixed = mixed;
  }
  const double per_iter = mixed ? 3 + 3.0 / kReplaceEvery : 3;
  int status = ELX_OK;
  std::vector<int> fallback;  // mixed columns to solve again in FP64
  std::vector<int> fallback_fp32_iters;
  for (int c0 = 0; c0 < nrhs; c0 += w) {
    const int nc = std::min(w, nrhs - c0);
    // b columns -> column-major staging (zero columns pad a short block)
    if (nc < w)
      ELX_CUDA(cudaMemsetAsync(c->bk_colmajor.p, 0, n * w * 8, c->stream));
    ELX_CUDA(cudaMemcpyAsync(c->bk_colmajor.p, b + (size_t)c0 * n, n * nc * 8,
                             device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                             c->stream));
    elx::launch_interleave((int)n, w, c->bk_colmajor.as<double>(), c->bk_b.as<double>(),
                           c->stream);
    elx::BlockHeader h{};
    h.tol = tol;
    // a cohort replacement is a full-width FP64 product: fewer pay here
    // (29.8 / 31.3 / 32.6 ms per case at 0.1 / 0.15 / 0.3, 96x96x48 plate)
    h.delta = 0.1;
    h.maxit = maxit;
    ELX_CUDA(cudaMemcpyAsync(v.hdr, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    elx::launch_block_start(k, v, mixed, c->stream);
    c->launches += 2;
    // batches of kBatch iterations until no column is active
    elx::BlockHeader hh{};
    const int max_batches = maxit / kBatch + 2;
    struct Gate {  // batch_gate(0) also when a launch or the poll throws
      elx_ctx *c;
      explicit Gate(elx_ctx *cc) : c(cc) {
        if (c->batch_gate) c->batch_gate(c->batch_gate_user, 1);
      }
      ~Gate() {
        if (c->batch_gate) c->batch_gate(c->batch_gate_user, 0);
      }
    };
    for (int bt = 0; bt < max_batches; bt++) {
      Gate gate(c);
      ELX_CUDA(cudaGraphLaunch(c->block_graph, c->stream));
      c->launches += (int64_t)(per_iter * kBatch + 0.5);
      ELX_CUDA(cudaMemcpyAsync(&hh, v.hdr, sizeof(hh), cudaMemcpyDeviceToHost, c->stream));
      c->sync();
      if (hh.active == 0) break;
    }
    elx::launch_block_diagnostics(k, v, c->bk_diag.as<double>(), c->stream);
    c->launches += 3;
    elx::launch_deinterleave((int)n, w, c->bk_x.as<double>(), c->bk_colmajor.as<double>(),
                             c->stream);
    c->launches += 1;
    ELX_CUDA(cudaMemcpyAsync(x + (size_t)c0 * n, c->bk_colmajor.p, n * nc * 8,
                             device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             c->stream));
    elx::ColScalars cs[kMaxBlockWidth];
    double dg[4 * kMaxBlockWidth];
    ELX_CUDA(cudaMemcpyAsync(cs, v.cols, sizeof(elx::ColScalars) * w, cudaMemcpyDeviceToHost,
                             c->stream));
    ELX_CUDA(cudaMemcpyAsync(dg, c->bk_diag.p, sizeof(double) * 4 * w, cudaMemcpyDeviceToHost,
                             c->stream));
    c->sync();
    const double secs =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int j = 0; j < nc; j++) {
      const elx::ColScalars &s = cs[j];
      int st = s.done ? s.status : ELX_ERR_NO_CONVERGENCE;
      if (mixed && s.failed) {
        fallback.push_back(c0 + j);
        fallback_fp32_iters.push_back(s.iters);
        st = ELX_OK;  // decided by the FP64 solve below
      }
      if (st != ELX_OK && status == ELX_OK) status = st;
      if (!infos) continue;
      elx_info &in = infos[c0 + j];
      std::memset(&in, 0, sizeof(in));
      in.iters = s.iters;
      in.status = st;
      in.xkx = dg[4 * j + 0];
      in.norm_x = std::sqrt(dg[4 * j + 1]);
      in.norm_m_r = std::sqrt(std::fabs(dg[4 * j + 2]));
      in.norm_r = std::sqrt(dg[4 * j + 3]);
      in.conv = s.conv;
      in.seconds = secs;
      in.refinements = mixed ? s.nupdates : 0;
      in.inner_iters = mixed ? s.iters : 0;
    }
  }
  if (!fallback.empty()) {
    // columns whose FP32 iteration diverged or stalled: FP64 PCG one by one
    // (the context's assembled b is kept aside meanwhile)
    ELX_CUDA(cudaMemcpyAsync(c->bk_z.p, c->b.p, n * 8, cudaMemcpyDeviceToDevice, c->stream));
    for (size_t f = 0; f < fallback.size(); f++) {
      const int col = fallback[f];
      ELX_CUDA(cudaMemcpyAsync(c->b.p, b + (size_t)col * n, n * 8,
                               device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               c->stream));
      elx_info in{};
      int st = ELX_OK;
      try {
        pcg64(c, tol, maxit, &in);
      } catch (const Error &e) {
        if (e.code != ELX_ERR_NO_CONVERGENCE) throw;
        st = e.code;
      }
      ELX_CUDA(cudaMemcpyAsync(x + (size_t)col * n, c->xs.p, n * 8,
                               device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               c->stream));
      c->sync();
      if (st != ELX_OK && status == ELX_OK) status = st;
      if (infos) {
        in.status = st;
        in.refinements = -1;
        in.inner_iters = fallback_fp32_iters[f];
        infos[col] = in;
      }
    }
    ELX_CUDA(cudaMemcpyAsync(c->b.p, c->bk_z.p, n * 8, cudaMemcpyDeviceToDevice, c->stream));
    c->sync();
  }
  if (status != ELX_OK) throw Error{status, "block PCG: a load case did not converge"};
}

void solve_resident(elx_ctx *c, int solver, int precision, double tol, int maxit, int ngram,
                    elx_info *info) {
  require(c->have_matrix, ELX_ERR_STATE, "solve before the matrix is assembled");
  require(tol > 0 && maxit >= 0, ELX_ERR_ARG, "tol must be > 0 and maxit >= 0");
  if (info) std::memset(info, 0, sizeof(*info));
  if (solver == ELX_SOLVER_PCG && precision == ELX_PREC_FP64) {
    pcg64(c, tol, maxit, info);
    return;
  }
  if (solver == ELX_SOLVER_PCG && precision == ELX_PREC_MIXED) {
    pcg_mixed(c, tol, maxit, info);
    return;
  }
  if ((solver == ELX_SOLVER_BICGSTAB || solver == ELX_SOLVER_BICGSTAB_NOPREC) &&
      precision == ELX_PREC_FP64) {
    bicgstab64(c, tol, maxit, info, solver == ELX_SOLVER_BICGSTAB_NOPREC);
    return;
  }
  if (solver == ELX_SOLVER_GMRES && precision == ELX_PREC_FP64) {
    gmres64(c, ngram, tol, maxit, info);
    return;
  }
  throw Error{ELX_ERR_ARG, "solver/precision combination not available"};
}

void check_mesh(int32_t ndm, int32_t ndf, int32_t nen, int32_t numel, int32_t nnode,
                const int32_t *ix, const int32_t *ie, int32_t numat, int32_t prop) {
  require(ndm >= 2 && ndm <= 3 && ndf == ndm && nen >= 3 && nen <= 8 && numel > 0 &&
              nnode > 0 && numat > 0 && prop >= 3,
          ELX_ERR_ARG, "invalid mesh sizes");
  for (int i = 0; i < numat; i++) {
    const int iel = ie[i];
    const int nv = elx::elem_nodes(iel);
    require(nv > 0, ELX_ERR_BAD_ELEMENT, "unsupported element type");
    require(nv <= nen, ELX_ERR_ARG, "element type needs more nodes than nen");
    require((iel <= 5) == (ndm == 2), ELX_ERR_ARG, "element type does not match ndm");
  }
  const int nen1 = nen + 1;
  for (int el = 0; el < numel; el++) {
    const int ma = ix[(size_t)el * nen1 + nen];
    require(ma >= 1 && ma <= numat, ELX_ERR_ARG, "material number out of range");
    const int nv = elx::elem_nodes(ie[ma - 1]);
    for (int a = 0; a < nv; a++) {
      const int no = ix[(size_t)el * nen1 + a];
      require(no >= 1 && no <= nnode, ELX_ERR_ARG, "node number out of range");
    }
  }
}

void fill_mesh(elx::Mesh &m, int32_t ndm, int32_t ndf, int32_t nen, int32_t numel,
               int32_t nnode, const int32_t *ix, const double *x, const int32_t *ie,
               const double *e, int32_t prop, int32_t numat) {
  const int nen1 = nen + 1;
  m.ndm = ndm; m.ndf = ndf; m.nen = nen; m.numel = numel; m.nnode = nnode;
  m.numat = numat; m.prop = prop;
  m.ix.assign(ix, ix + (size_t)nen1 * numel);
  m.x.assign(x, x + (size_t)ndm * nnode);
  m.ie.assign(ie, ie + numat);
  m.e.assign(e, e + (size_t)prop * numat);
}

// graph -> RCM (or natural order) -> numeq -> lower CSRC pattern, on the host.
void build_host_structure(const elx::Mesh &m, const int32_t *bc, bool reorder,
                          elx::Structure &s) {
  std::vector<int32_t> xadj, adj, perm0;
  elx::node_graph(m, xadj, adj);
  if (reorder) {
    elx::rcm_order(m.nnode, xadj, adj, perm0);
  } else {
    perm0.resize(m.nnode);
    for (int i = 0; i < m.nnode; i++) perm0[i] = i;
  }
  s.perm.resize(m.nnode);
  for (int i = 0; i < m.nnode; i++) s.perm[i] = perm0[i] + 1;
  s.neq = elx::number_equations(m, perm0, bc, s.id);
  require(s.neq > 0, ELX_ERR_ARG, "no free equations");
  elx::csrc_pattern(m, s, xadj, adj, s.ia, s.ja);
  s.nad = (int64_t)s.ia[s.neq] - 1;
  require(s.nad < INT_MAX, ELX_ERR_ARG, "nad exceeds 32-bit indexing");
}

}  // namespace elx_api

namespace elx {
namespace {
constexpr int kPoolDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kPoolDevices];
bool g_pool_probed[kPoolDevices];
int g_pool_users[kPoolDevices];
std::mutex g_pinned_mu;
std::vector<void *> g_pinned_free;
}  // namespace

cudaMemPool_t device_pool(int device) {
  if (device < 0 || device >= kPoolDevices) return nullptr;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pool_probed[device]) {
    g_pool_probed[device] = true;
    const char *env = std::getenv("ELX_DEVICE_POOL");
    int ok = 0;
    if (!(env && std::atoi(env) == 0) &&
        cudaDeviceGetAttribute(&ok, cudaDevAttrMemoryPoolsSupported, device) == cudaSuccess &&
        ok) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = device;
      cudaMemPool_t p = nullptr;
      if (cudaMemPoolCreate(&p, &props) == cudaSuccess) {
        // freed memory stays reserved for the next allocation (returned
        // when the last pool user goes, pool_users)
        uint64_t keep = UINT64_MAX;
        if (cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess)
          g_pool[device] = p;
        else
          cudaMemPoolDestroy(p);
      }
    }
    (void)cudaGetLastError();
  }
  return g_pool[device];
}

void pool_users(int device, int delta) {
  if (device < 0 || device >= kPoolDevices) return;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  g_pool_users[device] += delta;
  if (g_pool_users[device] == 0 && g_pool[device]) cudaMemPoolTrimTo(g_pool[device], 0);
}

void *pinned_block_get() {
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  if (g_pinned_free.empty()) {
    constexpr int kPerChunk = 64;
    void *chunk = nullptr;
    ELX_CUDA(cudaHostAlloc(&chunk, kPinnedBlock * kPerChunk, cudaHostAllocPortable));
    for (int i = kPerChunk - 1; i >= 0; i--)
      g_pinned_free.push_back(static_cast<char *>(chunk) + (size_t)i * kPinnedBlock);
  }
  void *p = g_pinned_free.back();
  g_pinned_free.pop_back();
  std::memset(p, 0, kPinnedBlock);
  return p;
}

void pinned_block_put(void *p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  g_pinned_free.push_back(p);
}
}  // namespace elx

using namespace elx_api;

extern "C" {

const char *elx_version(void) { return "elastic_gb300 0.1 (sm_103a)"; }

int elx_fp64_fma_rate(int32_t device, double *fma_per_s, double *per_clock_per_sm) {
  if (!fma_per_s) return ELX_ERR_ARG;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return ELX_ERR_CUDA;
  int code = ELX_OK;
  try {
    *fma_per_s = elx::measure_fp64_fma_rate(device, per_clock_per_sm);
  } catch (const Error &e) {
    code = e.code;
  }
  cudaSetDevice(prev);  // the caller's current device, as it was
  return code;
}

int elx_create(elx_ctx **out, const elx_opts *opts) {
  if (!out) return ELX_ERR_ARG;
  *out = nullptr;
  elx_ctx *c = new (std::nothrow) elx_ctx();
  if (!c) return ELX_ERR_OOM;
  if (opts) {
    c->device = opts->device;
    c->verbose = opts->verbose;
    c->budget = opts->hbm_budget;
  }
  int st = guarded(c, [&] {
    int ndev = 0;
    ELX_CUDA(cudaGetDeviceCount(&ndev));
    require(c->device >= 0 && c->device < ndev, ELX_ERR_ARG, "no such CUDA device");
    ELX_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->pool = elx::device_pool(c->device);
    elx::pool_users(c->device, 1);
    c->pool_user = true;
    // h_scal (2 PcgScalars), h_diag (8 doubles), h_flags (4 ints) in one
    // recycled pinned block
    static_assert(2 * sizeof(elx::PcgScalars) + 8 * sizeof(double) + 4 * sizeof(int32_t) <=
                      elx::kPinnedBlock,
                  "pinned block too small");
    c->pinned = elx::pinned_block_get();
    char *pb = static_cast<char *>(c->pinned);
    c->h_scal = reinterpret_cast<elx::PcgScalars *>(pb);
    c->h_diag = reinterpret_cast<double *>(pb + 2 * sizeof(elx::PcgScalars));
    c->h_flags = reinterpret_cast<int32_t *>(pb + 2 * sizeof(elx::PcgScalars) + 8 * sizeof(double));
    for (auto &e : c->ev) ELX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto &e : c->ev_t) ELX_CUDA(cudaEventCreate(&e));
  });
  if (st != ELX_OK) {
    // keep the context so that elx_last_error can report why
    *out = c;
    return st;
  }
  *out = c;
  return ELX_OK;
}

void elx_destroy(elx_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->drop_graphs();
  release_partitions(c);
  for (DBuf *d : {&c->conn, &c->mat, &c->elnum, &c->slot, &c->x, &c->eq, &c->e, &c->ia, &c->ja,
                  &c->iat, &c->jat, &c->pt, &c->ja16, &c->jat16, &c->alt, &c->alt32,
                  &c->tile_tgt, &c->tile_out, &c->tgt_col, &c->tgt_start, &c->tpos,
                  &c->halo_ptr, &c->halo_slot, &c->tile_desc, &c->part, &c->ad, &c->al,
                  &c->ad32, &c->al32, &c->m32, &c->p32, &c->q32, &c->r32, &c->x32,
                  &c->r0v, &c->tv, &c->unit, &c->gbasis, &c->garrays, &c->gstate,
                  &c->bia, &c->bt, &c->sell_ptr, &c->sell_col,
                  &c->sell_val, &c->sell_val64, &c->sell_d16,
                  &c->node_count, &c->tstress, &c->tx0buf, &c->fbuf, &c->ld_node, &c->ld_ptr,
                  &c->ld_ent, &c->ld_vec, &c->vtkbuf,
                  &c->u, &c->b0, &c->b, &c->xs, &c->r, &c->p, &c->q, &c->m, &c->z,
                  &c->scal, &c->partials, &c->counters, &c->flags, &c->diag})
    c->release(*d);
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto &e : c->ev_t)
    if (e) cudaEventDestroy(e);
  release_block(c);
  if (c->stream) cudaStreamSynchronize(c->stream);  // the stream-ordered frees
  elx::pinned_block_put(c->pinned);
  if (c->vtk_host) cudaFreeHost(c->vtk_host);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->pool_user) elx::pool_users(c->device, -1);
  delete c;
}

const char *elx_last_error(const elx_ctx *c) { return c ? c->err.c_str() : "null context"; }

void *elx_stream(elx_ctx *c) { return c ? (void *)c->stream : nullptr; }

int64_t elx_device_bytes(const elx_ctx *c) { return c ? c->used : 0; }

int64_t elx_kernel_launches(const elx_ctx *c) { return c ? c->launches : 0; }

int elx_set_mesh(elx_ctx *c, int32_t ndm, int32_t ndf, int32_t nen, int32_t numel,
                 int32_t nnode, const int32_t *ix, const double *x, const int32_t *ie,
                 const double *e, int32_t prop, int32_t numat) {
  return guarded(c, [&] {
    require(ix && x && ie && e, ELX_ERR_ARG, "null mesh array");
    check_mesh(ndm, ndf, nen, numel, nnode, ix, ie, numat, prop);
    fill_mesh(c->mesh, ndm, ndf, nen, numel, nnode, ix, x, ie, e, prop, numat);
    c->have_mesh = true;
    c->have_structure = false;
    c->have_matrix = false;
  });
}

int elx_set_structure(elx_ctx *c, int32_t neq, int64_t nad, const int32_t *id,
                      const int32_t *ia, const int32_t *ja) {
  return guarded(c, [&] {
    require(c->have_mesh, ELX_ERR_STATE, "set the mesh first");
    require(id && ia && (ja || nad == 0) && neq > 0 && nad >= 0 && nad < INT_MAX, ELX_ERR_ARG,
            "invalid structure arguments");
    require(ia[0] == 1 && (int64_t)ia[neq] - 1 == nad, ELX_ERR_ARG, "ia inconsistent with nad");
    const elx::Mesh &m = c->mesh;
    elx::Structure &s = c->s;
    s.neq = neq;
    s.nad = nad;
    s.id.assign(id, id + (size_t)m.ndf * m.nnode);
    for (int32_t q : s.id) require(q >= 0 && q <= neq, ELX_ERR_ARG, "id out of range");
    s.ia.assign(ia, ia + neq + 1);
    s.ja.assign(ja, ja + nad);
    for (int i = 0; i < neq; i++) {
      require(ia[i + 1] >= ia[i], ELX_ERR_ARG, "ia not monotone");
      for (int32_t k = ia[i]; k < ia[i + 1]; k++) {
        const int32_t col = ja[k - 1];
        require(col >= 1 && col <= i, ELX_ERR_ARG, "ja entry not strictly lower");
        require(k == ia[i] || ja[k - 2] < col, ELX_ERR_ARG, "ja row not ascending");
      }
    }
    s.perm.resize(m.nnode);
    for (int i = 0; i < m.nnode; i++) s.perm[i] = i + 1;
    upload_structure(c);
  });
}

int elx_build_structure(elx_ctx *c, const int32_t *bc, int32_t reorder) {
  return guarded(c, [&] {
    require(c->have_mesh, ELX_ERR_STATE, "set the mesh first");
    require(bc != nullptr, ELX_ERR_ARG, "null bc");
    build_host_structure(c->mesh, bc, reorder != 0, c->s);
    upload_structure(c);
  });
}

struct elx_host_structure {
  elx::Structure s;
  elx::Mesh m;  // connectivity only (coordinates and materials zero)
  int ndf = 0;
  std::string err;
};

int elx_host_structure_create(elx_host_structure **out, int32_t ndm, int32_t ndf, int32_t nen,
                              int32_t numel, int32_t nnode, const int32_t *ix, const int32_t *ie,
                              int32_t numat, const int32_t *bc, int32_t reorder) {
  if (!out || !ix || !ie || !bc) return ELX_ERR_ARG;
  *out = nullptr;
  try {
    elx::Mesh m;
    const std::vector<double> x((size_t)ndm * nnode, 0.0), e((size_t)3 * numat, 0.0);
    check_mesh(ndm, ndf, nen, numel, nnode, ix, ie, numat, 3);
    fill_mesh(m, ndm, ndf, nen, numel, nnode, ix, x.data(), ie, e.data(), 3, numat);
    auto *h = new elx_host_structure();
    h->ndf = ndf;
    build_host_structure(m, bc, reorder != 0, h->s);
    h->m = std::move(m);
    *out = h;
    return ELX_OK;
  } catch (const Error &e) {
    return e.code;
  } catch (const std::bad_alloc &) {
    return ELX_ERR_OOM;
  }
}

namespace {
int host_partition(const elx_host_structure *h, int32_t nparts, int32_t part,
                   elx::Partition &p) {
  if (!h || nparts < 1 || part < 0 || part >= nparts) return ELX_ERR_ARG;
  try {
    const std::vector<int32_t> b = elx::partition_bounds(h->s, h->ndf, nparts);
    if (b.empty()) return ELX_ERR_ARG;
    elx::build_partition(h->s, b[part], b[part + 1], p);
    return ELX_OK;
  } catch (const std::bad_alloc &) {
    return ELX_ERR_OOM;
  }
}
}  // namespace

int elx_host_partition_sizes(const elx_host_structure *h, int32_t nparts, int32_t part,
                             int32_t *eq0, int32_t *neq, int32_t *nhalo, int64_t *nad,
                             int64_t *nad1) {
  elx::Partition p;
  const int st = host_partition(h, nparts, part, p);
  if (st != ELX_OK) return st;
  if (eq0) *eq0 = p.eq0;
  if (neq) *neq = p.neq;
  if (nhalo) *nhalo = (int32_t)p.halo.size();
  if (nad) *nad = (int64_t)p.ja.size();
  if (nad1) *nad1 = (int64_t)p.ja1.size();
  return ELX_OK;
}

int elx_host_partition_get(const elx_host_structure *h, int32_t nparts, int32_t part,
                           int32_t *halo, int32_t *ia, int32_t *ja, int32_t *ia1,
                           int32_t *ja1, int64_t *pos, int64_t *pos1) {
  elx::Partition p;
  const int st = host_partition(h, nparts, part, p);
  if (st != ELX_OK) return st;
  auto put = [](auto *dst, const auto &v) {
    if (dst) std::copy(v.begin(), v.end(), dst);
  };
  put(halo, p.halo);
  put(ia, p.ia);
  put(ja, p.ja);
  put(ia1, p.ia1);
  put(ja1, p.ja1);
  put(pos, p.pos);
  put(pos1, p.pos1);
  return ELX_OK;
}

int elx_host_structure_sizes(const elx_host_structure *h, int32_t *neq, int64_t *nad) {
  if (!h) return ELX_ERR_ARG;
  if (neq) *neq = h->s.neq;
  if (nad) *nad = h->s.nad;
  return ELX_OK;
}

int elx_host_structure_get(const elx_host_structure *h, int32_t *perm, int32_t *id, int32_t *ia,
                           int32_t *ja) {
  if (!h) return ELX_ERR_ARG;
  const elx::Structure &s = h->s;
  if (perm) std::copy(s.perm.begin(), s.perm.end(), perm);
  if (id) std::copy(s.id.begin(), s.id.end(), id);
  if (ia) std::copy(s.ia.begin(), s.ia.end(), ia);
  if (ja) std::copy(s.ja.begin(), s.ja.end(), ja);
  return ELX_OK;
}

int elx_host_structure_colors(const elx_host_structure *h, int32_t *elcolor, int32_t *ncolors) {
  if (!h) return ELX_ERR_ARG;
  try {
    std::vector<int32_t> color;
    const int n = elx::color_elements(h->m, color);
    if (ncolors) *ncolors = n;
    if (elcolor)
      for (size_t el = 0; el < color.size(); el++) elcolor[el] = color[el] + 1;
    return ELX_OK;
  } catch (const std::bad_alloc &) {
    return ELX_ERR_OOM;
  }
}

void elx_host_structure_destroy(elx_host_structure *h) { delete h; }

int elx_get_sizes(const elx_ctx *c, int32_t *neq, int64_t *nad, int32_t *ncolors) {
  if (!c) return ELX_ERR_ARG;
  if (!c->have_structure) return ELX_ERR_STATE;
  if (neq) *neq = c->s.neq;
  if (nad) *nad = c->s.nad;
  if (ncolors) *ncolors = c->s.ncolors;
  return ELX_OK;
}

int elx_get_structure(const elx_ctx *c, int32_t *perm, int32_t *id, int32_t *ia, int32_t *ja) {
  if (!c) return ELX_ERR_ARG;
  if (!c->have_structure) return ELX_ERR_STATE;
  const elx::Structure &s = c->s;
  if (perm) std::copy(s.perm.begin(), s.perm.end(), perm);
  if (id) std::copy(s.id.begin(), s.id.end(), id);
  if (ia) std::copy(s.ia.begin(), s.ia.end(), ia);
  if (ja) std::copy(s.ja.begin(), s.ja.end(), ja);
  return ELX_OK;
}

int elx_set_state(elx_ctx *c, const double *u, const double *b0) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "set the structure first");
    if (u)
      ELX_CUDA(cudaMemcpyAsync(c->u.p, u, (size_t)c->mesh.ndf * c->mesh.nnode * 8,
                               cudaMemcpyHostToDevice, c->stream));
    else
      ELX_CUDA(cudaMemsetAsync(c->u.p, 0, c->u.bytes, c->stream));
    if (b0)
      ELX_CUDA(cudaMemcpyAsync(c->b0.p, b0, (size_t)c->s.neq * 8, cudaMemcpyHostToDevice,
                               c->stream));
    else
      ELX_CUDA(cudaMemsetAsync(c->b0.p, 0, c->b0.bytes, c->stream));
    c->sync();
  });
}

int elx_set_loads(elx_ctx *c, const double *f, const int32_t *eload, const double *loadvec,
                  int32_t nload) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "set the structure first");
    require(f != nullptr, ELX_ERR_ARG, "null f");
    const elx::Mesh &m = c->mesh;
    const size_t nf = (size_t)m.ndf * m.nnode;
    std::vector<int32_t> node, ptr, ent;
    if (eload) {
      require(m.ndm == 2 && m.ndf == 2, ELX_ERR_ARG,
              "distributed edge loads are 2-D only (the reference stops on 3-D element loads)");
      require(nload >= 0 && (nload == 0 || loadvec), ELX_ERR_ARG, "null loadvec");
      int32_t bad_el = 0;
      if (!elx::build_edge_lists(m, eload, nload, node, ptr, ent, bad_el))
        throw Error{ELX_ERR_ARG, "bad load number or unloadable side in element " +
                                     std::to_string(bad_el)};
    }
    if (!c->fbuf.p) c->alloc(c->fbuf, nf * 8);
    ELX_CUDA(cudaMemcpyAsync(c->fbuf.p, f, nf * 8, cudaMemcpyHostToDevice, c->stream));
    elx::launch_pload((int64_t)nf, c->eq.as<int32_t>(), c->fbuf.as<double>(), c->u.as<double>(),
                      c->b0.as<double>(), c->stream);
    c->launches += 1;
    if (!node.empty()) {
      c->upload(c->ld_node, node.data(), node.size());
      c->upload(c->ld_ptr, ptr.data(), ptr.size());
      c->upload(c->ld_ent, ent.data(), ent.size());
      c->upload(c->ld_vec, loadvec, (size_t)nload * 2);
      const int32_t big = INT_MAX;
      int32_t *bad = c->flags.as<int32_t>();
      ELX_CUDA(cudaMemcpyAsync(bad, &big, sizeof(big), cudaMemcpyHostToDevice, c->stream));
      elx::launch_edge_loads((int)node.size(), c->ld_node.as<int32_t>(), c->ld_ptr.as<int32_t>(),
                             c->ld_ent.as<int32_t>(), c->x.as<double>(), c->eq.as<int32_t>(),
                             c->ld_vec.as<double>(), c->b0.as<double>(), bad, c->stream);
      c->launches += 1;
      ELX_CUDA(cudaMemcpyAsync(c->h_flags, bad, sizeof(int32_t), cudaMemcpyDeviceToHost,
                               c->stream));
    }
    c->sync();
    if (!node.empty() && c->h_flags[0] != INT_MAX)
      throw Error{ELX_ERR_BAD_DET, "zero-length loaded side in element " +
                                       std::to_string(c->h_flags[0])};
  });
}

int elx_get_state(elx_ctx *c, double *u, double *b0) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "set the structure first");
    if (u)
      ELX_CUDA(cudaMemcpyAsync(u, c->u.p, (size_t)c->mesh.ndf * c->mesh.nnode * 8,
                               cudaMemcpyDeviceToHost, c->stream));
    if (b0)
      ELX_CUDA(cudaMemcpyAsync(b0, c->b0.p, (size_t)c->s.neq * 8, cudaMemcpyDeviceToHost,
                               c->stream));
    c->sync();
  });
}

int elx_assemble_resident(elx_ctx *c) { return guarded(c, [&] { assemble_resident(c); }); }

int elx_assemble(elx_ctx *c, const double *u, const double *b0, double *b_out, double *ad_out,
                 double *al_out) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "set the structure first");
    if (u)
      ELX_CUDA(cudaMemcpyAsync(c->u.p, u, (size_t)c->mesh.ndf * c->mesh.nnode * 8,
                               cudaMemcpyHostToDevice, c->stream));
    else
      ELX_CUDA(cudaMemsetAsync(c->u.p, 0, c->u.bytes, c->stream));
    if (b0)
      ELX_CUDA(cudaMemcpyAsync(c->b0.p, b0, (size_t)c->s.neq * 8, cudaMemcpyHostToDevice,
                               c->stream));
    else
      ELX_CUDA(cudaMemsetAsync(c->b0.p, 0, c->b0.bytes, c->stream));
    assemble_resident(c);
    const size_t n = (size_t)c->s.neq, nad = (size_t)c->s.nad;
    if (b_out) ELX_CUDA(cudaMemcpyAsync(b_out, c->b.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
    if (ad_out)
      ELX_CUDA(cudaMemcpyAsync(ad_out, c->ad.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
    if (al_out && nad)
      ELX_CUDA(cudaMemcpyAsync(al_out, c->al.p, nad * 8, cudaMemcpyDeviceToHost, c->stream));
    c->sync();
  });
}

int elx_set_matrix(elx_ctx *c, const double *ad, const double *al) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "set the structure first");
    require(ad && (al || c->s.nad == 0), ELX_ERR_ARG, "null matrix array");
    ELX_CUDA(cudaMemcpyAsync(c->ad.p, ad, (size_t)c->s.neq * 8, cudaMemcpyHostToDevice,
                             c->stream));
    if (c->s.nad)
      ELX_CUDA(cudaMemcpyAsync(c->al.p, al, (size_t)c->s.nad * 8, cudaMemcpyHostToDevice,
                               c->stream));
    refresh_derived_values(c);
    c->sync();
    c->have_matrix = true;
    c->have_fp32 = false;
  });
}

int elx_solve_resident(elx_ctx *c, int32_t solver, int32_t precision, double tol,
                       int32_t maxit, int32_t ngram, elx_info *info) {
  return guarded(c, [&] { solve_resident(c, solver, precision, tol, maxit, ngram, info); });
}

int elx_solve(elx_ctx *c, int32_t solver, int32_t precision, double tol, int32_t maxit,
              int32_t ngram, const double *b, double *x, elx_info *info) {
  return guarded(c, [&] {
    require(c->have_matrix, ELX_ERR_STATE, "solve before the matrix is assembled");
    require(b && x, ELX_ERR_ARG, "null b or x");
    ELX_CUDA(cudaMemcpyAsync(c->b.p, b, (size_t)c->s.neq * 8, cudaMemcpyHostToDevice,
                             c->stream));
    int st = ELX_OK;
    try {
      solve_resident(c, solver, precision, tol, maxit, ngram, info);
    } catch (const Error &e) {
      if (e.code != ELX_ERR_NO_CONVERGENCE) throw;
      st = e.code;
      c->err = e.msg;
    }
    ELX_CUDA(cudaMemcpyAsync(x, c->xs.p, (size_t)c->s.neq * 8, cudaMemcpyDeviceToHost,
                             c->stream));
    c->sync();
    if (st != ELX_OK) throw Error{st, c->err};
  });
}

int elx_stress(elx_ctx *c, const double *u, const double *tx0, double *t) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "stresses before the structure is set");
    require(t != nullptr, ELX_ERR_ARG, "null t");
    const elx::Mesh &m = c->mesh;
    const int ntn = m.ndm == 2 ? 4 : 6;
    const size_t nn = (size_t)m.nnode;
    if (!c->node_count.p) {
      // elements at each node (ic of Pform.f:400-403), once per mesh
      std::vector<int32_t> cnt(nn, 0);
      for (int el = 0; el < m.numel; el++)
        for (int a = 0; a < m.nen; a++) {
          const int no = m.ix[(size_t)el * (m.nen + 1) + a];
          if (no > 0) cnt[no - 1]++;
        }
      c->upload(c->node_count, cnt.data(), cnt.size());
      c->alloc(c->tstress, nn * ntn * 8);
      c->sync();
    }
    if (u)
      ELX_CUDA(cudaMemcpyAsync(c->u.p, u, (size_t)m.ndf * nn * 8, cudaMemcpyHostToDevice,
                               c->stream));
    const double *tx0d = nullptr;
    if (tx0) {
      if (!c->tx0buf.p) c->alloc(c->tx0buf, nn * ntn * 8);
      ELX_CUDA(cudaMemcpyAsync(c->tx0buf.p, tx0, nn * ntn * 8, cudaMemcpyHostToDevice,
                               c->stream));
      tx0d = c->tx0buf.as<double>();
    }
    ELX_CUDA(cudaMemsetAsync(c->tstress.p, 0, nn * ntn * 8, c->stream));
    const int32_t big = INT_MAX;
    int32_t *bad = c->flags.as<int32_t>();
    ELX_CUDA(cudaMemcpyAsync(bad, &big, sizeof(big), cudaMemcpyHostToDevice, c->stream));
    const elx::MeshDev md = c->mesh_dev();
    for (const elx::Segment &seg : c->s.segments)
      elx::launch_stress(md, seg, c->u.as<double>(), c->tstress.as<double>(), bad, c->stream);
    elx::launch_stress_average(m.nnode, ntn, c->node_count.as<int32_t>(), tx0d,
                               c->tstress.as<double>(), c->stream);
    c->launches += (int64_t)c->s.segments.size() + 1;
    ELX_CUDA(cudaMemcpyAsync(t, c->tstress.p, nn * ntn * 8, cudaMemcpyDeviceToHost, c->stream));
    ELX_CUDA(cudaMemcpyAsync(c->h_flags, bad, sizeof(int32_t), cudaMemcpyDeviceToHost,
                             c->stream));
    c->sync();
    c->have_stress = c->h_flags[0] == INT_MAX;
    if (c->h_flags[0] != INT_MAX)
      throw Error{ELX_ERR_BAD_DET, "non-positive Jacobian determinant in element " +
                                       std::to_string(c->h_flags[0])};
  });
}

// The result file (write_mesh_res_mec) formatted on the device into
// c->vtkbuf; returns its size.
int64_t format_vtk(elx_ctx *c, int format, int fields) {
  require(c->have_structure, ELX_ERR_STATE, "write results after the structure is set");
  require(format == 0 || format == 1, ELX_ERR_ARG,
          "format: 0 (XML VTU ASCII) or 1 (legacy binary VTK)");
  require((fields & ~3) == 0, ELX_ERR_ARG, "fields: 1 desloc, 2 stress");
  require(!(fields & 2) || c->have_stress, ELX_ERR_STATE,
          "stress output asked before elx_stress computed the nodal stresses");
  const elx::Mesh &m = c->mesh;
  int nnoel = 0, ctype = -1;
  for (int el = 0; el < m.numel; el++) {
    const int iel = m.ie[m.ix[(size_t)el * (m.nen + 1) + m.nen] - 1];
    int nn, ct;
    switch (iel) {
      case elx::TRIA3_STRAIN: case elx::TRIA3_STRESS: nn = 3, ct = 5; break;
      case elx::QUAD4_STRAIN: case elx::QUAD4_STRESS: nn = 4, ct = 9; break;
      case elx::TETRA4: nn = 4, ct = 10; break;
      default: nn = 8, ct = 12; break;
    }
    require(ctype < 0 || ct == ctype, ELX_ERR_ARG,
            "the result writer takes meshes of one cell type (as the reference's)");
    ctype = ct;
    nnoel = nn;
  }
  const elx::VtkLayout L =
      elx::vtk_layout(format, fields, m.nnode, m.numel, m.ndf, nnoel, ctype);
  if (c->vtkbuf.bytes < (size_t)L.size) c->alloc(c->vtkbuf, (size_t)L.size);
  elx::launch_vtk(L, c->vtkbuf.as<char>(), c->mesh_dev(), m.ndm == 2 ? 4 : 6, nnoel, ctype,
                  c->u.as<double>(), c->tstress.as<double>(), c->stream);
  c->launches += (int64_t)L.sections.size();
  return L.size;
}

int elx_format_vtk(elx_ctx *c, int32_t format, int32_t fields, char *out, int64_t capacity,
                   int64_t *bytes) {
  return guarded(c, [&] {
    require(bytes != nullptr, ELX_ERR_ARG, "null bytes");
    const int64_t n = format_vtk(c, format, fields);
    *bytes = n;
    if (out) {
      require(capacity >= n, ELX_ERR_ARG, "output buffer too small");
      ELX_CUDA(cudaMemcpyAsync(out, c->vtkbuf.p, (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    }
    c->sync();
  });
}

int elx_write_vtk(elx_ctx *c, const char *path, int32_t format, int32_t fields,
                  int64_t *bytes) {
  return guarded(c, [&] {
    require(path != nullptr, ELX_ERR_ARG, "null path");
    const int64_t n = format_vtk(c, format, fields);
    if (c->vtk_host_bytes < (size_t)n) {
      if (c->vtk_host) cudaFreeHost(c->vtk_host);
      c->vtk_host = nullptr;
      c->vtk_host_bytes = 0;
      ELX_CUDA(cudaMallocHost(&c->vtk_host, (size_t)n));
      c->vtk_host_bytes = (size_t)n;
    }
    ELX_CUDA(cudaMemcpyAsync(c->vtk_host, c->vtkbuf.p, (size_t)n, cudaMemcpyDeviceToHost,
                             c->stream));
    c->sync();
    FILE *f = std::fopen(path, "wb");
    require(f != nullptr, ELX_ERR_ARG, "cannot open the output file");
    const size_t w = std::fwrite(c->vtk_host, 1, (size_t)n, f);
    const int cl = std::fclose(f);
    require(w == (size_t)n && cl == 0, ELX_ERR_ARG, "short write of the output file");
    if (bytes) *bytes = n;
  });
}

int elx_partition_spmv(elx_ctx *c, int32_t nparts, const double *x, double *y) {
  return guarded(c, [&] {
    require(c->have_matrix, ELX_ERR_STATE, "no matrix");
    require(x && y && nparts >= 1, ELX_ERR_ARG, "null x or y, or nparts < 1");
    const size_t n = (size_t)c->s.neq;
    ELX_CUDA(cudaMemcpyAsync(c->p.p, x, n * 8, cudaMemcpyHostToDevice, c->stream));
    partition_product(c, nparts, c->p.as<double>(), c->q.as<double>());
    ELX_CUDA(cudaMemcpyAsync(y, c->q.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
    c->sync();
  });
}

int elx_partition_spmv_resident(elx_ctx *c, int32_t nparts, int32_t reps) {
  return guarded(c, [&] {
    require(c->have_matrix, ELX_ERR_STATE, "no matrix");
    require(nparts >= 1 && reps >= 0, ELX_ERR_ARG, "nparts < 1 or reps < 0");
    for (int i = 0; i < reps; i++)
      partition_product(c, nparts, c->p.as<double>(), c->q.as<double>());
  });
}

int elx_partition_info(elx_ctx *c, int32_t nparts, int32_t part, int32_t *eq0, int32_t *neq,
                       int32_t *nhalo) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "set the structure first");
    require(part >= 0 && part < nparts, ELX_ERR_ARG, "part outside 0..nparts-1");
    ensure_partitions(c, nparts);
    const elx_ctx::DevPartition &d = c->parts[part];
    const int B = c->s.bsize;
    if (eq0) *eq0 = d.I0 * B;
    if (neq) *neq = (d.I1 - d.I0) * B;
    if (nhalo) *nhalo = d.nhb * B;
  });
}

int elx_fortran_e(const double *x, int32_t n, int32_t w, int32_t d, int32_t e, char *out) {
  // a stand-alone test hook: no context, its own buffers on device 0's
  // current device
  if (!x || !out || n < 0 || w <= 0 || w > 40 || d < 1 || d > 9 || e < 0 || e > 4)
    return ELX_ERR_ARG;
  double *dx = nullptr;
  char *dout = nullptr;
  cudaError_t st = cudaMalloc(&dx, (size_t)n * 8 + 8);
  if (st == cudaSuccess) st = cudaMalloc(&dout, (size_t)n * w + 8);
  if (st == cudaSuccess) st = cudaMemcpy(dx, x, (size_t)n * 8, cudaMemcpyHostToDevice);
  if (st == cudaSuccess) {
    elx::launch_fortran_e(dx, n, w, d, e, dout, nullptr);
    st = cudaMemcpy(out, dout, (size_t)n * w, cudaMemcpyDeviceToHost);
  }
  cudaFree(dx);
  cudaFree(dout);
  return st == cudaSuccess ? ELX_OK : ELX_ERR_CUDA;
}

int elx_solve_block(elx_ctx *c, int32_t nrhs, int32_t precision, double tol, int32_t maxit,
                    int32_t width, const double *b, double *x, elx_info *info) {
  return guarded(c, [&] {
    require(b && x, ELX_ERR_ARG, "null b or x");
    solve_block(c, nrhs, precision, tol, maxit, width, b, x, info, false);
  });
}

int elx_solve_block_device(elx_ctx *c, int32_t nrhs, int32_t precision, double tol,
                           int32_t maxit, int32_t width, const double *b, double *x,
                           elx_info *info) {
  return guarded(c, [&] {
    require(b && x, ELX_ERR_ARG, "null b or x");
    solve_block(c, nrhs, precision, tol, maxit, width, b, x, info, true);
  });
}

int elx_autotune_block(elx_ctx *c, int32_t precision, int32_t *width, double *times_us) {
  return guarded(c, [&] {
    require(c->have_matrix, ELX_ERR_STATE, "autotune before the matrix is assembled");
    require(c->use_blocks, ELX_ERR_ARG, "block solves need node blocks");
    require(width, ELX_ERR_ARG, "null width");
    const bool mixed = precision == ELX_PREC_MIXED;
    if (times_us) c->tuned_width[mixed ? 1 : 0] = 0;
    *width = autotune_block_width(c, mixed, times_us);
  });
}

int elx_block_tiling(elx_ctx *c, int32_t precision, int32_t *unroll) {
  return guarded(c, [&] {
    require(unroll, ELX_ERR_ARG, "null unroll");
    const int slot = precision == ELX_PREC_MIXED ? 1 : 0;
    for (int i = 0; i < 5; i++) unroll[i] = c->tuned_unroll[slot][i];
  });
}

int elx_update(elx_ctx *c, const double *x, double *u) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "set the structure first");
    require(x && u, ELX_ERR_ARG, "null x or u");
    const std::vector<int32_t> &id = c->s.id;
    for (size_t q = 0; q < id.size(); q++)
      if (id[q] > 0) u[q] = x[id[q] - 1];
  });
}

int elx_update_resident(elx_ctx *c) {
  return guarded(c, [&] {
    require(c->have_structure, ELX_ERR_STATE, "set the structure first");
    elx::launch_update((int64_t)c->mesh.ndf * c->mesh.nnode, c->eq.as<int32_t>(),
                       c->xs.as<double>(), c->u.as<double>(), c->stream);
    c->launches += 1;
  });
}

int elx_spmv(elx_ctx *c, int32_t precision, const double *x, double *y) {
  return guarded(c, [&] {
    require(c->have_matrix, ELX_ERR_STATE, "no matrix");
    require(x && y, ELX_ERR_ARG, "null x or y");
    const size_t n = (size_t)c->s.neq;
    ELX_CUDA(cudaMemcpyAsync(c->p.p, x, n * 8, cudaMemcpyHostToDevice, c->stream));
    if (precision == ELX_PREC_FP64) {
      spmv64(c, c->p.as<double>(), c->q.as<double>());
    } else if (precision == ELX_PREC_MIXED) {
      // the FP32 product of the mixed-precision inner iteration
      ensure_fp32(c);
      elx::launch_convert((int)n, c->p.as<double>(), c->p32.as<float>(), c->stream);
      elx::launch_gather_spmv32(c->csrc_dev(), c->p32.as<float>(), c->q32.as<float>(), nullptr,
                                nullptr, nullptr, c->stream);
      elx::launch_widen((int)n, c->q32.as<float>(), c->q.as<double>(), c->stream);
      c->launches += 3;
    } else {
      throw Error{ELX_ERR_ARG, "precision not available"};
    }
    ELX_CUDA(cudaMemcpyAsync(y, c->q.p, n * 8, cudaMemcpyDeviceToHost, c->stream));
    c->sync();
    if (c->spmv_kind == elx::kSpmvTiled) check_pipe_waits(c);
  });
}

int elx_spmv_resident(elx_ctx *c, int32_t precision, int32_t reps) {
  return guarded(c, [&] {
    require(c->have_matrix, ELX_ERR_STATE, "no matrix");
    // the product as the solvers launch it: q = K p with the fused (p, q)
    // (fresh scalars, so that no finished-solve flag skips the work)
    set_scalars(c, 0.0, 0);
    auto *sc = c->scal.as<elx::PcgScalars>();
    if (precision == ELX_PREC_FP64) {
      for (int i = 0; i < reps; i++) {
        if (c->spmv_kind == elx::kSpmvTiled) {
          spmv64(c, c->p.as<double>(), c->q.as<double>());
        } else {
          elx::launch_gather_spmv64(c->csrc_dev(), c->p.as<double>(), c->q.as<double>(), sc,
                                    c->partials.as<double>(), c->counters.as<unsigned int>(),
                                    c->stream);
          c->launches += 1;
        }
      }
    } else if (precision == ELX_PREC_MIXED) {
      ensure_fp32(c);
      elx::launch_convert(c->s.neq, c->p.as<double>(), c->p32.as<float>(), c->stream);
      for (int i = 0; i < reps; i++)
        elx::launch_gather_spmv32(c->csrc_dev(), c->p32.as<float>(), c->q32.as<float>(), sc,
                                  c->partials.as<double>(), c->counters.as<unsigned int>(),
                                  c->stream);
      c->launches += 1 + reps;
    } else {
      throw Error{ELX_ERR_ARG, "precision not available"};
    }
  });
}

int elx_get_solution(elx_ctx *c, double *x) {
  return guarded(c, [&] {
    require(c->have_structure && x, ELX_ERR_ARG, "no structure or null x");
    ELX_CUDA(cudaMemcpyAsync(x, c->xs.p, (size_t)c->s.neq * 8, cudaMemcpyDeviceToHost,
                             c->stream));
    c->sync();
  });
}

int elx_get_rhs(elx_ctx *c, double *b) {
  return guarded(c, [&] {
    require(c->have_structure && b, ELX_ERR_ARG, "no structure or null b");
    ELX_CUDA(cudaMemcpyAsync(b, c->b.p, (size_t)c->s.neq * 8, cudaMemcpyDeviceToHost,
                             c->stream));
    c->sync();
  });
}

}  // extern "C"
