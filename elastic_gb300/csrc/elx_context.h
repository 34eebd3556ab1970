// The library context (elx_ctx of the C ABI) and the host-side operations on
// it that more than one translation unit uses (api.cu: the C ABI;
// server.cu: the solve server, which keeps one context per admitted
// request).
#pragma once

#include <string>

#include "elx_krylov.h"

using elx::DBuf;
using elx::Error;

struct elx_ctx {
  int device = 0;
  int verbose = 0;
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;  // the device's stream-ordered pool (or plain cudaMalloc)
  void *pinned = nullptr;        // the recycled pinned block of h_scal, h_diag, h_flags
  bool pool_user = false;        // counted among the pool's users
  int64_t budget = 0, used = 0;
  std::string err;

  elx::Mesh mesh;
  elx::Structure s;
  bool have_mesh = false, have_structure = false, have_matrix = false;
  // the FP32 copy of the matrix (sliced node blocks, or the scalar CSRC
  // arrays) was made since the last assembly
  bool have_fp32 = false;

  // mesh (colour order) and structure
  DBuf conn, mat, elnum, slot, x, eq, e;
  DBuf ia, ja, iat, jat, pt, ja16, jat16;
  // node blocks (when the numbering allows them): block row pointers and
  // mirror positions (read by the fill of the sliced copies)
  DBuf bia, bt;
  // the sliced copies of the node blocks (FP64, always; FP32 for the mixed
  // solvers) and their pattern; each read with streaming loads unless it
  // fits in 60 % of L2
  DBuf sell_ptr, sell_col, sell_val, sell_val64, sell_d16;
  bool sell_stream = true, sell64_stream = true;
  bool use_blocks = false;
  // tiled transposed index of the SpMV and its halo slots
  DBuf tile_tgt, tile_out, tgt_col, tgt_start, tpos, halo_ptr, halo_slot, tile_desc, part;
  // matrix
  DBuf ad, al, alt, ad32, al32, alt32;
  int spmv_kind = elx::kSpmvGather;  // FP64 SpMV kernel family
  bool use_delta = true;             // 16-bit column deltas when the bandwidth fits
  int gather_blocks = 0;             // gather SpMV grid (0: default)
  int spmm_unroll = 0;  // slot groups in flight in the block product (0: default)
  // state and solver vectors
  DBuf u, b0, b, xs, r, p, q, m, z;
  // mixed precision: FP32 inner PCG vectors and preconditioner
  DBuf m32, p32, q32, r32, x32;
  // stress recovery: elements per node, nodal stresses, initial stresses
  DBuf node_count, tstress, tx0buf;
  // device loads: nodal loads f, edge-load lists and load vectors
  DBuf fbuf, ld_node, ld_ptr, ld_ent, ld_vec;
  bool have_stress = false;  // tstress holds the last elx_stress result
  // row-block partitions of the node-block matrix (partition.cu): owned
  // block rows [I0, I1) = slices [s0, s1) of the sliced copy, values at voff,
  // local slice pointers and columns, halo blocks, the gathered x
  struct DevPartition {
    int32_t I0 = 0, I1 = 0, s0 = 0, s1 = 0, nhb = 0;
    int64_t voff = 0;
    DBuf sptr, scol, hb, xloc;
  };
  std::vector<DevPartition> parts;
  int parts_n = 0;
  // result writer: the formatted file on the device and its pinned copy
  DBuf vtkbuf;
  char *vtk_host = nullptr;
  size_t vtk_host_bytes = 0;
  // BiCGSTAB (r0, t) and GMRES (Krylov basis, small dense arrays, state)
  DBuf r0v, tv, unit, gbasis, garrays, gstate;
  // block PCG: multi-vectors of up to blk_cap columns, scalars, staging
  DBuf bk_b, bk_x, bk_r, bk_p, bk_q, bk_z, bk_xlo, bk_r32, bk_p32, bk_q32, bk_cols, bk_hdr,
      bk_part, bk_cnt, bk_diag, bk_colmajor;
  int blk_cap = 0;
  int tuned_width[2] = {0, 0};  // autotuned block width (FP64, mixed)
  // autotuned slot groups in flight of the block product per width
  // ([FP64, mixed][log2 W]; 0: the default)
  int tuned_unroll[2][5] = {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}};
  cudaGraphExec_t block_graph = nullptr;
  // called with 1 before and 0 after each batch of block iterations (launch
  // and poll); a solve server holds a block solve's batches back here while
  // small requests need the GPU
  void (*batch_gate)(void *user, int enter) = nullptr;
  void *batch_gate_user = nullptr;
  int block_graph_w = 0;
  bool block_graph_mixed = false;
  // scalars, partials, counters, flags
  DBuf scal, partials, counters, flags, diag;
  elx::PcgScalars *h_scal = nullptr;  // pinned, 2 slots
  double *h_diag = nullptr;           // pinned
  int32_t *h_flags = nullptr;         // pinned

  int64_t launches = 0;  // kernels of this library launched by this context

  cudaGraphExec_t pcg_graph = nullptr;    // kBatch FP64 PCG iterations
  cudaGraphExec_t pcg32_graph = nullptr;  // kBatch FP32 inner PCG iterations
  cudaGraphExec_t bicg_graph = nullptr;   // kBatch BiCGSTAB iterations
  bool bicg_plain = false;                // bicg_graph has M = I (no preconditioner)
  cudaGraphExec_t gmres_graph = nullptr;  // one GMRES(gmres_k) restart cycle
  int gmres_k = 0, gmres_launches = 0;
  int pcg_graph_iters = 0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaEvent_t ev_t[2] = {nullptr, nullptr};  // timing (autotuner)

  void alloc(DBuf &d, size_t bytes) {
    release(d);
    if (bytes == 0) bytes = 16;
    if (budget > 0 && used + (int64_t)bytes > budget)
      throw Error{ELX_ERR_OOM, "HBM budget exceeded: need " + std::to_string(bytes) +
                                   " more bytes, " + std::to_string(budget - used) + " left"};
    cudaError_t me =
        pool ? cudaMallocFromPoolAsync(&d.p, bytes, pool, stream) : cudaMalloc(&d.p, bytes);
    if (me != cudaSuccess && pool) {
      // the pool keeps freed memory reserved: hand what none of its users
      // holds back to the device (this stream's own frees done first) and
      // try once more
      (void)cudaGetLastError();
      cudaStreamSynchronize(stream);
      cudaMemPoolTrimTo(pool, 0);
      me = cudaMallocFromPoolAsync(&d.p, bytes, pool, stream);
    }
    if (me != cudaSuccess) {
      d.p = nullptr;
      (void)cudaGetLastError();
      throw Error{ELX_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(me)};
    }
    d.bytes = bytes;
    used += (int64_t)bytes;
  }
  void release(DBuf &d) {
    if (d.p) {
      // stream-ordered: the memory returns to the pool once the context's
      // stream has passed its last use
      if (pool)
        cudaFreeAsync(d.p, stream);
      else
        cudaFree(d.p);
      used -= (int64_t)d.bytes;
    }
    d.p = nullptr;
    d.bytes = 0;
  }
  // Arrays read by bulk copies get 64 bytes of slack: a copy rounded out to
  // 16-byte boundaries may read up to 15 bytes past the last element.
  template <class T>
  void upload(DBuf &d, const T *src, size_t n) {
    alloc(d, n * sizeof(T) + 64);
    if (n) ELX_CUDA(cudaMemcpyAsync(d.p, src, n * sizeof(T), cudaMemcpyHostToDevice, stream));
  }
  void sync() { ELX_CUDA(cudaStreamSynchronize(stream)); }
  void drop_graphs() {
    if (pcg_graph) cudaGraphExecDestroy(pcg_graph);
    if (pcg32_graph) cudaGraphExecDestroy(pcg32_graph);
    if (bicg_graph) cudaGraphExecDestroy(bicg_graph);
    if (gmres_graph) cudaGraphExecDestroy(gmres_graph);
    if (block_graph) cudaGraphExecDestroy(block_graph);
    pcg_graph = pcg32_graph = bicg_graph = gmres_graph = block_graph = nullptr;
    block_graph_w = 0;
    gmres_k = gmres_launches = 0;
    pcg_graph_iters = 0;
  }

  elx::MeshDev mesh_dev() const {
    elx::MeshDev md;
    md.ndm = mesh.ndm; md.ndf = mesh.ndf; md.nen = mesh.nen; md.numel = mesh.numel;
    md.nnode = mesh.nnode; md.numat = mesh.numat; md.prop = mesh.prop;
    md.conn = conn.as<int32_t>(); md.mat = mat.as<int32_t>(); md.elnum = elnum.as<int32_t>();
    md.slot = slot.as<int32_t>(); md.x = x.as<double>(); md.eq = eq.as<int32_t>();
    md.e = e.as<double>(); md.npairs = s.npairs;
    return md;
  }
  elx::CsrcDev csrc_dev() const {
    elx::CsrcDev k;
    k.neq = s.neq; k.nad = s.nad;
    k.ia = ia.as<int32_t>(); k.ja = ja.as<int32_t>();
    k.iat = iat.as<int32_t>(); k.jat = jat.as<int32_t>(); k.pt = pt.as<int32_t>();
    k.ja16 = s.bw16 && use_delta ? ja16.as<uint16_t>() : nullptr;
    k.jat16 = s.bw16 && use_delta ? jat16.as<uint16_t>() : nullptr;
    k.ad = ad.as<double>(); k.al = al.as<double>(); k.alt = alt.as<double>();
    k.ad32 = ad32.as<float>(); k.al32 = al32.as<float>(); k.alt32 = alt32.as<float>();
    k.gather_blocks = gather_blocks;
    k.max_grid = elx::grid_cap(8);
    k.spmm_unroll = spmm_unroll;
    for (int i = 0; i < 5; i++) {
      k.spmm_unroll_w64[i] = tuned_unroll[0][i];
      k.spmm_unroll_w32[i] = tuned_unroll[1][i];
    }
    if (use_blocks) {
      k.bsize = s.bsize; k.nb = s.nb; k.nnzb = s.nnzb;
      k.bia = bia.as<int32_t>(); k.bt = bt.as<int32_t>();
      k.nslices = s.nslices;
      k.sell_ptr = sell_ptr.as<int32_t>(); k.sell_col = sell_col.as<int32_t>();
      k.sell_val = sell_val.as<float>();
      k.sell_stream = sell_stream;
      k.sell_val64 = sell_val64.as<double>();
      k.sell64_stream = sell64_stream;
      k.sell_d16 = static_cast<const int16_t *>(sell_d16.p);
    }
    return k;
  }
  elx::TileDev tile_dev() const {
    elx::TileDev t;
    t.rows = s.tile_rows; t.ntiles = s.ntiles; t.max_nnz = s.max_tile_nnz;
    t.max_tgt = s.max_tile_tgt; t.lanes = s.lanes;
    t.desc = tile_desc.as<int32_t>();
    t.tile_tgt = tile_tgt.as<int32_t>(); t.tile_out = tile_out.as<int32_t>();
    t.tgt_col = tgt_col.as<int32_t>(); t.tgt_start = tgt_start.as<int32_t>();
    t.halo_ptr = halo_ptr.as<int32_t>(); t.halo_slot = halo_slot.as<int32_t>();
    t.tpos = tpos.as<uint16_t>();
    return t;
  }
};

namespace elx_api {

void require(bool c, int code, const char *what);
// Derives (unless `prederived`) and uploads the structure of c->mesh / c->s.
void upload_structure(elx_ctx *c, bool prederived = false);
void assemble_resident(elx_ctx *c);
void build_preconditioner(elx_ctx *c);
void release_block(elx_ctx *c);
// Row-block partitions on one device (partition.cu).
void ensure_partitions(elx_ctx *c, int nparts);
void release_partitions(elx_ctx *c);
void partition_product(elx_ctx *c, int nparts, const double *x, double *y);
// Block PCG of nrhs load cases (api.cu); b, x column-major neq x nrhs.
void solve_block(elx_ctx *c, int nrhs, int precision, double tol, int maxit, int width,
                 const double *b, double *x, elx_info *infos, bool device_ptrs);
void check_mesh(int32_t ndm, int32_t ndf, int32_t nen, int32_t numel, int32_t nnode,
                const int32_t *ix, const int32_t *ie, int32_t numat, int32_t prop);
void fill_mesh(elx::Mesh &m, int32_t ndm, int32_t ndf, int32_t nen, int32_t numel,
               int32_t nnode, const int32_t *ix, const double *x, const int32_t *ie,
               const double *e, int32_t prop, int32_t numat);

}  // namespace elx_api
