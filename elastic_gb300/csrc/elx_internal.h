// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "elastic_gb300.h"

namespace elx {

// ---------------------------------------------------------------- errors
struct Error {
  int code;
  std::string msg;
};

#define ELX_CUDA(call)                                                      \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess)                                                  \
      throw ::elx::Error{ELX_ERR_CUDA, std::string(#call) + ": " +          \
                                           cudaGetErrorString(e_)};         \
  } while (0)

#define ELX_REQUIRE(cond, code, what)                                       \
  do {                                                                      \
    if (!(cond)) throw ::elx::Error{(code), (what)};                        \
  } while (0)

// ------------------------------------------------------- device buffers
// Owning device allocation; every allocation of a context goes through
// Ctx::alloc so that the HBM budget is enforced in one place.
struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  template <class T>
  T *as() const { return static_cast<T *>(p); }
};

// ------------------------------------------------------ host structure
// Element type codes of the reference (Elmlib.f:43-144).
enum ElemType : int32_t {
  TRIA3_STRAIN = 2,
  TRIA3_STRESS = 3,
  QUAD4_STRAIN = 4,
  QUAD4_STRESS = 5,
  TETRA4 = 6,
  HEXA8 = 7
};
int elem_nodes(int iel);  // vertex count, 0 if unsupported

struct Mesh {
  int32_t ndm = 0, ndf = 0, nen = 0, numel = 0, nnode = 0, numat = 0, prop = 0;
  std::vector<int32_t> ix;  // (nen+1, numel), 1-based contents
  std::vector<double> x;    // (ndm, nnode)
  std::vector<int32_t> ie;  // (numat)
  std::vector<double> e;    // (prop, numat)
};

// One launch segment of the assembly: elements [begin, end) of the colour-
// ordered element list, all of the same element type.
struct Segment {
  int32_t iel, begin, end;
};

struct Structure {
  int32_t neq = 0;
  int64_t nad = 0;
  std::vector<int32_t> perm;  // (nnode) 1-based, RCM order (identity if given)
  std::vector<int32_t> id;    // (ndf, nnode) 1-based equation numbers, 0 = fixed
  std::vector<int32_t> ia;    // (neq+1) 1-based
  std::vector<int32_t> ja;    // (nad)   1-based
  // derived, 0-based
  std::vector<int32_t> elem_order;      // colour-ordered element list (0-based)
  std::vector<Segment> segments;        // per colour and element type
  std::vector<int32_t> color_of_segment;
  int32_t ncolors = 0;
  std::vector<int32_t> slot;            // (npairs, numel) in colour order
  int32_t npairs = 0;
  // Tiled transposed index of the strict lower part (see spmv.cu): rows in
  // tiles of tile_rows; per tile its distinct columns ("targets", ascending:
  // first those left of the tile, then those inside), per target the tile-
  // local positions of its entries, and per row the halo slots that the
  // tiles to its right fill for it.
  int32_t tile_rows = 0, ntiles = 0, max_tile_nnz = 0, max_tile_tgt = 0, lanes = 8;
  std::vector<int32_t> tile_desc;  // (8, ntiles): base, nnz, g0, ng, o0, nout, r0, nr
  std::vector<int32_t> tile_tgt;   // (ntiles+1) first target of each tile
  std::vector<int32_t> tile_out;   // (ntiles+1) first halo slot of each tile
  std::vector<int32_t> tgt_col;    // (ntargets) 0-based column
  std::vector<int32_t> tgt_start;  // (ntargets+1) start of the target's positions in tpos
  std::vector<uint16_t> tpos;      // (nad) tile-local entry positions, target order
  std::vector<int32_t> halo_ptr;   // (neq+1)
  std::vector<int32_t> halo_slot;  // (nhalo) slots, tile order within a row
  // Global transposed index of the strict lower part (CSR of the upper
  // part): for each row c the entries of column c of L, by ascending row:
  // their rows jat and their positions pt in al.
  std::vector<int32_t> iat, jat, pt;
  // 16-bit column deltas of both parts (row - col below, col - row above),
  // used when the matrix bandwidth fits (bw16 = true)
  bool bw16 = false;
  std::vector<uint16_t> ja16, jat16;
  // Node blocks (BCSR): when the equations come in runs of B = ndf per node
  // (every node all free or all fixed), K is a matrix of B x B node blocks.
  // Block row I holds equations B I .. B I + B - 1; its blocks in ascending
  // block column: the lower blocks (the order of the CSRC row B I), the
  // diagonal block, the upper blocks.  bt: for an upper block the position
  // of its mirror (a lower block), for a lower or diagonal block -1 - I.
  bool blocked = false;
  int32_t bsize = 0, nb = 0;
  int64_t nnzb = 0;
  std::vector<int32_t> bia, bja, bt;
  // Sliced copy of the node blocks for the FP32 product: block rows in
  // slices of kSliceRows; slice s is sell_ptr[s + 1] - sell_ptr[s] slot
  // groups wide (its longest row), and slot (g, t) is block g - sell_ptr[s]
  // of block row kSliceRows s + t, with block column sell_col[kSliceRows g + t]
  // (padding slots: the row's own column, zero values).
  int32_t nslices = 0;
  std::vector<int32_t> sell_ptr, sell_col;
};

constexpr int kSliceRows = 32;

// Streaming multiprocessors of the current device (read once per device).
int sm_count();

// Device memory of the contexts: one stream-ordered pool per device
// (cudaMallocFromPoolAsync / cudaFreeAsync on the context's stream), so
// that a context's allocations and frees wait for its own stream only --
// cudaFree waits for the whole device, which stalls every other context
// (a solve server's admissions behind its large solves).  Freed memory
// stays in the pool for the next allocation while a pool user (a context
// or a server) lives; the last one to go returns it to the device.
// nullptr where the device has no memory pools (plain cudaMalloc then).
cudaMemPool_t device_pool(int device);
void pool_users(int device, int delta);
// A context's small pinned host scalars: blocks of kPinnedBlock bytes,
// carved from larger pinned allocations and recycled, so that creating and
// destroying contexts pins and unpins no memory once warm.
constexpr size_t kPinnedBlock = 1024;
void *pinned_block_get();
void pinned_block_put(void *p);
// Grid bound of the grid-stride kernels: per_sm CTAs on every SM.
inline int grid_cap(int per_sm) { return sm_count() * per_sm; }

// One row-block partition of the CSRC (structure.cpp): owned global
// equations [eq0, eq0 + neq), local numbering owned 1..neq then the halo
// (equations outside the block that owned rows couple to, ascending) from
// neq + 1; the lower CSRC among owned equations (ia, ja) and the rectangular
// part (ia1, ja1), 1-based as csrstruct(lower, right) lays them out
// (Csr.f:13-305); pos / pos1: each entry's 0-based position in the global al.
struct Partition {
  int32_t eq0 = 0, neq = 0;
  std::vector<int32_t> halo;
  std::vector<int32_t> ia, ja, ia1, ja1;
  std::vector<int64_t> pos, pos1;
};

// host structure routines (structure.cpp)
void node_graph(const Mesh &m, std::vector<int32_t> &xadj, std::vector<int32_t> &adj);
void rcm_order(int32_t n, const std::vector<int32_t> &xadj,
               const std::vector<int32_t> &adj, std::vector<int32_t> &perm);
int32_t number_equations(const Mesh &m, const std::vector<int32_t> &perm,
                         const int32_t *bc, std::vector<int32_t> &id);
void csrc_pattern(const Mesh &m, const Structure &s, const std::vector<int32_t> &xadj,
                  const std::vector<int32_t> &adj, std::vector<int32_t> &ia,
                  std::vector<int32_t> &ja);
int color_elements(const Mesh &m, std::vector<int32_t> &color);
void derive_structure(const Mesh &m, Structure &s);
void build_tiles(Structure &s, int tile_rows);
void build_transpose(Structure &s);
std::vector<int32_t> partition_bounds(const Structure &s, int ndf, int nparts);
void build_partition(const Structure &s, int32_t eq0, int32_t eq1, Partition &p);
void build_blocks(Structure &s, int bsize);

// ------------------------------------------------------------- kernels
struct MeshDev {
  int32_t ndm, ndf, nen, numel, nnode, numat, prop;
  const int32_t *conn;   // (nen, numel) 0-based node, colour order, SoA
  const int32_t *mat;    // (numel) 0-based material, colour order
  const int32_t *elnum;  // (numel) original 1-based element number
  const int32_t *slot;   // (npairs, numel) colour order
  const double *x;       // (ndm, nnode)
  const int32_t *eq;     // (ndf, nnode) 0-based equation or -1
  const double *e;       // (prop, numat)
  int32_t npairs;
};

struct CsrcDev {
  int32_t neq;
  int64_t nad;
  const int32_t *ia;   // (neq+1) 0-based positions
  const int32_t *ja;   // (nad)   0-based columns
  const int32_t *iat;  // (neq+1) upper part (transposed index) row pointers
  const int32_t *jat;  // (nad)   upper part columns
  const int32_t *pt;   // (nad)   position in al of each upper entry
  const uint16_t *ja16, *jat16;  // 16-bit column deltas (null: use ja/jat)
  double *ad, *al, *alt;
  float *ad32, *al32, *alt32;
  int32_t gather_blocks = 0;  // grid of the gather SpMV (0: default)
  // node blocks (bsize 0: none); see Structure
  int32_t bsize = 0, nb = 0;
  int64_t nnzb = 0;
  const int32_t *bia = nullptr, *bt = nullptr;
  int32_t nslices = 0;
  const int32_t *sell_ptr = nullptr, *sell_col = nullptr;
  float *sell_val = nullptr;
  bool sell_stream = true;  // streaming loads (the copy does not stay in L2)
  double *sell_val64 = nullptr;  // sliced FP64 copy
  bool sell64_stream = true;     // streaming loads of the FP64 copy
  // slot groups whose loads the block product issues together (0: default)
  int32_t spmm_unroll = 0;
  // the autotuner's slot groups in flight per block width (index log2 W;
  // 0: the default), for the FP32 and the FP64 block products
  int32_t spmm_unroll_w32[5] = {0, 0, 0, 0, 0};
  int32_t spmm_unroll_w64[5] = {0, 0, 0, 0, 0};
  // grid bound of the products with fused dots: eight CTAs per SM (the
  // partial sums hold one row per CTA)
  int32_t max_grid = 1;
  // the sliced columns as 16-bit offsets from the block row (null: the
  // matrix's block bandwidth does not fit, or the copies stay in L2;
  // sell_col is read)
  const int16_t *sell_d16 = nullptr;
};

struct TileDev {
  int32_t rows, ntiles, max_nnz, max_tgt, lanes;
  const int32_t *tile_tgt, *tile_out, *tgt_col, *tgt_start, *halo_ptr, *halo_slot;
  const int32_t *desc;  // (8, ntiles)
  const uint16_t *tpos;
};

// assemble.cu
void launch_assembly(const MeshDev &m, const CsrcDev &k, const Segment &seg,
                     const double *u, double *b, int32_t *bad_elem,
                     cudaStream_t st);
// spmv.cu: y = K x in two launches (tiles, then halo); the halo launch can
// also form (p, y) and alpha for the PCG (sc != nullptr).
struct PcgScalars;
size_t tile_smem_bytes(const TileDev &t, bool fp32);
size_t pipe_smem_bytes(int max_nnz, int max_tgt, int rows, bool fp32);
void prepare_tile_kernels(const TileDev &t);
// sc (nullable): the launch does nothing once the solve it belongs to is done
void launch_tile_spmv64(const CsrcDev &k, const TileDev &t, const double *x, double *ytile,
                        double *part, int32_t *err, cudaStream_t st,
                        const PcgScalars *sc = nullptr);
void launch_tile_spmv32(const CsrcDev &k, const TileDev &t, const float *x, float *ytile,
                        float *part, int32_t *err, cudaStream_t st);
// Stress recovery (stress.cu): nodal stress sums of one colour segment, then
// the per-node average + tx0.
void launch_stress(const MeshDev &m, const Segment &seg, const double *u, double *ts,
                   int32_t *bad, cudaStream_t st);
void launch_stress_average(int nnode, int ntn, const int32_t *count, const double *tx0,
                           double *ts, cudaStream_t st);
void launch_update(int64_t n, const int32_t *eq, const double *x, double *u, cudaStream_t st);
// Result writer (vtk.cu): the file of write_mesh_res_mec as host text pieces
// and fixed-width device sections, formatted on the GPU.
struct VtkLayout {
  struct Text {
    int64_t off;
    std::string s;
  };
  struct Section {
    int kind;
    int64_t off;
    int count;
  };
  std::vector<Text> texts;
  std::vector<Section> sections;
  int64_t size = 0;
  void add_text(const std::string &s);
  void add_section(int kind, int count, int nnoel, int ndf);
};
VtkLayout vtk_layout(int format, int fields, int nnode, int numel, int ndf, int nnoel, int ctype);
void launch_vtk(const VtkLayout &L, char *dbuf, const MeshDev &m, int ntn, int nnoel, int ctype,
                const double *u, const double *tx, cudaStream_t st);
void launch_fortran_e(const double *x, int n, int w, int d, int e, char *out, cudaStream_t st);
// Loads (loads.cu): pload_mec into the resident b0/u, then the 2-D edge
// loads of pform_mec isw = 4 from host-built integer lists.
constexpr int kEdgeEntryInts = 8;
bool build_edge_lists(const Mesh &m, const int32_t *eload, int32_t nload,
                      std::vector<int32_t> &node, std::vector<int32_t> &ptr,
                      std::vector<int32_t> &ent, int32_t &bad_el);
void launch_pload(int64_t n, const int32_t *eq, const double *f, double *u, double *b0,
                  cudaStream_t st);
void launch_edge_loads(int nnodes, const int32_t *node, const int32_t *ptr, const int32_t *ent,
                       const double *x, const int32_t *eq, const double *loadvec, double *b0,
                       int32_t *bad, cudaStream_t st);
void launch_demote_values(const CsrcDev &k, cudaStream_t st);
void launch_transpose_values(const CsrcDev &k, cudaStream_t st);
// The sliced node-block copies from the CSRC arrays: FP64 (k.sell_val64),
// FP32 (k.sell_val).
void launch_fill_sell64(const CsrcDev &k, cudaStream_t st);
void launch_fill_sell32(const CsrcDev &k, cudaStream_t st);
// FP64 FMAs per second of the device (a register-only probe kernel, best of
// five timed launches) and, optionally, per clock per SM at the device's
// maximum SM clock.
double measure_fp64_fma_rate(int device, double *per_clock_per_sm);
// y = K x with the sliced FP64 kernel on explicit arrays (a partition's
// local slices; no dot product)
void launch_sell64_local(int nb, int nslices, int bsize, const int32_t *sell_ptr,
                         const int32_t *sell_col, const double *sval, const double *x,
                         double *y, cudaStream_t st);
// Two-sided gather SpMV: y = K x reading the lower part (ja, al) and the
// upper part through the transposed copy (jat, alt); with sc != nullptr it
// also forms (x, y) and alpha = d / (x, y).
void launch_gather_spmv64(const CsrcDev &k, const double *x, double *y, PcgScalars *sc,
                          double *partials, unsigned int *counter, cudaStream_t st,
                          const int32_t *gate = nullptr);
void launch_gather_spmv32(const CsrcDev &k, const float *x, float *y, PcgScalars *sc,
                          double *partials, unsigned int *counter, cudaStream_t st);

// Epilogues of the gather SpMV: what it does with y = K x besides storing it.
enum GatherEpi : int {
  kEpiNone = 0,       // nothing
  kEpiPcg = 1,        // pq = (x, y), alpha = d / pq
  kEpiBicgAlpha = 2,  // pq = (w, y), alpha = rho / pq, iters += 1   (w = r0)
  kEpiBicgOmega = 3,  // omega = (w, y) / (y, y)                      (w = r)
  kEpiScale = 4,      // y = w .* (K x), no dot                       (w = M)
};
void launch_gather_epi64(const CsrcDev &k, int epi, const double *x, double *y, const double *w,
                         PcgScalars *sc, double *partials, unsigned int *counter,
                         const int32_t *gate, cudaStream_t st);
// The node-block product (bcsr.cu), with the same epilogues.
template <class T, int EPI>
void launch_bcsr(const CsrcDev &k, const T *x, T *y, const T *w, PcgScalars *sc,
                 double *partials, unsigned int *counter, const int32_t *gate, cudaStream_t st);

}  // namespace elx
