/*
 * elastic_gb300.h -- C ABI of the GB300 (sm_103a) linear-elasticity solve
 * library: element stiffness integration for TRIA3/QUAD4/TETRA4/HEXA8,
 * assembly into CSRC storage, the CSRC matrix-vector product and Jacobi-PCG
 * (with BiCGSTAB and GMRES on the same kernels).
 *
 * It replaces two calls of the Fortran driver of lmn-labest/Elastic:
 *   pform_mec(..., lhs=.true., rhs=.true., isw=2, ...)   mef/src/Pform.f:1-11,
 *                                                         called at Main.f:791-802
 *   solv(neq,nad,ip,ja,ad,au,al,m,b,x,tol,maxit,ngram,...) mef/src/Solv.f:13-15,
 *                                                         called at Main.f:820-826
 * Everything else in the driver (deck reading, RCM, numeq, load vectors,
 * output) stays where it is.
 *
 * Conventions (the reference's): every array is passed by plain pointer; all
 * index CONTENTS are 1-based (node, material, equation numbers, ia/ja
 * positions); multi-dimensional arrays are Fortran column-major, e.g.
 * ix(nen+1,numel) with the material number in the last row, x(ndm,nnode),
 * id(ndf,nnode), e(prop,numat), u(ndf,nnode).  Integers are int32 unless
 * stated; reals are double.  CSRC = diagonal ad(neq) + strict lower part in CSR
 * (ia(neq+1), ja(nad), al(nad)); the upper part is al mirrored.
 *
 * Errors: every call returns ELX_OK (0) or an ELX_ERR_* code and never exits
 * the process; elx_last_error() returns the message of the context's last
 * failure.  The Fortran glue calls stop_mef on a non-zero status, which keeps
 * the reference's behaviour (Paralelo.f:1123-1130).
 *
 * Threading: one context per host thread; calls are synchronous to the host
 * unless named *_async.  Device memory is owned by the context.
 */
#ifndef ELASTIC_GB300_H
#define ELASTIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define ELX_OK 0
#define ELX_ERR_ZERO_DIAG 1      /* ad(i) == 0 (Iters.f:337-342)              */
#define ELX_ERR_NO_CONVERGENCE 2 /* maxit reached (Iters.f:429-431)           */
#define ELX_ERR_BAD_DET 3        /* element det <= 1e-14 (Elmlib.f:1826-1829) */
#define ELX_ERR_OOM 4            /* device allocation or HBM budget           */
#define ELX_ERR_TIMEOUT 5        /* a bounded device wait gave up             */
#define ELX_ERR_ARG 6            /* invalid argument                          */
#define ELX_ERR_BAD_ELEMENT 7    /* unknown element type (Elmlib.f:151-153)   */
#define ELX_ERR_CUDA 8           /* CUDA runtime error                        */
#define ELX_ERR_STATE 9          /* call out of order (e.g. solve before mesh)*/

/* solver codes (the reference's `solver` variable, Main.f:177-198) */
#define ELX_SOLVER_PCG 1
#define ELX_SOLVER_GMRES 2
#define ELX_SOLVER_BICGSTAB 4
/* BiCGSTAB without a preconditioner (bicgstab, Iters.f:812-1075): the
 * reference has no solver code for it (its only call is commented out at
 * Solv.f:334); stops on ||r|| < tol ||b||; info->norm_m_r = ||b - K x||. */
#define ELX_SOLVER_BICGSTAB_NOPREC 5

/* precision of the Krylov iteration */
#define ELX_PREC_FP64 0  /* everything in FP64, as the reference          */
#define ELX_PREC_MIXED 1 /* FP32 inner PCG inside FP64 iterative refinement */

typedef struct elx_ctx elx_ctx;

typedef struct elx_opts {
  int32_t device;     /* CUDA device ordinal                                */
  int32_t verbose;    /* 0 silent                                            */
  int64_t hbm_budget; /* bytes the context may allocate; 0 = no limit        */
} elx_opts;

/* Post-solve diagnostics, the fields PCG prints at Iters.f:473-490. */
typedef struct elx_info {
  int32_t iters;      /* Krylov iterations (GMRES: inner steps)              */
  int32_t status;     /* ELX_* status of this solve                          */
  double xkx;         /* x . K x                                             */
  double norm_x;      /* ||x||_2                                             */
  double norm_r;      /* ||b - K x||_2                                       */
  double norm_m_r;    /* ||b - K x||_M, M = diag(K)^-1                       */
  double conv;        /* stopping threshold tol * ||b||_M (GMRES/BiCGSTAB: 2-norm) */
  double seconds;     /* wall time of the solve on the device                */
  double mflops;      /* flop_cg(neq,nad,iters,2) / seconds (Matvec.f:1499) */
  int32_t refinements;/* mixed precision: FP64 residual replacements; -1 when */
                      /* the FP32 iteration diverged or stalled and the case  */
                      /* was solved in FP64 instead                           */
  int32_t inner_iters;/* mixed precision: total FP32 inner iterations        */
} elx_info;

/* ---- context ---------------------------------------------------------- */
int elx_create(elx_ctx **out, const elx_opts *opts);
void elx_destroy(elx_ctx *ctx);
const char *elx_last_error(const elx_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time or
 * order device work around the library's. */
void *elx_stream(elx_ctx *ctx);
/* Bytes of device memory the context holds. */
int64_t elx_device_bytes(const elx_ctx *ctx);
/* Number of this library's kernels the context has launched so far
 * (a CUDA graph launch counts the kernels it contains). */
int64_t elx_kernel_launches(const elx_ctx *ctx);
const char *elx_version(void);

/* ---- mesh and structure ------------------------------------------------ */
/* Mesh arrays as read by rdat (Rdata.f:1-740).  ix(nen+1,numel); x(ndm,nnode);
 * ie(numat) element type per material (2,3 TRIA3; 4,5 QUAD4; 6 TETRA4;
 * 7 HEXA8); e(prop,numat) with E, nu, thickness in rows 1..3.  Copies them to
 * the device.  Element types are checked here (ELX_ERR_BAD_ELEMENT). */
int elx_set_mesh(elx_ctx *ctx, int32_t ndm, int32_t ndf, int32_t nen,
                 int32_t numel, int32_t nnode, const int32_t *ix,
                 const double *x, const int32_t *ie, const double *e,
                 int32_t prop, int32_t numat);

/* Structure computed by the caller, as the reference driver does
 * (reord Reord.f:1, numeq Numeq.f:139, csrstruct Csr.f:13 lower-only):
 * id(ndf,nnode) equation numbers (0 = constrained), ia(neq+1), ja(nad).
 * The library derives the transposed index, the element colouring and the
 * per-element slot map from them and uploads everything once. */
int elx_set_structure(elx_ctx *ctx, int32_t neq, int64_t nad,
                      const int32_t *id, const int32_t *ia, const int32_t *ja);

/* Structure computed by the library on the host from the mesh: node graph
 * (Graph.f:20), RCM when reorder != 0 (Reord.f:1), equation numbering
 * (Numeq.f:139) from bc(ndf,nnode) with 1 = constrained, and the lower CSRC
 * pattern (Csr.f:13).  Same output as the reference, bit for bit. */
int elx_build_structure(elx_ctx *ctx, const int32_t *bc, int32_t reorder);

/* Host-only form of elx_build_structure, usable without a GPU (for example
 * by a driver that replaces reord/numeq/csrstruct, Main.f:412-491): builds
 * the structure into a host handle; read it back with the two getters.
 * ix, ie as for elx_set_mesh, bc(ndf,nnode) with 1 = constrained. */
typedef struct elx_host_structure elx_host_structure;
int elx_host_structure_create(elx_host_structure **out, int32_t ndm, int32_t ndf,
                              int32_t nen, int32_t numel, int32_t nnode,
                              const int32_t *ix, const int32_t *ie, int32_t numat,
                              const int32_t *bc, int32_t reorder);
int elx_host_structure_sizes(const elx_host_structure *h, int32_t *neq,
                             int64_t *nad);
int elx_host_structure_get(const elx_host_structure *h, int32_t *perm,
                           int32_t *id, int32_t *ia, int32_t *ja);
/* The element colours the assembly kernels use (in place of colormsh's
 * elcolor, Colormsh.f:9-308: elements of one colour share no node, so their
 * blocks are added without atomics): elcolor(numel) 1-based colours
 * (nullable), *ncolors their number (nullable). */
int elx_host_structure_colors(const elx_host_structure *h, int32_t *elcolor,
                              int32_t *ncolors);
void elx_host_structure_destroy(elx_host_structure *h);

/* Row-block partitions for a multi-GPU run (one partition per GPU), in the
 * layout of the reference's overlapping MPI partitions: csrstruct with
 * lower = right = .true. (Csr.f:13-305) on the partition's local numbering
 * -- owned equations 1..neq (global eq0+1 .. eq0+neq of the RCM order),
 * then the halo (the equations outside the block that owned rows couple
 * to, ascending) from neq+1.  ia(neq+1)/ja(nad): the lower CSRC among owned
 * equations; ia1(neq+1)/ja1(nad1): the rectangular part (owned rows x halo
 * columns) that matvec_csrcrsym1 (Matvec.f:1090-1191) reads; pos/pos1: each
 * entry's 0-based position in the global al (the values); halo(nhalo):
 * 0-based global equations.  Cuts on node boundaries (multiples of 32 nodes
 * with node blocks), balancing full-row nonzeros.  Host only, no GPU.
 * ELX_ERR_ARG if there are fewer cut units than nparts. */
int elx_host_partition_sizes(const elx_host_structure *h, int32_t nparts, int32_t part,
                             int32_t *eq0, int32_t *neq, int32_t *nhalo, int64_t *nad,
                             int64_t *nad1);
int elx_host_partition_get(const elx_host_structure *h, int32_t nparts, int32_t part,
                           int32_t *halo, int32_t *ia, int32_t *ja, int32_t *ia1,
                           int32_t *ja1, int64_t *pos, int64_t *pos1);

/* Sizes and copies of the structure (any pointer may be NULL). */
int elx_get_sizes(const elx_ctx *ctx, int32_t *neq, int64_t *nad,
                  int32_t *ncolors);
int elx_get_structure(const elx_ctx *ctx, int32_t *perm, int32_t *id,
                      int32_t *ia, int32_t *ja);

/* ---- assembly: pform_mec(isw=2, lhs=.true., rhs=.true.) ----------------- */
/* u(ndf,nnode) current displacements (prescribed values in constrained dofs),
 * b0(neq) load vector.  Forms K (ad, al, device-resident) and
 * b_out = b0 - K_e u_e summed over elements (Assbly.f:116-118).  ad_out and
 * al_out are optional host copies (NULL = keep on the device only). */
int elx_assemble(elx_ctx *ctx, const double *u, const double *b0,
                 double *b_out, double *ad_out, double *al_out);

/* ---- solve: solv(...) -------------------------------------------------- */
/* Solves K x = b with the resident K.  solver: ELX_SOLVER_*; precision:
 * ELX_PREC_*; tol, maxit, ngram as in the reference (Main.f:177-198).
 * b and x are host arrays of length neq; x need not be initialised (x0 = 0). */
int elx_solve(elx_ctx *ctx, int32_t solver, int32_t precision, double tol,
              int32_t maxit, int32_t ngram, const double *b, double *x,
              elx_info *info);

/* Block PCG: nrhs load cases of the resident matrix, solved `width`
 * columns at a time over one read of the matrix per iteration (each column is
 * the reference's Jacobi PCG with its own scalars and stopping test; pcg,
 * Iters.f:252-524).  b and x are neq x nrhs, column-major; info has nrhs
 * entries (refinements = FP64 residual replacements of the mixed solver).
 * width 0 = autotuned (elx_autotune_block); otherwise 1, 2, 4, 8 or 16.
 * Needs node blocks: every node all free or all fixed.  No reference
 * counterpart (the reference solves one load case per solv call,
 * Main.f:820-826).  _device: b and x are device pointers. */
int elx_solve_block(elx_ctx *ctx, int32_t nrhs, int32_t precision, double tol,
                    int32_t maxit, int32_t width, const double *b, double *x,
                    elx_info *info);
int elx_solve_block_device(elx_ctx *ctx, int32_t nrhs, int32_t precision, double tol,
                           int32_t maxit, int32_t width, const double *b, double *x,
                           elx_info *info);
/* The block width with the least product time per column on the resident
 * matrix (FP32 product for ELX_PREC_MIXED, FP64 otherwise); times_us
 * (nullable, 5 entries) gets the product times of widths 1, 2, 4, 8, 16 and
 * forces a new measurement. */
int elx_autotune_block(elx_ctx *ctx, int32_t precision, int32_t *width, double *times_us);
/* The tiling the autotuner chose for the block product of each width
 * (unroll[i] for W = 2^i, 5 entries): the slot groups of matrix loads kept in
 * flight (1-3; 0 = not tuned, the library's default).  No reference
 * counterpart (the reference has no block product). */
int elx_block_tiling(elx_ctx *ctx, int32_t precision, int32_t *unroll);

/* ---- solve server ----------------------------------------------------- */
/* A request loop over many meshes at once (no reference counterpart: the
 * reference runs one deck per process).  Requests are solved with the
 * reference's FP64 Jacobi PCG; structures are built on host threads while
 * the GPU works; a request is admitted when its device memory fits the HBM
 * budget; the PCG iterations of all admitted requests (every load case) run
 * as one packed set of kernels per iteration, each load case with its own
 * scalars and stopping test; requests join and leave between polls
 * (continuous batching).  Requests of large_dofs equations or more are
 * instead solved whole, several at once on their own streams, by the block
 * PCG over all their load cases (see large_mode).
 * A result is bitwise the same alone and in a mix. */
typedef struct elx_server elx_server;
typedef struct elx_server_opts {
  int32_t device;
  int32_t prep_threads; /* host threads building structures (0: 4)          */
  int64_t hbm_budget;   /* device bytes for admitted requests (0: no limit)  */
  int32_t poll_steps;   /* PCG iterations between polls (0: 8)               */
  int32_t max_slots;    /* load cases in flight at most (0: 4096)            */
  int32_t large_dofs;   /* requests with at least this many equations are   */
                        /* solved whole, not packed (0: 100000)             */
  int32_t large_mode;   /* those: block PCG, 0 auto (mixed precision in     */
                        /* 3-D, FP64 in 2-D), 1 FP64, 2 mixed (FP32 inner,  */
                        /* FP64 replacements and test), -1 packed like the  */
                        /* others                                           */
  int32_t large_workers;/* large requests solved at once (0: 2)             */
} elx_server_opts;
typedef struct elx_server_stats {
  int64_t submitted, completed;
  int64_t peak_bytes;     /* most device bytes held by admitted requests      */
  int64_t resident_bytes; /* bytes held now                                   */
  int64_t peak_slots;     /* most load cases in one packed iteration         */
  int64_t iterations;     /* packed iterations run                           */
  int64_t large_solved;   /* requests solved whole (block PCG)               */
  /* [0] packed, [1] block: finished requests and their summed seconds from
   * submit to prepared (host structure), to admission start (waiting for
   * memory / slots), to admitted (uploads, assembly, preconditioner), to
   * the solve's start (joining the pack / a block-solve thread), to done */
  int64_t phase_n[2];
  double phase_s[2][5];
} elx_server_stats;
int elx_server_create(elx_server **out, const elx_server_opts *opts);
/* Queues a request (the arrays are copied): a mesh as for elx_set_mesh,
 * bc(ndf,nnode) with 1 = constrained (whole nodes: a node's dofs all free or
 * all fixed), f(ndf,nnode,nrhs) nodal forces per load case.  Returns at
 * once with a ticket. */
int elx_server_submit(elx_server *srv, int32_t ndm, int32_t ndf, int32_t nen,
                      int32_t numel, int32_t nnode, const int32_t *ix, const double *x,
                      const int32_t *ie, const double *e, int32_t prop, int32_t numat,
                      const int32_t *bc, int32_t nrhs, const double *f, double tol,
                      int32_t maxit, int64_t *ticket);
/* Waits (timeout_s < 0: without limit) for a request; u(ndf,nnode,nrhs)
 * gets the displacements (0 on fixed dofs), info[nrhs] the per-load-case
 * iterations, status and threshold, latency_s submit-to-done seconds.
 * Returns the request's status (ELX_ERR_TIMEOUT: not done yet; the ticket
 * stays valid).  Each ticket can be collected once. */
int elx_server_wait(elx_server *srv, int64_t ticket, double timeout_s, double *u,
                    elx_info *info, double *latency_s);
int elx_server_get_stats(elx_server *srv, elx_server_stats *stats);
void elx_server_destroy(elx_server *srv);

/* Stress recovery, tform_mec (Pform.f:258-421, called for isw = 3 at
 * Main.f:893-901): t(ntn,nnode) = for each node the average over its
 * elements of their stresses at the node (elmt02-07_mec isw = 3) + tx0
 * (ntn = 4: sxx syy szz sxy in 2-D; 6: sxx syy szz sxy syz sxz in 3-D).
 * u(ndf,nnode) the nodal displacements (NULL: the resident u of
 * elx_set_state); tx0(ntn,nnode) initial stresses (NULL: zero). */
int elx_stress(elx_ctx *ctx, const double *u, const double *tx0, double *t);

/* update_mec (Predict.f:183-209): u(j,i) = x(id(j,i)) for free dofs. */
int elx_update(elx_ctx *ctx, const double *x, double *u);

/* ---- lower-level calls on resident data (benchmarks, tests) ------------ */
/* y = K x with the resident K (matvec_csrcsym1, Matvec.f:528-621).
 * precision ELX_PREC_FP64 or ELX_PREC_MIXED (FP32 values and vectors). */
int elx_spmv(elx_ctx *ctx, int32_t precision, const double *x, double *y);

/* Upload the matrix directly (ad(neq), al(nad)) instead of assembling it. */
int elx_set_matrix(elx_ctx *ctx, const double *ad, const double *al);

/* Device-resident steps, no host copies: assembly from the resident u and b0
 * (elx_set_state), a solve from the resident b into the resident x, and
 * `reps` SpMVs y = K x on resident vectors, launched as the solvers launch
 * them (with the fused dot product (x, y)).  All are stream-ordered on
 * elx_stream(ctx) and return once enqueued, except elx_solve_resident which
 * waits for convergence. */
int elx_set_state(elx_ctx *ctx, const double *u, const double *b0);
int elx_assemble_resident(elx_ctx *ctx);
int elx_solve_resident(elx_ctx *ctx, int32_t solver, int32_t precision,
                       double tol, int32_t maxit, int32_t ngram,
                       elx_info *info);
int elx_spmv_resident(elx_ctx *ctx, int32_t precision, int32_t reps);
/* update_mec (Predict.f:183-209) on the resident state: u(j,i) =
 * x(id(j,i)) for the free dofs, from the resident solution; with it a
 * solvm pass (assemble, solve, update) and the stresses (elx_stress with
 * u = NULL) never leave the device.  Stream-ordered like the calls above. */
int elx_update_resident(elx_ctx *ctx);
int elx_get_solution(elx_ctx *ctx, double *x);
int elx_get_rhs(elx_ctx *ctx, double *b);

/* ---- the steps around the solve -------------------------------------- */
/* The load step on the device (replaces the host's pload_mec, Pload.f:2-58,
 * and pform_mec with isw = 4, Pform.f:1-11 / Elmlib02.f:260-314, 856-910):
 * f(ndf,nnode) evaluated nodal loads -> b0(id) = f for free dofs, u = f for
 * prescribed ones (free dofs of u keep their value); then, if eload is not
 * NULL, the 2-D distributed edge loads: eload(7,numel) 1-based load numbers
 * per element side (0: unloaded), loadvec(2,nload) the loads' traction
 * vectors (type 40); b0(k) -= the element vectors, bitwise as the reference
 * forms them.  The results stay resident for elx_assemble_resident.
 * ELX_ERR_ARG for a load number outside 1..nload, a loaded side an element
 * does not have, or edge loads on a 3-D mesh; ELX_ERR_BAD_DET for a
 * zero-length loaded side. */
int elx_set_loads(elx_ctx *ctx, const double *f, const int32_t *eload,
                  const double *loadvec, int32_t nload);
/* Copy the resident u(ndf,nnode) and b0(neq) to the host (either NULL). */
int elx_get_state(elx_ctx *ctx, double *u, double *b0);

/* Result writer: the file of write_mesh_res_mec (Write_vtk.f:742-985 with
 * the record writers of Vtk.f), formatted on the GPU from the resident mesh,
 * the resident u (fields & 1: "desloc", fprint(2)) and the nodal stresses of
 * the last elx_stress call (fields & 2: "stress", fprint(3)).  format 0: the
 * reference's default XML VTU ASCII file (legacy_vtk = bvtk = .false.);
 * format 1: its legacy binary VTK file (legacy_vtk = bvtk = .true., big-
 * endian).  Byte for byte the reference's records, numbers as gfortran
 * prints the Ew.d[Ee] / Iw edit descriptors.  The mesh must be of one cell
 * type (as the reference's writer assumes).  elx_write_vtk writes `path`;
 * elx_format_vtk returns the size in *bytes and, if out != NULL, copies the
 * file into out (capacity bytes).  ELX_ERR_STATE for stresses not yet
 * computed. */
int elx_write_vtk(elx_ctx *ctx, const char *path, int32_t format, int32_t fields,
                  int64_t *bytes);
int elx_format_vtk(elx_ctx *ctx, int32_t format, int32_t fields, char *out,
                   int64_t capacity, int64_t *bytes);
/* The partitioned product on one GPU: y = K x formed partition by partition
 * as a multi-GPU run forms it (elx_host_partition_* gives the same cuts),
 * each partition gathering its halo of x (the exchange) and multiplying its
 * owned block rows with the sliced node-block kernel on its local numbering
 * (owned + halo columns: matvec_csrcrsym1, Matvec.f:1090-1191).  Bitwise
 * equal to elx_spmv's FP64 product.  Node blocks required.
 * elx_partition_spmv_resident runs `reps` products on the resident vectors
 * (for timing); elx_partition_info gives a partition's owned equations and
 * halo size. */
int elx_partition_spmv(elx_ctx *ctx, int32_t nparts, const double *x, double *y);
int elx_partition_spmv_resident(elx_ctx *ctx, int32_t nparts, int32_t reps);
int elx_partition_info(elx_ctx *ctx, int32_t nparts, int32_t part, int32_t *eq0,
                       int32_t *neq, int32_t *nhalo);

/* The FP64 pipe's rate on `device`, measured: FMAs per second of a
 * register-only probe kernel (eight independent FMA chains per thread, one
 * resident wave, best of five timed launches) and, if per_clock_per_sm is
 * not NULL, that rate per clock per SM at the device's maximum SM clock.
 * No reference counterpart: the FP64 product's floor (one FMA per stored
 * entry of the full matrix) is this rate.  The call allocates and frees one
 * output buffer (a double per probe thread) and leaves the calling thread's
 * current device as it found it. */
int elx_fp64_fma_rate(int32_t device, double *fma_per_s, double *per_clock_per_sm);

/* Test hook of the device number formatter: n fields Ew.d (e = 0) or
 * Ew.dEe of x into out (n * w chars), as the writer prints them. */
int elx_fortran_e(const double *x, int32_t n, int32_t w, int32_t d, int32_t e, char *out);

/* ---- allocation-free SpMV + dot ---------------------------------------- */
/* No counterpart in the reference: this entry point is for callers that
 * cannot let the library allocate device memory -- a driver that, like the
 * reference's own memory manager, keeps every device array in one pool it
 * allocated up front, or code that must not call cudaMalloc because that
 * would synchronise the device in the middle of its asynchronous work.  It
 * needs no context: every input and output is a DEVICE pointer owned by the
 * caller, and it computes y = K x (the CSRC product of matvec_csrcsym1) and
 * *xy = (x, y), the product and dot of one PCG step, deterministically.
 *   ia, ja, ad, al  the CSRC matrix, index contents 1-based as above;
 *   iat, jat, alt   its upper part in CSR form, i.e. the transpose of the
 *                   lower part (iat(neq+1) 1-based positions, jat(nad)
 *                   1-based row numbers, alt(nad) the values of al in that
 *                   order), e.g. from a counting sort of ja;
 *   x (neq), y (neq), xy (1 double); stream: a cudaStream_t (NULL = default).
 * Limit: neq <= 1048576 (ELX_ERR_ARG above; nothing is launched).  The
 * scratch (one partial sum per 64 rows, a ticket and a scalar slot, about
 * 130 KB) is a static device array that every GPU loading this library
 * holds until the process exits.  The first call on a device looks up that
 * array's device address (with the device current): make that first call
 * before any stream capture.  The address is that of the device's primary
 * context (the CUDA runtime's): a caller that makes its own driver-API
 * context current must not call this entry point from it.  All calls share the scratch, so calls that
 * overlap on the GPU race; serialise them on one stream.  Returns ELX_OK
 * once the work is enqueued on `stream`. */
int elx_spmv_dot_noalloc(int32_t neq, const int32_t *ia, const int32_t *ja,
                         const double *ad, const double *al, const int32_t *iat,
                         const int32_t *jat, const double *alt, const double *x,
                         double *y, double *xy, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ELASTIC_GB300_H */
