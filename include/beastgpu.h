/*
 * beastgpu.h -- C ABI of libbeastgpu.so, the GB300 (sm_103a) replacement for BEAST.jl's
 * Galerkin assembly and dense solve.
 *
 * Plain C types only.  Every call returns an int status (BEAST_OK = 0); on failure,
 * beast_last_error() gives a message.  Matrices are column-major complex arrays with
 * interleaved (re, im) pairs -- bit-compatible with Julia's Matrix{ComplexF64}
 * (BEAST_C128) or Matrix{ComplexF32} (BEAST_C64).  Rows are test dofs, columns trial
 * dofs, in the order of the caller's assembly data (BEAST's `tfs.fns` order).
 *
 * Ownership: host pointers are borrowed for the duration of a call.  Handles
 * (ctx, mesh, space, lu) own device memory and are freed by the matching *_free call.
 * A context may be used from several host threads; calls on one context serialise
 * on its stream.  Nothing here calls back into the caller.
 */
#ifndef BEASTGPU_H
#define BEASTGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the Julia shim turns non-zero codes into error(beast_last_error)) */
enum {
  BEAST_OK = 0,
  BEAST_ERR_ARG = 1,        /* invalid argument (the reference raises @assert/error)   */
  BEAST_ERR_OOM = 2,        /* device allocation failed                                 */
  BEAST_ERR_CUDA = 3,       /* CUDA runtime error                                       */
  BEAST_ERR_TIMEOUT = 4,    /* a bounded device wait gave up (no GPU fault is raised)   */
  BEAST_ERR_NOCONV = 5,     /* iterative solver/refinement did not converge            */
  BEAST_ERR_SINGULAR = 6,   /* exactly singular pivot (LAPACK info > 0)                 */
  BEAST_ERR_UNSUPPORTED = 7 /* operator / space / strategy combination not implemented */
};

/* ---- operator kinds (reference types) */
enum {
  BEAST_MW_SL = 1,   /* MWSingleLayer3D(gamma, alpha, beta)  src/maxwell/mwops.jl:11-24     */
  BEAST_MW_DL = 2,   /* MWDoubleLayer3D(alpha, gamma)        src/maxwell/mwops.jl:61-81     */
  BEAST_MW_NXDL = 3, /* DoubleLayerRotatedMW3D (n x K)        src/maxwell/nxdbllayer.jl:17-44*/
  BEAST_HH_SL = 4,   /* HH3DSingleLayerFDBIO(alpha, gamma)   src/helmholtz3d/hh3dops.jl:47-50*/
  BEAST_HH_DL = 5,   /* HH3DDoubleLayerFDBIO(alpha, gamma)   src/helmholtz3d/hh3dops.jl:62-65*/
  BEAST_HH_DLT = 6   /* HH3DDoubleLayerTransposedFDBIO      src/helmholtz3d/hh3dops.jl:77-80*/
};

/* ---- space kinds (local reference spaces) */
enum {
  BEAST_P0 = 0, /* LagrangeRefSpace{T,0,3}  src/bases/local/laglocal.jl:17-18  */
  BEAST_P1 = 1, /* LagrangeRefSpace{T,1,3}  src/bases/local/laglocal.jl:214-228 */
  BEAST_RT = 2  /* RTRefSpace               src/bases/local/rtlocal.jl:1-29     */
};

/* ---- quadrature strategy kinds */
enum {
  BEAST_QS_WILTON_SAUTER = 1, /* DoubleNumWiltonSauterQStrat src/quadrature/doublenumwiltonsauterqstrat.jl:1-69 */
  BEAST_QS_SAUTER = 2,        /* DoubleNumSauterQstrat src/quadrature/doublenumsauterqstrat.jl:1-27          */
  BEAST_QS_DOUBLENUM = 3,     /* DoubleNumQStrat src/quadrature/doublenumqstrat.jl:1-32                     */
  BEAST_QS_TEST_REFINES_TRIAL = 4, /* TestRefinesTrialQStrat(DoubleNumWiltonSauterQStrat(...)),
                                 src/quadrature/strategies/testrefinestrialqstrat.jl:1-17 with
                                 rules/testrefinestrialqrule.jl:1-52: the test space lives on a
                                 refinement of the trial space's mesh (beast_mesh_set_children on
                                 the trial mesh); a pair that shares a vertex integrates the trial
                                 cell's children with the wrapped strategy, every other pair the
                                 wrapped strategy on the trial cell itself.  RT x RT; orders as for
                                 DoubleNumWiltonSauter. */
  BEAST_QS_TRIAL_REFINES_TEST = 5  /* TrialRefinesTestQStrat(DoubleNumWiltonSauterQStrat(...)),
                                 src/quadrature/strategies/trialrefinestestqstrat.jl:1-17 with
                                 rules/trialrefinestestqrule.jl:1-40: the same with the roles
                                 swapped (the trial space on the refinement, the test cell split
                                 into its children; children registered on the test mesh). */
};

/* ---- precision of assembly and solve */
enum {
  BEAST_FP64 = 0, /* everything complex FP64 (the reference's arithmetic)                    */
  BEAST_MIXED = 1, /* far pairs in FP32, Sauter-Schwab RT Maxwell pairs with FP32 moments
                      (double-float partial sums), other near pairs FP64, c64 storage; solve:
                      FP32 panels with FP16-operand tensor-core trailing updates of a c64
                      copy, FP64 iterative refinement against the c64 matrix                 */
  BEAST_MIXED_ACCURATE = 2, /* assembly as BEAST_FP64 (c128 matrix); solve as BEAST_MIXED, the
                      refinement residual taken against the c128 matrix, so the solution is
                      the FP64 one to the refinement tolerance                               */
  BEAST_MIXED_BALANCED = 3 /* as BEAST_MIXED_ACCURATE, but the far pairs of the RT Maxwell
                      single layer keep double-float arithmetic only where the gather cancels:
                      the Green's function values and the divergence (beta) term of each cell
                      pair; the vector-potential (alpha) terms run in FP32 (about 1e-7 of the
                      largest entry of a block).  Other operators: as BEAST_MIXED_ACCURATE    */
};

/* ---- element type of a dense matrix / vector argument */
enum { BEAST_C128 = 0, BEAST_C64 = 1 };

/* ---- where a matrix / vector argument lives */
enum { BEAST_HOST = 0, BEAST_DEVICE = 1 };

/* excitation kinds */
enum {
  BEAST_EXC_TANGTRACE_E = 0,  /* TangTraceMW(PlaneWaveMW): ((n x E) x n)   src/excitation.jl:176-181 */
  BEAST_EXC_CROSSTRACE_H = 1, /* CrossTraceMW of H = -1/(ik) curl E: n x H  src/excitation.jl:166-174 */
  BEAST_EXC_HH_DIRICHLET = 2  /* Helmholtz plane-wave Dirichlet trace      src/helmholtz3d/hh3dexc.jl */
};

typedef struct beast_ctx beast_ctx;
typedef struct beast_mesh beast_mesh;
typedef struct beast_space beast_space;
typedef struct beast_lu beast_lu;
typedef struct beast_system beast_system;

/* operator parameters: MW_SL uses gamma, alpha, beta; MW_DL / MW_NXDL use gamma (alpha is
 * carried but, as in the reference integrands, not applied); HH_* use gamma and alpha. */
typedef struct {
  int kind;
  double gamma_re, gamma_im;
  double alpha_re, alpha_im;
  double beta_re, beta_im;
} beast_op_desc;

/* rule orders: the eight fields of DoubleNumWiltonSauterQStrat.  For DoubleNumSauterQstrat
 * (outer, inner, tetr, face, edge, vert) pass outer/inner in both the far and near slots;
 * for DoubleNumQStrat(outer, inner) set the far slots. */
typedef struct {
  int kind;
  int outer_far, inner_far, outer_near, inner_near;
  int ss_tetr, ss_face, ss_edge, ss_vert;
} beast_qs_desc;

/* ---- context ------------------------------------------------------------------------ */
/* replaces: nothing in the reference (it has no device); owns stream, workspace, errors */
int beast_ctx_create(int device, beast_ctx** out);
int beast_ctx_destroy(beast_ctx* ctx);
/* copies the last error message of this context into buf (always NUL-terminated) */
int beast_last_error(beast_ctx* ctx, char* buf, size_t len);
/* use this CUDA stream (cudaStream_t passed as void*) for all later work; NULL = own stream */
int beast_ctx_set_stream(beast_ctx* ctx, void* stream);
/* upper bound in bytes for the assembly workspace (default: 25% of free device memory) */
int beast_ctx_set_workspace_limit(beast_ctx* ctx, size_t bytes);
/* wait for all work queued on the context stream */
int beast_ctx_synchronize(beast_ctx* ctx);
/* bound on the polls of one flag wait in the triangular solves (0 = the library default,
 * about 4 million).  A wait that runs out makes the solve return BEAST_ERR_TIMEOUT; the
 * context stays usable.  For tests of that error path; no reference counterpart. */
int beast_ctx_set_wait_limit(beast_ctx* ctx, int64_t polls);

/* ---- geometry and spaces ------------------------------------------------------------ */
/* replaces the mesh arrays a CompScienceMeshes.Mesh carries into assemble (vertices,
 * faces).  verts: [nv][3] float64; cells: [nc][3] vertex indices with base 0 or 1. */
int beast_mesh_upload(beast_ctx* ctx, const double* verts, int64_t nv, const int32_t* cells,
                      int64_t nc, int index_base, beast_mesh** out);
int beast_mesh_free(beast_mesh* mesh);
/* the children of every cell of `coarse` in a refinement (CompScienceMeshes.children of the
 * barycentric refinement that Buffa-Christiansen spaces live on): child_verts [nc][nchild][3][3]
 * float64, the vertices of each child triangle, oriented like its parent; nchild <= 8.
 * Needed by BEAST_QS_TEST_REFINES_TRIAL (trial space on `coarse`) and
 * BEAST_QS_TRIAL_REFINES_TEST (test space on `coarse`).  A second call replaces the first. */
int beast_mesh_set_children(beast_ctx* ctx, beast_mesh* coarse, int nchild, const double* child_verts);

/* replaces assemblydata(basis) (src/bases/basis.jl:235-294): the active cells
 * (act_to_global, `cells`, [ncells]) and AssemblyData.data split into two arrays of
 * layout [ncells][nshapes][maxfn] (Julia's data[k, r, c] memory order): dof indices
 * (empty slot: < index_base) and coefficients.  nfuncs = numfunctions(basis). */
int beast_space_upload(beast_ctx* ctx, const beast_mesh* mesh, int kind, int64_t ncells,
                       const int64_t* cells, int maxfn, int nshapes, const int64_t* ad_dof,
                       const double* ad_coeff, int64_t nfuncs, int index_base,
                       beast_space** out);
int beast_space_free(beast_space* space);

/* ---- assembly ----------------------------------------------------------------------- */
/* replaces assemble!(op, tfs, bfs, store, threading) + assemblechunk! for integral
 * operators (src/operator.jl:215-231, src/integralop.jl:69-184) with the dense store
 * closure of allocatestorage (src/operator.jl:168-183) lowered to arguments:
 *   Z[row_off + m, col_off + n]  (=|+=)  coeff * a(m, n)
 * Z: ldz leading dimension, element type z_dtype (BEAST_C128/C64), location z_loc.
 * accumulate = 0 overwrites the addressed block, 1 adds (linear combinations,
 * src/operator.jl:294-304).  precision: BEAST_FP64 or BEAST_MIXED (BEAST_MIXED_ACCURATE
 * assembles as BEAST_FP64, BEAST_MIXED_BALANCED as described at its enum).  Singularity-extraction pairs (DoubleNumWiltonSauterQStrat) are
 * available for the Maxwell operators on RT and the Helmholtz single, double and transposed
 * double layers on any P0 / P1 combination. */
int beast_assemble(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs,
                   const beast_space* test, const beast_space* trial, int precision, void* Z,
                   int64_t ldz, int z_dtype, int z_loc, int64_t row_off, int64_t col_off,
                   double coeff_re, double coeff_im, int accumulate);

/* replaces blockassembler(op, tfs, bfs)(test_ids, trial_ids, store) and assemblerow! /
 * assemblecol! (src/integralop.jl:228-320, 593-702; reduce_assembly_data,
 * src/bases/basis.jl:486-499): the block a(test_ids[i], trial_ids[j]) for i < ntest,
 * j < ntrial into Z[i, j] (block-local rows / columns, ldz, like beast_assemble with zero
 * offsets).  Ids are function indices of the two spaces with the given index_base; a
 * repeated id gives a repeated row / column.  Every entry equals the full assembly's. */
int beast_assemble_block(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs,
                         const beast_space* test, const beast_space* trial, const int64_t* test_ids,
                         int64_t ntest, const int64_t* trial_ids, int64_t ntrial, int index_base,
                         int precision, void* Z, int64_t ldz, int z_dtype, int z_loc, double coeff_re,
                         double coeff_im, int accumulate);

/* replaces assemble!(::LocalOperator, ...) for Identity (which = 0) and NCross
 * (which = 1) on RT x RT (src/identityop.jl:7-24, 66-67; src/localop.jl:107-155):
 * adds coeff * block into Z (same addressing as beast_assemble).  degree: SingleNumQStrat. */
int beast_assemble_local(beast_ctx* ctx, int which, const beast_space* test,
                         const beast_space* trial, int degree, void* Z, int64_t ldz,
                         int z_dtype, int z_loc, int64_t row_off, int64_t col_off,
                         double coeff_re, double coeff_im);

/* replaces assemble(field, tfs) for plane-wave excitations (src/excitation.jl:17-65,
 * 91-115; src/maxwell/mwexc.jl:36-52).  b: complex FP64 vector [nfuncs] (overwritten),
 * location b_loc.  dir/pol: 3 doubles (pol ignored for BEAST_EXC_HH_DIRICHLET). */
int beast_rhs_planewave(beast_ctx* ctx, int kind, const beast_space* test, const double* dir,
                        const double* pol, double gamma_re, double gamma_im, double amp_re,
                        double amp_im, int degree, double* b, int b_loc);

/* ---- dense solve -------------------------------------------------------------------- */
/* replaces LinearAlgebra.lu / `\` (zgetrf + zgetrs; src/solvers/lu.jl:40-47,
 * src/solvers/lusolver.jl:30).  A: n x n device matrix (dtype) factored IN PLACE with
 * partial pivoting; the handle keeps the pivots. */
int beast_lu_factor(beast_ctx* ctx, int64_t n, void* A, int64_t lda, int dtype, beast_lu** out);
/* solve with the factors: B (device, same dtype as the factors, n x nrhs) overwritten;
 * blocks until done; BEAST_ERR_TIMEOUT if a bounded wait of the triangular solves ran out */
int beast_lu_solve(beast_ctx* ctx, const beast_lu* lu, int64_t nrhs, void* B, int64_t ldb);
int beast_lu_free(beast_lu* lu);

/* Same result as beast_lu_solve, but the call allocates no device memory: its scratch (one
 * permuted right-hand side and the wavefront flags) is a fixed array inside the library,
 * sized for n <= 65536 (about 1 MiB, held by every GPU that loads the library until the
 * process exits).  For callers that cannot allocate at solve time: a host runtime that owns
 * the device memory pool (such as Julia's CUDA.jl allocator) or a serving loop that reserves
 * all memory up front.  Larger n is rejected with BEAST_ERR_ARG.  The first call on a device
 * looks up the array's device address; make that first call before any stream capture.
 * All calls share the one array and it keeps the previous call's contents: calls that
 * overlap on the GPU (other streams, other host threads) race -- serialise them.
 * Like every call here it makes the context's device current on the calling thread, and it
 * blocks that thread until the solve has finished (it reads the solve's status word).
 * No counterpart in the reference (it has no device memory). */
int beast_lu_solve_noalloc(beast_ctx* ctx, const beast_lu* lu, int64_t nrhs, void* B, int64_t ldb);

/* x = A \ b for a device matrix A (c128 or c64).  precision BEAST_FP64: FP64 LU;
 * BEAST_MIXED (or BEAST_MIXED_ACCURATE / BALANCED, the same here): FP32 LU of a c64 copy + FP64
 * iterative refinement to `tol` relative residual (residual matvec and update in FP64,
 * against A as stored: c128 for the FP64 solution to the tolerance).
 * b, x: complex FP64 [n x nrhs], location bx_loc.  iters/resid (may be NULL) report the
 * refinement steps and the final relative residual. */
int beast_solve_dense(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int a_dtype,
                      int precision, const double* b, double* x, int64_t nrhs, int bx_loc,
                      double tol, int maxiter, int* iters, double* resid);

/* replaces GMRESSolver / gmres (src/solvers/itsolver.jl:5-176, src/solvers/gmres.jl:1-83):
 * restarted GMRES, x0 = 0, stop when ||r|| <= reltol ||b||; FP64 orthogonalisation.
 * A: device matrix (c128 or c64); b, x: complex FP64 [n], location bx_loc. */
int beast_gmres(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int a_dtype,
                const double* b, double* x, int bx_loc, double reltol, int restart,
                int maxiter, int* iters, double* resid);

/* ---- post-processing ------------------------------------------------------------------ */
/* replaces potential(MWFarField3D(gamma), points, u, X) (src/postproc.jl:138-211,
 * 273-288; src/maxwell/farfield.jl:60-63): ff[p] (3 complex) for unit directions pts[p].
 * u, ff: complex FP64, location loc. */
int beast_farfield(beast_ctx* ctx, const beast_space* space, const double* u, const double* pts,
                   int64_t npts, double gamma_re, double gamma_im, int degree, double* ff,
                   int loc);

/* ---- one assemble + excitation + solve job (the `solve(eq)` path, src/solvers/lusolver.jl:9-39)
 * Host-facing: mesh/space handles are already resident; the matrix, RHS and factors
 * live on the device only; x (host or device, complex FP64 [nfuncs]) receives u. */
int beast_solve_job(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs,
                    const beast_space* space, int exc_kind, const double* dir, const double* pol,
                    double exc_gamma_re, double exc_gamma_im, int precision, double tol,
                    double* x, int x_loc, int* iters, double* resid);

/* ---- batched assembly: many meshes in one persistent launch ---------------------------
 * Helmholtz single layer (BEAST_HH_SL) or transposed double layer (BEAST_HH_DLT) on P0
 * spaces (one cell per function, coefficient 1): job j assembles ops[j] on spaces[j] x
 * spaces[j] into the device matrix Z[j] (column-major, ld = nfuncs, c64 for BEAST_MIXED, else
 * c128; overwritten).  Every job shares the quadrature strategy `qs` and one operator kind.
 * The far pairs of all jobs run as one persistent kernel over a tile list (tile_m test cells x
 * tile_q trial cells of one job per CTA step; 0 = defaults 128 x 16) in the order `order`
 * (0: job by job, 1: largest jobs first, 2: jobs interleaved), the near pairs of all jobs as a
 * second one; the pair list length stays on the device.  beast_batch_assemble captures both
 * launches in a CUDA graph on its first call and replays the graph afterwards (the calls
 * replace, for a batch of meshes, one assemble(op, X, X) per mesh: src/operator.jl:100-116).
 * No reference counterpart for the handle. */
typedef struct beast_batch beast_batch;
int beast_batch_create(beast_ctx* ctx, const beast_qs_desc* qs, int64_t njobs, const beast_space* const* spaces,
                       const beast_op_desc* ops, void* const* Z, int precision, int tile_m, int tile_q, int order,
                       beast_batch** out);
int beast_batch_assemble(beast_ctx* ctx, beast_batch* batch);
int beast_batch_free(beast_batch* batch);

/* ---- resident systems: the `solve(eq)` path split so that the matrix and its factors stay
 * on the device between requests (serving: a request on a system already resident skips
 * assembly and factorisation; src/solvers/lusolver.jl:9-39 assembles and factors per call).
 * beast_system_create assembles op (+ local_coeff * Identity / NCross when local_which is 0 /
 * 1; -1: none) on space x space in `precision` and factors it (the mixed factorisation for
 * BEAST_MIXED / BEAST_MIXED_ACCURATE / BEAST_MIXED_BALANCED, FP64 LU for BEAST_FP64).  beast_system_solve builds nrhs
 * plane-wave excitations (dirs, pols: [nrhs][3]; same gamma) and solves them against the
 * kept factors (FP64 refinement to `tol` on the mixed paths); x: complex FP64 [nrhs][nfuncs],
 * location x_loc.  beast_system_bytes: device memory the system holds (matrix, factors,
 * pivots).  The space must outlive the system.  No reference counterpart for the handle. */
int beast_system_create(beast_ctx* ctx, const beast_op_desc* op, const beast_qs_desc* qs,
                        const beast_space* space, int local_which, double local_coeff_re,
                        double local_coeff_im, int precision, beast_system** out);
int beast_system_solve(beast_ctx* ctx, beast_system* sys, int exc_kind, int64_t nrhs,
                       const double* dirs, const double* pols, double exc_gamma_re,
                       double exc_gamma_im, double tol, double* x, int x_loc, int* iters,
                       double* resid);
int beast_system_bytes(const beast_system* sys, size_t* bytes);
int beast_system_free(beast_system* sys);

/* ---- instrumentation (no reference counterpart: the reference has no device) ---------
 * When enabled, every instrumented kernel launch on the context stream is bracketed by
 * CUDA events.  Kinds: 0 geometry, 1 far pairs, 2 near pairs, 3 gather/scatter, 4 local
 * operators, 5 excitation, 6 far field, 7 LU panel, 8 row swaps, 9 TRSM, 10 trailing GEMM,
 * 11 triangular solves, 12 FP64 matvec, 13 vector ops, 14 precision conversion,
 * 15 tensor-core trailing update (tcgen05).
 * beast_prof_read sums event time (ms), bracketed launches and algorithmic work (flops for
 * compute kinds, bytes for memory kinds) over the records since the last enable. */
int beast_prof_enable(beast_ctx* ctx, int on);
/* as beast_prof_enable(ctx, 1), recording only the kinds whose bit (1 << kind) is set */
int beast_prof_enable_kinds(beast_ctx* ctx, unsigned int mask);
int beast_prof_read(beast_ctx* ctx, int kind, double* ms, int64_t* launches, double* work);
/* kernels launched by this context since the last beast_prof_enable (counted always) */
int beast_prof_launches(beast_ctx* ctx, int64_t* n);
/* factorisation that produced the result of the last beast_solve_dense / beast_solve_job on
 * this context: 0 LU with partial pivoting, 1 unpivoted LU (mixed), 2 symmetric LDL^T-type
 * (mixed, near complex-symmetric matrix), -1 none yet */
int beast_last_factor_mode(beast_ctx* ctx, int* mode);

/* the device's stream-ordered memory pool that every allocation of the library's calls comes
 * from: bytes reserved from the device and bytes in use, now and at their highest (since the
 * process started).  Serving admission reads it to check that its footprint model bounds the
 * device memory actually held.  No reference counterpart. */
int beast_pool_stats(beast_ctx* ctx, size_t* reserved, size_t* reserved_high, size_t* used,
                     size_t* used_high);

/* library version string */
const char* beast_version(void);

#ifdef __cplusplus
}
#endif
#endif
