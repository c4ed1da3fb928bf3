// internal.h -- shared host/device declarations of libbeastgpu (not part of the ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/beastgpu.h"

#define BEAST_CUDA_TRY(ctx, expr)                                                  \
  do {                                                                             \
    cudaError_t e_ = (expr);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return beast_fail((ctx), e_ == cudaErrorMemoryAllocation ? BEAST_ERR_OOM      \
                                                               : BEAST_ERR_CUDA,  \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));       \
  } while (0)

// kernel classes timed by the optional profiler (beast_prof_*)
enum {
  PK_GEOM = 0, PK_FAR, PK_NEAR, PK_GATHER, PK_LOCAL, PK_RHS, PK_FARFIELD, PK_PANEL, PK_LASWP,
  PK_TRSM, PK_GEMM, PK_TRSV, PK_GEMV, PK_VEC, PK_CONVERT, PK_TCGEMM, PK_COUNT
};
struct ProfRec {
  int kind;
  cudaEvent_t a, b;
  double work;
};

struct beast_ctx {
  int device = 0;
  int num_sms = 0;
  // SMs a tensor-core update leaves free (its persistent grid has num_sms - tc_sm_reserve
  // CTAs): set while kernels of the lookahead stream are meant to run beside the update
  int tc_sm_reserve = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  size_t ws_limit = 0;   // assembly workspace byte limit
  std::string err;
  // reusable device workspace
  void* ws = nullptr;
  size_t ws_size = 0;
  int* d_flag = nullptr;  // device error / status word
  // profiler: CUDA events around instrumented launches on `stream`
  bool prof_on = false;
  uint32_t prof_mask = 0xffffffffu;  // kinds recorded while prof_on
  std::vector<ProfRec> prof;
  std::vector<cudaEvent_t> evpool;
  int64_t launches = 0;   // kernels launched by this context (counted always)
  int last_factor_mode = -1;  // factorisation of the last dense solve (beast_last_factor_mode)
  long long trsv_spin_max = 0;  // polls of one triangular-solve flag wait (0: library default)
  // second (high-priority) stream and events of the factorisation's lookahead, made on first use
  cudaStream_t aux = nullptr;
  cudaEvent_t la_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // Sauter-Schwab node tables as double-float pairs, built on first use: key 64 class + order
  std::map<int, void*> ss_tabs;
};

// the lookahead stream and events of ctx (created once); false when they cannot be made
bool ctx_lookahead_streams(beast_ctx* ctx);

// brackets one or more launches of class `kind`; `work` = algorithmic flops or bytes
struct ProfScope {
  beast_ctx* ctx;
  int kind;
  double work;
  cudaEvent_t a = nullptr;
  ProfScope(beast_ctx* c, int k, double w, int nlaunch = 1);
  ~ProfScope();
};

constexpr int MAX_CHILDREN = 8;
struct beast_mesh {
  beast_ctx* ctx = nullptr;
  int64_t nv = 0, nc = 0;
  double* verts = nullptr;   // [nv][3]
  int* cells = nullptr;      // [nc][3] 0-based
  // the cells' children in a refinement (beast_mesh_set_children): [nc][nchild][9] or null
  double* children = nullptr;
  int nchild = 0;
};

// per active cell geometry, 16 doubles: v0 v1 v2 (9) | centroid (3) | unit normal (3) | area
enum { GEO_STRIDE = 16 };

struct beast_space {
  beast_ctx* ctx = nullptr;
  const beast_mesh* mesh = nullptr;
  int kind = 0, nshapes = 0, maxfn = 0;
  int64_t ncells = 0, nfuncs = 0;
  int* cells = nullptr;        // active -> mesh cell
  int* cell2act = nullptr;     // mesh cell -> active index (-1 if inactive)
  int* ad_dof = nullptr;       // [ncells][nshapes][maxfn], -1 empty
  double* ad_coeff = nullptr;
  double* geo = nullptr;       // [ncells][GEO_STRIDE]
  float* geof = nullptr;       // [ncells][4]: centroid (3), circumradius about centroid
  // dof -> (active cell, local shape, coefficient), CSR
  int64_t* fn_ptr = nullptr;
  int* fn_cell = nullptr;
  int* fn_shape = nullptr;
  double* fn_coeff = nullptr;
  std::vector<int64_t> h_fn_ptr;
  std::vector<int> h_fn_cell, h_fn_shape;
  std::vector<double> h_fn_coeff;
  // Zcell row order of the test side: active cells sorted by their first function
  int* tperm = nullptr;        // position -> active cell
  int* tpos = nullptr;         // active cell -> position
  // (active cell, shape) -> its entry in the function CSR (fn_*), -1 for none; `injective`
  // when no (cell, shape) belongs to two entries (RT on a closed or open surface, P0, P1): the
  // cell-pair blocks can then be laid out by entries (ZLAYOUT_ENTRY)
  bool injective = false;
  bool unit_coef = false;  // every function coefficient is +1 or -1 (RT, P0, P1 spaces)
  std::vector<int> h_cs2e;
  int* zrow_entry = nullptr;   // [ncells][nshapes] by Zcell position: the entry, or -1
  std::vector<int> h_ad_dof;   // host copy of the assembly data
  std::vector<double> h_ad_coeff;
};

struct beast_lu {
  beast_ctx* ctx = nullptr;
  int64_t n = 0, lda = 0;
  int dtype = 0;
  void* A = nullptr;     // factors (not owned)
  int* ipiv = nullptr;   // device, 0-based
  int info = 0;
};

int beast_fail(beast_ctx* ctx, int code, const std::string& msg);

// quadrature rule set passed by value to kernels
enum { RULE_MAXPTS = 25 };
struct TriRuleDev {
  int n;
  double u[RULE_MAXPTS], v[RULE_MAXPTS], w[RULE_MAXPTS];
};
bool make_trirule(int degree, TriRuleDev* r);

struct OpParams {
  int kind;
  double gr, gi;   // gamma
  double ar, ai;   // alpha
  double br, bi;   // beta
};

// element format of the cell-pair blocks (Zcell): complex FP64 (plain path), complex FP32
// (mixed path), or double-float pairs (mixed-accurate path: re.hi, re.lo, im.hi, im.lo as one
// float4, written and summed on the FP32 pipes)
enum { ZCELL_C128 = 0, ZCELL_C64 = 1, ZCELL_DF = 2 };

// near-pair list entry
struct NearPair {
  int p, q;       // test active cell, trial cell (chunk-local index)
  int cls;        // 3/2/1 Sauter-Schwab face/edge/vertex, -1 Wilton SE
  int pad;
};

// ---- assembly launchers (assemble.cu)
struct AsmArgs {
  OpParams op;
  beast_qs_desc qs;
  const beast_space* ts;
  const beast_space* bs;
  int precision;
  // chunk description
  const int* qcells;   // device: trial active cell ids of this chunk [nq]
  int nq;
  void* zcell;         // device Zcell [ns_t*ncells_t x ns_b*nq], in format zcell_fmt
  int zcell_fmt;       // ZCELL_C128, ZCELL_C64 or ZCELL_DF
  int64_t ldc;
  NearPair* near;      // device near list
  int near_cap;
  int* near_count;     // device counter
  int* flag;           // device error flag
  // where the block of (test position pp, shape i) x (chunk trial cell ql, shape j) goes:
  // row zrow[pp * nst + i], column zcol[ql * nsb + j] (-1: not stored); null: the cell layout,
  // row nst pp + i, column nsb ql + j
  const int* zrow;
  const int* zcol;
  std::map<int, void*>* ss_tabs = nullptr;  // the context's Sauter-Schwab node tables
};
cudaError_t launch_geometry(const beast_space* s, cudaStream_t st);
cudaError_t launch_far(const AsmArgs& a, const TriRuleDev& ro, const TriRuleDev& ri,
                       cudaStream_t st);
// ro_far / ri_far: the far rules, for the children of the refines strategies
cudaError_t launch_near(const AsmArgs& a, int nnear, const TriRuleDev& ro_near,
                        const TriRuleDev& ri_near, const TriRuleDev& ro_far, const TriRuleDev& ri_far,
                        cudaStream_t st);
struct GatherArgs {
  const beast_space* ts;
  const beast_space* bs;
  const void* zcell;
  int zcell_fmt;
  int64_t ldc;
  const int* qlocal;      // device: trial active cell -> chunk-local index (-1 absent)
  const int* tpos;        // device: test active cell -> Zcell position
  int64_t n0, n1;         // trial dof range of this chunk
  void* Z;
  int64_t ldz;
  int z_c64;
  int64_t row_off, col_off;
  double cr, ci;
  int accumulate;
  // entry layout (ZLAYOUT_ENTRY): Zcell row = test entry, column = trial entry - f0
  int entry_layout;
  int64_t f0;
};
cudaError_t launch_gather(const GatherArgs& g, cudaStream_t st);
cudaError_t launch_local_impl(int which, const beast_space* ts, const beast_space* bs,
                              const int* b_cell2act, const TriRuleDev& r, void* Z, int64_t ldz,
                              int z_c64, int64_t row_off, int64_t col_off, double cr, double ci,
                              int* flag, cudaStream_t st);
cudaError_t launch_rhs(int kind, const beast_space* ts, const double* dir, const double* pol,
                       double gr, double gi, double ar, double ai, const TriRuleDev& r,
                       double* b, cudaStream_t st);
cudaError_t launch_farfield(const beast_space* s, const double* u, const double* pts,
                            int64_t npts, double gr, double gi, const TriRuleDev& r, double* ff,
                            cudaStream_t st);

// ---- batched assembly of many meshes (assemble.cu / api.cu): Helmholtz operators on P0
// spaces, every cell-pair value written straight into its job's matrix
struct BatchJobDev {
  OpParams op;
  double k2;
  const double* geo;   // the job space's geometry ([ncells][GEO_STRIDE])
  const float* geof;   // centroid and radius per cell
  const int* tperm;    // position -> active cell
  const int* zrow;     // [position]: matrix row (the space's entry of the cell)
  const int* zcol;     // [active cell]: matrix column
  int64_t ncells;
  void* Z;             // the job's matrix (column-major, ld ldz)
  int64_t ldz;
};
struct BatchTile {
  int job, p0, q0, pad;  // test positions p0 .. p0 + tile_m, trial cells q0 .. q0 + tile_q
};
struct NearPairB {
  int job, p, q, cls;
};
struct BatchLaunch {
  const BatchJobDev* jobs;
  const BatchTile* tiles;
  int ntiles;
  int qs_kind;
  beast_qs_desc qs;
  TriRuleDev ro, ri, ron, rin;  // far and near rules
  int precision;
  int zfmt;                     // matrix element format (ZCELL_C64 or ZCELL_C128)
  int op_kind;                  // one operator kind for the whole batch
  NearPairB* near;
  int near_cap;
  int* near_count;
  int* flag;
  int tile_m, tile_q;           // test cells per CTA (= threads), trial cells staged per CTA
  int grid_far, grid_near;      // persistent CTAs
  // single-layer Sauter-Schwab pairs in double-float (not on the FP64 path): node tables per
  // class 1..3 (ss_tables)
  int ssdf = 0;
  const float2* ssdf_tab[4] = {nullptr, nullptr, nullptr, nullptr};
  int ssdf_items[4] = {0, 0, 0, 0};
};
// the double-float Sauter-Schwab node tables of the strategy's orders (class 1..3: vertex,
// edge, face), from the context's cache or built now on `st` (not inside a graph capture)
cudaError_t ss_tables(std::map<int, void*>* cache, const beast_qs_desc& qs, cudaStream_t st,
                      const float2** tab, int* items);
cudaError_t launch_far_batch(const BatchLaunch& L, cudaStream_t st);
// the constant tables of the near-pair kernels (Gauss-Legendre nodes), once per device; must
// run before a launch that is captured in a graph
cudaError_t upload_tables(cudaStream_t st);
cudaError_t launch_near_batch(const BatchLaunch& L, cudaStream_t st);

// ---- dense linear algebra (linalg.cu)
// bytes of the auxiliary allocation of a factorisation (pivots, permutation, inverses of the
// diagonal blocks); lu_dinv locates the inverses inside it
size_t lu_aux_bytes(int64_t n, int dtype);
void* lu_dinv(const int* ipiv, int64_t n);
// pivot = false: no row interchanges (the mixed path; guarded by refinement and a
// fall-back to partial pivoting in the caller)
// sym (c64, unpivoted): the symmetric variant for a near complex-symmetric A (only its lower
// triangle is used; the factors approximate those of (A + A^T) / 2)
int lu_factor_dev(beast_ctx* ctx, int64_t n, void* A, int64_t lda, int dtype, int* ipiv,
                  int* info, bool pivot = true, bool sym = false);
// relative asymmetry ||A - A^T|| / ||A|| (Frobenius) estimated on about 10^6 sampled pairs
double asym_sample(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int dtype);
int lu_solve_dev(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int dtype,
                 const int* ipiv, void* B, int64_t ldb, int64_t nrhs);
// synchronises the context stream; BEAST_ERR_TIMEOUT when a triangular-solve wait of the
// solves queued since the last lu_solve_dev gave up
int trsv_check(beast_ctx* ctx);
// y = alpha * A x + beta * y (FP64 arithmetic, A c128 or c64, x/y c128)
cudaError_t gemv_dev(int64_t n, const void* A, int64_t lda, int a_c64, const double* x,
                     double* y, double alpha, double beta, cudaStream_t st);
// the block-lower part of a c64 matrix (column j from row 64 floor(j / 64)), for the
// symmetric factorisation's copy
cudaError_t copy_lower_c64(int64_t n, const void* A, int64_t lda, void* F, int64_t ldf, cudaStream_t st);
// the same from a c128 matrix into a c64 copy (round to nearest)
cudaError_t convert_lower_c128_to_c64(int64_t n, const void* A, int64_t lda, void* F, int64_t ldf, cudaStream_t st);
cudaError_t convert_c128_to_c64(int64_t rows, int64_t cols, const double* src, int64_t lds,
                                float* dst, int64_t ldd, cudaStream_t st);
cudaError_t convert_c64_to_c128(int64_t rows, int64_t cols, const float* src, int64_t lds,
                                double* dst, int64_t ldd, cudaStream_t st);
// complex FP64 vector helpers
cudaError_t vec_axpy(int64_t n, double ar, double ai, const double* x, double* y, cudaStream_t st);
cudaError_t vec_copy(int64_t n, const double* x, double* y, cudaStream_t st);
// reduction: sum of |x|^2 into out (device double), deterministic
cudaError_t vec_norm2(int64_t n, const double* x, double* out, cudaStream_t st);
// h[k] = <v_k, w> for k < m (columns of V with ld), FP64
cudaError_t vec_dots(int64_t n, int m, const double* V, int64_t ldv, const double* w, double* h,
                     cudaStream_t st);
// w -= V h (m columns)
cudaError_t vec_gemv_sub(int64_t n, int m, const double* V, int64_t ldv, const double* h,
                         double* w, cudaStream_t st);

// ---- FP16 operands of the tensor-core LU update (tc_gemm.cu)
// work layout of an M x K by K x N update: A' (2M rows of K half2), B' (N columns of K half2),
// the row scales 1/s (M floats), the column scales 1/t (N floats)
// largest K of a symmetric (D-scaled) tensor-core update: its pivots are staged in shared memory
constexpr int TC_SYM_KMAX = 2048;
void tc_gemm_operands(void* work, int64_t M, int64_t N, int K, void** Ap, float** inv_sa, void** Bp,
                      float** inv_sb);
#ifdef __CUDACC__
// power-of-two scale 2^sh that brings a largest magnitude mx into [2^13, 2^14) (sh = 0 for
// mx = 0): the FP16 operands then never clip and keep 11 significant bits
__device__ __forceinline__ int tc_scale_shift(float mx) {
  if (!(mx > 0.f)) return 0;
  int e;
  frexpf(mx, &e);  // mx = f 2^e, f in [0.5, 1)
  return max(-120, min(120, 14 - e));
}
#endif
