/*
 * oracle.h -- CPU FP64 restatement of BEAST.jl's Galerkin assembly path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness checker for the
 * GB300 kernels and the timed CPU baseline.  Only tests/, the smoke() entry of
 * __graft_entry__.py and bench.py (cpu_baseline / --impl reference) may load it.
 * The product library (libbeastgpu.so) never links or calls it.
 *
 * Parity status: the reference (Julia) cannot run in this build environment.
 * The restatement is pinned to the reference's own test cases and tolerances
 * (test/test_wiltonints.jl, test/test_sauterschwabints.jl, test/test_hh3dints.jl,
 * test/test_rt.jl, test/test_itsolver.jl).  The triangle rule point sets of
 * CompScienceMeshes.trgauss and the region split of SauterSchwabQuadrature.jl
 * live in un-vendored dependencies; here they are restated from the published
 * methods (symmetric Gauss rules on the triangle indexed by polynomial degree;
 * Sauter & Schwab, Boundary Element Methods, 2011, ch. 5), so per-entry parity
 * with the real BEAST is pinned only to those tests' tolerances.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* operator kinds (mirror beastgpu.h) */
enum {
  ORC_MW_SL = 1,    /* MWSingleLayer3D      src/maxwell/mwops.jl:11-24, 101-117 */
  ORC_MW_DL = 2,    /* MWDoubleLayer3D      src/maxwell/mwops.jl:61-81, 141-155 */
  ORC_MW_NXDL = 3,  /* DoubleLayerRotatedMW3D src/maxwell/nxdbllayer.jl:17-44 */
  ORC_HH_SL = 4,    /* HH3DSingleLayerFDBIO src/helmholtz3d/hh3dops.jl:47-50,119-138 */
  ORC_HH_DL = 5,    /* HH3DDoubleLayerFDBIO src/helmholtz3d/hh3dops.jl:62-65,142-161 */
  ORC_HH_DLT = 6,   /* HH3DDoubleLayerTransposedFDBIO hh3dops.jl:77-80,164-182 */
  /* regular parts used by singularity extraction (internal, exposed for tests) */
  ORC_MW_SL_REG = 11, ORC_MW_DL_REG = 12, ORC_HH_SL_REG = 14, ORC_HH_DL_REG = 15,
  ORC_HH_DLT_REG = 16
};

/* space kinds */
enum { ORC_P0 = 0, ORC_P1 = 1, ORC_RT = 2 };

/* quadrature strategy kinds */
enum {
  ORC_QS_WILTON_SAUTER = 1, /* DoubleNumWiltonSauterQStrat doublenumwiltonsauterqstrat.jl:1-69 */
  ORC_QS_SAUTER = 2,        /* DoubleNumSauterQstrat doublenumsauterqstrat.jl:1-27 */
  ORC_QS_DOUBLENUM = 3      /* DoubleNumQStrat doublenumqstrat.jl:1-32 */
};

/* rule kinds for orc_cellpair (single triangle pair) */
enum { ORC_RULE_DQ = 0, ORC_RULE_SE = 1, ORC_RULE_SS_FACE = 2, ORC_RULE_SS_EDGE = 3,
       ORC_RULE_SS_VERT = 4 };

typedef struct {
  int kind;
  double gamma_re, gamma_im;
  double alpha_re, alpha_im;
  double beta_re, beta_im;
} orc_op;

typedef struct {
  int kind;
  int outer_far, inner_far, outer_near, inner_near;
  int ss_tetr, ss_face, ss_edge, ss_vert;
} orc_qs;

typedef struct {
  int kind;                 /* ORC_P0 / ORC_P1 / ORC_RT */
  int64_t ncells;           /* active cells */
  const int64_t* cells;     /* active cell -> mesh cell (0-based) */
  int maxfn, nshapes;
  const int64_t* ad_dof;    /* [ncells][nshapes][maxfn], 0-based dof or -1 */
  const double* ad_coeff;   /* same layout */
  int64_t nfuncs;
} orc_space;

typedef struct {
  const double* verts;      /* [nv][3] */
  int64_t nv;
  const int32_t* cells;     /* [nc][3] 0-based */
  int64_t nc;
} orc_mesh;

/* symmetric triangle rule exact to polynomial `degree` (1,2,3,4,5,6,7,8,10) or a
 * collapsed Gauss product rule for other degrees.  uv: [n][2] barycentric (u,v)
 * of x = u*v1 + v*v2 + (1-u-v)*v3; w sums to 1.  Returns n, or -needed if cap small. */
int orc_trirule(int degree, double* uv, double* w, int cap);
/* n-point Gauss-Legendre on [0,1] */
int orc_gausslegendre(int n, double* x, double* w);

/* Wilton et al. 1984 analytic potential integrals over triangle (p1,p2,p3) seen from x.
 * scal[6], vec[6][3], grad[4][3] in the layout of the reference's in-tree copy
 * (test/test_wiltonints.jl:60-232). */
void orc_wiltonints(const double* p1, const double* p2, const double* p3, const double* x,
                    double* scal, double* vec, double* grad);

/* one local block for a triangle pair with an explicit rule.
 * tv, bv: 9 doubles (vertices) of test and trial triangle.
 * deg_o/deg_i: triangle rule degrees (DQ, SE); gl: Gauss-Legendre order (SS).
 * out: complex interleaved, [nt][nb] row-major (out[2*(i*nb+j)]). */
int orc_cellpair(const orc_op* op, int tkind, int bkind, const double* tv, const double* bv,
                 int rule, int deg_o, int deg_i, int gl, double* out);

/* classify a pair like quadrule(..., ::DoubleNumWiltonSauterQStrat):
 * returns 3/2/1 hits (SS face/edge/vertex), 0 for far DQ, -1 for Wilton SE */
int orc_classify(const orc_op* op, const orc_qs* qs, const double* tv, const double* bv);

/* dense assembly  Z[m + n*ldz] (complex interleaved, column-major) for test dofs
 * m in [row_lo,row_hi) (row_hi<0 means all).  Z must be zeroed by the caller.
 * nthreads: worker threads (dof splitting, src/operator.jl:215-231). */
int orc_assemble(const orc_op* op, const orc_qs* qs, const orc_mesh* mesh,
                 const orc_space* tspace, const orc_space* bspace,
                 double* Z, int64_t ldz, int64_t row_lo, int64_t row_hi, int nthreads);

/* TestRefinesTrialQStrat (split_test 0: test space on the refinement of the trial mesh) or
 * TrialRefinesTestQStrat (split_test 1) wrapping the DoubleNumWiltonSauterQStrat `qs`, RT x RT.
 * children: [coarse mesh cell][nchild][3][3] vertices of each coarse cell's children.
 * Z as orc_assemble (all rows), zeroed by the caller. */
int orc_assemble_refines(const orc_op* op, const orc_qs* qs, const orc_mesh* tmesh,
                         const orc_mesh* bmesh, const orc_space* tspace, const orc_space* bspace,
                         const double* children, int nchild, int split_test, double* Z, int64_t ldz,
                         int nthreads);

/* local identity / ncross operator on same-cell pairs (src/identityop.jl), RT x RT.
 * which: 0 Identity, 1 NCross.  Adds coeff * block into Z. */
int orc_assemble_local(int which, const orc_mesh* mesh, const orc_space* tspace,
                       const orc_space* bspace, int degree, double coeff_re, double coeff_im,
                       double* Z, int64_t ldz);

/* excitation (src/excitation.jl:38-115): plane wave
 * kind 0: TangTraceMW of PlaneWaveMW  ((n x E) x n), test RT
 * kind 1: CrossTraceMW of the magnetic field H = -1/(i k) curl E  (n x H), test RT
 * kind 2: Helmholtz plane wave Dirichlet trace, test P0/P1
 * b: complex interleaved, length nfuncs (zeroed by caller). */
int orc_rhs_planewave(int kind, const orc_mesh* mesh, const orc_space* tspace,
                      const double* dir, const double* pol, double gamma_re, double gamma_im,
                      double amp_re, double amp_im, int degree, double* b);

/* dense complex LU with partial pivoting (LAPACK zgetrf semantics) and solve.
 * A: n x n complex interleaved column-major, overwritten with factors; B: n x nrhs,
 * overwritten with the solution.  ipiv: 0-based pivot rows.  Returns 0 or info>0. */
int orc_lu_factor(int64_t n, double* A, int64_t lda, int64_t* ipiv, int nthreads);
int orc_lu_solve(int64_t n, const double* A, int64_t lda, const int64_t* ipiv, int64_t nrhs,
                 double* B, int64_t ldb);

/* restarted GMRES (IterativeSolvers semantics, src/solvers/itsolver.jl:83-125):
 * x0 = 0, stop when ||r|| <= reltol * ||b||.  Returns iterations, or -iters if not converged */
int orc_gmres(int64_t n, const double* A, int64_t lda, const double* b, double* x,
              double reltol, int restart, int maxiter, int nthreads, double* resnorm);

/* far field of an RT current u (src/postproc.jl:174-211, 273-288,
 * src/maxwell/farfield.jl:60-63): ff[p] = sum over cells of
 * a * (yhat x (exp(gamma yhat.x) f(x)) ) x yhat with SingleNumQStrat(degree). */
int orc_farfield(const orc_mesh* mesh, const orc_space* space, const double* u,
                 const double* pts, int64_t npts, double gamma_re, double gamma_im,
                 int degree, double* ff);

#ifdef __cplusplus
}
#endif
