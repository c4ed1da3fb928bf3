// assemble.cu -- GB300 kernels of the Galerkin assembly path.
//
// Pipeline of one beast_assemble call (per trial-dof chunk):
//   k_far     every (test cell p, trial cell q) pair of the chunk: pair classification
//             (quadrule, src/quadrature/doublenumwiltonsauterqstrat.jl:32-69) and, for far
//             pairs, the DoubleQuadRule block (src/quadrature/doublenumints.jl:12-43) in FP64
//             or FP32.  The per-point-pair work is reduced algebraically: for RT shapes
//             f_i = (x - v_i)/2A the 3x3 block is a fixed combination of 8 (single layer) or
//             10/16 (double layer, n x K) complex moments of the kernel, accumulated with
//             coordinates relative to the cell centroids.  Near pairs go to a list.
//   k_near    one warp per listed pair: Sauter-Schwab (touching) or Wilton singularity
//             extraction (near), FP64 (src/quadrature/sauterschwabints.jl:156-182,
//             src/quadrature/singularityextractionints.jl:4-22).
//   k_gather  Z[m,n] = sum over the shapes of dof m and dof n of a*b*Zcell: the RT/P0/P1
//             local-to-global scatter (src/integralop.jl:173-184) as an owner-computes
//             gather: every output entry written once, no atomics, deterministic.
#include <cuda_runtime.h>

#include <mutex>
#include <type_traits>

#include <cmath>

#include "fsplit.h"
#include "internal.h"
#include "se_p1.h"
#include "far_df.h"
#include "se_core.h"

namespace {

#define DEV __device__ __forceinline__


// exp(-gamma R) / (4 pi R) for gamma = gr + i gi
DEV C2<double> green_d(double gr, double gi, double R, double iR) {
  double s, c;
  sincos(gi * R, &s, &c);
  double a = (gr == 0.0 ? 1.0 : exp(-gr * R)) * I4PI * iR;
  return {a * c, -a * s};
}
DEV C2<float> green_f(float gr, float gi, float R, float iR) {
  float s, c;
  sincosf(gi * R, &s, &c);
  float a = (gr == 0.0f ? 1.0f : expf(-gr * R)) * (float)I4PI * iR;
  return {a * c, -a * s};
}
template <typename R>
DEV C2<R> green(R gr, R gi, R Rr, R iR);
template <>
DEV C2<double> green<double>(double gr, double gi, double Rr, double iR) {
  return green_d(gr, gi, Rr, iR);
}
template <>
DEV C2<float> green<float>(float gr, float gi, float Rr, float iR) {
  return green_f(gr, gi, Rr, iR);
}
template <typename R>
DEV R rsq(R x);
template <>
DEV double rsq<double>(double x) {
  return rsqrt(x);
}
template <>
DEV float rsq<float>(float x) {
  return rsqrtf(x);
}

// expm1 of a complex argument (accurate for small |z|)
DEV C2<double> cexpm1_d(C2<double> z) {
  double s, c, sh;
  sincos(z.im, &s, &c);
  sh = sin(0.5 * z.im);
  double ea = exp(z.re), em = expm1(z.re);
  return {em * c - 2.0 * sh * sh, ea * s};
}
DEV C2<double> cexp_d(C2<double> z) {
  double s, c;
  sincos(z.im, &s, &c);
  double e = z.re == 0.0 ? 1.0 : exp(z.re);
  return {e * c, e * s};
}


// ------------------------------------------------------------------------------------
// per-cell geometry (chart: x = u v1 + v v2 + (1-u-v) v3, normal (v1-v3)x(v2-v3)/|.|)
// ------------------------------------------------------------------------------------
__global__ void k_geometry(const double* verts, const int* mcells, const int* act, int64_t n,
                           double* geo, float* geof) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= n) return;
  int mc = act[c];
  V3<double> v[3];
  for (int i = 0; i < 3; ++i) {
    const double* p = verts + 3 * (int64_t)mcells[3 * (int64_t)mc + i];
    v[i] = mk(p[0], p[1], p[2]);
  }
  V3<double> cr = cross(v[0] - v[2], v[1] - v[2]);
  double j = sqrt(dot(cr, cr));
  V3<double> cen = (1.0 / 3.0) * (v[0] + v[1] + v[2]);
  double* g = geo + c * GEO_STRIDE;
  for (int i = 0; i < 3; ++i) {
    g[3 * i] = v[i].x;
    g[3 * i + 1] = v[i].y;
    g[3 * i + 2] = v[i].z;
  }
  g[9] = cen.x; g[10] = cen.y; g[11] = cen.z;
  g[12] = cr.x / j; g[13] = cr.y / j; g[14] = cr.z / j;
  g[15] = 0.5 * j;
  double rad = 0;
  for (int i = 0; i < 3; ++i) {
    V3<double> d = v[i] - cen;
    rad = fmax(rad, sqrt(dot(d, d)));
  }
  geof[4 * c] = (float)cen.x;
  geof[4 * c + 1] = (float)cen.y;
  geof[4 * c + 2] = (float)cen.z;
  geof[4 * c + 3] = (float)(rad * (1.0 + 1e-6));
}

// ------------------------------------------------------------------------------------
// pair classification: quadrule(..., ::DoubleNumWiltonSauterQStrat)
// returns 3/2/1 (common face/edge/vertex), -1 (Wilton SE) or 0 (far DQ)
// ------------------------------------------------------------------------------------
DEV int classify_exact(const Geo& t, const Geo& s, int qs_kind, double k2) {
  const double dtol = 1.0e3 * 2.220446049250313e-16;
  int hits = 0;
  double dmin2 = 1e308;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      V3<double> d = t.v[i] - s.v[j];
      double d2 = dot(d, d);
      dmin2 = fmin(dmin2, d2);
      if (sqrt(d2) < dtol) ++hits;
    }
  if (qs_kind == BEAST_QS_DOUBLENUM) return 0;
  if (hits > 0) return hits;
  if (qs_kind == BEAST_QS_SAUTER) return 0;
  double h2 = s.area;
  if (fmax(dmin2 * k2, dmin2 / (16.0 * h2)) < 0.2 * 0.2) return -1;
  return 0;
}

// TestRefinesTrialQStrat / TrialRefinesTestQStrat (src/quadrature/strategies/
// testrefinestrialqstrat.jl:9-17, trialrefinestestqstrat.jl:9-17): a pair that shares a vertex
// becomes class 5 (split the trial cell into its children) or 6 (split the test cell); every
// other pair keeps the wrapped strategy's class
DEV int refines_class(int cls, int qs_kind) {
  if (cls > 0 && qs_kind == BEAST_QS_TEST_REFINES_TRIAL) return 5;
  if (cls > 0 && qs_kind == BEAST_QS_TRIAL_REFINES_TEST) return 6;
  return cls;
}

// squared distance below which a pair can be near (strategy threshold of the trial cell)
DEV double near_threshold2(int qs_kind, double k2, double area) {
  if (qs_kind == BEAST_QS_DOUBLENUM) return -1.0;
  if (qs_kind == BEAST_QS_SAUTER) return 0.0;
  // max(d^2 k2, d^2/(16 A)) < 0.04  <=>  d^2 < 0.04 min(1/k2, 16 A)
  double t = 0.04 * 16.0 * area;
  if (k2 > 0) t = fmin(t, 0.04 / k2);
  return t;
}

// ------------------------------------------------------------------------------------
// far-pair kernel
// ------------------------------------------------------------------------------------
struct FarParams {
  OpParams op;
  int qs_kind;
  double k2;
  const int* tperm;  // Zcell position -> test active cell
  const double* tgeo;
  const float* tgeof;
  int64_t np;
  const double* bgeo;
  const float* bgeof;
  const int* qcells;
  int nq;
  void* zcell;
  int64_t ldc;
  const int* zrow;  // Zcell row of (position, test shape) / column of (chunk cell, trial
  const int* zcol;  // shape); null: the cell layout (see AsmArgs)
  NearPair* near;
  int near_cap;
  int* near_count;
  int* flag;
  TriRuleDev ro, ri;
};

// Zcell rows / columns (-1: the block entry is not stored)
DEV int64_t zrow_of(const int* zrow, int64_t pp, int nst, int i) { return zrow ? zrow[pp * nst + i] : nst * pp + i; }
DEV int64_t zcol_of(const int* zcol, int ql, int nsb, int j) { return zcol ? zcol[(int64_t)ql * nsb + j] : nsb * ql + j; }
DEV int64_t zidx(int64_t row, int64_t col, int64_t ldc) { return (row < 0 || col < 0) ? -1 : col * ldc + row; }

constexpr int FAR_THREADS = 128;
constexpr int FAR_QT = 16;  // trial cells staged per CTA

// one cell-pair value into Zcell in its format (ZCELL_*); an FP64 value enters the
// double-float format through the integer split of fsplit.h (no FP64 instruction)
template <typename R>
DEV void store_c(void* z, int64_t idx, C2<R> v, int fmt) {
  if (idx < 0) return;
  if (fmt == ZCELL_C64) {
    reinterpret_cast<float2*>(z)[idx] = make_float2((float)v.re, (float)v.im);
  } else if (fmt == ZCELL_DF) {
    float4 o;
    if (sizeof(R) == 8) {
      fsplit::split_f64((double)v.re, &o.x, &o.y);
      fsplit::split_f64((double)v.im, &o.z, &o.w);
    } else {
      o = make_float4((float)v.re, 0.f, (float)v.im, 0.f);
    }
    reinterpret_cast<float4*>(z)[idx] = o;
  } else {
    reinterpret_cast<double2*>(z)[idx] = make_double2((double)v.re, (double)v.im);
  }
}

// shared trial-cell record (in the arithmetic type R): sigma_j = s_j - c (9), centroid hi
// (3) and lo (3) parts, unit normal (3), area, near-test radius (radius + threshold
// distance); then per inner rule point eta_b = y_b - c (3) and weight
constexpr int QREC_HDR = 20;

template <int OPK, int TK, int BK, typename R, int FMT>
__global__ void __launch_bounds__(FAR_THREADS) k_far(FarParams P) {
  extern __shared__ unsigned char smraw[];
  R* sm = reinterpret_cast<R*>(smraw);
  const int ni = P.ri.n;
  const int rec = QREC_HDR + 4 * ni;
  const int q0 = blockIdx.y * FAR_QT;
  const int nqt = min(FAR_QT, P.nq - q0);
  // rule points in the arithmetic type, converted once per CTA (a double -> float conversion
  // runs on the FP64 pipe)
  __shared__ R ro_s[3 * RULE_MAXPTS], ri_s[2 * RULE_MAXPTS];
  for (int k = threadIdx.x; k < P.ro.n; k += blockDim.x) {
    ro_s[3 * k] = (R)P.ro.u[k];
    ro_s[3 * k + 1] = (R)P.ro.v[k];
    ro_s[3 * k + 2] = (R)P.ro.w[k];
  }
  for (int k = threadIdx.x; k < ni; k += blockDim.x) {
    ri_s[2 * k] = (R)P.ri.u[k];
    ri_s[2 * k + 1] = (R)P.ri.v[k];
  }
  // ---- stage trial cells
  for (int k = threadIdx.x; k < nqt * (1 + ni); k += blockDim.x) {
    int qi = k / (1 + ni), b = k % (1 + ni);
    const int qc = P.qcells[q0 + qi];
    const double* g = P.bgeo + (int64_t)qc * GEO_STRIDE;
    R* r = sm + qi * rec;
    const double cx = g[9], cy = g[10], cz = g[11];
    if (b == 0) {
      for (int j = 0; j < 3; ++j) {
        r[3 * j] = (R)(g[3 * j] - cx);
        r[3 * j + 1] = (R)(g[3 * j + 1] - cy);
        r[3 * j + 2] = (R)(g[3 * j + 2] - cz);
      }
      r[9] = (R)cx; r[10] = (R)cy; r[11] = (R)cz;
      r[12] = (R)(cx - (double)(R)cx); r[13] = (R)(cy - (double)(R)cy); r[14] = (R)(cz - (double)(R)cz);
      r[15] = (R)g[12]; r[16] = (R)g[13]; r[17] = (R)g[14];
      r[18] = (R)g[15];
      double thr2 = near_threshold2(P.qs_kind, P.k2, g[15]);
      r[19] = (R)((double)P.bgeof[4 * qc + 3] + sqrt(fmax(thr2, 0.0)));
    } else {
      int bb = b - 1;
      double u = P.ri.u[bb], v = P.ri.v[bb], w = 1.0 - u - v;
      R* pt = r + QREC_HDR + 4 * bb;
      pt[0] = (R)(u * (g[0] - cx) + v * (g[3] - cx) + w * (g[6] - cx));
      pt[1] = (R)(u * (g[1] - cy) + v * (g[4] - cy) + w * (g[7] - cy));
      pt[2] = (R)(u * (g[2] - cz) + v * (g[5] - cz) + w * (g[8] - cz));
      pt[3] = (R)P.ri.w[bb];
    }
  }
  __shared__ int s_zc[FAR_QT][3];
  for (int k = threadIdx.x; k < nqt * 3; k += blockDim.x)
    s_zc[k / 3][k % 3] = (int)zcol_of(P.zcol, q0 + k / 3, (BK == BEAST_P0) ? 1 : 3, k % 3);
  __syncthreads();
  // pp: the test cell's Zcell position (cells in the order of their first function, so that
  // the rows a warp of the gather reads are close together); p: the active cell
  const int64_t pp = blockIdx.x * (int64_t)FAR_THREADS + threadIdx.x;
  if (pp >= P.np) return;
  const int64_t p = P.tperm[pp];
  int64_t zr[3];
  for (int i = 0; i < 3; ++i) zr[i] = i < ((TK == BEAST_P0) ? 1 : 3) ? zrow_of(P.zrow, pp, (TK == BEAST_P0) ? 1 : 3, i) : -1;
  const double* tg = P.tgeo + p * GEO_STRIDE;
  const double cpx = tg[9], cpy = tg[10], cpz = tg[11];
  const V3<R> chp = mk((R)cpx, (R)cpy, (R)cpz);
  const V3<R> clp = mk((R)(cpx - (double)(R)cpx), (R)(cpy - (double)(R)cpy), (R)(cpz - (double)(R)cpz));
  V3<R> tau[3];
  for (int i = 0; i < 3; ++i)
    tau[i] = mk((R)(tg[3 * i] - cpx), (R)(tg[3 * i + 1] - cpy), (R)(tg[3 * i + 2] - cpz));
  const V3<R> nn = mk((R)tg[12], (R)tg[13], (R)tg[14]);
  const double Ap = tg[15];
  const R radp = (R)P.tgeof[4 * p + 3];
  const R gr = (R)P.op.gr, gi = (R)P.op.gi;
  const C2<R> alpha{(R)P.op.ar, (R)P.op.ai}, beta{(R)P.op.br, (R)P.op.bi};
  const R ApR = (R)Ap;
  const int nst = (TK == BEAST_P0) ? 1 : 3, nsb = (BK == BEAST_P0) ? 1 : 3;
  const int no = P.ro.n;

  for (int qi = 0; qi < nqt; ++qi) {
    const R* rq = sm + qi * rec;
    const int ql = q0 + qi;
    // d = c_p - c_q from hi/lo parts
    const V3<R> d = mk((chp.x - rq[9]) + (clp.x - rq[12]), (chp.y - rq[10]) + (clp.y - rq[13]),
                       (chp.z - rq[11]) + (clp.z - rq[14]));
    // ---- near test (candidate filter on centroid distance, exact FP64 classification).
    // DoubleNumQStrat applies one rule to every pair; the pairs whose circumspheres about the
    // centroids meet (every touching pair among them) go to k_near as class 4, the same rule
    // evaluated point by point in FP64: the moment form loses digits when rule points of the
    // two cells come close.
    {
      const R lim = radp + rq[19];
      if (dot(d, d) <= lim * lim * (R)1.0001 + (R)1e-30) {
        int cls = 4;
        if (P.qs_kind != BEAST_QS_DOUBLENUM) {
          Geo t = load_geo(tg);
          Geo s = load_geo(P.bgeo + (int64_t)P.qcells[ql] * GEO_STRIDE);
          cls = refines_class(classify_exact(t, s, P.qs_kind, P.k2), P.qs_kind);
        }
        if (cls != 0) {
          int idx = atomicAdd(P.near_count, 1);
          if (idx < P.near_cap)
            P.near[idx] = NearPair{(int)pp, ql, cls, 0};
          else
            atomicOr(P.flag, 1);
          for (int i = 0; i < nst; ++i)
            for (int j = 0; j < nsb; ++j)
              store_c<R>(P.zcell, zidx(zr[i], s_zc[qi][j], P.ldc), C2<R>{0, 0}, FMT);
          continue;
        }
      }
    }
    const R Aq = rq[18];
    const R* pts = rq + QREC_HDR;

    if (OPK == BEAST_MW_SL || OPK == BEAST_MW_DL || OPK == BEAST_MW_NXDL) {
      // ---- RT x RT with moment reduction
      C2<R> M0{0, 0}, M1{0, 0}, M2{0, 0}, M3{0, 0};  // scalar moments
      CV<R> V1, V2, V3_, V4, V5, V6;                   // vector moments
      cv_zero(V1); cv_zero(V2); cv_zero(V3_); cv_zero(V4); cv_zero(V5); cv_zero(V6);
      for (int a = 0; a < no; ++a) {
        const R ua = ro_s[3 * a], va = ro_s[3 * a + 1], wa3 = (R)1 - ua - va;
        const V3<R> xi = mk(ua * tau[0].x + va * tau[1].x + wa3 * tau[2].x,
                            ua * tau[0].y + va * tau[1].y + wa3 * tau[2].y,
                            ua * tau[0].z + va * tau[1].z + wa3 * tau[2].z);
        const R wa = ro_s[3 * a + 2];
        const V3<R> dx = d + xi;
        // inner sums over trial points: U0 = sum w K, U1 = sum w K eta,
        // U2 = sum w K eta (n.eta), U3 = sum w K (n.eta)   (K = G or grad coefficient)
        C2<R> U0{0, 0}, U3{0, 0};
        CV<R> U1, U2;
        cv_zero(U1); cv_zero(U2);
        for (int b = 0; b < ni; ++b) {
          const R* pb = pts + 4 * b;
          const V3<R> eta = mk(pb[0], pb[1], pb[2]);
          const R wb = pb[3];
          const V3<R> r = dx - eta;
          const R R2 = dot(r, r);
          const R iR = rsq<R>(R2);
          const R Rr = R2 * iR;
          C2<R> G = green<R>(gr, gi, Rr, iR);
          C2<R> K;
          if (OPK == BEAST_MW_SL) {
            K = cscale(wb, G);
          } else {  // grad G = c r, c = -(gamma + 1/R) G / R
            C2<R> c = cmul(C2<R>{-(gr + iR), -gi}, G);
            K = cscale(wb * iR, c);
          }
          U0 = cadd(U0, K);
          cv_axpy(K, eta, U1);
          if (OPK == BEAST_MW_NXDL) {
            R ne = dot(nn, eta);
            C2<R> Kn = cscale(ne, K);
            U3 = cadd(U3, Kn);
            cv_axpy(Kn, eta, U2);
          }
        }
        // fold the inner sums into the pair moments
        if (OPK == BEAST_MW_SL) {
          // M0 = sum G, V1 = sum G xi, V2 = sum G eta, M1 = sum G xi.eta
          C2<R> s0 = cscale(wa, U0);
          M0 = cadd(M0, s0);
          cv_axpy(s0, xi, V1);
          V2.x = cadd(V2.x, cscale(wa, U1.x));
          V2.y = cadd(V2.y, cscale(wa, U1.y));
          V2.z = cadd(V2.z, cscale(wa, U1.z));
          M1 = cadd(M1, cscale(wa, rdot(xi, U1)));
        } else if (OPK == BEAST_MW_DL) {
          // D0 = sum c xi.(d x eta) = xi.(d x U1) ; Dxr = sum c (xi x r) = (xi x d) U0 - xi x U1
          // Drh = sum c (r x eta) = (d + xi) x U1 ; Dr = sum c r = (d + xi) U0 - U1
          M0 = cadd(M0, cscale(wa, rdot(xi, rcross_cv(d, U1))));
          CV<R> xu = rcross_cv(xi, U1);
          V3<R> xd = cross(xi, d);
          V1.x = cadd(V1.x, cscale(wa, csub(cscale(xd.x, U0), xu.x)));
          V1.y = cadd(V1.y, cscale(wa, csub(cscale(xd.y, U0), xu.y)));
          V1.z = cadd(V1.z, cscale(wa, csub(cscale(xd.z, U0), xu.z)));
          CV<R> du = rcross_cv(dx, U1);
          V2.x = cadd(V2.x, cscale(wa, du.x));
          V2.y = cadd(V2.y, cscale(wa, du.y));
          V2.z = cadd(V2.z, cscale(wa, du.z));
          V3_.x = cadd(V3_.x, cscale(wa, csub(cscale(dx.x, U0), U1.x)));
          V3_.y = cadd(V3_.y, cscale(wa, csub(cscale(dx.y, U0), U1.y)));
          V3_.z = cadd(V3_.z, cscale(wa, csub(cscale(dx.z, U0), U1.z)));
        } else {  // n x K, n = test normal
          const R xr = dot(xi, dx);     // xi.(d + xi)
          const R nd = dot(nn, dx);     // n.(d + xi)
          C2<R> xU1 = rdot(xi, U1), xU2 = rdot(xi, U2);
          // N1 = (xi.(d+xi)) U3 - xi.U2
          M0 = cadd(M0, cscale(wa, csub(cscale(xr, U3), xU2)));
          // N2 = (xi.(d+xi)) U0 - xi.U1
          M1 = cadd(M1, cscale(wa, csub(cscale(xr, U0), xU1)));
          // N3 = (d + xi) U3 - U2
          V1.x = cadd(V1.x, cscale(wa, csub(cscale(dx.x, U3), U2.x)));
          V1.y = cadd(V1.y, cscale(wa, csub(cscale(dx.y, U3), U2.y)));
          V1.z = cadd(V1.z, cscale(wa, csub(cscale(dx.z, U3), U2.z)));
          // N4 = (d + xi) U0 - U1
          V2.x = cadd(V2.x, cscale(wa, csub(cscale(dx.x, U0), U1.x)));
          V2.y = cadd(V2.y, cscale(wa, csub(cscale(dx.y, U0), U1.y)));
          V2.z = cadd(V2.z, cscale(wa, csub(cscale(dx.z, U0), U1.z)));
          // N5 = n.(d+xi) xi.U1 - xi.U2
          M2 = cadd(M2, cscale(wa, csub(cscale(nd, xU1), xU2)));
          // N6 = xi (n.(d+xi) U0 - U3)
          C2<R> t6 = cscale(wa, csub(cscale(nd, U0), U3));
          cv_axpy(t6, xi, V3_);
          // N7 = n.(d+xi) U1 - U2
          V4.x = cadd(V4.x, cscale(wa, csub(cscale(nd, U1.x), U2.x)));
          V4.y = cadd(V4.y, cscale(wa, csub(cscale(nd, U1.y), U2.y)));
          V4.z = cadd(V4.z, cscale(wa, csub(cscale(nd, U1.z), U2.z)));
          // N8 = n.(d+xi) U0 - U3
          M3 = cadd(M3, t6);
        }
      }
      // ---- finalize the 3x3 block (x Ap Aq from the rule weights, / (4 Ap Aq) from the shapes)
      for (int i = 0; i < 3; ++i) {
        const V3<R> ti = tau[i];
        for (int j = 0; j < 3; ++j) {
          const V3<R> sj = mk(rq[3 * j], rq[3 * j + 1], rq[3 * j + 2]);
          C2<R> z;
          if (OPK == BEAST_MW_SL) {
            // alpha/4 (Mxe - Mx.s - t.Me + (t.s) M0) + beta M0
            C2<R> f = csub(csub(M1, rdot(sj, V1)), rdot(ti, V2));
            f = cadd(f, cscale(dot(ti, sj), M0));
            z = cadd(cscale((R)0.25, cmul(alpha, f)), cmul(beta, M0));
          } else if (OPK == BEAST_MW_DL) {
            // 1/4 [D0 - Dxr.s - t.Drh + (s x t).Dr]
            C2<R> f = csub(csub(M0, rdot(sj, V1)), rdot(ti, V2));
            f = cadd(f, rdot(cross(sj, ti), V3_));
            z = cscale((R)0.25, f);
          } else {
            const R ns = dot(nn, sj);
            // 1/4 [N1 - N2 n.s - t.N3 + (t.N4) n.s - N5 + N6.s + t.N7 - (t.s) N8]
            C2<R> f = csub(M0, cscale(ns, M1));
            f = csub(f, rdot(ti, V1));
            f = cadd(f, cscale(ns, rdot(ti, V2)));
            f = csub(f, M2);
            f = cadd(f, rdot(sj, V3_));
            f = cadd(f, rdot(ti, V4));
            f = csub(f, cscale(dot(ti, sj), M3));
            z = cscale((R)0.25, f);
          }
          store_c<R>(P.zcell, zidx(zr[i], s_zc[qi][j], P.ldc), z, FMT);
        }
      }
    } else {
      // ---- Helmholtz kernels on P0/P1: per point pair with shape products
      C2<R> acc[9];
      for (int k = 0; k < 9; ++k) acc[k] = C2<R>{0, 0};
      const V3<R> nq = mk(rq[15], rq[16], rq[17]);
      for (int a = 0; a < no; ++a) {
        const R ua = ro_s[3 * a], va = ro_s[3 * a + 1], wa3 = (R)1 - ua - va;
        const V3<R> xi = mk(ua * tau[0].x + va * tau[1].x + wa3 * tau[2].x,
                            ua * tau[0].y + va * tau[1].y + wa3 * tau[2].y,
                            ua * tau[0].z + va * tau[1].z + wa3 * tau[2].z);
        const R lt[3] = {ua, va, wa3};
        const R wa = ro_s[3 * a + 2];
        const V3<R> dx = d + xi;
        for (int b = 0; b < ni; ++b) {
          const R* pb = pts + 4 * b;
          const V3<R> eta = mk(pb[0], pb[1], pb[2]);
          const R wb = pb[3] * wa;
          const V3<R> r = dx - eta;
          const R R2 = dot(r, r);
          const R iR = rsq<R>(R2);
          const R Rr = R2 * iR;
          C2<R> G = green<R>(gr, gi, Rr, iR);
          C2<R> K;
          const C2<R> al = alpha;
          if (OPK == BEAST_HH_SL) {
            K = cmul(al, G);
          } else {
            C2<R> c = cscale(iR, cmul(C2<R>{-(gr + iR), -gi}, G));  // grad G = c r
            c = cmul(al, c);
            if (OPK == BEAST_HH_DL)
              K = cscale(-dot(nq, r), c);
            else
              K = cscale(dot(nn, r), c);
          }
          K = cscale(wb, K);
          const R ub = ri_s[2 * b], vb = ri_s[2 * b + 1];
          const R lb[3] = {ub, vb, (R)1 - ub - vb};
          for (int i = 0; i < nst; ++i)
            for (int j = 0; j < nsb; ++j) {
              R s = (TK == BEAST_P0 ? (R)1 : lt[i]) * (BK == BEAST_P0 ? (R)1 : lb[j]);
              acc[i * nsb + j] = cadd(acc[i * nsb + j], cscale(s, K));
            }
        }
      }
      const R ApAq = ApR * Aq;
      for (int i = 0; i < nst; ++i)
        for (int j = 0; j < nsb; ++j)
          store_c<R>(P.zcell, zidx(zr[i], s_zc[qi][j], P.ldc), cscale(ApAq, acc[i * nsb + j]), FMT);
    }
  }
}

// ------------------------------------------------------------------------------------
// near pairs (FP64): generic per-point integrand
// ------------------------------------------------------------------------------------
struct Shp {
  double s[3];
  V3<double> v[3];
  double div[3];
};

DEV void shapes(int kind, const Geo& g, V3<double> x, const double* bary, Shp& S) {
  if (kind == BEAST_RT) {
    double ij = 0.5 / g.area;
    for (int i = 0; i < 3; ++i) {
      S.v[i] = ij * (x - g.v[i]);
      S.div[i] = 2.0 * ij;
    }
  } else if (kind == BEAST_P0) {
    S.s[0] = 1.0;
  } else {
    for (int i = 0; i < 3; ++i) S.s[i] = bary[i];
  }
}

// operator kinds for the regular parts of singularity extraction
enum { REG = 100 };

// adds w * k_ij(x, y) to acc[i*nb + j]
DEV void integrand(int kind, const OpParams& op, V3<double> x, V3<double> y, V3<double> nx,
                   V3<double> ny, int tk, const Shp& f, int bk, const Shp& g, double w,
                   C2<double>* acc) {
  const int nt = tk == BEAST_P0 ? 1 : 3, nb = bk == BEAST_P0 ? 1 : 3;
  V3<double> r = x - y;
  // one reciprocal square root instead of a square root and a division (both long FP64
  // sequences on GB300)
  const double R2 = dot(r, r);
  const double iR = rsqrt(R2);
  const double R = R2 * iR;
  C2<double> gR{op.gr * R, op.gi * R};
  C2<double> al{op.ar, op.ai}, be{op.br, op.bi};
  switch (kind) {
    case BEAST_MW_SL:
    case REG + BEAST_MW_SL: {
      C2<double> G;
      if (kind == BEAST_MW_SL) {
        G = cexp_d(C2<double>{-gR.re, -gR.im});
        G = cscale(I4PI * iR, G);
      } else {  // (expm1(-gR) + gR - gR^2/2) / (4 pi R)
        C2<double> e = cexpm1_d(C2<double>{-gR.re, -gR.im});
        C2<double> g2 = cmul(gR, gR);
        G = cadd(e, csub(gR, cscale(0.5, g2)));
        G = cscale(I4PI * iR, G);
      }
      C2<double> aG = cmul(al, G), bG = cmul(be, G);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          C2<double> t = cadd(cscale(dot(f.v[i], g.v[j]), aG), cscale(f.div[i] * g.div[j], bG));
          acc[i * 3 + j] = cadd(acc[i * 3 + j], cscale(w, t));
        }
      break;
    }
    case BEAST_MW_DL:
    case REG + BEAST_MW_DL:
    case BEAST_MW_NXDL: {
      C2<double> c;
      if (kind == REG + BEAST_MW_DL) {
        C2<double> ex = cexp_d(C2<double>{-gR.re, -gR.im});
        C2<double> g2 = cmul(gR, gR);
        C2<double> t = cmul(C2<double>{-(gR.re + 1.0), -gR.im}, ex);
        t = cadd(t, C2<double>{1.0 - 0.5 * g2.re, -0.5 * g2.im});
        c = cscale(I4PI * iR * iR * iR, t);
      } else {
        C2<double> G = cscale(I4PI * iR, cexp_d(C2<double>{-gR.re, -gR.im}));
        c = cscale(iR, cmul(C2<double>{-(op.gr + iR), -op.gi}, G));
      }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double t;
          if (kind == BEAST_MW_NXDL)
            t = dot(f.v[i], cross(nx, cross(r, g.v[j])));
          else
            t = dot(f.v[i], cross(r, g.v[j]));
          acc[i * 3 + j] = cadd(acc[i * 3 + j], cscale(w * t, c));
        }
      break;
    }
    case BEAST_HH_SL:
    case REG + BEAST_HH_SL: {
      C2<double> G;
      if (kind == BEAST_HH_SL) {
        G = cscale(I4PI * iR, cexp_d(C2<double>{-gR.re, -gR.im}));
      } else {  // (expm1(-gR) - gR^2/2) / (4 pi R)
        C2<double> e = cexpm1_d(C2<double>{-gR.re, -gR.im});
        C2<double> g2 = cmul(gR, gR);
        G = cscale(1.0 / (4.0 * PI * R), csub(e, cscale(0.5, g2)));
      }
      C2<double> aG = cmul(al, G);
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nb; ++j)
          acc[i * nb + j] = cadd(acc[i * nb + j], cscale(w * f.s[i] * g.s[j], aG));
      break;
    }
    default: {  // HH DL / DLT and their regular parts
      bool reg = kind >= REG;
      int base = reg ? kind - REG : kind;
      C2<double> c;
      if (reg) {
        C2<double> ex = cexp_d(C2<double>{-gR.re, -gR.im});
        C2<double> g2 = cmul(gR, gR);
        C2<double> t = cmul(C2<double>{-(gR.re + 1.0), -gR.im}, ex);
        t = cadd(t, C2<double>{1.0 - 0.5 * g2.re, -0.5 * g2.im});
        c = cscale(I4PI * iR * iR * iR, t);  // the reference's regular part omits alpha
      } else {
        C2<double> G = cscale(I4PI * iR, cexp_d(C2<double>{-gR.re, -gR.im}));
        c = cmul(al, cscale(iR, cmul(C2<double>{-(op.gr + iR), -op.gi}, G)));
      }
      C2<double> k = base == BEAST_HH_DL ? cscale(-dot(ny, r), c) : cscale(dot(nx, r), c);
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nb; ++j)
          acc[i * nb + j] = cadd(acc[i * nb + j], cscale(w * f.s[i] * g.s[j], k));
      break;
    }
  }
}

__constant__ double c_gl_x[210];
__constant__ double c_gl_w[210];
__constant__ int c_gl_off[21];

// one Sauter-Schwab node: map index -> reference points X, Y on {0<=x2<=x1<=1} and weight
DEV void ss_node(int cls, int n, int64_t item, const double* glx, const double* glw, double* X,
                 double* Y, double* w) {
  int nreg = cls == 1 ? 2 : 6;
  int reg = (int)(item % nreg);
  int64_t k = item / nreg;
  int i4 = (int)(k % n); k /= n;
  int i3 = (int)(k % n); k /= n;
  int i2 = (int)(k % n); k /= n;
  int i1 = (int)k;
  double xi = glx[i1], e1 = glx[i2], e2 = glx[i3], e3 = glx[i4];
  double ww = glw[i1] * glw[i2] * glw[i3] * glw[i4];
  double A[2], B[2], wt;
  int sub = reg >> 1;
  bool swap = reg & 1;
  if (cls == 1) {  // common vertex: 2 regions
    wt = ww * xi * xi * xi * e2;
    A[0] = xi; A[1] = xi * e1;
    B[0] = xi * e2; B[1] = xi * e2 * e3;
  } else if (cls == 2) {  // common edge: x1 = xi, x2 = xi b, y1 = xi(1-a'), y2 = xi(1-a')c
    double ap, bb, cc;
    if (sub == 0) { ap = e1; bb = e1 * e2; cc = e1 * e3; }
    else if (sub == 1) { bb = e1; ap = e1 * e2; cc = e1 * e3; }
    else { cc = e1; ap = e1 * e2; bb = e1 * e3; }
    wt = ww * xi * xi * xi * (1.0 - ap) * e1 * e1;
    A[0] = xi; A[1] = xi * bb;
    B[0] = xi * (1.0 - ap); B[1] = xi * (1.0 - ap) * cc;
  } else {  // common face
    double s = e1, t = e2, u = e3;
    wt = ww * xi * xi * xi * s * (1.0 - s);
    if (sub == 0) {
      double ap = s * t, e = s * (1.0 - t), b = (1.0 - s) * u;
      A[0] = xi; A[1] = xi * b;
      B[0] = xi * (1.0 - ap); B[1] = xi * (b + e);
    } else if (sub == 1) {
      double ap = s, ep = s * t, cp = (1.0 - s) * u;
      A[0] = xi; A[1] = xi * (cp + ep);
      B[0] = xi * (1.0 - ap); B[1] = xi * cp;
    } else {
      double ep = s, ap = s * t, cp = (1.0 - s) * u;
      A[0] = xi; A[1] = xi * (cp + ep);
      B[0] = xi * (1.0 - ap); B[1] = xi * cp;
    }
  }
  if (swap) {
    X[0] = B[0]; X[1] = B[1]; Y[0] = A[0]; Y[1] = A[1];
  } else {
    X[0] = A[0]; X[1] = A[1]; Y[0] = B[0]; Y[1] = B[1];
  }
  *w = wt;
}

// ss_node in FP32 for the mixed path, with D = X - Y formed from the maps' own factors (it
// scales with xi, so x - y keeps its relative precision near the singularity)
DEV void ss_node_f(int cls, int n, int item, const float* glx, const float* glw, float* X, float* Y,
                   float* D, float* w) {
  const int nreg = cls == 1 ? 2 : 6;
  const int reg = item % nreg;
  int k = item / nreg;
  const int i4 = k % n;
  k /= n;
  const int i3 = k % n;
  k /= n;
  const int i2 = k % n;
  const int i1 = k / n;
  const float xi = glx[i1], e1 = glx[i2], e2 = glx[i3], e3 = glx[i4];
  const float ww = glw[i1] * glw[i2] * glw[i3] * glw[i4];
  float A[2], B[2], AB[2], wt;
  const int sub = reg >> 1;
  const bool swap = reg & 1;
  if (cls == 1) {  // common vertex
    wt = ww * xi * xi * xi * e2;
    A[0] = xi; A[1] = xi * e1;
    B[0] = xi * e2; B[1] = xi * e2 * e3;
    AB[0] = xi * (1.0f - e2); AB[1] = xi * (e1 - e2 * e3);
  } else if (cls == 2) {  // common edge
    float ap, bb, cc;
    if (sub == 0) { ap = e1; bb = e1 * e2; cc = e1 * e3; }
    else if (sub == 1) { bb = e1; ap = e1 * e2; cc = e1 * e3; }
    else { cc = e1; ap = e1 * e2; bb = e1 * e3; }
    wt = ww * xi * xi * xi * (1.0f - ap) * e1 * e1;
    A[0] = xi; A[1] = xi * bb;
    B[0] = xi * (1.0f - ap); B[1] = xi * (1.0f - ap) * cc;
    AB[0] = xi * ap; AB[1] = xi * (bb - (1.0f - ap) * cc);
  } else {  // common face
    const float s = e1, t = e2, u = e3;
    wt = ww * xi * xi * xi * s * (1.0f - s);
    if (sub == 0) {
      const float ap = s * t, e = s * (1.0f - t), b = (1.0f - s) * u;
      A[0] = xi; A[1] = xi * b;
      B[0] = xi * (1.0f - ap); B[1] = xi * (b + e);
      AB[0] = xi * ap; AB[1] = -xi * e;
    } else {
      const float ap = sub == 1 ? s : s * t, ep = sub == 1 ? s * t : s, cp = (1.0f - s) * u;
      A[0] = xi; A[1] = xi * (cp + ep);
      B[0] = xi * (1.0f - ap); B[1] = xi * cp;
      AB[0] = xi * ap; AB[1] = xi * ep;
    }
  }
  if (swap) {
    X[0] = B[0]; X[1] = B[1]; Y[0] = A[0]; Y[1] = A[1];
    D[0] = -AB[0]; D[1] = -AB[1];
  } else {
    X[0] = A[0]; X[1] = A[1]; Y[0] = B[0]; Y[1] = B[1];
    D[0] = AB[0]; D[1] = AB[1];
  }
  *w = wt;
}

// ss_node_f's maps in FP64 (X, Y, D = X - Y from the maps' own factors, weight): the node
// tables of k_near_ss_df are built from it once
DEV void ss_node_fd(int cls, int n, int item, const double* glx, const double* glw, double* X, double* Y,
                    double* D, double* w) {
  const int nreg = cls == 1 ? 2 : 6;
  const int reg = item % nreg;
  int k = item / nreg;
  const int i4 = k % n;
  k /= n;
  const int i3 = k % n;
  k /= n;
  const int i2 = k % n;
  const int i1 = k / n;
  const double xi = glx[i1], e1 = glx[i2], e2 = glx[i3], e3 = glx[i4];
  const double ww = glw[i1] * glw[i2] * glw[i3] * glw[i4];
  double A[2], B[2], AB[2], wt;
  const int sub = reg >> 1;
  const bool swap = reg & 1;
  if (cls == 1) {
    wt = ww * xi * xi * xi * e2;
    A[0] = xi; A[1] = xi * e1;
    B[0] = xi * e2; B[1] = xi * e2 * e3;
    AB[0] = xi * (1.0 - e2); AB[1] = xi * (e1 - e2 * e3);
  } else if (cls == 2) {
    double ap, bb, cc;
    if (sub == 0) { ap = e1; bb = e1 * e2; cc = e1 * e3; }
    else if (sub == 1) { bb = e1; ap = e1 * e2; cc = e1 * e3; }
    else { cc = e1; ap = e1 * e2; bb = e1 * e3; }
    wt = ww * xi * xi * xi * (1.0 - ap) * e1 * e1;
    A[0] = xi; A[1] = xi * bb;
    B[0] = xi * (1.0 - ap); B[1] = xi * (1.0 - ap) * cc;
    AB[0] = xi * ap; AB[1] = xi * (bb - (1.0 - ap) * cc);
  } else {
    const double s = e1, t = e2, u = e3;
    wt = ww * xi * xi * xi * s * (1.0 - s);
    if (sub == 0) {
      const double ap = s * t, e = s * (1.0 - t), b = (1.0 - s) * u;
      A[0] = xi; A[1] = xi * b;
      B[0] = xi * (1.0 - ap); B[1] = xi * (b + e);
      AB[0] = xi * ap; AB[1] = -xi * e;
    } else {
      const double ap = sub == 1 ? s : s * t, ep = sub == 1 ? s * t : s, cp = (1.0 - s) * u;
      A[0] = xi; A[1] = xi * (cp + ep);
      B[0] = xi * (1.0 - ap); B[1] = xi * cp;
      AB[0] = xi * ap; AB[1] = xi * ep;
    }
  }
  if (swap) {
    X[0] = B[0]; X[1] = B[1]; Y[0] = A[0]; Y[1] = A[1];
    D[0] = -AB[0]; D[1] = -AB[1];
  } else {
    X[0] = A[0]; X[1] = A[1]; Y[0] = B[0]; Y[1] = B[1];
    D[0] = AB[0]; D[1] = AB[1];
  }
  *w = wt;
}

DEV V3<float> v3f(V3<double> a) { return V3<float>{(float)a.x, (float)a.y, (float)a.z}; }

struct NearParams {
  OpParams op;
  beast_qs_desc qs;
  int tk, bk;
  const int* tperm;  // Zcell position -> test active cell
  const double* tgeo;
  const double* bgeo;
  const int* qcells;
  const NearPair* near;
  int nnear;
  void* zcell;
  int zfmt;  // Zcell format (ZCELL_*)
  int ss32;  // Sauter-Schwab moments of RT Maxwell pairs in FP32 (mixed precision)
  int ssdf;  // Sauter-Schwab pairs of RT Maxwell operators in double-float (k_near_ss_df)
  const float2* ssdf_tab[4];  // per class 1..3: node table [7][items] (ss_table)
  int ssdf_items[4];
  int64_t ldc;
  const int* zrow;  // as in FarParams
  const int* zcol;
  int* flag;
  TriRuleDev ro, ri;
  // the refines strategies: the wrapped strategy's far rules (children far from the other
  // cell), the coarse side's active cell -> mesh cell and the coarse mesh's children
  TriRuleDev fro, fri;
  const int* bcells;        // trial active cell -> trial mesh cell
  const double* bchildren;  // [trial mesh cell][bnchild][9]
  int bnchild;
  const int* tcells;        // test active cell -> test mesh cell
  const double* tchildren;  // [test mesh cell][tnchild][9]
  int tnchild;
};

constexpr int NEAR_WARPS = 4;

// Sauter-Schwab pairs of RT x RT Maxwell single / double layers on the mixed path: the 22
// moments in FP32 (FP64 partial sums every 16 points), the 3 x 3 block from them in FP64.
// A kernel of its own so that its register budget (and occupancy) is not set by the FP64
// paths of k_near; k_near skips these pairs.
DEV bool near_is_ss32(const NearParams& P, int cls) {
  return P.ss32 && cls >= 1 && cls <= 3 && P.tk == BEAST_RT && P.bk == BEAST_RT &&
         (P.op.kind == BEAST_MW_SL || (P.op.kind == BEAST_MW_DL && cls != 3));
}

// the same pairs in double-float arithmetic on the mixed-accurate path (real wavenumber):
// k_near_ss_df; the double layer's common-face blocks (identically zero) stay with k_near;
// (k_near_ss_df), and the Helmholtz single layer's Sauter-Schwab pairs on P0 / P1 on the
// mixed and mixed-accurate paths (k_near_hh_df, k_near_batch_df)
DEV bool near_is_ssdf(const NearParams& P, int cls) {
  if (!P.ssdf || cls < 1 || cls > 3) return false;
  if (P.tk == BEAST_RT && P.bk == BEAST_RT)
    return P.op.kind == BEAST_MW_SL || (P.op.kind == BEAST_MW_DL && cls != 3);
  return P.op.kind == BEAST_HH_SL && P.tk != BEAST_RT && P.bk != BEAST_RT;
}

// sh + sl += p, the rounding error of the addition kept (Knuth's TwoSum; no contraction)
__device__ __forceinline__ void two_sum_f(float& sh, float& sl, float p) {
  const float t = __fadd_rn(sh, p);
  const float bb = __fsub_rn(t, sh);
  sl = __fadd_rn(sl, __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(p, bb)));
  sh = t;
}

__global__ void __launch_bounds__(32 * NEAR_WARPS) k_near_ss32(NearParams P) {
  __shared__ float s_glxf[210], s_glwf[210];
  __shared__ float2 s_mom[NEAR_WARPS][22][33];  // per warp: each lane's double-float moments
  __shared__ double s_tot[NEAR_WARPS][22];      // the warp's totals
  for (int k = threadIdx.x; k < 210; k += blockDim.x) {
    s_glxf[k] = (float)c_gl_x[k];
    s_glwf[k] = (float)c_gl_w[k];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * (int64_t)NEAR_WARPS + warp;
  if (e >= P.nnear) return;
  const NearPair np_ = P.near[e];
  if (!near_is_ss32(P, np_.cls)) return;
  const Geo t = load_geo(P.tgeo + (int64_t)P.tperm[np_.p] * GEO_STRIDE);
  const Geo s = load_geo(P.bgeo + (int64_t)P.qcells[np_.q] * GEO_STRIDE);
  {
    // ---- Sauter-Schwab: shared vertices first, same order (SauterSchwabQuadrature.reorder).
    // Lanes 0..8 test one vertex pair each (i = lane / 3, j = lane % 3; squared distances:
    // shared vertices coincide exactly); the first three hits in (i, j) order from the ballot.
    // (FP64 is a small fraction of the FP32 rate: per-pair FP64 work is spread over lanes.)
    const double dtol = 1.0e3 * 2.220446049250313e-16;
    bool hit = false;
    if (lane < 9) {
      const V3<double> dd = t.v[lane / 3] - s.v[lane % 3];
      hit = dot(dd, dd) < dtol * dtol;
    }
    const unsigned hmask = __ballot_sync(0xffffffffu, hit);
    int pt[3], ps[3], hits = 0, ti[3], si[3];
    for (int b = 0; b < 9; ++b)
      if (((hmask >> b) & 1u) && hits < 3) {
        ti[hits] = b / 3;
        si[hits] = b % 3;
        ++hits;
      }
    int k = 0;
    for (int h = 0; h < hits; ++h) pt[k++] = ti[h];
    for (int i = 0; i < 3; ++i) {
      bool used = false;
      for (int h = 0; h < hits; ++h) used |= ti[h] == i;
      if (!used) pt[k++] = i;
    }
    k = 0;
    for (int h = 0; h < hits; ++h) ps[k++] = si[h];
    for (int j = 0; j < 3; ++j) {
      bool used = false;
      for (int h = 0; h < hits; ++h) used |= si[h] == j;
      if (!used) ps[k++] = j;
    }
    const int n = np_.cls == 3 ? P.qs.ss_face : (np_.cls == 2 ? P.qs.ss_edge : P.qs.ss_vert);
    const int nreg = np_.cls == 1 ? 2 : 6;
    const int64_t items = (int64_t)nreg * n * n * n * n;
    const bool sl = P.op.kind == BEAST_MW_SL;
    const V3<double> cp = t.c, cq = s.c;
    const double gi = P.op.gi, gr = P.op.gr;
    double m[22];
#pragma unroll
    for (int k = 0; k < 22; ++k) m[k] = 0.0;
    const V3<double> d = cp - cq;
    {
        // FP32: x - y = X0 Et1 + X1 Et2 - Y0 Es1 - Y1 Es2 over the edge vectors of the two
        // charts from the shared first vertex (common terms folded into D = X - Y)
        // edge vectors as FP32 pairs hi + lo: the rounding of the geometry to FP32 would
        // otherwise be one systematic perturbation of every point of the pair
        const V3<double> Et1 = t.v[pt[1]] - t.v[pt[0]], Et2 = t.v[pt[2]] - t.v[pt[1]];
        const V3<double> Es1 = s.v[ps[1]] - s.v[ps[0]], Es2 = s.v[ps[2]] - s.v[ps[1]];
        const V3<float> a0 = v3f(t.v[pt[0]] - cp), et1 = v3f(Et1), et2 = v3f(Et2);
        const V3<float> b0 = v3f(s.v[ps[0]] - cq), es1 = v3f(Es1), es2 = v3f(Es2);
        const V3<float> et1l = v3f(Et1 - mk<double>(et1.x, et1.y, et1.z)),
                        et2l = v3f(Et2 - mk<double>(et2.x, et2.y, et2.z)),
                        es1l = v3f(Es1 - mk<double>(es1.x, es1.y, es1.z)),
                        es2l = v3f(Es2 - mk<double>(es2.x, es2.y, es2.z));
        const V3<float> df = v3f(d);
        const float gif = (float)gi, grf = (float)gr;
        const float* glxf = s_glxf + c_gl_off[n - 1];
        const float* glwf = s_glwf + c_gl_off[n - 1];
        // FP32 partial moments over at most 16 points, flushed into double-float moments
        // (mh + ml, the rounding error of each addition kept by TwoSum) so that the FP32
        // rounding of the sums stays at the level of a 16-term sum -- without FP64
        // arithmetic in the point loop (the FP64 pipe is a small fraction of the FP32 rate)
        float mf[22], mh[22], ml[22];
#pragma unroll
        for (int k = 0; k < 22; ++k) mf[k] = mh[k] = ml[k] = 0.0f;
        int cnt = 0;
        for (int it = lane; it < (int)items; it += 32) {
          float X[2], Y[2], D[2], w;
          ss_node_f(np_.cls, n, it, glxf, glwf, X, Y, D, &w);
          const V3<float> xi = a0 + X[0] * et1 + X[1] * et2;
          const V3<float> eta = b0 + Y[0] * es1 + Y[1] * es2;
          V3<float> r;
          if (np_.cls == 3)
            r = (D[0] * et1 + D[1] * et2) + (D[0] * et1l + D[1] * et2l);
          else if (np_.cls == 2)
            r = (D[0] * et1 + (X[1] * et2 - Y[1] * es2)) + (D[0] * et1l + (X[1] * et2l - Y[1] * es2l));
          else
            r = ((X[0] * et1 + X[1] * et2) - (Y[0] * es1 + Y[1] * es2)) +
                ((X[0] * et1l + X[1] * et2l) - (Y[0] * es1l + Y[1] * es2l));
          const float R = sqrtf(dot(r, r));
          const float iR = 1.0f / R;
          float sn, cs;
          sincosf(gif * R, &sn, &cs);
          const float amp = (grf == 0.0f ? 1.0f : expf(-grf * R)) * (float)I4PI * iR * w;
          float cr = amp * cs, ci = -amp * sn;
          V3<float> a, b, c3;
          float s0;
          if (sl) {
            s0 = dot(xi, eta);
            a = xi;
            b = eta;
            c3 = V3<float>{0, 0, 0};
            mf[0] += cr;
            mf[1] += ci;
          } else {
            const float pr = -(grf + iR) * iR, pi = -gif * iR;
            const float nr = pr * cr - pi * ci, ni = pr * ci + pi * cr;
            cr = nr;
            ci = ni;
            s0 = dot(xi, cross(df, eta));
            a = cross(xi, r);
            b = cross(r, eta);
            c3 = r;
          }
          mf[2] += s0 * cr; mf[3] += s0 * ci;
          mf[4] += a.x * cr; mf[5] += a.x * ci; mf[6] += a.y * cr; mf[7] += a.y * ci; mf[8] += a.z * cr; mf[9] += a.z * ci;
          mf[10] += b.x * cr; mf[11] += b.x * ci; mf[12] += b.y * cr; mf[13] += b.y * ci; mf[14] += b.z * cr; mf[15] += b.z * ci;
          mf[16] += c3.x * cr; mf[17] += c3.x * ci; mf[18] += c3.y * cr; mf[19] += c3.y * ci; mf[20] += c3.z * cr; mf[21] += c3.z * ci;
          if (++cnt == 16) {
#pragma unroll
            for (int k = 0; k < 22; ++k) {
              two_sum_f(mh[k], ml[k], mf[k]);
              mf[k] = 0.0f;
            }
            cnt = 0;
          }
        }
        // the lanes' double-float moments through shared memory: lane k < 22 sums moment k
        // over the 32 lanes (TwoSum) and converts it to FP64 once
#pragma unroll
        for (int k = 0; k < 22; ++k) {
          two_sum_f(mh[k], ml[k], mf[k]);
          s_mom[warp][k][lane] = make_float2(mh[k], ml[k]);
        }
        __syncwarp();
        if (lane < 22) {
          float th = 0.0f, tl = 0.0f;
          for (int l = 0; l < 32; ++l) {
            const float2 v = s_mom[warp][lane][l];
            two_sum_f(th, tl, v.x);
            tl = __fadd_rn(tl, v.y);
          }
          s_tot[warp][lane] = (double)th + (double)tl;
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 22; ++k) m[k] = s_tot[warp][k];
          }
      const C2<double> M0{m[0], m[1]}, M1{m[2], m[3]};
      CV<double> V1, V2, V3_;
      V1.x = {m[4], m[5]}; V1.y = {m[6], m[7]}; V1.z = {m[8], m[9]};
      V2.x = {m[10], m[11]}; V2.y = {m[12], m[13]}; V2.z = {m[14], m[15]};
      V3_.x = {m[16], m[17]}; V3_.y = {m[18], m[19]}; V3_.z = {m[20], m[21]};
      if (lane < 9) {  // lane 3 i + j: entry (i, j) of the 3 x 3 block
        const C2<double> al{P.op.ar, P.op.ai}, be{P.op.br, P.op.bi};
        const int i = lane / 3, j = lane % 3;
        const V3<double> ti = t.v[i] - cp;
        const V3<double> sj = s.v[j] - cq;
        C2<double> z;
        if (sl) {
          C2<double> fm = csub(csub(M1, rdot(sj, V1)), rdot(ti, V2));
          fm = cadd(fm, cscale(dot(ti, sj), M0));
          z = cadd(cmul(al, fm), cscale(4.0, cmul(be, M0)));
        } else {
          C2<double> fm = csub(csub(M1, rdot(sj, V1)), rdot(ti, V2));
          z = cadd(fm, rdot(cross(sj, ti), V3_));
        }
        store_c<double>(P.zcell, zidx(zrow_of(P.zrow, np_.p, 3, i), zcol_of(P.zcol, np_.q, 3, j), P.ldc), z, P.zfmt);
      }
  }
}

// ---- per-node paths of a near pair, shared by near_pair and the children of the refines
// strategies.  Each adds its lane's share of the block (lanes over nodes) to acc[i * nb + j].

// DoubleQuadRule (src/quadrature/doublenumints.jl:12-43) of rules ro x ri point by point in
// FP64 with the integrand of `kind` (REG + kind: the regular part of singularity extraction)
DEV void dq_points(const NearParams& P, int kind, const Geo& t, const Geo& s, const TriRuleDev& ro,
                   const TriRuleDev& ri, int lane, C2<double>* acc) {
  Shp f, g;
  const int no = ro.n, ni = ri.n;
  for (int it = lane; it < no * ni; it += 32) {
    const int a = it / ni, b = it % ni;
    double bx[3] = {ro.u[a], ro.v[a], 1.0 - ro.u[a] - ro.v[a]};
    double by[3] = {ri.u[b], ri.v[b], 1.0 - ri.u[b] - ri.v[b]};
    V3<double> x = bx[0] * t.v[0] + bx[1] * t.v[1] + bx[2] * t.v[2];
    V3<double> y = by[0] * s.v[0] + by[1] * s.v[1] + by[2] * s.v[2];
    shapes(P.tk, t, x, bx, f);
    shapes(P.bk, s, y, by, g);
    integrand(kind, P.op, x, y, t.n, s.n, P.tk, f, P.bk, g, ro.w[a] * t.area * ri.w[b] * s.area, acc);
  }
}

// Sauter-Schwab vertex order: shared vertices first, same order (SauterSchwabQuadrature.reorder)
DEV void ss_order(const Geo& t, const Geo& s, int* pt, int* ps) {
  const double dtol = 1.0e3 * 2.220446049250313e-16;
  int hits = 0, ti[3], si[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      V3<double> dd = t.v[i] - s.v[j];
      if (sqrt(dot(dd, dd)) < dtol && hits < 3) {
        ti[hits] = i;
        si[hits] = j;
        ++hits;
      }
    }
  int k = 0;
  for (int h = 0; h < hits; ++h) pt[k++] = ti[h];
  for (int i = 0; i < 3; ++i) {
    bool used = false;
    for (int h = 0; h < hits; ++h) used |= ti[h] == i;
    if (!used) pt[k++] = i;
  }
  k = 0;
  for (int h = 0; h < hits; ++h) ps[k++] = si[h];
  for (int j = 0; j < 3; ++j) {
    bool used = false;
    for (int h = 0; h < hits; ++h) used |= si[h] == j;
    if (!used) ps[k++] = j;
  }
}

// Sauter-Schwab rule of class cls (3 face, 2 edge, 1 vertex) node by node
DEV void ss_points(const NearParams& P, const Geo& t, const Geo& s, int cls, const int* pt, const int* ps,
                   const double* s_glx, const double* s_glw, int lane, C2<double>* acc) {
  Shp f, g;
  const int n = cls == 3 ? P.qs.ss_face : (cls == 2 ? P.qs.ss_edge : P.qs.ss_vert);
  const int nreg = cls == 1 ? 2 : 6;
  const int64_t items = (int64_t)nreg * n * n * n * n;
  const double jac = 4.0 * t.area * s.area;
  const double* glx = s_glx + c_gl_off[n - 1];
  const double* glw = s_glw + c_gl_off[n - 1];
  for (int64_t it = lane; it < items; it += 32) {
    double X[2], Y[2], w;
    ss_node(cls, n, it, glx, glw, X, Y, &w);
    double lt[3] = {1.0 - X[0], X[0] - X[1], X[1]}, ls[3] = {1.0 - Y[0], Y[0] - Y[1], Y[1]};
    double bx[3], by[3];
    for (int q = 0; q < 3; ++q) {
      bx[pt[q]] = lt[q];
      by[ps[q]] = ls[q];
    }
    V3<double> x = lt[0] * t.v[pt[0]] + lt[1] * t.v[pt[1]] + lt[2] * t.v[pt[2]];
    V3<double> y = ls[0] * s.v[ps[0]] + ls[1] * s.v[ps[1]] + ls[2] * s.v[ps[2]];
    shapes(P.tk, t, x, bx, f);
    shapes(P.bk, s, y, by, g);
    integrand(P.op.kind, P.op, x, y, t.n, s.n, P.tk, f, P.bk, g, w * jac, acc);
  }
}

// singularity extraction: the regular part by the near rules, the analytic inner part per
// outer point
DEV void se_points(const NearParams& P, const Geo& t, const Geo& s, int lane, C2<double>* acc) {
  dq_points(P, REG + P.op.kind, t, s, P.ro, P.ri, lane, acc);
  for (int a = lane; a < P.ro.n; a += 32) {
    double bx[3] = {P.ro.u[a], P.ro.v[a], 1.0 - P.ro.u[a] - P.ro.v[a]};
    V3<double> x = bx[0] * t.v[0] + bx[1] * t.v[1] + bx[2] * t.v[2];
    if (!se_singular(P.op, P.tk, P.bk, t, s, x, bx, P.ro.w[a] * t.area, acc)) atomicOr(P.flag, 2);
  }
}

// double-layer type kernels vanish identically on a flat common face
DEV bool dl_type(int kind) { return kind == BEAST_MW_DL || kind == BEAST_HH_DL || kind == BEAST_HH_DLT; }

// the wrapped DoubleNumWiltonSauterQStrat on one pair of triangles, any class
DEV void pair_points(const NearParams& P, const Geo& t, const Geo& s, int cls, const double* s_glx,
                     const double* s_glw, int lane, C2<double>* acc) {
  if (cls == 0) {
    dq_points(P, P.op.kind, t, s, P.fro, P.fri, lane, acc);
  } else if (cls > 0) {
    if (cls == 3 && dl_type(P.op.kind)) return;
    int pt[3], ps[3];
    ss_order(t, s, pt, ps);
    ss_points(P, t, s, cls, pt, ps, s_glx, s_glw, lane, acc);
  } else {
    se_points(P, t, s, lane, acc);
  }
}

// the triangle of 9 vertex coordinates as a Geo
DEV Geo geo_of_triangle(const double* v) {
  Geo g;
  for (int i = 0; i < 3; ++i) g.v[i] = mk(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
  const V3<double> cr = cross(g.v[0] - g.v[2], g.v[1] - g.v[2]);
  const double j = sqrt(dot(cr, cr));
  g.c = (1.0 / 3.0) * (g.v[0] + g.v[1] + g.v[2]);
  g.n = (1.0 / j) * cr;
  g.area = 0.5 * j;
  return g;
}

// RT shape j of `parent` on its child `ch`: sum_k Q[j][k] (child shape k), Q[j][k] the flux of
// shape j through the child's edge k (an RT shape has unit outward flux through its own edge):
// |e_k| (m_k - v_j).n_k / (2 A), n_k the edge's outward unit normal, m_k a point of the edge
// (the RT interpolation of src/bases/local/rtlocal.jl:82-111)
DEV void rt_restriction(const Geo& parent, const Geo& ch, double Q[3][3]) {
  for (int k = 0; k < 3; ++k) {
    const V3<double> a = ch.v[(k + 1) % 3], b = ch.v[(k + 2) % 3];
    V3<double> nk = cross(b - a, ch.n);
    nk = (1.0 / sqrt(dot(nk, nk))) * nk;
    if (dot(ch.v[k] - a, nk) > 0) nk = -1.0 * nk;
    const double len = sqrt(dot(b - a, b - a));
    for (int j = 0; j < 3; ++j) Q[j][k] = len * dot(a - parent.v[j], nk) / (2.0 * parent.area);
  }
}

// one near pair, by one warp (lane = its lane); s_glx / s_glw: the Gauss-Legendre table in
// shared memory (lanes read different nodes: a constant-memory read would serialise)
DEV void near_pair(const NearParams& P, const NearPair np_, const double* s_glx, const double* s_glw, int lane) {
  if (near_is_ss32(P, np_.cls) || near_is_ssdf(P, np_.cls)) return;  // k_near_ss32 / k_near_ss_df
  const Geo t = load_geo(P.tgeo + (int64_t)P.tperm[np_.p] * GEO_STRIDE);
  const Geo s = load_geo(P.bgeo + (int64_t)(P.qcells ? P.qcells[np_.q] : np_.q) * GEO_STRIDE);
  const int nt = P.tk == BEAST_P0 ? 1 : 3, nb = P.bk == BEAST_P0 ? 1 : 3;
  C2<double> acc[9];
  for (int k = 0; k < 9; ++k) acc[k] = C2<double>{0, 0};
  const bool dl_face = np_.cls == 3 && dl_type(P.op.kind);
  if (np_.cls >= 5) return;  // k_near_refines
  if (np_.cls == 4) {
    // ---- DoubleNumQStrat pair close to its partner: the pair's own DoubleQuadRule
    // (src/quadrature/doublenumints.jl:12-43) point by point in FP64, lanes over point pairs.
    // Double-layer type kernels vanish identically on a common face (every vector of the
    // triple product lies in the flat triangle): that block stays 0 rather than summed noise.
    const bool dl_kind = dl_type(P.op.kind) || P.op.kind == BEAST_MW_NXDL;
    int hits = 0;
    if (dl_kind)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const V3<double> dd = t.v[i] - s.v[j];
          hits += sqrt(dot(dd, dd)) < 1.0e3 * 2.220446049250313e-16;
        }
    if (!(dl_kind && hits == 3)) dq_points(P, P.op.kind, t, s, P.ro, P.ri, lane, acc);
  } else if (np_.cls >= 1 && !dl_face) {
    int pt[3], ps[3];
    ss_order(t, s, pt, ps);
    const int n = np_.cls == 3 ? P.qs.ss_face : (np_.cls == 2 ? P.qs.ss_edge : P.qs.ss_vert);
    const int nreg = np_.cls == 1 ? 2 : 6;
    const int64_t items = (int64_t)nreg * n * n * n * n;
    const double* glx = s_glx + c_gl_off[n - 1];
    const double* glw = s_glw + c_gl_off[n - 1];
    const bool mw_rt = P.tk == BEAST_RT && P.bk == BEAST_RT &&
                       (P.op.kind == BEAST_MW_SL || P.op.kind == BEAST_MW_DL);
    if (mw_rt) {
      // moment form: with xi = x - c_p, eta = y - c_q and W = node weight x kernel,
      //  single layer: z_ij = alpha (Mxe - s_j.Mx - t_i.Me + (t_i.s_j) M0) + 4 beta M0
      //  double layer: z_ij = D0 - s_j.Dxr - t_i.Dre + (s_j x t_i).Dr
      // (t_i = v_i - c_p, s_j = w_j - c_q; the shape normalisations cancel the Jacobian)
      const bool sl = P.op.kind == BEAST_MW_SL;
      const V3<double> cp = t.c, cq = s.c;
      const double gi = P.op.gi, gr = P.op.gr;
      // m[0..1] M0, m[2..3] M1 (SL) ; m[4..9] V1, m[10..15] V2, m[16..21] V3 as (re, im) per axis
      double m[22];
#pragma unroll
      for (int k = 0; k < 22; ++k) m[k] = 0.0;
      const V3<double> d = cp - cq;
      for (int64_t it = lane; it < items; it += 32) {
        double X[2], Y[2], w;
        ss_node(np_.cls, n, it, glx, glw, X, Y, &w);
        const double lt[3] = {1.0 - X[0], X[0] - X[1], X[1]}, ls[3] = {1.0 - Y[0], Y[0] - Y[1], Y[1]};
        const V3<double> xi = lt[0] * (t.v[pt[0]] - cp) + lt[1] * (t.v[pt[1]] - cp) + lt[2] * (t.v[pt[2]] - cp);
        const V3<double> eta = ls[0] * (s.v[ps[0]] - cq) + ls[1] * (s.v[ps[1]] - cq) + ls[2] * (s.v[ps[2]] - cq);
        const V3<double> r = (d + xi) - eta;
        const double R2 = dot(r, r);
        const double iR = rsqrt(R2);
        const double R = R2 * iR;
        double sn, cs;
        sincos(gi * R, &sn, &cs);
        const double amp = (gr == 0.0 ? 1.0 : exp(-gr * R)) * I4PI * iR * w;
        double cr = amp * cs, ci = -amp * sn;  // w e^{-gamma R} / (4 pi R)
        V3<double> a, b, c3;
        double s0;
        if (sl) {
          s0 = dot(xi, eta);
          a = xi;
          b = eta;
          c3 = V3<double>{0, 0, 0};
          m[0] += cr;
          m[1] += ci;
        } else {
          // grad G = c r with c = -(gamma + 1/R) G / R
          const double pr = -(gr + iR) * iR, pi = -gi * iR;
          const double nr = pr * cr - pi * ci, ni = pr * ci + pi * cr;
          cr = nr;
          ci = ni;
          s0 = dot(xi, cross(d, eta));  // xi.(r x eta) = xi.(d x eta)
          a = cross(xi, r);
          b = cross(r, eta);
          c3 = r;
        }
        m[2] += s0 * cr; m[3] += s0 * ci;
        m[4] += a.x * cr; m[5] += a.x * ci; m[6] += a.y * cr; m[7] += a.y * ci; m[8] += a.z * cr; m[9] += a.z * ci;
        m[10] += b.x * cr; m[11] += b.x * ci; m[12] += b.y * cr; m[13] += b.y * ci; m[14] += b.z * cr; m[15] += b.z * ci;
        m[16] += c3.x * cr; m[17] += c3.x * ci; m[18] += c3.y * cr; m[19] += c3.y * ci; m[20] += c3.z * cr; m[21] += c3.z * ci;
      }
#pragma unroll
      for (int k = 0; k < 22; ++k) {
        double v = m[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        m[k] = v;
      }
      const C2<double> M0{m[0], m[1]}, M1{m[2], m[3]};
      CV<double> V1, V2, V3_;
      V1.x = {m[4], m[5]}; V1.y = {m[6], m[7]}; V1.z = {m[8], m[9]};
      V2.x = {m[10], m[11]}; V2.y = {m[12], m[13]}; V2.z = {m[14], m[15]};
      V3_.x = {m[16], m[17]}; V3_.y = {m[18], m[19]}; V3_.z = {m[20], m[21]};
      if (lane == 0) {
        const C2<double> al{P.op.ar, P.op.ai}, be{P.op.br, P.op.bi};
        for (int i = 0; i < 3; ++i) {
          const V3<double> ti = t.v[i] - cp;
          for (int j = 0; j < 3; ++j) {
            const V3<double> sj = s.v[j] - cq;
            C2<double> z;
            if (sl) {
              C2<double> fm = csub(csub(M1, rdot(sj, V1)), rdot(ti, V2));
              fm = cadd(fm, cscale(dot(ti, sj), M0));
              z = cadd(cmul(al, fm), cscale(4.0, cmul(be, M0)));
            } else {
              C2<double> fm = csub(csub(M1, rdot(sj, V1)), rdot(ti, V2));
              z = cadd(fm, rdot(cross(sj, ti), V3_));
            }
            store_c<double>(P.zcell, zidx(zrow_of(P.zrow, np_.p, 3, i), zcol_of(P.zcol, np_.q, 3, j), P.ldc), z, P.zfmt);
          }
        }
      }
      return;
    }
    ss_points(P, t, s, np_.cls, pt, ps, s_glx, s_glw, lane, acc);
  } else if (np_.cls == -1) {
    se_points(P, t, s, lane, acc);
  }
  // ---- warp reduction and store
  for (int k = 0; k < nt * nb; ++k) {
    double re = acc[k].re, im = acc[k].im;
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    acc[k] = C2<double>{re, im};
  }
  if (lane == 0) {
    for (int i = 0; i < nt; ++i)
      for (int j = 0; j < nb; ++j)
        store_c<double>(P.zcell, zidx(zrow_of(P.zrow, np_.p, nt, i), zcol_of(P.zcol, np_.q, nb, j), P.ldc),
                        acc[i * nb + j], P.zfmt);
  }
}

__global__ void __launch_bounds__(32 * NEAR_WARPS) k_near(NearParams P) {
  __shared__ double s_glx[210], s_glw[210];
  for (int k = threadIdx.x; k < 210; k += blockDim.x) {
    s_glx[k] = c_gl_x[k];
    s_glw[k] = c_gl_w[k];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * (int64_t)NEAR_WARPS + warp;
  if (e >= P.nnear) return;
  near_pair(P, P.near[e], s_glx, s_glw, lane);
}

// the pairs of the refines strategies (classes 5 and 6), one per warp: a kernel of their own
// so that the children loop does not set k_near's register budget
__global__ void __launch_bounds__(32 * NEAR_WARPS) k_near_refines(NearParams P) {
  __shared__ double s_glx[210], s_glw[210];
  for (int k = threadIdx.x; k < 210; k += blockDim.x) {
    s_glx[k] = c_gl_x[k];
    s_glw[k] = c_gl_w[k];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * (int64_t)NEAR_WARPS + warp;
  if (e >= P.nnear) return;
  const NearPair np_ = P.near[e];
  if (np_.cls < 5) return;
  const Geo t = load_geo(P.tgeo + (int64_t)P.tperm[np_.p] * GEO_STRIDE);
  const Geo s = load_geo(P.bgeo + (int64_t)(P.qcells ? P.qcells[np_.q] : np_.q) * GEO_STRIDE);
  C2<double> acc[9];
  for (int k = 0; k < 9; ++k) acc[k] = C2<double>{0, 0};
  // ---- the refines strategies (src/quadrature/rules/testrefinestrialqrule.jl:6-52,
  // trialrefinestestqrule.jl:6-40): the pair shares a vertex, so the coarse cell (trial for
  // class 5, test for class 6) is split into its children, each child integrated against the
  // other cell with the wrapped strategy (its own class), the coarse RT shapes restricted to
  // the child.  The restriction is linear, so it applies to each lane's share.
  const bool split_trial = np_.cls == 5;
  const Geo& parent = split_trial ? s : t;
  const int nchild = split_trial ? P.bnchild : P.tnchild;
  const double* ch = split_trial
                         ? P.bchildren + (int64_t)P.bcells[P.qcells ? P.qcells[np_.q] : np_.q] * nchild * 9
                         : P.tchildren + (int64_t)P.tcells[P.tperm[np_.p]] * nchild * 9;
  const double k2 = P.op.gr * P.op.gr + P.op.gi * P.op.gi;
  for (int c = 0; c < nchild; ++c) {
    const Geo g = geo_of_triangle(ch + 9 * c);
    const Geo& tt = split_trial ? t : g;
    const Geo& ss = split_trial ? g : s;
    C2<double> B[9];
    for (int k = 0; k < 9; ++k) B[k] = C2<double>{0, 0};
    pair_points(P, tt, ss, classify_exact(tt, ss, BEAST_QS_WILTON_SAUTER, k2), s_glx, s_glw, lane, B);
    double Q[3][3];
    rt_restriction(parent, g, Q);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k)
          acc[i * 3 + j] = cadd(acc[i * 3 + j], split_trial ? cscale(Q[j][k], B[i * 3 + k])
                                                            : cscale(Q[i][k], B[k * 3 + j]));
  }
  for (int k = 0; k < 9; ++k) {
    double re = acc[k].re, im = acc[k].im;
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    acc[k] = C2<double>{re, im};
  }
  if (lane == 0)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        store_c<double>(P.zcell, zidx(zrow_of(P.zrow, np_.p, 3, i), zcol_of(P.zcol, np_.q, 3, j), P.ldc),
                        acc[i * 3 + j], P.zfmt);
}

// ------------------------------------------------------------------------------------
// gather: Z[m, n] = sum_{(p,r,a) of m} sum_{(q,s,b) of n} a b Zcell[nst p + r, nsb q' + s]
// ------------------------------------------------------------------------------------
// A thread owns one test function m and a run of GATHER_NCOL consecutive trial functions: its
// test entries (Zcell row, coefficient) are loaded once into registers, the trial entries are
// warp-uniform loads, and each output is a sum of (#test x #trial) products.  With a complex
// FP32 Zcell and output (the mixed path) the sums are FP32; otherwise FP64.
constexpr int GATHER_NCOL = 16, GATHER_MAXE = 8;
template <int ZC64, int OC64>
__global__ void __launch_bounds__(256) k_gather(GatherArgs G, const int64_t* tptr, const int* tcell,
                                                const int* tshape, const double* tcoef,
                                                const int64_t* bptr, const int* bcell, const int* bshape,
                                                const double* bcoef, int nst, int nsb, int64_t nrows) {
  typedef typename std::conditional<ZC64 && OC64, float, double>::type A;
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nb0 = G.n0 + (int64_t)blockIdx.y * GATHER_NCOL;
  const int64_t nb1 = nb0 + GATHER_NCOL < G.n1 ? nb0 + GATHER_NCOL : G.n1;
  // the CTA's trial functions with at most two entries: Zcell column offsets and coefficients
  // staged once in shared memory (s_cnt = -1: more entries, taken by the general loop)
  // (both for c64 -> c64, with FP32 sums, and c128 -> c128, with FP64 sums)
  constexpr bool FAST = ZC64 == OC64;
  typedef typename std::conditional<ZC64, float2, double2>::type Z2;
  constexpr int GRP = ZC64 ? 8 : 4;  // trial functions whose Zcell values are requested together
  __shared__ int64_t s_col[GATHER_NCOL][2];
  __shared__ A s_b[GATHER_NCOL][2];
  __shared__ int s_cnt[GATHER_NCOL];
  if (FAST && threadIdx.x < GATHER_NCOL) {
    const int64_t n = nb0 + threadIdx.x;
    int cnt = 0;
    if (n < nb1) {
      const int64_t f0 = bptr[n];
      const int c = (int)(bptr[n + 1] - f0);
      cnt = c <= 2 ? c : -1;
      for (int k = 0; k < 2 && k < c; ++k) {
        s_col[threadIdx.x][k] = ((int64_t)nsb * G.qlocal[bcell[f0 + k]] + bshape[f0 + k]) * G.ldc;
        s_b[threadIdx.x][k] = (A)bcoef[f0 + k];
      }
    }
    s_cnt[threadIdx.x] = cnt;
  }
  if (FAST) __syncthreads();
  if (m >= nrows) return;
  const int64_t e0 = tptr[m], ne = tptr[m + 1] - e0;
  int64_t trow[GATHER_MAXE];
  A tc[GATHER_MAXE];
#pragma unroll
  for (int j = 0; j < GATHER_MAXE; ++j) {
    trow[j] = 0;
    tc[j] = 0;
    if (j < ne) {
      trow[j] = (int64_t)nst * G.tpos[tcell[e0 + j]] + tshape[e0 + j];
      tc[j] = (A)tcoef[e0 + j];
    }
  }
  int64_t nstart = nb0;
  if (FAST && ne <= 2) {
    // fast path: the Zcell values of GRP trial functions (<= 2 x 2 each) are requested before
    // any is used
    bool all2 = true;
    for (int nn = 0; nn < nb1 - nb0; ++nn) all2 &= s_cnt[nn] >= 0;
    if (all2) {
      const Z2* zc = reinterpret_cast<const Z2*>(G.zcell);
      for (int g0 = 0; g0 < (int)(nb1 - nb0); g0 += GRP) {
        Z2 z[GRP][2][2];
#pragma unroll
        for (int u = 0; u < GRP; ++u)
#pragma unroll
          for (int k = 0; k < 2; ++k)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int nn = g0 + u;
              const bool ok = nn < nb1 - nb0 && k < s_cnt[nn] && j < ne;
              Z2 v;
              v.x = 0;
              v.y = 0;
              z[u][k][j] = ok ? zc[s_col[nn][k] + trow[j]] : v;
            }
#pragma unroll
        for (int u = 0; u < GRP; ++u) {
          const int nn = g0 + u;
          if (nn >= nb1 - nb0) break;
          A re = 0, im = 0;
#pragma unroll
          for (int k = 0; k < 2; ++k)
#pragma unroll
            for (int j = 0; j < 2; ++j)
              if (k < s_cnt[nn] && j < ne) {
                const A ab = tc[j] * s_b[nn][k];
                re += ab * z[u][k][j].x;
                im += ab * z[u][k][j].y;
              }
          const A cr = (A)G.cr, ci = (A)G.ci;
          A vr = cr * re - ci * im, vi = cr * im + ci * re;
          Z2* Z = reinterpret_cast<Z2*>(G.Z);
          const int64_t o = (G.row_off + m) + (G.col_off + nb0 + nn) * G.ldz;
          if (G.accumulate) {
            const Z2 old = Z[o];
            vr += old.x;
            vi += old.y;
          }
          Z2 out;
          out.x = vr;
          out.y = vi;
          Z[o] = out;
        }
      }
      nstart = nb1;
    }
  }
  for (int64_t n = nstart; n < nb1; ++n) {
    A re = 0, im = 0;
    for (int64_t f = bptr[n]; f < bptr[n + 1]; ++f) {
      const int ql = G.qlocal[bcell[f]];
      const int64_t col = ((int64_t)nsb * ql + bshape[f]) * G.ldc;
      const A b = (A)bcoef[f];
      if (ne <= GATHER_MAXE) {
#pragma unroll
        for (int j = 0; j < GATHER_MAXE; ++j) {
          if (j < ne) {
            const A ab = tc[j] * b;
            if (ZC64) {
              const float2 z = reinterpret_cast<const float2*>(G.zcell)[col + trow[j]];
              re += ab * (A)z.x;
              im += ab * (A)z.y;
            } else {
              const double2 z = reinterpret_cast<const double2*>(G.zcell)[col + trow[j]];
              re += ab * (A)z.x;
              im += ab * (A)z.y;
            }
          }
        }
      } else {
        for (int64_t e = e0; e < e0 + ne; ++e) {
          const A ab = (A)tcoef[e] * b;
          const int64_t idx = col + (int64_t)nst * G.tpos[tcell[e]] + tshape[e];
          if (ZC64) {
            const float2 z = reinterpret_cast<const float2*>(G.zcell)[idx];
            re += ab * (A)z.x;
            im += ab * (A)z.y;
          } else {
            const double2 z = reinterpret_cast<const double2*>(G.zcell)[idx];
            re += ab * (A)z.x;
            im += ab * (A)z.y;
          }
        }
      }
    }
    const A cr = (A)G.cr, ci = (A)G.ci;
    A vr = cr * re - ci * im, vi = cr * im + ci * re;
    const int64_t o = (G.row_off + m) + (G.col_off + n) * G.ldz;
    if (OC64) {
      float2* Z = reinterpret_cast<float2*>(G.Z);
      if (G.accumulate) {
        const float2 old = Z[o];
        vr += (A)old.x;
        vi += (A)old.y;
      }
      Z[o] = make_float2((float)vr, (float)vi);
    } else {
      double2* Z = reinterpret_cast<double2*>(G.Z);
      if (G.accumulate) {
        const double2 old = Z[o];
        vr += (A)old.x;
        vi += (A)old.y;
      }
      Z[o] = make_double2((double)vr, (double)vi);
    }
  }
}

// The same gather from double-float cell-pair blocks (ZCELL_DF, the mixed-accurate path): the
// sums run on the FP32 pipes as sloppy pair sums, coefficients enter as pairs from the
// integer split, and the result reaches the c128 output through exact integer float-to-double
// conversions and one FP64 addition per real part (or rounds to c64).  The far entries of RT
// functions cancel by about (h/R)^2 in these sums; the pair sums keep about 2^-44 of the
// largest term, below the cell-pair values' own error.
__device__ __forceinline__ dfl::df df_coef(double c) {
  float h, l;
  fsplit::split_f64(c, &h, &l);
  return dfl::fast_two_sum(h, l);
}
// one term c z of a double-float gather sum (running sums, as k_gather_e): UC, c = +-1
template <int UC>
__device__ __forceinline__ void df_term(dfl::df& re, dfl::df& im, float4 z, dfl::df c) {
  if (UC) {
    dfl::acc(re, dfl::df{c.hi * z.x, c.hi * z.y});
    dfl::acc(im, dfl::df{c.hi * z.z, c.hi * z.w});
  } else {
    dfl::acc(re, dfl::mul(dfl::df{z.x, z.y}, c));
    dfl::acc(im, dfl::mul(dfl::df{z.z, z.w}, c));
  }
}
template <int OC64, int UC>
__global__ void __launch_bounds__(256) k_gather_df(GatherArgs G, const int64_t* tptr, const int* tcell,
                                                   const int* tshape, const double* tcoef, const int64_t* bptr,
                                                   const int* bcell, const int* bshape, const double* bcoef, int nst,
                                                   int nsb, int64_t nrows) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nb0 = G.n0 + (int64_t)blockIdx.y * GATHER_NCOL;
  const int64_t nb1 = nb0 + GATHER_NCOL < G.n1 ? nb0 + GATHER_NCOL : G.n1;
  __shared__ int64_t s_col[GATHER_NCOL][2];
  __shared__ dfl::df s_b[GATHER_NCOL][2];
  __shared__ int s_cnt[GATHER_NCOL];
  if (threadIdx.x < GATHER_NCOL) {
    const int64_t n = nb0 + threadIdx.x;
    int cnt = 0;
    if (n < nb1) {
      const int64_t f0 = bptr[n];
      const int c = (int)(bptr[n + 1] - f0);
      cnt = c <= 2 ? c : -1;
      for (int k = 0; k < 2 && k < c; ++k) {
        s_col[threadIdx.x][k] = ((int64_t)nsb * G.qlocal[bcell[f0 + k]] + bshape[f0 + k]) * G.ldc;
        s_b[threadIdx.x][k] = df_coef(bcoef[f0 + k]);
      }
    }
    s_cnt[threadIdx.x] = cnt;
  }
  __syncthreads();
  if (m >= nrows) return;
  const int64_t e0 = tptr[m], ne = tptr[m + 1] - e0;
  const float4* zc = reinterpret_cast<const float4*>(G.zcell);
  const bool unit = G.cr == 1.0 && G.ci == 0.0;
  auto finish = [&](int64_t n, dfl::df re, dfl::df im) {
    const int64_t o = (G.row_off + m) + (G.col_off + n) * G.ldz;
    if (OC64) {
      float vr = dfl::add_rn(re.hi, re.lo), vi = dfl::add_rn(im.hi, im.lo);
      if (!unit) {
        const float cr = (float)G.cr, ci = (float)G.ci;
        const float tr = cr * vr - ci * vi;
        vi = cr * vi + ci * vr;
        vr = tr;
      }
      float2* Z = reinterpret_cast<float2*>(G.Z);
      if (G.accumulate) {
        const float2 old = Z[o];
        vr += old.x;
        vi += old.y;
      }
      Z[o] = make_float2(vr, vi);
    } else {
      double vr = fsplit::f2d(re.hi) + fsplit::f2d(re.lo), vi = fsplit::f2d(im.hi) + fsplit::f2d(im.lo);
      if (!unit) {
        const double tr = G.cr * vr - G.ci * vi;
        vi = G.cr * vi + G.ci * vr;
        vr = tr;
      }
      double2* Z = reinterpret_cast<double2*>(G.Z);
      if (G.accumulate) {
        const double2 old = Z[o];
        vr += old.x;
        vi += old.y;
      }
      Z[o] = make_double2(vr, vi);
    }
  };
  const dfl::df z0 = dfl::make(0.f);
  int64_t nstart = nb0;
  if (ne <= 2) {
    bool all2 = true;
    for (int nn = 0; nn < nb1 - nb0; ++nn) all2 &= s_cnt[nn] >= 0;
    if (all2) {
      int64_t trow[2] = {0, 0};
      dfl::df tc[2] = {z0, z0};
      for (int j = 0; j < ne; ++j) {
        trow[j] = (int64_t)nst * G.tpos[tcell[e0 + j]] + tshape[e0 + j];
        tc[j] = df_coef(tcoef[e0 + j]);
      }
      // the Zcell values of four trial functions (<= 2 x 2 each) are requested before any is used
      for (int g0 = 0; g0 < (int)(nb1 - nb0); g0 += 4) {
        float4 z[4][2][2];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int k = 0; k < 2; ++k)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int nn = g0 + u;
              const bool ok = nn < nb1 - nb0 && k < s_cnt[nn] && j < ne;
              z[u][k][j] = ok ? zc[s_col[nn][k] + trow[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int nn = g0 + u;
          if (nn >= nb1 - nb0) break;
          dfl::df re = z0, im = z0;
#pragma unroll
          for (int k = 0; k < 2; ++k)
#pragma unroll
            for (int j = 0; j < 2; ++j)
              if (k < s_cnt[nn] && j < ne) df_term<UC>(re, im, z[u][k][j], dfl::mul(tc[j], s_b[nn][k]));
          finish(nb0 + nn, dfl::norm(re), dfl::norm(im));
        }
      }
      nstart = nb1;
    }
  }
  for (int64_t n = nstart; n < nb1; ++n) {
    dfl::df re = z0, im = z0;
    for (int64_t f = bptr[n]; f < bptr[n + 1]; ++f) {
      const int64_t col = ((int64_t)nsb * G.qlocal[bcell[f]] + bshape[f]) * G.ldc;
      const dfl::df b = df_coef(bcoef[f]);
      for (int64_t e = e0; e < e0 + ne; ++e)
        df_term<UC>(re, im, zc[col + (int64_t)nst * G.tpos[tcell[e]] + tshape[e]], dfl::mul(df_coef(tcoef[e]), b));
    }
    finish(n, dfl::norm(re), dfl::norm(im));
  }
}

// Gather from cell-pair blocks laid out by function entries (the entry layout of AsmArgs):
//   Z[m, n] = sum over the entries e of m and f of n of c_e c_f Zcell[(f - f0) ldc + e].
// A thread owns a test function m and GATHER_NCOL consecutive trial functions.  The entries of
// a function are consecutive rows (columns), so for functions with the same number of entries
// (RT: two) the rows a warp reads in one column are one contiguous run: every Zcell byte is
// read once, in full sectors.  Sums in FP32 for c64 -> c64, in pairs of floats (sloppy sums,
// as k_gather_df) for double-float blocks, else in FP64.
constexpr int GATHER_E_MAX = 4;  // entries per function handled from registers
// UC (double-float blocks only): every coefficient is +1 or -1, so a term is the block value
// with a sign and the sums need no pair products.
template <int ZC, int OC64, int UC = 0>
__global__ void __launch_bounds__(256) k_gather_e(GatherArgs G, const int64_t* tptr, const double* tcoef,
                                                  const int64_t* bptr, const double* bcoef, int64_t nrows) {
  typedef typename std::conditional<ZC == ZCELL_C64 && OC64, float, double>::type A;
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nb0 = G.n0 + (int64_t)blockIdx.y * GATHER_NCOL;
  const int64_t nb1 = nb0 + GATHER_NCOL < G.n1 ? nb0 + GATHER_NCOL : G.n1;
  __shared__ int64_t s_c0[GATHER_NCOL];  // first Zcell column (element offset) of trial function n
  __shared__ int s_nc[GATHER_NCOL];
  __shared__ double s_b[GATHER_NCOL][GATHER_E_MAX];
  __shared__ dfl::df s_bd[GATHER_NCOL][GATHER_E_MAX];  // the same as pairs (double-float blocks)
  if (threadIdx.x < GATHER_NCOL) {
    const int64_t n = nb0 + threadIdx.x;
    if (n < nb1) {
      const int64_t f0 = bptr[n];
      const int c = (int)(bptr[n + 1] - f0);
      s_c0[threadIdx.x] = (f0 - G.f0) * G.ldc;
      s_nc[threadIdx.x] = c;
      for (int k = 0; k < GATHER_E_MAX; ++k) {
        s_b[threadIdx.x][k] = k < c ? bcoef[f0 + k] : 0.0;
        if (ZC == ZCELL_DF) s_bd[threadIdx.x][k] = df_coef(s_b[threadIdx.x][k]);
      }
    }
  }
  __syncthreads();
  if (m >= nrows) return;
  const int64_t e0 = tptr[m];
  const int ne = (int)(tptr[m + 1] - e0);
  dfl::df tcd[GATHER_E_MAX];  // the test coefficients as pairs, split once per thread
  if (ZC == ZCELL_DF)
    for (int e = 0; e < GATHER_E_MAX; ++e) tcd[e] = e < ne ? df_coef(tcoef[e0 + e]) : dfl::make(0.f);
  const bool unit = G.cr == 1.0 && G.ci == 0.0;
  auto out = [&](int64_t n, double vr, double vi) {
    if (!unit) {
      const double tr = G.cr * vr - G.ci * vi;
      vi = G.cr * vi + G.ci * vr;
      vr = tr;
    }
    const int64_t o = (G.row_off + m) + (G.col_off + n) * G.ldz;
    if (OC64) {
      float2* Z = reinterpret_cast<float2*>(G.Z);
      float r = (float)vr, i = (float)vi;
      if (G.accumulate) {
        const float2 old = Z[o];
        r += old.x;
        i += old.y;
      }
      Z[o] = make_float2(r, i);
    } else {
      double2* Z = reinterpret_cast<double2*>(G.Z);
      if (G.accumulate) {
        const double2 old = Z[o];
        vr += old.x;
        vi += old.y;
      }
      Z[o] = make_double2(vr, vi);
    }
  };
  for (int64_t n = nb0; n < nb1; ++n) {
    const int nn = (int)(n - nb0);
    const int nc = s_nc[nn];
    const int64_t c0 = s_c0[nn] + e0;
    if (ZC == ZCELL_DF) {
      const float4* zc = reinterpret_cast<const float4*>(G.zcell);
      dfl::df re = dfl::make(0.f), im = dfl::make(0.f);
      for (int f = 0; f < nc; ++f) {
        if (UC) {
          const float sb = f < GATHER_E_MAX ? s_bd[nn][f].hi : fsplit::to_float_rn(bcoef[bptr[n] + f]);
          for (int e = 0; e < ne; ++e) {
            const float sg = sb * (e < GATHER_E_MAX ? tcd[e].hi : fsplit::to_float_rn(tcoef[e0 + e]));
            df_term<1>(re, im, zc[c0 + (int64_t)f * G.ldc + e], dfl::make(sg));
          }
        } else {
          const dfl::df b = f < GATHER_E_MAX ? s_bd[nn][f] : df_coef(bcoef[bptr[n] + f]);
          for (int e = 0; e < ne; ++e) {
            df_term<0>(re, im, zc[c0 + (int64_t)f * G.ldc + e],
                       dfl::mul(e < GATHER_E_MAX ? tcd[e] : df_coef(tcoef[e0 + e]), b));
          }
        }
      }
      re = dfl::norm(re);
      im = dfl::norm(im);
      if (OC64) {
        out(n, (double)dfl::add_rn(re.hi, re.lo), (double)dfl::add_rn(im.hi, im.lo));
      } else {
        // exact float -> double by integer operations, one FP64 addition per part
        const double vr = fsplit::f2d(re.hi) + fsplit::f2d(re.lo), vi = fsplit::f2d(im.hi) + fsplit::f2d(im.lo);
        if (unit && !G.accumulate) {
          reinterpret_cast<double2*>(G.Z)[(G.row_off + m) + (G.col_off + n) * G.ldz] = make_double2(vr, vi);
        } else {
          out(n, vr, vi);
        }
      }
    } else {
      typedef typename std::conditional<ZC == ZCELL_C64, float2, double2>::type Z2;
      const Z2* zc = reinterpret_cast<const Z2*>(G.zcell);
      A re = 0, im = 0;
      for (int f = 0; f < nc; ++f) {
        const A b = (A)(f < GATHER_E_MAX ? s_b[nn][f] : bcoef[bptr[n] + f]);
        for (int e = 0; e < ne; ++e) {
          const Z2 z = zc[c0 + (int64_t)f * G.ldc + e];
          const A ab = (A)tcoef[e0 + e] * b;
          re += ab * (A)z.x;
          im += ab * (A)z.y;
        }
      }
      out(n, (double)re, (double)im);
    }
  }
}

// ------------------------------------------------------------------------------------
// local operators (Identity / NCross on RT x RT), deterministic per test dof
// ------------------------------------------------------------------------------------
constexpr int LOCAL_MAXCOLS = 64;

__global__ void k_local(int which, const int64_t* tptr, const int* tcell, const int* tshape,
                        const double* tcoef, const int* tcells_mesh, const double* tgeo,
                        const int* b_cell2act, const int* bad_dof, const double* bad_coef,
                        int bmaxfn, TriRuleDev r, int64_t nrows, void* Z, int64_t ldz, int zc64,
                        int64_t row_off, int64_t col_off, double cr, double ci, int* flag) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= nrows) return;
  // the distinct trial functions of this row (a Buffa-Christiansen row meets about 25 coarse
  // RT functions written on the refinement; an RT row at most 5)
  int cols[LOCAL_MAXCOLS];
  double vals[LOCAL_MAXCOLS];
  int nc = 0;
  for (int64_t e = tptr[m]; e < tptr[m + 1]; ++e) {
    int pa = tcell[e], ra = tshape[e];
    double a = tcoef[e];
    int qb = b_cell2act[tcells_mesh[pa]];
    if (qb < 0) continue;
    Geo g = load_geo(tgeo + (int64_t)pa * GEO_STRIDE);
    double gram[3] = {0, 0, 0};
    for (int k = 0; k < r.n; ++k) {
      double bx[3] = {r.u[k], r.v[k], 1.0 - r.u[k] - r.v[k]};
      V3<double> x = bx[0] * g.v[0] + bx[1] * g.v[1] + bx[2] * g.v[2];
      double w = r.w[k] * g.area;
      Shp f;
      shapes(BEAST_RT, g, x, bx, f);
      for (int j = 0; j < 3; ++j)
        gram[j] += w * (which == 0 ? dot(f.v[ra], f.v[j]) : dot(f.v[ra], cross(g.n, f.v[j])));
    }
    for (int j = 0; j < 3; ++j)
      for (int kb = 0; kb < bmaxfn; ++kb) {
        int n = bad_dof[((int64_t)qb * 3 + j) * bmaxfn + kb];
        if (n < 0) continue;
        double v = a * gram[j] * bad_coef[((int64_t)qb * 3 + j) * bmaxfn + kb];
        int slot = -1;
        for (int s = 0; s < nc; ++s)
          if (cols[s] == n) slot = s;
        if (slot < 0) {
          if (nc == LOCAL_MAXCOLS) {  // more distinct columns than the buffer holds: reported
            atomicOr(flag, 16);
            continue;
          }
          slot = nc++;
          cols[slot] = n;
          vals[slot] = 0;
        }
        vals[slot] += v;
      }
  }
  for (int s = 0; s < nc; ++s) {
    int64_t o = (row_off + m) + (col_off + cols[s]) * ldz;
    if (zc64) {
      float2* z = reinterpret_cast<float2*>(Z);
      float2 old = z[o];
      z[o] = make_float2((float)(old.x + cr * vals[s]), (float)(old.y + ci * vals[s]));
    } else {
      double2* z = reinterpret_cast<double2*>(Z);
      double2 old = z[o];
      z[o] = make_double2(old.x + cr * vals[s], old.y + ci * vals[s]);
    }
  }
}

// ------------------------------------------------------------------------------------
// excitation: b[m] = sum_{(p,r,a) of m} a * int f_r . F  (deterministic per dof)
// ------------------------------------------------------------------------------------
__global__ void k_rhs(int kind, int tk, const int64_t* tptr, const int* tcell, const int* tshape,
                      const double* tcoef, const double* tgeo, double dx, double dy, double dz,
                      double px, double py, double pz, double gr, double gi, double ar, double ai,
                      TriRuleDev r, int64_t nrows, double* b) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= nrows) return;
  V3<double> d = mk(dx, dy, dz), u = mk(px, py, pz);
  C2<double> gam{gr, gi}, amp{ar, ai};
  C2<double> pref{1.0, 0.0};
  V3<double> fu = u;
  if (kind == BEAST_EXC_CROSSTRACE_H) {
    // H = -1/(i k) curl E, curl E = -gamma (d x u) E0 ; with k = -i gamma: H = (d x u) E0 gamma/(i k)
    C2<double> k{gi, -gr};                 // k = -i gamma
    C2<double> ik{-k.im, k.re};            // i k
    double den = ik.re * ik.re + ik.im * ik.im;
    pref = C2<double>{(gam.re * ik.re + gam.im * ik.im) / den, (gam.im * ik.re - gam.re * ik.im) / den};
    fu = cross(d, u);
  }
  double re = 0, im = 0;
  for (int64_t e = tptr[m]; e < tptr[m + 1]; ++e) {
    int pa = tcell[e], ra = tshape[e];
    double a = tcoef[e];
    Geo g = load_geo(tgeo + (int64_t)pa * GEO_STRIDE);
    for (int k = 0; k < r.n; ++k) {
      double bx[3] = {r.u[k], r.v[k], 1.0 - r.u[k] - r.v[k]};
      V3<double> x = bx[0] * g.v[0] + bx[1] * g.v[1] + bx[2] * g.v[2];
      double w = r.w[k] * g.area;
      C2<double> ph = cmul(amp, cexp_d(C2<double>{-(gr * dot(d, x)), -(gi * dot(d, x))}));
      double val;
      if (kind == BEAST_EXC_HH_DIRICHLET) {
        val = tk == BEAST_P0 ? 1.0 : bx[ra];
      } else {
        Shp f;
        shapes(BEAST_RT, g, x, bx, f);
        if (kind == BEAST_EXC_TANGTRACE_E)
          val = dot(f.v[ra], cross(cross(g.n, fu), g.n));
        else
          val = dot(f.v[ra], cross(g.n, fu));
      }
      C2<double> t = cscale(w * val * a, cmul(pref, ph));
      re += t.re;
      im += t.im;
    }
  }
  b[2 * m] = re;
  b[2 * m + 1] = im;
}

// ------------------------------------------------------------------------------------
// far field (src/postproc.jl:174-211, 273-288; src/maxwell/farfield.jl:60-63)
// ------------------------------------------------------------------------------------
__global__ void k_farfield(const double* geo, const int* ad_dof, const double* ad_coef, int maxfn,
                           int64_t ncells, const double* u, const double* pts, double gr,
                           double gi, TriRuleDev r, double* ff) {
  const int p = blockIdx.x;
  V3<double> yh = mk(pts[3 * p], pts[3 * p + 1], pts[3 * p + 2]);
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t c = threadIdx.x; c < ncells; c += blockDim.x) {
    Geo g = load_geo(geo + c * GEO_STRIDE);
    for (int k = 0; k < r.n; ++k) {
      double bx[3] = {r.u[k], r.v[k], 1.0 - r.u[k] - r.v[k]};
      V3<double> x = bx[0] * g.v[0] + bx[1] * g.v[1] + bx[2] * g.v[2];
      double w = r.w[k] * g.area;
      double ph = dot(yh, x);
      C2<double> krn = cexp_d(C2<double>{gr * ph, gi * ph});  // exp(gamma yhat.x)
      Shp f;
      shapes(BEAST_RT, g, x, bx, f);
      for (int i = 0; i < 3; ++i) {
        C2<double> cu{0, 0};
        for (int kk = 0; kk < maxfn; ++kk) {
          int mdof = ad_dof[(c * 3 + i) * maxfn + kk];
          if (mdof < 0) continue;
          double a = ad_coef[(c * 3 + i) * maxfn + kk];
          cu = cadd(cu, cscale(a, C2<double>{u[2 * mdof], u[2 * mdof + 1]}));
        }
        C2<double> s = cscale(w, cmul(krn, cu));
        V3<double> tr = cross(cross(yh, f.v[i]), yh);
        acc[0] += s.re * tr.x; acc[1] += s.im * tr.x;
        acc[2] += s.re * tr.y; acc[3] += s.im * tr.y;
        acc[4] += s.re * tr.z; acc[5] += s.im * tr.z;
      }
    }
  }
  __shared__ double red[6][256];
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) ff[6 * p + k] = red[k][0];
}

}  // namespace

#include "rules_gen.h"

bool make_trirule(int degree, TriRuleDev* r) {
  if (degree < 1 || degree > BEAST_TRI_MAXDEG) return false;
  int off = beast_tri_off[degree], cnt = beast_tri_cnt[degree];
  r->n = cnt;
  for (int i = 0; i < cnt; ++i) {
    r->u[i] = beast_tri_pts[off + i][0];
    r->v[i] = beast_tri_pts[off + i][1];
    r->w[i] = beast_tri_pts[off + i][2];
  }
  return true;
}

cudaError_t launch_geometry(const beast_space* s, cudaStream_t st) {
  if (s->ncells == 0) return cudaSuccess;
  int th = 256;
  int64_t bl = (s->ncells + th - 1) / th;
  k_geometry<<<(unsigned)bl, th, 0, st>>>(s->mesh->verts, s->mesh->cells, s->cells, s->ncells,
                                           s->geo, s->geof);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// batched far pairs: many meshes in one persistent launch (Helmholtz operators, P0 spaces)
// ------------------------------------------------------------------------------------
// The grid walks a tile list (job, first test position, first trial cell), tile t on CTA
// t mod gridDim.x: a CTA stages tile_q trial cells of the tile's job in shared memory and
// each of its tile_m threads takes one test cell against them, as k_far does for one mesh.
// P0 functions have one cell each, so every cell-pair value is a matrix entry and goes
// straight to the job's matrix (row zrow[position], column zcol[trial cell]).  Near pairs go
// to one list for the whole batch (k_near_batch).
template <int OPK, typename R, int FMT>
__global__ void k_far_batch(BatchLaunch L) {
  extern __shared__ unsigned char smraw[];
  R* sm = reinterpret_cast<R*>(smraw);
  const int ni = L.ri.n, no = L.ro.n;
  const int rec = 8 + 4 * ni;  // per trial cell: centroid hi (3) lo (3), area, near radius; points
  int* s_col = reinterpret_cast<int*>(sm + (size_t)L.tile_q * rec);
  __shared__ R ro_s[3 * RULE_MAXPTS];
  for (int k = threadIdx.x; k < no; k += blockDim.x) {
    ro_s[3 * k] = (R)L.ro.u[k];
    ro_s[3 * k + 1] = (R)L.ro.v[k];
    ro_s[3 * k + 2] = (R)L.ro.w[k];
  }
  for (int t = blockIdx.x; t < L.ntiles; t += gridDim.x) {
    const BatchTile tile = L.tiles[t];
    const BatchJobDev J = L.jobs[tile.job];
    const int nqt = (int)min((int64_t)L.tile_q, J.ncells - tile.q0);
    __syncthreads();  // the previous tile's records are no longer read
    for (int k = threadIdx.x; k < nqt * (1 + ni); k += blockDim.x) {
      const int qi = k / (1 + ni), b = k % (1 + ni);
      const int qc = tile.q0 + qi;
      const double* g = J.geo + (int64_t)qc * GEO_STRIDE;
      R* r = sm + qi * rec;
      const double cx = g[9], cy = g[10], cz = g[11];
      if (b == 0) {
        r[0] = (R)cx; r[1] = (R)cy; r[2] = (R)cz;
        r[3] = (R)(cx - (double)(R)cx); r[4] = (R)(cy - (double)(R)cy); r[5] = (R)(cz - (double)(R)cz);
        r[6] = (R)g[15];
        const double thr2 = near_threshold2(L.qs_kind, J.k2, g[15]);
        r[7] = (R)((double)J.geof[4 * qc + 3] + sqrt(fmax(thr2, 0.0)));
        s_col[qi] = J.zcol[qc];
      } else {
        const int bb = b - 1;
        const double u = L.ri.u[bb], v = L.ri.v[bb], w = 1.0 - u - v;
        R* pt = r + 8 + 4 * bb;
        pt[0] = (R)(u * (g[0] - cx) + v * (g[3] - cx) + w * (g[6] - cx));
        pt[1] = (R)(u * (g[1] - cy) + v * (g[4] - cy) + w * (g[7] - cy));
        pt[2] = (R)(u * (g[2] - cz) + v * (g[5] - cz) + w * (g[8] - cz));
        pt[3] = (R)L.ri.w[bb];
      }
    }
    __syncthreads();
    const int64_t pp = tile.p0 + threadIdx.x;
    if (pp >= J.ncells || threadIdx.x >= L.tile_m) continue;
    const int64_t p = J.tperm[pp];
    const double* tg = J.geo + p * GEO_STRIDE;
    const double cpx = tg[9], cpy = tg[10], cpz = tg[11];
    const V3<R> chp = mk((R)cpx, (R)cpy, (R)cpz);
    const V3<R> clp = mk((R)(cpx - (double)(R)cpx), (R)(cpy - (double)(R)cpy), (R)(cpz - (double)(R)cpz));
    V3<R> tau[3];
    for (int i = 0; i < 3; ++i)
      tau[i] = mk((R)(tg[3 * i] - cpx), (R)(tg[3 * i + 1] - cpy), (R)(tg[3 * i + 2] - cpz));
    const V3<R> nn = mk((R)tg[12], (R)tg[13], (R)tg[14]);
    const R ApR = (R)tg[15];
    const R radp = (R)J.geof[4 * p + 3];
    const R gr = (R)J.op.gr, gi = (R)J.op.gi;
    const C2<R> al{(R)J.op.ar, (R)J.op.ai};
    const int64_t zr = J.zrow[pp];
    for (int qi = 0; qi < nqt; ++qi) {
      const R* rq = sm + qi * rec;
      const V3<R> d = mk((chp.x - rq[0]) + (clp.x - rq[3]), (chp.y - rq[1]) + (clp.y - rq[4]),
                         (chp.z - rq[2]) + (clp.z - rq[5]));
      const int64_t o = zidx(zr, s_col[qi], J.ldz);
      const R lim = radp + rq[7];
      if (dot(d, d) <= lim * lim * (R)1.0001 + (R)1e-30) {
        int cls = 4;
        if (L.qs_kind != BEAST_QS_DOUBLENUM) {
          Geo ta = load_geo(tg);
          Geo sb = load_geo(J.geo + (int64_t)(tile.q0 + qi) * GEO_STRIDE);
          cls = classify_exact(ta, sb, L.qs_kind, J.k2);
        }
        if (cls != 0) {
          const int idx = atomicAdd(L.near_count, 1);
          if (idx < L.near_cap)
            L.near[idx] = NearPairB{tile.job, (int)pp, tile.q0 + qi, cls};
          else
            atomicOr(L.flag, 1);
          continue;  // k_near_batch writes the entry
        }
      }
      const R* pts = rq + 8;
      const V3<R> nq = mk((R)0, (R)0, (R)0);  // trial normal: only the double layer needs it
      C2<R> acc{0, 0};
      for (int a = 0; a < no; ++a) {
        const R ua = ro_s[3 * a], va = ro_s[3 * a + 1], wa3 = (R)1 - ua - va;
        const V3<R> xi = mk(ua * tau[0].x + va * tau[1].x + wa3 * tau[2].x,
                            ua * tau[0].y + va * tau[1].y + wa3 * tau[2].y,
                            ua * tau[0].z + va * tau[1].z + wa3 * tau[2].z);
        const R wa = ro_s[3 * a + 2];
        const V3<R> dx = d + xi;
        for (int b = 0; b < ni; ++b) {
          const R* pb = pts + 4 * b;
          const V3<R> r = dx - mk(pb[0], pb[1], pb[2]);
          const R R2 = dot(r, r);
          const R iR = rsq<R>(R2);
          const C2<R> G = green<R>(gr, gi, R2 * iR, iR);
          C2<R> K;
          if (OPK == BEAST_HH_SL) {
            K = cmul(al, G);
          } else {  // transposed double layer: n_x . grad G (the double layer takes the trial
                    // normal from the geometry below)
            const C2<R> c = cmul(al, cscale(iR, cmul(C2<R>{-(gr + iR), -gi}, G)));
            K = cscale(dot(nn, r), c);
          }
          acc = cadd(acc, cscale(pb[3] * wa, K));
        }
      }
      (void)nq;
      store_c<R>(J.Z, o, cscale(ApR * rq[6], acc), FMT);
    }
  }
}

// near pairs of a batch: one warp per pair, pairs dealt over the warps of a fixed grid
// (the list length is read on the device, so the launch needs no host round trip)
__global__ void __launch_bounds__(32 * NEAR_WARPS) k_near_batch(BatchLaunch L) {
  __shared__ double s_glx[210], s_glw[210];
  for (int k = threadIdx.x; k < 210; k += blockDim.x) {
    s_glx[k] = c_gl_x[k];
    s_glw[k] = c_gl_w[k];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = min(*L.near_count, L.near_cap);
  for (int64_t e = blockIdx.x * (int64_t)NEAR_WARPS + warp; e < n; e += (int64_t)gridDim.x * NEAR_WARPS) {
    const NearPairB nb = L.near[e];
    const BatchJobDev J = L.jobs[nb.job];
    NearParams P;
    P.op = J.op;
    P.qs = L.qs;
    P.tk = BEAST_P0;
    P.bk = BEAST_P0;
    P.tperm = J.tperm;
    P.tgeo = J.geo;
    P.bgeo = J.geo;
    P.qcells = nullptr;
    P.near = nullptr;
    P.nnear = 0;
    P.zcell = J.Z;
    P.zfmt = L.zfmt;
    P.ss32 = 0;
    P.ldc = J.ldz;
    P.zrow = J.zrow;
    P.zcol = J.zcol;
    P.flag = L.flag;
    P.ro = L.ron;
    P.ri = L.rin;
    P.ssdf = L.ssdf && J.op.gr == 0.0;  // those pairs run in k_near_batch_df
    P.bcells = P.tcells = nullptr;  // no refines strategies in a batch
    P.bchildren = P.tchildren = nullptr;
    P.bnchild = P.tnchild = 0;
    near_pair(P, NearPair{nb.p, nb.q, nb.cls, 0}, s_glx, s_glw, lane);
  }
}

template <int OPK, int TK, int BK, typename R, int FMT>
static cudaError_t far_t(const FarParams& P, cudaStream_t st) {
  dim3 grid((unsigned)((P.np + FAR_THREADS - 1) / FAR_THREADS), (unsigned)((P.nq + FAR_QT - 1) / FAR_QT));
  size_t sm = (size_t)FAR_QT * (QREC_HDR + 4 * P.ri.n) * sizeof(R);
  k_far<OPK, TK, BK, R, FMT><<<grid, FAR_THREADS, sm, st>>>(P);
  return cudaGetLastError();
}

template <int OPK, int TK, int BK>
static cudaError_t far_prec(const FarParams& P, int precision, int fmt, cudaStream_t st) {
  if (precision == BEAST_MIXED) return far_t<OPK, TK, BK, float, ZCELL_C64>(P, st);
  if (fmt == ZCELL_C64) return far_t<OPK, TK, BK, double, ZCELL_C64>(P, st);
  if (fmt == ZCELL_DF) return far_t<OPK, TK, BK, double, ZCELL_DF>(P, st);
  return far_t<OPK, TK, BK, double, ZCELL_C128>(P, st);
}

// ---- EFIE far pairs in double-float arithmetic (FP64-quality values on the FP32 pipes) -------
// Same pair loop, near filter and Zcell layout (c128) as k_far<MW_SL, RT, RT, double, 0>; the
// block of a far pair comes from dfl::efie_far_pair (far_df.h) on pair-split geometry.
struct FarDfRecord {
  dfl::df sig[3][3];  // trial vertices minus centroid
  dfl::df c[3];       // trial centroid
  float lim;          // near-test radius (radius + threshold distance)
  float pad;
  dfl::df eta[RULE_MAXPTS][3];  // inner rule points minus centroid
  dfl::df w[RULE_MAXPTS];       // inner rule weights
  dfl::df eta2[RULE_MAXPTS];    // |eta_b|^2
};

DEV dfl::df df_of(double x) {
  float h, l;
  fsplit::split_f64(x, &h, &l);
  return dfl::fast_two_sum(h, l);
}

// The EFIE far pairs of the mixed-accurate path: k_far's tiling (one test cell per thread,
// FAR_QT trial cells staged in shared memory), every operation on FP32 pairs (dfloat.h), the
// cell-pair blocks stored as double-float pairs (ZCELL_DF).  NO x NI > 0: the rule sizes known
// at compile time (the default 3 x 4 far rules; efie_far_pair_fast), else the general core.
// BETA: the balanced core (efie_far_pair_beta: Green's function values and the beta term of
// the pair in double-float, the alpha terms in FP32; BEAST_MIXED_BALANCED)
// (five CTAs per SM for the cores of the default rule sizes: 96 registers, no spills)
template <int NO, int NI, bool BETA = false>
__global__ void __launch_bounds__(FAR_THREADS, NO > 0 ? 5 : 1) k_far_efie_df(FarParams P) {
  __shared__ FarDfRecord rec[FAR_QT];
  __shared__ float s_tab[64][4];  // sin / cos(m pi/32): lanes read different entries
  __shared__ int s_zc[FAR_QT][3];
  constexpr int NOW = NO > 0 ? NO : 1, NIW = NI > 0 ? NI : 1;
  __shared__ dfl::df s_wab[NOW][NIW];  // w_a w_b / (4 pi) of the fast core
  for (int k = threadIdx.x; k < 256; k += blockDim.x) s_tab[k >> 2][k & 3] = dfl::sincos_tab_dev[k >> 2][k & 3];
  if constexpr (NO > 0) {
    if (threadIdx.x == 0) {
      dfl::df w1[NOW], w2[NIW];
      for (int a = 0; a < NO; ++a) w1[a] = df_of(P.ro.w[a]);
      for (int b = 0; b < NI; ++b) w2[b] = df_of(P.ri.w[b]);
      dfl::efie_far_weights<NOW, NIW>(w1, w2, s_wab);
    }
  }
  const int ni = P.ri.n, no = P.ro.n;
  const int q0 = blockIdx.y * FAR_QT;
  const int nqt = min(FAR_QT, P.nq - q0);
  for (int k = threadIdx.x; k < nqt * (1 + ni); k += blockDim.x) {
    const int qi = k / (1 + ni), b = k % (1 + ni);
    const int qc = P.qcells[q0 + qi];
    const double* g = P.bgeo + (int64_t)qc * GEO_STRIDE;
    FarDfRecord& r = rec[qi];
    const double cx = g[9], cy = g[10], cz = g[11];
    if (b == 0) {
      for (int j = 0; j < 3; ++j) {
        r.sig[j][0] = df_of(g[3 * j] - cx);
        r.sig[j][1] = df_of(g[3 * j + 1] - cy);
        r.sig[j][2] = df_of(g[3 * j + 2] - cz);
      }
      r.c[0] = df_of(cx);
      r.c[1] = df_of(cy);
      r.c[2] = df_of(cz);
      const double thr2 = near_threshold2(P.qs_kind, P.k2, g[15]);
      r.lim = (float)((double)P.bgeof[4 * qc + 3] + sqrt(fmax(thr2, 0.0)));
    } else {
      const int bb = b - 1;
      const double u = P.ri.u[bb], v = P.ri.v[bb], w = 1.0 - u - v;
      r.eta[bb][0] = df_of(u * (g[0] - cx) + v * (g[3] - cx) + w * (g[6] - cx));
      r.eta[bb][1] = df_of(u * (g[1] - cy) + v * (g[4] - cy) + w * (g[7] - cy));
      r.eta[bb][2] = df_of(u * (g[2] - cz) + v * (g[5] - cz) + w * (g[8] - cz));
      r.w[bb] = df_of(P.ri.w[bb]);
      r.eta2[bb] = dfl::dot3s(r.eta[bb], r.eta[bb]);
    }
  }
  for (int k = threadIdx.x; k < nqt * 3; k += blockDim.x) s_zc[k / 3][k % 3] = (int)zcol_of(P.zcol, q0 + k / 3, 3, k % 3);
  __syncthreads();
  const int64_t pp = blockIdx.x * (int64_t)FAR_THREADS + threadIdx.x;
  if (pp >= P.np) return;
  const int64_t p = P.tperm[pp];
  int64_t zr[3];
  for (int i = 0; i < 3; ++i) zr[i] = zrow_of(P.zrow, pp, 3, i);
  const double* tg = P.tgeo + p * GEO_STRIDE;
  const double cpx = tg[9], cpy = tg[10], cpz = tg[11];
  const dfl::df cp[3] = {df_of(cpx), df_of(cpy), df_of(cpz)};
  constexpr int NOA = NO > 0 ? NO : RULE_MAXPTS;
  dfl::df tau[3][3], xi[NOA][3], wo[NOA];
  for (int i = 0; i < 3; ++i) {
    tau[i][0] = df_of(tg[3 * i] - cpx);
    tau[i][1] = df_of(tg[3 * i + 1] - cpy);
    tau[i][2] = df_of(tg[3 * i + 2] - cpz);
  }
#pragma unroll
  for (int a = 0; a < NOA; ++a) {
    if (NO == 0 && a >= no) break;
    const double u = P.ro.u[a], v = P.ro.v[a], w = 1.0 - u - v;
    xi[a][0] = df_of(u * (tg[0] - cpx) + v * (tg[3] - cpx) + w * (tg[6] - cpx));
    xi[a][1] = df_of(u * (tg[1] - cpy) + v * (tg[4] - cpy) + w * (tg[7] - cpy));
    xi[a][2] = df_of(u * (tg[2] - cpz) + v * (tg[5] - cpz) + w * (tg[8] - cpz));
    wo[a] = df_of(P.ro.w[a]);
  }
  const float radp = P.tgeof[4 * p + 3];
  const dfl::df kk = df_of(P.op.gi);
  const dfl::cdf alpha{df_of(P.op.ar), df_of(P.op.ai)}, beta{df_of(P.op.br), df_of(P.op.bi)};
  float4* zc = reinterpret_cast<float4*>(P.zcell);
  for (int qi = 0; qi < nqt; ++qi) {
    const FarDfRecord& r = rec[qi];
    const int ql = q0 + qi;
    // far pairs: |c_p - c_q| is at least a cell size, so the sloppy difference (error 2^-44 of the
    // coordinates) keeps the pair's distance to about 1e-11 relative
    const dfl::df d[3] = {dfl::subs(cp[0], r.c[0]), dfl::subs(cp[1], r.c[1]), dfl::subs(cp[2], r.c[2])};
    if (P.qs_kind != BEAST_QS_DOUBLENUM) {
      const float lim = radp + r.lim;
      const float dd = d[0].hi * d[0].hi + d[1].hi * d[1].hi + d[2].hi * d[2].hi;
      if (dd <= lim * lim * 1.0001f + 1e-30f) {
        Geo t = load_geo(tg);
        Geo s = load_geo(P.bgeo + (int64_t)P.qcells[ql] * GEO_STRIDE);
        const int cls = refines_class(classify_exact(t, s, P.qs_kind, P.k2), P.qs_kind);
        if (cls != 0) {
          const int idx = atomicAdd(P.near_count, 1);
          if (idx < P.near_cap)
            P.near[idx] = NearPair{(int)pp, ql, cls, 0};
          else
            atomicOr(P.flag, 1);
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
              const int64_t o = zidx(zr[i], s_zc[qi][j], P.ldc);
              if (o >= 0) zc[o] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
          continue;
        }
      }
    }
    dfl::cdf z[9];
    if constexpr (NO > 0 && BETA)
      dfl::efie_far_pair_beta<NO, NI>(d, tau, r.sig, xi, s_wab, r.eta, r.eta2, kk, alpha, beta, s_tab, z);
    else if constexpr (NO > 0)
      dfl::efie_far_pair_fast<NO, NI>(d, tau, r.sig, xi, s_wab, r.eta, r.eta2, kk, alpha, beta, s_tab, z);
    else
      dfl::efie_far_pair(d, tau, r.sig, no, xi, wo, ni, r.eta, r.w, kk, alpha, beta, z);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const dfl::cdf& v = z[3 * i + j];
        const int64_t o = zidx(zr[i], s_zc[qi][j], P.ldc);
        if (o >= 0) zc[o] = make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo);
      }
  }
}

// balanced: the balanced core for the default rule sizes (3 x 4 points); other rule sizes run
// the general double-float core in both modes
static cudaError_t far_efie_df(const FarParams& P, bool balanced, cudaStream_t st) {
  dim3 grid((unsigned)((P.np + FAR_THREADS - 1) / FAR_THREADS), (unsigned)((P.nq + FAR_QT - 1) / FAR_QT));
  if (P.ro.n == 3 && P.ri.n == 4 && balanced)
    k_far_efie_df<3, 4, true><<<grid, FAR_THREADS, 0, st>>>(P);
  else if (P.ro.n == 3 && P.ri.n == 4)
    k_far_efie_df<3, 4><<<grid, FAR_THREADS, 0, st>>>(P);
  else
    k_far_efie_df<0, 0><<<grid, FAR_THREADS, 0, st>>>(P);
  return cudaGetLastError();
}

template <int OPK>
static cudaError_t far_hh(const FarParams& P, int tk, int bk, int precision, int fmt, cudaStream_t st) {
  if (tk == BEAST_P0 && bk == BEAST_P0) return far_prec<OPK, BEAST_P0, BEAST_P0>(P, precision, fmt, st);
  if (tk == BEAST_P0 && bk == BEAST_P1) return far_prec<OPK, BEAST_P0, BEAST_P1>(P, precision, fmt, st);
  if (tk == BEAST_P1 && bk == BEAST_P0) return far_prec<OPK, BEAST_P1, BEAST_P0>(P, precision, fmt, st);
  if (tk == BEAST_P1 && bk == BEAST_P1) return far_prec<OPK, BEAST_P1, BEAST_P1>(P, precision, fmt, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_far(const AsmArgs& a, const TriRuleDev& ro, const TriRuleDev& ri, cudaStream_t st) {
  FarParams P;
  P.op = a.op;
  P.qs_kind = a.qs.kind;
  P.k2 = a.op.gr * a.op.gr + a.op.gi * a.op.gi;
  P.tgeo = a.ts->geo;
  P.tgeof = a.ts->geof;
  P.np = a.ts->ncells;
  P.tperm = a.ts->tperm;
  P.bgeo = a.bs->geo;
  P.bgeof = a.bs->geof;
  P.qcells = a.qcells;
  P.nq = a.nq;
  P.zcell = a.zcell;
  P.ldc = a.ldc;
  P.zrow = a.zrow;
  P.zcol = a.zcol;
  P.near = a.near;
  P.near_cap = a.near_cap;
  P.near_count = a.near_count;
  P.flag = a.flag;
  P.ro = ro;
  P.ri = ri;
  if (P.np == 0 || P.nq == 0) return cudaSuccess;
  const int tk = a.ts->kind, bk = a.bs->kind;
  const int kind = a.op.kind;
  if (kind == BEAST_MW_SL || kind == BEAST_MW_DL || kind == BEAST_MW_NXDL) {
    if (tk != BEAST_RT || bk != BEAST_RT) return cudaErrorInvalidValue;
    const bool balanced = a.precision == BEAST_MIXED_BALANCED;
    if (kind == BEAST_MW_SL && (a.precision == BEAST_MIXED_ACCURATE || balanced) && a.zcell_fmt == ZCELL_DF &&
        P.op.gr == 0.0) {
      // mixed-accurate EFIE assemblies (real wavenumber): far pairs in double-float arithmetic
      // on the FP32 pipes (about 1e-12 relative to the FP64 values, at a fraction of the FP64
      // kernel's time on GB300); BEAST_FAR_DF=0 selects the FP64 kernel instead.  Balanced:
      // the alpha terms in FP32 (about 1e-7 of a block's largest entry)
      const char* e = getenv("BEAST_FAR_DF");
      if (!(e && e[0] == '0')) return far_efie_df(P, balanced, st);
    }
    if (kind == BEAST_MW_SL) return far_prec<BEAST_MW_SL, BEAST_RT, BEAST_RT>(P, a.precision, a.zcell_fmt, st);
    if (kind == BEAST_MW_DL) return far_prec<BEAST_MW_DL, BEAST_RT, BEAST_RT>(P, a.precision, a.zcell_fmt, st);
    return far_prec<BEAST_MW_NXDL, BEAST_RT, BEAST_RT>(P, a.precision, a.zcell_fmt, st);
  }
  if (kind == BEAST_HH_SL) return far_hh<BEAST_HH_SL>(P, tk, bk, a.precision, a.zcell_fmt, st);
  if (kind == BEAST_HH_DL) return far_hh<BEAST_HH_DL>(P, tk, bk, a.precision, a.zcell_fmt, st);
  if (kind == BEAST_HH_DLT) return far_hh<BEAST_HH_DLT>(P, tk, bk, a.precision, a.zcell_fmt, st);
  return cudaErrorInvalidValue;
}

static cudaError_t upload_gl(cudaStream_t st) {
  static bool done[64] = {false};
  static std::mutex mtx;
  std::lock_guard<std::mutex> lk(mtx);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (done[dev]) return cudaSuccess;
  double x[210], w[210];
  for (int i = 0; i < 210; ++i) {
    x[i] = beast_gl_pts[i][0];
    w[i] = beast_gl_pts[i][1];
  }
  cudaError_t e = cudaMemcpyToSymbol(c_gl_x, x, sizeof(x));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gl_w, w, sizeof(w));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gl_off, beast_gl_off, sizeof(int) * 21);
  if (e == cudaSuccess) done[dev] = true;
  (void)st;
  return e;
}

cudaError_t launch_far_batch(const BatchLaunch& L, cudaStream_t st) {
  if (L.ntiles == 0) return cudaSuccess;
  const size_t sm_f = (size_t)L.tile_q * (8 + 4 * L.ri.n) * sizeof(float) + sizeof(int) * L.tile_q;
  const size_t sm_d = (size_t)L.tile_q * (8 + 4 * L.ri.n) * sizeof(double) + sizeof(int) * L.tile_q;
  const int th = ((L.tile_m + 31) / 32) * 32;
  const bool f32 = L.precision == BEAST_MIXED;
  if (L.op_kind == BEAST_HH_SL) {
    if (f32) k_far_batch<BEAST_HH_SL, float, ZCELL_C64><<<L.grid_far, th, sm_f, st>>>(L);
    else k_far_batch<BEAST_HH_SL, double, ZCELL_C128><<<L.grid_far, th, sm_d, st>>>(L);
  } else if (L.op_kind == BEAST_HH_DLT) {
    if (f32) k_far_batch<BEAST_HH_DLT, float, ZCELL_C64><<<L.grid_far, th, sm_f, st>>>(L);
    else k_far_batch<BEAST_HH_DLT, double, ZCELL_C128><<<L.grid_far, th, sm_d, st>>>(L);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t upload_tables(cudaStream_t st) { return upload_gl(st); }

__global__ void __launch_bounds__(32 * NEAR_WARPS) k_near_batch_df(BatchLaunch L);  // below

cudaError_t launch_near_batch(const BatchLaunch& L, cudaStream_t st) {
  // the Gauss-Legendre table is uploaded before (upload_tables): this launch may be captured
  k_near_batch<<<L.grid_near, 32 * NEAR_WARPS, 0, st>>>(L);
  if (L.ssdf) k_near_batch_df<<<L.grid_near, 32 * NEAR_WARPS, 0, st>>>(L);
  return cudaGetLastError();
}

// ---- Sauter-Schwab pairs in double-float arithmetic (mixed-accurate path)
// The node table of class cls and order n: for node `it` of the pair's rule (ss_node's order),
// tab[k * items + it] = (hi, lo) of X0, X1, Y0, Y1, D0, D1, w (k = 0..6), built once in FP64.
constexpr int SSDF_VALS = 7;
__global__ void k_ss_table(int cls, int n, int items, float2* tab) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= items) return;
  double X[2], Y[2], D[2], w;
  ss_node_fd(cls, n, it, c_gl_x + c_gl_off[n - 1], c_gl_w + c_gl_off[n - 1], X, Y, D, &w);
  const double v[SSDF_VALS] = {X[0], X[1], Y[0], Y[1], D[0], D[1], w};
  for (int k = 0; k < SSDF_VALS; ++k) {
    const dfl::df p = df_of(v[k]);
    tab[(int64_t)k * items + it] = make_float2(p.hi, p.lo);
  }
}

// the table of (cls, n) from the context's cache, built on first use (after upload_gl)
static cudaError_t ss_table(std::map<int, void*>* cache, int cls, int n, cudaStream_t st, const float2** out,
                            int* items) {
  const int nreg = cls == 1 ? 2 : 6;
  *items = nreg * n * n * n * n;
  const int key = 64 * cls + n;
  auto f = cache->find(key);
  if (f != cache->end()) {
    *out = (const float2*)f->second;
    return cudaSuccess;
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, sizeof(float2) * SSDF_VALS * (size_t)*items);
  if (e != cudaSuccess) return e;
  k_ss_table<<<(*items + 255) / 256, 256, 0, st>>>(cls, n, *items, (float2*)p);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFree(p);
    return e;
  }
  (*cache)[key] = p;
  *out = (const float2*)p;
  return cudaSuccess;
}

cudaError_t ss_tables(std::map<int, void*>* cache, const beast_qs_desc& qs, cudaStream_t st, const float2** tab,
                      int* items) {
  cudaError_t e = upload_gl(st);
  if (e != cudaSuccess) return e;
  const int ord[4] = {0, qs.ss_vert, qs.ss_edge, qs.ss_face};
  tab[0] = nullptr;
  items[0] = 0;
  for (int c = 1; c <= 3; ++c) {
    e = ss_table(cache, c, ord[c], st, &tab[c], &items[c]);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

DEV void dfv3(const V3<double>& a, dfl::df* o) {
  o[0] = df_of(a.x);
  o[1] = df_of(a.y);
  o[2] = df_of(a.z);
}

// The moment form of k_near's Sauter-Schwab path for RT x RT Maxwell pairs, every node in
// double-float arithmetic on the FP32 pipes (GB300's FP64 pipe is a small fraction of its FP32
// rate): one warp per pair, lanes over the nodes, x - y from the maps' own factors (D = X - Y)
// on double-float edge vectors, 1/R by the pair reciprocal square root, exp(-ikR) from the
// shared-memory sine table; per-lane moments as running pair sums, the warp's totals as exact
// pair sums, the 3 x 3 block from them in FP64 (nine lanes).  Real wavenumbers (the caller
// keeps complex ones on k_near).
// shared vertices of a touching pair first, in the same order (SauterSchwabQuadrature.reorder):
// lanes 0..8 test one vertex pair each (shared vertices coincide exactly), the first three
// hits in (i, j) order from the ballot
DEV void ss_order_warp(const Geo& t, const Geo& s, int lane, int* pt, int* ps) {
  const double dtol = 1.0e3 * 2.220446049250313e-16;
  bool hit = false;
  if (lane < 9) {
    const V3<double> dd = t.v[lane / 3] - s.v[lane % 3];
    hit = dot(dd, dd) < dtol * dtol;
  }
  const unsigned hmask = __ballot_sync(0xffffffffu, hit);
  int hits = 0, ti[3], si[3];
  for (int b = 0; b < 9; ++b)
    if (((hmask >> b) & 1u) && hits < 3) {
      ti[hits] = b / 3;
      si[hits] = b % 3;
      ++hits;
    }
  int k = 0;
  for (int h = 0; h < hits; ++h) pt[k++] = ti[h];
  for (int i = 0; i < 3; ++i) {
    bool used = false;
    for (int h = 0; h < hits; ++h) used |= ti[h] == i;
    if (!used) pt[k++] = i;
  }
  k = 0;
  for (int h = 0; h < hits; ++h) ps[k++] = si[h];
  for (int j = 0; j < 3; ++j) {
    bool used = false;
    for (int h = 0; h < hits; ++h) used |= si[h] == j;
    if (!used) ps[k++] = j;
  }
}

// the warp's total of a double-float value (exact pair sums over the butterfly), as FP64
DEV double warp_total_df(dfl::df x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const dfl::df y{__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)};
    x = dfl::add(x, y);
  }
  return fsplit::f2d(x.hi) + fsplit::f2d(x.lo);
}

// The Helmholtz single layer alpha G on a touching pair of P0 / P1 cells by the Sauter-Schwab
// rule of class cls, every node in double-float arithmetic (real wavenumber kk): lanes over the
// nodes, per shape pair (a, b) of the reordered vertices the moment sum_k w_k G_k lt_a ls_b
// (P0: one moment, shape value 1), the warp's totals in FP64 on every lane.  z[i * nb + j]:
// the block in the cells' own vertex order (alpha and the Jacobian 4 A_t A_s included).
// (Here and in k_near_ss_df every product inside the node loop feeds a pair sum, a running
// sum or another product, so all of them are the unnormalised dfl::mulu.)
template <int TP1, int BP1>
DEV void hh_sl_ss_df(const OpParams& op, const Geo& t, const Geo& s, int cls, const float2* tab, int items,
                     const float (*s_tab)[4], int lane, C2<double>* z) {
  constexpr int NT = TP1 ? 3 : 1, NB = BP1 ? 3 : 1;
  int pt[3], ps[3];
  ss_order_warp(t, s, lane, pt, ps);
  dfl::df et1[3], et2[3], es1[3], es2[3];
  dfv3(t.v[pt[1]] - t.v[pt[0]], et1);
  dfv3(t.v[pt[2]] - t.v[pt[1]], et2);
  dfv3(s.v[ps[1]] - s.v[ps[0]], es1);
  dfv3(s.v[ps[2]] - s.v[ps[1]], es2);
  const dfl::df kk = df_of(op.gi);
  const dfl::df i4pi{DF_I4PI_HI, DF_I4PI_LO};
  const dfl::df one = dfl::make(1.f);
  dfl::df m[NT * NB][2];
#pragma unroll
  for (int q = 0; q < NT * NB; ++q) m[q][0] = m[q][1] = dfl::make(0.f);
  for (int it = lane; it < items; it += 32) {
    dfl::df v[SSDF_VALS];
#pragma unroll
    for (int q = 0; q < SSDF_VALS; ++q) {
      const float2 f = tab[(int64_t)q * items + it];
      v[q] = dfl::df{f.x, f.y};
    }
    const dfl::df X0 = v[0], X1 = v[1], Y0 = v[2], Y1 = v[3], D0 = v[4], D1 = v[5], w = v[6];
    dfl::df r[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (cls == 3)
        r[c] = dfl::adds(dfl::mulu(D0, et1[c]), dfl::mulu(D1, et2[c]));
      else if (cls == 2)
        r[c] = dfl::adds(dfl::mulu(D0, et1[c]), dfl::subs(dfl::mulu(X1, et2[c]), dfl::mulu(Y1, es2[c])));
      else
        r[c] = dfl::subs(dfl::adds(dfl::mulu(X0, et1[c]), dfl::mulu(X1, et2[c])),
                         dfl::adds(dfl::mulu(Y0, es1[c]), dfl::mulu(Y1, es2[c])));
    }
    const dfl::df R2 = dfl::dot3u(r, r);
    const dfl::df iR = dfl::rsqrt(R2);
    const dfl::df R = dfl::mulu(R2, iR);
    dfl::df sn, cs;
    dfl::sincos_tab(dfl::mulu(kk, R), s_tab, &sn, &cs);
    const dfl::df amp = dfl::mulu(dfl::mulu(iR, w), i4pi);  // w / (4 pi R)
    const dfl::df cr = dfl::mulu(amp, cs), ci = dfl::neg(dfl::mulu(amp, sn));
    // shape values at the node in the reordered vertex order: lt = (1 - X0, X0 - X1, X1)
    const dfl::df lt[3] = {dfl::sub(one, X0), dfl::sub(X0, X1), X1};
    const dfl::df ls[3] = {dfl::sub(one, Y0), dfl::sub(Y0, Y1), Y1};
#pragma unroll
    for (int a = 0; a < NT; ++a)
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        dfl::df f = TP1 ? lt[a] : one;
        if (BP1) f = BP1 && TP1 ? dfl::mulu(f, ls[b]) : ls[b];
        dfl::acc(m[a * NB + b][0], TP1 || BP1 ? dfl::mulu(f, cr) : cr);
        dfl::acc(m[a * NB + b][1], TP1 || BP1 ? dfl::mulu(f, ci) : ci);
      }
  }
  const C2<double> al{op.ar, op.ai};
  const double jac = 4.0 * t.area * s.area;
#pragma unroll
  for (int a = 0; a < NT; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const C2<double> M{warp_total_df(dfl::norm(m[a * NB + b][0])), warp_total_df(dfl::norm(m[a * NB + b][1]))};
      const int i = TP1 ? pt[a] : 0, j = BP1 ? ps[b] : 0;
      z[i * NB + j] = cscale(jac, cmul(al, M));
    }
}

// the Helmholtz single layer's Sauter-Schwab pairs (P0 / P1) of one assembly in double-float
// (near_is_ssdf), one warp per pair
template <int TP1, int BP1>
__global__ void __launch_bounds__(32 * NEAR_WARPS) k_near_hh_df(NearParams P) {
  __shared__ float s_tab[64][4];
  for (int k = threadIdx.x; k < 256; k += blockDim.x) s_tab[k >> 2][k & 3] = dfl::sincos_tab_dev[k >> 2][k & 3];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * (int64_t)NEAR_WARPS + warp;
  if (e >= P.nnear) return;
  const NearPair np_ = P.near[e];
  if (!near_is_ssdf(P, np_.cls)) return;
  const Geo t = load_geo(P.tgeo + (int64_t)P.tperm[np_.p] * GEO_STRIDE);
  const Geo s = load_geo(P.bgeo + (int64_t)P.qcells[np_.q] * GEO_STRIDE);
  constexpr int NT = TP1 ? 3 : 1, NB = BP1 ? 3 : 1;
  C2<double> z[NT * NB];
  hh_sl_ss_df<TP1, BP1>(P.op, t, s, np_.cls, P.ssdf_tab[np_.cls], P.ssdf_items[np_.cls], s_tab, lane, z);
  if (lane == 0)
    for (int i = 0; i < NT; ++i)
      for (int j = 0; j < NB; ++j)
        store_c<double>(P.zcell, zidx(zrow_of(P.zrow, np_.p, NT, i), zcol_of(P.zcol, np_.q, NB, j), P.ldc),
                        z[i * NB + j], P.zfmt);
}

// the batch's P0 single-layer Sauter-Schwab pairs in double-float (the pairs k_near_batch
// skips), persistent over the device-counted near list
__global__ void __launch_bounds__(32 * NEAR_WARPS) k_near_batch_df(BatchLaunch L) {
  __shared__ float s_tab[64][4];
  for (int k = threadIdx.x; k < 256; k += blockDim.x) s_tab[k >> 2][k & 3] = dfl::sincos_tab_dev[k >> 2][k & 3];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = min(*L.near_count, L.near_cap);
  for (int64_t e = blockIdx.x * (int64_t)NEAR_WARPS + warp; e < n; e += (int64_t)gridDim.x * NEAR_WARPS) {
    const NearPairB nb = L.near[e];
    const BatchJobDev& J = L.jobs[nb.job];
    if (!(J.op.gr == 0.0 && nb.cls >= 1 && nb.cls <= 3)) continue;
    const Geo t = load_geo(J.geo + (int64_t)J.tperm[nb.p] * GEO_STRIDE);
    const Geo s = load_geo(J.geo + (int64_t)nb.q * GEO_STRIDE);
    C2<double> z[1];
    hh_sl_ss_df<0, 0>(J.op, t, s, nb.cls, L.ssdf_tab[nb.cls], L.ssdf_items[nb.cls], s_tab, lane, z);
    if (lane == 0)
      store_c<double>(J.Z, zidx(zrow_of(J.zrow, nb.p, 1, 0), zcol_of(J.zcol, nb.q, 1, 0), J.ldz), z[0], L.zfmt);
  }
}

// five CTAs per SM (96 registers, a few spilled): measured 9.9 -> 9.6 ms per C2 solve against
// four CTAs at 128 registers
template <bool SL>
__global__ void __launch_bounds__(32 * NEAR_WARPS, 5) k_near_ss_df(NearParams P) {
  __shared__ float s_tab[64][4];  // sin / cos(m pi/32)
  for (int k = threadIdx.x; k < 256; k += blockDim.x) s_tab[k >> 2][k & 3] = dfl::sincos_tab_dev[k >> 2][k & 3];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * (int64_t)NEAR_WARPS + warp;
  if (e >= P.nnear) return;
  const NearPair np_ = P.near[e];
  if (!near_is_ssdf(P, np_.cls)) return;
  const Geo t = load_geo(P.tgeo + (int64_t)P.tperm[np_.p] * GEO_STRIDE);
  const Geo s = load_geo(P.bgeo + (int64_t)P.qcells[np_.q] * GEO_STRIDE);
  int pt[3], ps[3];
  ss_order_warp(t, s, lane, pt, ps);
  const int cls = np_.cls;
  const float2* tab = P.ssdf_tab[cls];
  const int items = P.ssdf_items[cls];
  const V3<double> cp = t.c, cq = s.c;
  dfl::df a0[3], et1[3], et2[3], b0[3], es1[3], es2[3], dd[3];
  dfv3(t.v[pt[0]] - cp, a0);
  dfv3(t.v[pt[1]] - t.v[pt[0]], et1);
  dfv3(t.v[pt[2]] - t.v[pt[1]], et2);
  dfv3(s.v[ps[0]] - cq, b0);
  dfv3(s.v[ps[1]] - s.v[ps[0]], es1);
  dfv3(s.v[ps[2]] - s.v[ps[1]], es2);
  dfv3(cp - cq, dd);
  const dfl::df kk = df_of(P.op.gi);
  const dfl::df i4pi{DF_I4PI_HI, DF_I4PI_LO};
  constexpr int NM = SL ? 16 : 22;  // M0 (SL only), M1, V1, V2 (+ V3 for the double layer)
  dfl::df m[22];
#pragma unroll
  for (int q = 0; q < 22; ++q) m[q] = dfl::make(0.f);
  for (int it = lane; it < items; it += 32) {
    dfl::df v[SSDF_VALS];
#pragma unroll
    for (int q = 0; q < SSDF_VALS; ++q) {
      const float2 f = tab[(int64_t)q * items + it];
      v[q] = dfl::df{f.x, f.y};
    }
    const dfl::df X0 = v[0], X1 = v[1], Y0 = v[2], Y1 = v[3], D0 = v[4], D1 = v[5], w = v[6];
    dfl::df xi[3], eta[3], r[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      xi[c] = dfl::adds(a0[c], dfl::adds(dfl::mulu(X0, et1[c]), dfl::mulu(X1, et2[c])));
      eta[c] = dfl::adds(b0[c], dfl::adds(dfl::mulu(Y0, es1[c]), dfl::mulu(Y1, es2[c])));
      if (cls == 3)
        r[c] = dfl::adds(dfl::mulu(D0, et1[c]), dfl::mulu(D1, et2[c]));
      else if (cls == 2)
        r[c] = dfl::adds(dfl::mulu(D0, et1[c]), dfl::subs(dfl::mulu(X1, et2[c]), dfl::mulu(Y1, es2[c])));
      else
        r[c] = dfl::subs(dfl::adds(dfl::mulu(X0, et1[c]), dfl::mulu(X1, et2[c])),
                         dfl::adds(dfl::mulu(Y0, es1[c]), dfl::mulu(Y1, es2[c])));
    }
    const dfl::df R2 = dfl::dot3u(r, r);
    const dfl::df iR = dfl::rsqrt(R2);
    const dfl::df R = dfl::mulu(R2, iR);
    dfl::df sn, cs;
    dfl::sincos_tab(dfl::mulu(kk, R), s_tab, &sn, &cs);
    const dfl::df amp = dfl::mulu(dfl::mulu(iR, w), i4pi);  // w / (4 pi R)
    dfl::df cr = dfl::mulu(amp, cs), ci = dfl::neg(dfl::mulu(amp, sn));
    dfl::df s0, a[3], b[3];
    if (SL) {
      s0 = dfl::dot3u(xi, eta);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a[c] = xi[c];
        b[c] = eta[c];
      }
      dfl::acc(m[0], cr);
      dfl::acc(m[1], ci);
    } else {
      // grad G = c r, c = -(i k + 1/R) G / R
      const dfl::df pr = dfl::neg(dfl::mulu(iR, iR)), pi = dfl::neg(dfl::mulu(kk, iR));
      const dfl::df nr = dfl::subs(dfl::mulu(pr, cr), dfl::mulu(pi, ci));
      const dfl::df ni = dfl::adds(dfl::mulu(pr, ci), dfl::mulu(pi, cr));
      cr = nr;
      ci = ni;
      // xi.(r x eta) = xi.(d x eta); a = xi x r, b = r x eta
      const dfl::df de[3] = {dfl::subs(dfl::mulu(dd[1], eta[2]), dfl::mulu(dd[2], eta[1])),
                             dfl::subs(dfl::mulu(dd[2], eta[0]), dfl::mulu(dd[0], eta[2])),
                             dfl::subs(dfl::mulu(dd[0], eta[1]), dfl::mulu(dd[1], eta[0]))};
      s0 = dfl::dot3u(xi, de);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
        a[c] = dfl::subs(dfl::mulu(xi[c1], r[c2]), dfl::mulu(xi[c2], r[c1]));
        b[c] = dfl::subs(dfl::mulu(r[c1], eta[c2]), dfl::mulu(r[c2], eta[c1]));
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        dfl::acc(m[16 + 2 * c], dfl::mulu(r[c], cr));
        dfl::acc(m[17 + 2 * c], dfl::mulu(r[c], ci));
      }
    }
    dfl::acc(m[2], dfl::mulu(s0, cr));
    dfl::acc(m[3], dfl::mulu(s0, ci));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dfl::acc(m[4 + 2 * c], dfl::mulu(a[c], cr));
      dfl::acc(m[5 + 2 * c], dfl::mulu(a[c], ci));
      dfl::acc(m[10 + 2 * c], dfl::mulu(b[c], cr));
      dfl::acc(m[11 + 2 * c], dfl::mulu(b[c], ci));
    }
  }
  // the warp's totals (exact pair sums), then FP64
  double md[22];
#pragma unroll
  for (int q = 0; q < 22; ++q) {
    if ((q < 2 && !SL) || (q >= NM && SL)) {  // moments this operator does not have: no butterfly
      md[q] = 0.0;
      continue;
    }
    dfl::df x = dfl::norm(m[q]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const dfl::df y{__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)};
      x = dfl::add(x, y);
    }
    md[q] = fsplit::f2d(x.hi) + fsplit::f2d(x.lo);
  }
  if (lane < 9) {  // lane 3 i + j: entry (i, j) of the 3 x 3 block, as k_near's moment form
    const C2<double> M0{md[0], md[1]}, M1{md[2], md[3]};
    CV<double> V1, V2, V3_;
    V1.x = {md[4], md[5]}; V1.y = {md[6], md[7]}; V1.z = {md[8], md[9]};
    V2.x = {md[10], md[11]}; V2.y = {md[12], md[13]}; V2.z = {md[14], md[15]};
    V3_.x = {md[16], md[17]}; V3_.y = {md[18], md[19]}; V3_.z = {md[20], md[21]};
    const int i = lane / 3, j = lane % 3;
    const V3<double> tv = t.v[i] - cp, sv = s.v[j] - cq;
    C2<double> z;
    C2<double> fm = csub(csub(M1, rdot(sv, V1)), rdot(tv, V2));
    if (SL) {
      const C2<double> al{P.op.ar, P.op.ai}, be{P.op.br, P.op.bi};
      fm = cadd(fm, cscale(dot(tv, sv), M0));
      z = cadd(cmul(al, fm), cscale(4.0, cmul(be, M0)));
    } else {
      z = cadd(fm, rdot(cross(sv, tv), V3_));
    }
    store_c<double>(P.zcell, zidx(zrow_of(P.zrow, np_.p, 3, i), zcol_of(P.zcol, np_.q, 3, j), P.ldc), z, P.zfmt);
  }
}

cudaError_t launch_near(const AsmArgs& a, int nnear, const TriRuleDev& ro, const TriRuleDev& ri,
                        const TriRuleDev& fro, const TriRuleDev& fri, cudaStream_t st) {
  if (nnear <= 0) return cudaSuccess;
  cudaError_t e = upload_gl(st);
  if (e != cudaSuccess) return e;
  NearParams P;
  P.op = a.op;
  P.qs = a.qs;
  P.tk = a.ts->kind;
  P.bk = a.bs->kind;
  P.tperm = a.ts->tperm;
  P.tgeo = a.ts->geo;
  P.bgeo = a.bs->geo;
  P.qcells = a.qcells;
  P.near = a.near;
  P.nnear = nnear;
  P.zcell = a.zcell;
  P.zfmt = a.zcell_fmt;
  P.ss32 = a.precision == BEAST_MIXED;
  P.ldc = a.ldc;
  P.zrow = a.zrow;
  P.zcol = a.zcol;
  P.flag = a.flag;
  P.ro = ro;
  P.ri = ri;
  P.fro = fro;
  P.fri = fri;
  // Sauter-Schwab pairs in double-float arithmetic (real wavenumber): RT Maxwell single and
  // double layers on the mixed-accurate path, the Helmholtz single layer on P0 / P1 off the
  // FP64 path; their node tables first
  const bool rt_mw = a.zcell_fmt == ZCELL_DF && a.ts->kind == BEAST_RT && a.bs->kind == BEAST_RT &&
                     (a.op.kind == BEAST_MW_SL || a.op.kind == BEAST_MW_DL);
  const bool hh_sl = a.precision != BEAST_FP64 && a.op.kind == BEAST_HH_SL && a.ts->kind != BEAST_RT &&
                     a.bs->kind != BEAST_RT;
  P.ssdf = (rt_mw || hh_sl) && a.op.gr == 0.0 && a.ss_tabs != nullptr && a.qs.kind != BEAST_QS_DOUBLENUM;
  for (int c = 0; c < 4; ++c) {
    P.ssdf_tab[c] = nullptr;
    P.ssdf_items[c] = 0;
  }
  if (P.ssdf) {
    e = ss_tables(a.ss_tabs, a.qs, st, P.ssdf_tab, P.ssdf_items);
    if (e != cudaSuccess) return e;
  }
  P.bcells = a.bs->cells;
  P.bchildren = a.bs->mesh->children;
  P.bnchild = a.bs->mesh->nchild;
  P.tcells = a.ts->cells;
  P.tchildren = a.ts->mesh->children;
  P.tnchild = a.ts->mesh->nchild;
  unsigned blocks = (unsigned)((nnear + NEAR_WARPS - 1) / NEAR_WARPS);
  if (P.ss32) k_near_ss32<<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
  if (P.ssdf) {
    if (rt_mw && a.op.kind == BEAST_MW_SL)
      k_near_ss_df<true><<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
    else if (rt_mw)
      k_near_ss_df<false><<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
    else if (P.tk == BEAST_P1 && P.bk == BEAST_P1)
      k_near_hh_df<1, 1><<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
    else if (P.tk == BEAST_P1)
      k_near_hh_df<1, 0><<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
    else if (P.bk == BEAST_P1)
      k_near_hh_df<0, 1><<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
    else
      k_near_hh_df<0, 0><<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
  }
  k_near<<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
  if (P.qs.kind == BEAST_QS_TEST_REFINES_TRIAL || P.qs.kind == BEAST_QS_TRIAL_REFINES_TEST)
    k_near_refines<<<blocks, 32 * NEAR_WARPS, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_gather(const GatherArgs& g, cudaStream_t st) {
  const beast_space* ts = g.ts;
  const beast_space* bs = g.bs;
  int64_t nrows = ts->nfuncs;
  if (nrows == 0 || g.n1 <= g.n0) return cudaSuccess;
  int th = 256;
  const int64_t ncb = (g.n1 - g.n0 + GATHER_NCOL - 1) / GATHER_NCOL;
  if (ncb > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((unsigned)((nrows + th - 1) / th), (unsigned)ncb);
  int nst = ts->kind == BEAST_P0 ? 1 : 3, nsb = bs->kind == BEAST_P0 ? 1 : 3;
#define GATHER(ZC, OC)                                                                       \
  k_gather<ZC, OC><<<grid, th, 0, st>>>(g, ts->fn_ptr, ts->fn_cell, ts->fn_shape, ts->fn_coeff, \
                                        bs->fn_ptr, bs->fn_cell, bs->fn_shape, bs->fn_coeff, nst, \
                                        nsb, nrows)
  if (g.entry_layout) {
#define GATHER_E(ZC, OC, UC) \
  k_gather_e<ZC, OC, UC><<<grid, th, 0, st>>>(g, ts->fn_ptr, ts->fn_coeff, bs->fn_ptr, bs->fn_coeff, nrows)
    const bool uc = ts->unit_coef && bs->unit_coef;
    if (g.zcell_fmt == ZCELL_DF) {
      if (uc) {
        if (g.z_c64) GATHER_E(ZCELL_DF, 1, 1); else GATHER_E(ZCELL_DF, 0, 1);
      } else {
        if (g.z_c64) GATHER_E(ZCELL_DF, 1, 0); else GATHER_E(ZCELL_DF, 0, 0);
      }
    } else if (g.zcell_fmt == ZCELL_C64) {
      if (g.z_c64) GATHER_E(ZCELL_C64, 1, 0); else GATHER_E(ZCELL_C64, 0, 0);
    } else {
      if (g.z_c64) GATHER_E(ZCELL_C128, 1, 0); else GATHER_E(ZCELL_C128, 0, 0);
    }
#undef GATHER_E
  } else if (g.zcell_fmt == ZCELL_DF) {
#define GATHER_DF(OC, UC)                                                                              \
  k_gather_df<OC, UC><<<grid, th, 0, st>>>(g, ts->fn_ptr, ts->fn_cell, ts->fn_shape, ts->fn_coeff, bs->fn_ptr, \
                                           bs->fn_cell, bs->fn_shape, bs->fn_coeff, nst, nsb, nrows)
    const bool uc = ts->unit_coef && bs->unit_coef;
    if (uc) {
      if (g.z_c64) GATHER_DF(1, 1); else GATHER_DF(0, 1);
    } else {
      if (g.z_c64) GATHER_DF(1, 0); else GATHER_DF(0, 0);
    }
#undef GATHER_DF
  } else if (g.zcell_fmt == ZCELL_C64) {
    if (g.z_c64) GATHER(1, 1); else GATHER(1, 0);
  } else {
    if (g.z_c64) GATHER(0, 1); else GATHER(0, 0);
  }
#undef GATHER
  return cudaGetLastError();
}

cudaError_t launch_rhs(int kind, const beast_space* ts, const double* dir, const double* pol,
                       double gr, double gi, double ar, double ai, const TriRuleDev& r, double* b,
                       cudaStream_t st) {
  int64_t n = ts->nfuncs;
  if (n == 0) return cudaSuccess;
  int th = 128;
  k_rhs<<<(unsigned)((n + th - 1) / th), th, 0, st>>>(kind, ts->kind, ts->fn_ptr, ts->fn_cell,
                                                    ts->fn_shape, ts->fn_coeff, ts->geo, dir[0],
                                                    dir[1], dir[2], pol[0], pol[1], pol[2], gr, gi,
                                                    ar, ai, r, n, b);
  return cudaGetLastError();
}

cudaError_t launch_farfield(const beast_space* s, const double* u, const double* pts, int64_t npts,
                            double gr, double gi, const TriRuleDev& r, double* ff, cudaStream_t st) {
  if (npts == 0) return cudaSuccess;
  k_farfield<<<(unsigned)npts, 256, 0, st>>>(s->geo, s->ad_dof, s->ad_coeff, s->maxfn, s->ncells, u,
                                             pts, gr, gi, r, ff);
  return cudaGetLastError();
}

cudaError_t launch_local_impl(int which, const beast_space* ts, const beast_space* bs,
                              const int* b_cell2act, const TriRuleDev& r, void* Z, int64_t ldz,
                              int z_c64, int64_t row_off, int64_t col_off, double cr, double ci,
                              int* flag, cudaStream_t st) {
  int64_t n = ts->nfuncs;
  if (n == 0) return cudaSuccess;
  int th = 128;
  k_local<<<(unsigned)((n + th - 1) / th), th, 0, st>>>(which, ts->fn_ptr, ts->fn_cell, ts->fn_shape,
                                                      ts->fn_coeff, ts->cells, ts->geo, b_cell2act,
                                                      bs->ad_dof, bs->ad_coeff, bs->maxfn, r, n, Z,
                                                      ldz, z_c64, row_off, col_off, cr, ci, flag);
  return cudaGetLastError();
}
