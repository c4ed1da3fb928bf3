// oracle.cpp -- CPU FP64 restatement of BEAST.jl's Galerkin BEM assembly and dense solve.
//
// TEST INFRASTRUCTURE ONLY: the correctness checker for the GB300 kernels and the timed
// CPU baseline.  Nothing in the product library links or calls this file.
//
// Every function names the reference code it restates (paths relative to the BEAST.jl
// project root).  The per-point-pair integrands are evaluated exactly as the reference
// writes them (shape values times kernel, accumulated per local pair), deliberately NOT
// in the algebraically reduced form the GPU kernels use, so that the two are independent.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

typedef std::complex<double> cplx;

namespace {

const double PI = 3.14159265358979323846264338327950288;
const double I4PI = 1.0 / (4.0 * PI);

struct V3 {
  double x, y, z;
};
inline V3 v3(const double* p) { return V3{p[0], p[1], p[2]}; }
inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

struct CV3 {
  cplx x, y, z;
};

// ------------------------------------------------------------------------------------
// Quadrature rules.
// CompScienceMeshes.trgauss(n) (un-vendored) returns the symmetric triangle rule exact to
// polynomial degree n; call sites: src/quadrature/doublenumwiltonsauterqstrat.jl:20-21,
// src/identityop.jl:41.  Restated here from the published structure of the symmetric
// (Dunavant 1985) rules: orbits of the centroid (S3), (a,a,1-2a) (S21) and (a,b,1-a-b)
// (S111).  The published orbit parameters serve as starting values; Gauss-Newton on the
// moment equations refines them to full double precision.
// ------------------------------------------------------------------------------------
struct Orbit {
  int type;  // 0 = S3, 1 = S21, 2 = S111
  double a, b, w;
};

struct SymRuleSpec {
  int degree;
  std::vector<Orbit> orbits;
};

const std::vector<SymRuleSpec>& sym_specs() {
  static std::vector<SymRuleSpec> s = {
      {1, {{0, 0, 0, 1.0}}},
      {2, {{1, 0.166666666666667, 0, 1.0 / 3}}},
      {3, {{0, 0, 0, -0.5625}, {1, 0.2, 0, 0.520833333333333}}},
      {4, {{1, 0.445948490915965, 0, 0.223381589678011}, {1, 0.091576213509771, 0, 0.109951743655322}}},
      {5, {{0, 0, 0, 0.225}, {1, 0.470142064105115, 0, 0.132394152788506},
           {1, 0.101286507323456, 0, 0.125939180544827}}},
      {6, {{1, 0.249286745170910, 0, 0.116786275726379}, {1, 0.063089014491502, 0, 0.050844906370207},
           {2, 0.053145049844817, 0.310352451033784, 0.082851075618374}}},
      {7, {{0, 0, 0, -0.149570044467682}, {1, 0.260345966079040, 0, 0.175615257433208},
           {1, 0.065130102902216, 0, 0.053347235608838},
           {2, 0.048690315425316, 0.312865496004874, 0.077113760890257}}},
      {8, {{0, 0, 0, 0.144315607677787}, {1, 0.459292588292723, 0, 0.095091634267285},
           {1, 0.170569307751760, 0, 0.103217370534718}, {1, 0.050547228317031, 0, 0.032458497623198},
           {2, 0.008394777409958, 0.263112829634638, 0.027230314174435}}},
      {10, {{0, 0, 0, 0.090817990382754}, {1, 0.485577633383657, 0, 0.036725957756467},
            {1, 0.109481575485037, 0, 0.045321059435528},
            {2, 0.141707219414880, 0.307939838764121, 0.072757916845420},
            {2, 0.025003534762686, 0.246672560639903, 0.028327242531057},
            {2, 0.009540815400299, 0.066803251012200, 0.009421666963733}}},
  };
  return s;
}

double fact(int n) {
  double r = 1;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}

// points of an orbit in barycentric (l1,l2,l3)
int orbit_points(const Orbit& o, double (*pts)[3]) {
  if (o.type == 0) {
    pts[0][0] = pts[0][1] = pts[0][2] = 1.0 / 3;
    return 1;
  }
  if (o.type == 1) {
    double a = o.a, c = 1 - 2 * a;
    double P[3][3] = {{a, a, c}, {a, c, a}, {c, a, a}};
    memcpy(pts, P, sizeof(P));
    return 3;
  }
  double a = o.a, b = o.b, c = 1 - a - b;
  double P[6][3] = {{a, b, c}, {b, a, c}, {a, c, b}, {c, a, b}, {b, c, a}, {c, b, a}};
  memcpy(pts, P, sizeof(P));
  return 6;
}

// monomial moments u^p v^q over the triangle, normalised to unit area
double moment(int p, int q) { return 2.0 * fact(p) * fact(q) / fact(p + q + 2); }

void solve_dense(std::vector<double>& A, std::vector<double>& b, int n) {
  // Gaussian elimination with partial pivoting, A row-major n x n
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > std::fabs(A[piv * n + k])) piv = i;
    if (piv != k) {
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[piv * n + j]);
      std::swap(b[k], b[piv]);
    }
    for (int i = k + 1; i < n; ++i) {
      double f = A[i * n + k] / A[k * n + k];
      for (int j = k; j < n; ++j) A[i * n + j] -= f * A[k * n + j];
      b[i] -= f * b[k];
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    double s = b[k];
    for (int j = k + 1; j < n; ++j) s -= A[k * n + j] * b[j];
    b[k] = s / A[k * n + k];
  }
}

void refine_rule(SymRuleSpec& spec) {
  // unknown vector: per orbit w (+a for S21, +a,b for S111)
  std::vector<int> off;
  int nun = 0;
  for (auto& o : spec.orbits) {
    off.push_back(nun);
    nun += 1 + (o.type == 1 ? 1 : 0) + (o.type == 2 ? 2 : 0);
  }
  std::vector<std::pair<int, int>> mons;
  for (int p = 0; p <= spec.degree; ++p)
    for (int q = 0; p + q <= spec.degree; ++q) mons.push_back({p, q});
  int neq = (int)mons.size();
  auto eval = [&](std::vector<double>& res, std::vector<double>& J) {
    res.assign(neq, 0.0);
    J.assign((size_t)neq * nun, 0.0);
    for (size_t oi = 0; oi < spec.orbits.size(); ++oi) {
      const Orbit& o = spec.orbits[oi];
      double pts[6][3];
      int np = orbit_points(o, pts);
      const double h = 1e-7;
      for (int e = 0; e < neq; ++e) {
        int p = mons[e].first, q = mons[e].second;
        double s = 0;
        for (int k = 0; k < np; ++k) s += std::pow(pts[k][0], p) * std::pow(pts[k][1], q);
        res[e] += o.w * s;
        J[(size_t)e * nun + off[oi]] += s;
        // derivatives wrt a, b by central differences of the analytic orbit sum
        for (int d = 0; d < (o.type == 1 ? 1 : (o.type == 2 ? 2 : 0)); ++d) {
          Orbit op = o, om = o;
          if (d == 0) { op.a += h; om.a -= h; } else { op.b += h; om.b -= h; }
          double pp[6][3], pm[6][3];
          orbit_points(op, pp);
          orbit_points(om, pm);
          double sp = 0, sm = 0;
          for (int k = 0; k < np; ++k) {
            sp += std::pow(pp[k][0], p) * std::pow(pp[k][1], q);
            sm += std::pow(pm[k][0], p) * std::pow(pm[k][1], q);
          }
          J[(size_t)e * nun + off[oi] + 1 + d] += o.w * (sp - sm) / (2 * h);
        }
      }
    }
    for (int e = 0; e < neq; ++e) res[e] -= moment(mons[e].first, mons[e].second);
  };
  std::vector<double> res, J;
  for (int it = 0; it < 60; ++it) {
    eval(res, J);
    double rn = 0;
    for (double r : res) rn = std::max(rn, std::fabs(r));
    if (rn < 1e-17) break;
    // normal equations J^T J dx = -J^T r
    std::vector<double> A((size_t)nun * nun, 0.0), b(nun, 0.0);
    for (int i = 0; i < nun; ++i) {
      for (int j = 0; j < nun; ++j) {
        double s = 0;
        for (int e = 0; e < neq; ++e) s += J[(size_t)e * nun + i] * J[(size_t)e * nun + j];
        A[i * nun + j] = s;
      }
      double s = 0;
      for (int e = 0; e < neq; ++e) s += J[(size_t)e * nun + i] * res[e];
      b[i] = -s;
    }
    solve_dense(A, b, nun);
    for (size_t oi = 0; oi < spec.orbits.size(); ++oi) {
      Orbit& o = spec.orbits[oi];
      o.w += b[off[oi]];
      if (o.type >= 1) o.a += b[off[oi] + 1];
      if (o.type == 2) o.b += b[off[oi] + 2];
    }
  }
}

struct TriRule {
  std::vector<double> u, v, w;
};

void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w) {
  // Newton iteration on P_n (Golub-Welsch-free classic form); FastGaussQuadrature's
  // gausslegendre, mapped to [0,1] as _legendre does (src/maxwell/mwops.jl:46-51)
  x.assign(n, 0);
  w.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    double z = std::cos(PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1; }
      double dp = n * (z * p1 - p0) / (z * z - 1);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    double p0 = 1, p1 = z;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    double dp = n * (z * p1 - p0) / (z * z - 1);
    double wz = 2.0 / ((1 - z * z) * dp * dp);
    // ascending order on [0,1]
    x[n - 1 - i] = 0.5 * (z + 1);
    w[n - 1 - i] = 0.5 * wz;
  }
}

const TriRule& trirule(int degree) {
  static std::mutex mtx;
  static std::vector<TriRule*> cache(64, nullptr);
  std::lock_guard<std::mutex> lk(mtx);
  if (degree < 1) degree = 1;
  if (degree >= 64) degree = 63;
  if (cache[degree]) return *cache[degree];
  TriRule* r = new TriRule();
  bool done = false;
  for (auto spec : sym_specs()) {
    if (spec.degree != degree) continue;
    refine_rule(spec);
    for (auto& o : spec.orbits) {
      double pts[6][3];
      int np = orbit_points(o, pts);
      for (int k = 0; k < np; ++k) {
        r->u.push_back(pts[k][0]);
        r->v.push_back(pts[k][1]);
        r->w.push_back(o.w);
      }
    }
    done = true;
  }
  if (!done) {
    // collapsed (Duffy) product rule: u = s, v = (1-s) t, exact to degree 2n-2
    // (odd degrees collapse onto another vertex so that rules of neighbouring degrees
    // never share points)
    int n = degree / 2 + 2;
    std::vector<double> x, w;
    gauss_legendre01(n, x, w);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double a = x[i], b = (1 - x[i]) * x[j];
        if (degree % 2) { r->u.push_back(1 - a - b); r->v.push_back(a); }
        else { r->u.push_back(a); r->v.push_back(b); }
        r->w.push_back(2.0 * w[i] * w[j] * (1 - x[i]));
      }
  }
  cache[degree] = r;
  return *r;
}

// ------------------------------------------------------------------------------------
// Geometry of one triangle (CompScienceMeshes chart: x = u v1 + v v2 + (1-u-v) v3,
// tangents t_u = v1 - v3, t_v = v2 - v3, jacobian = |t_u x t_v| = 2 area)
// ------------------------------------------------------------------------------------
struct Tri {
  V3 v[3];
  V3 n;      // unit normal (t_u x t_v) / |.|
  double area;
};

Tri make_tri(const double* p) {
  Tri t;
  for (int i = 0; i < 3; ++i) t.v[i] = v3(p + 3 * i);
  V3 c = cross(t.v[0] - t.v[2], t.v[1] - t.v[2]);
  double j = norm(c);
  t.area = 0.5 * j;
  t.n = (1.0 / j) * c;
  return t;
}

// local shape values at a point: src/bases/local/rtlocal.jl:8-27 (RT: (x - v_i)/(2A),
// divergence 1/A), src/bases/local/laglocal.jl:17-18 (P0: 1), laglocal.jl:214-228 (P1:
// barycentric coordinates).
struct Shapes {
  int n;
  double s[3];
  V3 v[3];
  double div[3];
};

void eval_shapes(int kind, const Tri& t, V3 x, const double* bary, Shapes& S) {
  if (kind == ORC_RT) {
    S.n = 3;
    double ij = 1.0 / (2 * t.area);
    for (int i = 0; i < 3; ++i) {
      S.v[i] = ij * (x - t.v[i]);
      S.div[i] = 2 * ij;
    }
  } else if (kind == ORC_P0) {
    S.n = 1;
    S.s[0] = 1;
  } else {
    S.n = 3;
    for (int i = 0; i < 3; ++i) S.s[i] = bary[i];
  }
}

// complex exp(-gamma R) and expm1(-gamma R)
inline cplx cexpm1(cplx z) {
  double a = z.real(), b = z.imag();
  double ea = std::exp(a), em = std::expm1(a);
  double sb = std::sin(b), sh = std::sin(0.5 * b);
  return cplx(em * std::cos(b) - 2 * sh * sh, ea * sb);
}

struct Op {
  int kind;
  cplx gamma, alpha, beta;
};

Op make_op(const orc_op* o) {
  Op op;
  op.kind = o->kind;
  op.gamma = cplx(o->gamma_re, o->gamma_im);
  op.alpha = cplx(o->alpha_re, o->alpha_im);
  op.beta = cplx(o->beta_re, o->beta_im);
  return op;
}

// Integrand(biop)(x,y,f,g) for each operator; adds w * k_ij into out[i*nb + j].
// MW SL: src/maxwell/mwops.jl:101-117; Reg: 121-138
// MW DL: mwops.jl:141-155 (alpha is not applied there); Reg: 158-174
// n x K: src/maxwell/nxdbllayer.jl:27-44 (alpha not applied)
// HH SL/DL/DLT: src/helmholtz3d/hh3dops.jl:119-182; Reg: src/helmholtz3d/wiltonints.jl:2-17,
// 141-159, 293-312
void integrand(const Op& op, V3 x, V3 y, V3 nx, V3 ny, const Shapes& f, const Shapes& g, double w,
               cplx* out) {
  V3 r = x - y;
  double R = norm(r);
  double iR = 1.0 / R;
  cplx gR = op.gamma * R;
  const int nb = g.n;
  switch (op.kind) {
    case ORC_MW_SL:
    case ORC_MW_SL_REG: {
      cplx green;
      if (op.kind == ORC_MW_SL)
        green = std::exp(-gR) * (I4PI * iR);
      else
        green = (cexpm1(-gR) + gR - 0.5 * gR * gR) / (4 * PI * R);
      cplx aG = op.alpha * green, bG = op.beta * green;
      for (int i = 0; i < f.n; ++i)
        for (int j = 0; j < nb; ++j)
          out[i * nb + j] += w * (aG * dot(f.v[i], g.v[j]) + bG * (f.div[i] * g.div[j]));
      break;
    }
    case ORC_MW_DL:
    case ORC_MW_DL_REG:
    case ORC_MW_NXDL: {
      cplx c;
      if (op.kind == ORC_MW_DL_REG) {
        cplx expo = std::exp(-gR);
        c = (-(gR + 1.0) * expo + (1.0 - 0.5 * gR * gR)) * (I4PI * iR * iR * iR);
      } else {
        cplx green = std::exp(-gR) * (iR * I4PI);
        c = -(op.gamma + iR) * green * iR;  // gradgreen = c * r
      }
      for (int i = 0; i < f.n; ++i)
        for (int j = 0; j < nb; ++j) {
          double t;
          if (op.kind == ORC_MW_NXDL)
            t = dot(f.v[i], cross(nx, cross(r, g.v[j])));
          else
            t = dot(f.v[i], cross(r, g.v[j]));
          out[i * nb + j] += w * (c * t);
        }
      break;
    }
    case ORC_HH_SL:
    case ORC_HH_SL_REG: {
      cplx green;
      if (op.kind == ORC_HH_SL)
        green = std::exp(-gR) * (I4PI * iR);
      else
        green = (cexpm1(-gR) - 0.5 * gR * gR) / (4 * PI * R);
      cplx aG = op.alpha * green;
      for (int i = 0; i < f.n; ++i)
        for (int j = 0; j < nb; ++j) out[i * nb + j] += w * (g.s[j] * (aG * f.s[i]));
      break;
    }
    case ORC_HH_DL:
    case ORC_HH_DL_REG:
    case ORC_HH_DLT:
    case ORC_HH_DLT_REG: {
      cplx c;
      bool reg = (op.kind == ORC_HH_DL_REG || op.kind == ORC_HH_DLT_REG);
      if (reg) {
        cplx expo = std::exp(-gR);
        c = (-(gR + 1.0) * expo + (1.0 - 0.5 * gR * gR)) * (I4PI * iR * iR * iR);
      } else {
        cplx green = std::exp(-gR) * (iR * I4PI);
        c = -(op.gamma + iR) * green * iR * op.alpha;  // alpha * gradgreen = c r
      }
      cplx k;
      if (op.kind == ORC_HH_DL || op.kind == ORC_HH_DL_REG)
        k = -c * dot(ny, r);
      else
        k = c * dot(nx, r);
      for (int i = 0; i < f.n; ++i)
        for (int j = 0; j < nb; ++j) out[i * nb + j] += w * (k * (f.s[i] * g.s[j]));
      break;
    }
  }
}

int nshapes(int kind) { return kind == ORC_P0 ? 1 : 3; }

// point of a rule on a triangle
inline V3 rule_point(const Tri& t, double u, double v, double* bary) {
  bary[0] = u;
  bary[1] = v;
  bary[2] = 1 - u - v;
  return u * t.v[0] + v * t.v[1] + (1 - u - v) * t.v[2];
}

// DoubleQuadRule: src/quadrature/doublenumints.jl:12-43
void dq_block(const Op& op, int tk, int bk, const Tri& t, const Tri& s, int deg_o, int deg_i,
              cplx* out) {
  const TriRule& ro = trirule(deg_o);
  const TriRule& ri = trirule(deg_i);
  Shapes f, g;
  for (size_t a = 0; a < ro.w.size(); ++a) {
    double bx[3], by[3];
    V3 x = rule_point(t, ro.u[a], ro.v[a], bx);
    eval_shapes(tk, t, x, bx, f);
    double jx = ro.w[a] * t.area;
    for (size_t b = 0; b < ri.w.size(); ++b) {
      V3 y = rule_point(s, ri.u[b], ri.v[b], by);
      eval_shapes(bk, s, y, by, g);
      double jy = ri.w[b] * s.area;
      integrand(op, x, y, t.n, s.n, f, g, jx * jy, out);
    }
  }
}

}  // namespace

// ------------------------------------------------------------------------------------
// Wilton et al. (1984) potential integrals.  Restates the reference's in-tree copy
// test/test_wiltonints.jl:60-232 (WiltonInts84.wiltonints is un-vendored).
// scal: [d/R^3, 1/R, 1, R, R^2, R^3], vec: [(rho'-rho)/R^3, /R, 1, R, R^2, -], grad: as the
// in-tree copy ([grad'(1/R), grad' R, grad' R^2, grad' R^3]).
// ------------------------------------------------------------------------------------
extern "C" void orc_wiltonints(const double* p1, const double* p2, const double* p3,
                               const double* xp, double* scal, double* vec, double* grad) {
  const double tol = 2.220446049250313e-16 * 1e3;
  V3 P[3] = {v3(p1), v3(p2), v3(p3)};
  V3 x = v3(xp);
  V3 t1 = P[1] - P[0], t2 = P[2] - P[0];
  V3 n = cross(t1, t2);
  n = (1.0 / norm(n)) * n;
  double d = dot(x - P[0], n);
  double D = std::fabs(d);
  V3 c = x - d * n;
  double s[6] = {0, 0, 0, 0, 0, 0};
  V3 v[6] = {};
  bool c_inside = true;
  int nthru = 0;
  int thru[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i) {
    V3 a = P[i], b = P[(i + 1) % 3];
    V3 ab = b - a;
    double l = norm(ab);
    V3 t = (1.0 / l) * ab;
    V3 m = cross(t, n);
    V3 ca = a - c, cb = b - c;
    double xa = dot(ca, t), xb = dot(cb, t);
    double p = dot(ca, m);
    double Pabs = std::fabs(p);
    if (p < 0) c_inside = false;
    double w2 = p * p + d * d;
    double ra = std::sqrt(xa * xa + w2), rb = std::sqrt(xb * xb + w2);
    double w = std::sqrt(w2);
    auto add = [&](int k, double sc) { v[k] = v[k] + sc * m; };
    if (Pabs > tol) {
      double lg = std::log((xb + rb) / (xa + ra));
      double at = std::atan(d * xb / (p * rb)) - std::atan(d * xa / (p * ra));
      s[0] += -at;
      s[1] += p * lg + d * at;
      s[2] += 0.5 * p * (xb - xa);
      s[3] += p * (xb * rb - xa * ra) / 6 + (0.5 * d * d + p * p / 6) * p * lg + d * d * d * at / 3;
      s[4] += 0.5 * xb * p * (xb * xb / 6 + 0.5 * p * p + d * d) -
              0.5 * xa * p * (xa * xa / 6 + 0.5 * p * p + d * d);
      s[5] += (p * xb * rb * (xb * xb + 0.5 * (9 * d * d + 5 * p * p)) -
               p * xa * ra * (xa * xa + 0.5 * (9 * d * d + 5 * p * p))) / 20 +
              p * (15 * d * d * d * d + 10 * d * d * p * p + 3 * p * p * p * p) * lg / 40 +
              0.2 * d * d * d * d * d * at;
      add(0, -lg);
      add(1, 0.5 * ((xb * rb - xa * ra) + w * w * lg));
      add(2, 0.5 * xb * (xb * xb / 3 + p * p) - 0.5 * xa * (xa * xa / 3 + p * p));
      add(3, (xb * rb * rb * rb - xa * ra * ra * ra) / 12 + w * w * (xb * rb - xa * ra) / 8 +
                 w * w * w * w * lg / 8);
      double q5b = xb * xb * xb * xb * xb / 20 + p * p * xb * xb * xb / 6 + 0.25 * p * p * p * p * xb +
                   0.5 * d * d * (xb * xb * xb / 3 + p * p * xb);
      double q5a = xa * xa * xa * xa * xa / 20 + p * p * xa * xa * xa / 6 + 0.25 * p * p * p * p * xa +
                   0.5 * d * d * (xa * xa * xa / 3 + p * p * xa);
      add(4, q5b - q5a);
    } else {
      if (xa * xb < tol * tol) thru[nthru++] = i;
      double lg;
      if (D > tol)
        lg = std::log((xb + rb) / (xa + ra));
      else
        lg = (xb > 0) ? std::log(xb / xa) : std::log(xa / xb);
      add(0, -lg);
      if (D > tol)
        add(1, 0.5 * (xb * rb - xa * ra) + 0.5 * w * w * lg);
      else
        add(1, 0.5 * (xb * rb - xa * ra));
      add(2, xb * xb * xb / 6 - xa * xa * xa / 6);
      add(3, (xb * rb * rb * rb - xa * ra * ra * ra) / 12 + w * w * (xb * rb - xa * ra) / 8 +
                 w * w * w * w * lg / 8);
      double q5b = xb * xb * xb * xb * xb / 20 + p * p * xb * xb * xb / 6 + 0.25 * p * p * p * p * xb +
                   0.5 * d * d * (xb * xb * xb / 3 + p * p * xb);
      double q5a = xa * xa * xa * xa * xa / 20 + p * p * xa * xa * xa / 6 + 0.25 * p * p * p * p * xa +
                   0.5 * d * d * (xa * xa * xa / 3 + p * p * xa);
      add(4, q5b - q5a);
    }
  }
  double sgn = D < tol ? 0.0 : (d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0));
  double alpha = 0;
  if (nthru == 0 && c_inside)
    alpha = 2 * PI;
  else if (nthru == 1)
    alpha = PI;
  else if (nthru == 2) {
    V3 e1 = P[(thru[0] + 1) % 3] - P[thru[0]];
    V3 e2 = P[(thru[1] + 1) % 3] - P[thru[1]];
    double ca = dot(-1.0 * e1, e2) / (norm(e1) * norm(e2));
    alpha = std::acos(std::max(-1.0, std::min(1.0, ca)));
  }
  s[0] += alpha * sgn;
  s[1] += -alpha * D;
  s[3] += -alpha * D * D * D / 3;
  s[5] += -alpha * D * D * D * D * D / 5;
  for (int k = 0; k < 6; ++k) scal[k] = s[k];
  for (int k = 0; k < 6; ++k) {
    vec[3 * k] = v[k].x;
    vec[3 * k + 1] = v[k].y;
    vec[3 * k + 2] = v[k].z;
  }
  V3 g[4];
  g[0] = -1.0 * (v[0] - s[0] * n);
  g[1] = v[1] - (d * s[1]) * n;
  g[2] = 2.0 * (v[2] - (d * s[2]) * n);
  g[3] = 3.0 * (v[3] - (d * s[3]) * n);
  for (int k = 0; k < 4; ++k) {
    grad[3 * k] = g[k].x;
    grad[3 * k + 1] = g[k].y;
    grad[3 * k + 2] = g[k].z;
  }
}

namespace {

// Singular part of the singularity-extraction rule at one test point x with weight dx.
// MW SL: src/maxwell/wiltonints.jl:8-52.  MW DL: wiltonints.jl:55-84 (grad of the
// singular kernel (1/R + gamma^2 R/2)/(4pi); the gradient of R enters as  grad' R).
// HH SL P0xP0: src/helmholtz3d/wiltonints.jl:19-40; HH DL P0xP0: wiltonints.jl:349-378;
// HH DLT P0xP0: wiltonints.jl:162-190.
bool se_singular(const Op& op, int tk, int bk, const Tri& t, const Tri& s, V3 x, const double* bx,
                 double dx, cplx* out) {
  double scal[6], vec[18], grad[12];
  double sv[9];
  for (int i = 0; i < 3; ++i) {
    sv[3 * i] = s.v[i].x;
    sv[3 * i + 1] = s.v[i].y;
    sv[3 * i + 2] = s.v[i].z;
  }
  double xp[3] = {x.x, x.y, x.z};
  orc_wiltonints(sv, sv + 3, sv + 6, xp, scal, vec, grad);
  V3 ns = s.n;
  V3 rho = x - dot(x - s.v[0], ns) * ns;
  cplx g = op.gamma;
  auto VEC = [&](int k) { return V3{vec[3 * k], vec[3 * k + 1], vec[3 * k + 2]}; };
  // grad'(1/R) and grad' R over the trial triangle
  V3 gm1 = V3{grad[0], grad[1], grad[2]};
  V3 gR = VEC(1) - (dot(x - s.v[0], ns) * scal[1]) * ns;
  switch (op.kind) {
    case ORC_MW_SL: {
      cplx iG = (scal[1] - g * scal[2] + 0.5 * g * g * scal[3]) / (4 * PI);
      V3 v1 = VEC(1), v2 = VEC(2), v3_ = VEC(3);
      CV3 iGy;
      iGy.x = (v1.x + scal[1] * rho.x - g * (v2.x + scal[2] * rho.x) + 0.5 * g * g * (v3_.x + scal[3] * rho.x)) / (4 * PI);
      iGy.y = (v1.y + scal[1] * rho.y - g * (v2.y + scal[2] * rho.y) + 0.5 * g * g * (v3_.y + scal[3] * rho.y)) / (4 * PI);
      iGy.z = (v1.z + scal[1] * rho.z - g * (v2.z + scal[2] * rho.z) + 0.5 * g * g * (v3_.z + scal[3] * rho.z)) / (4 * PI);
      double a = 1.0 / t.area / s.area / 4;
      for (int i = 0; i < 3; ++i) {
        V3 gi = x - t.v[i];
        for (int j = 0; j < 3; ++j) {
          V3 b = s.v[j];
          cplx fx = iGy.x - iG * b.x, fy = iGy.y - iG * b.y, fz = iGy.z - iG * b.z;
          cplx dg = gi.x * fx + gi.y * fy + gi.z * fz;
          cplx idf = 2.0 * iG;
          out[i * 3 + j] += (a * op.alpha * dg + a * op.beta * 2.0 * idf) * dx;
        }
      }
      return true;
    }
    case ORC_MW_DL: {
      // integral of grad_x of (1/R + gamma^2 R / 2)/(4 pi) = -(grad'(1/R) + gamma^2/2 grad' R)/(4 pi)
      CV3 iDG;
      cplx h = 0.5 * g * g;
      iDG.x = (-gm1.x - h * gR.x) / (4 * PI);
      iDG.y = (-gm1.y - h * gR.y) / (4 * PI);
      iDG.z = (-gm1.z - h * gR.z) / (4 * PI);
      double a = 1.0 / t.area / s.area / 4;
      for (int i = 0; i < 3; ++i) {
        V3 gi = x - t.v[i];
        for (int j = 0; j < 3; ++j) {
          V3 cr = cross(x - s.v[j], gi);
          out[i * 3 + j] += (a * (cr.x * iDG.x + cr.y * iDG.y + cr.z * iDG.z)) * dx;
        }
      }
      return true;
    }
    case ORC_HH_SL: {
      // src/helmholtz3d/wiltonints.jl:19-135: P0 or P1 on either side.  A P1 trial shape is
      // affine in the plane, lambda_j(y) = lambda_j(rho) + grad lambda_j . (rho' - rho), so its
      // integrals against 1/R and R follow from scal and vec (the reference takes them from
      // WiltonInts84.higherorder); a P1 test shape is the barycentric coordinate of x.
      const cplx h = 0.5 * g * g;
      const int nt = tk == ORC_P0 ? 1 : 3, nb = bk == ORC_P0 ? 1 : 3;
      cplx iG[3];
      if (bk == ORC_P0) {
        iG[0] = (scal[1] + h * scal[3]) / (4 * PI);
      } else {
        const double twoA = dot(cross(s.v[1] - s.v[0], s.v[2] - s.v[0]), ns);
        for (int j = 0; j < 3; ++j) {
          const V3 a = s.v[(j + 1) % 3], b = s.v[(j + 2) % 3];
          const double lr = dot(cross(a - rho, b - rho), ns) / twoA;
          const V3 gl = (1.0 / twoA) * cross(ns, b - a);
          const double i1 = lr * scal[1] + dot(gl, VEC(1)), i3 = lr * scal[3] + dot(gl, VEC(3));
          iG[j] = (i1 + h * i3) / (4 * PI);
        }
      }
      for (int i = 0; i < nt; ++i) {
        const double ft = tk == ORC_P0 ? 1.0 : bx[i];
        for (int j = 0; j < nb; ++j) out[i * nb + j] += op.alpha * ft * iG[j] * dx;
      }
      return true;
    }
    case ORC_HH_DL:
    case ORC_HH_DLT: {
      // P0 or P1 test shapes (a factor: the barycentric coordinate of x).  Trial P1 for the
      // double layer: the source normal is constant on the flat trial triangle, so
      // n.grad'(1/R) = d/R^3 and n.grad' R = -d/R with d = n.(x - y) fixed, and the shape
      // moments follow from scal / vec as for the single layer.  The transposed double layer
      // with P1 trial shapes needs in-plane second moments (the reference takes them from
      // WiltonInts84.higherorder): built here from the divergence theorem in the plane.
      const cplx h = 0.5 * g * g;
      const int nt = tk == ORC_P0 ? 1 : 3, nb = bk == ORC_P0 ? 1 : 3;
      cplx v[3];
      if (bk == ORC_P0) {
        CV3 iDG;
        iDG.x = -(gm1.x + h * gR.x) / (4 * PI);
        iDG.y = -(gm1.y + h * gR.y) / (4 * PI);
        iDG.z = -(gm1.z + h * gR.z) / (4 * PI);
        const V3 nn = op.kind == ORC_HH_DL ? ns : t.n;
        const cplx ndg = nn.x * iDG.x + nn.y * iDG.y + nn.z * iDG.z;
        v[0] = op.kind == ORC_HH_DL ? -ndg : ndg;
      } else {
        const double twoA = dot(cross(s.v[1] - s.v[0], s.v[2] - s.v[0]), ns);
        const double d = dot(x - s.v[0], ns);
        // transposed double layer: in-plane second moments of u = rho' - rho,
        //   Q3 = int u u^T / R^3 = P S1 - sum_e (int_e u / R) m_e^T,
        //   Q1 = int u u^T / R   = sum_e (int_e u R) m_e^T - P S3
        // (divergence theorem on d_l(u_k / R) and d_l(u_k R)); their products with a vector w
        V3 q3w[3], q1w[3];
        const V3 nt = t.n;
        auto Q = [&](V3 w, V3* o3, V3* o1) {
          const V3 pw = w - dot(w, ns) * ns;
          *o3 = scal[1] * pw;
          *o1 = (-scal[3]) * pw;
          for (int e = 0; e < 3; ++e) {
            const V3 a = s.v[e], b = s.v[(e + 1) % 3];
            const double len = norm(b - a);
            const V3 te = (1.0 / len) * (b - a);
            const V3 me = cross(te, ns);
            const double sa = dot(a - rho, te), sb = dot(b - rho, te), pe = dot(a - rho, me);
            const double w2 = pe * pe + d * d;
            const double ra = std::sqrt(sa * sa + w2), rb = std::sqrt(sb * sb + w2);
            const double lg = (sa + sb >= 0) ? std::log((sb + rb) / (sa + ra)) : std::log((ra - sa) / (rb - sb));
            const double ir = 0.5 * (sb * rb - sa * ra + w2 * lg);
            const V3 f1 = (pe * lg) * me + (rb - ra) * te;
            const V3 f3 = (pe * ir) * me + ((rb * rb * rb - ra * ra * ra) / 3.0) * te;
            *o3 = *o3 - dot(me, w) * f1;
            *o1 = *o1 + dot(me, w) * f3;
          }
        };
        for (int j = 0; j < 3; ++j) {
          const V3 a = s.v[(j + 1) % 3], b = s.v[(j + 2) % 3];
          const double lr = dot(cross(a - rho, b - rho), ns) / twoA;
          const V3 gl = (1.0 / twoA) * cross(ns, b - a);
          const double iA = lr * scal[0] + d * dot(gl, VEC(0));  // int lambda_j d / R^3
          const double iB = d * (lr * scal[1] + dot(gl, VEC(1)));  // int lambda_j d / R
          if (op.kind == ORC_HH_DL) {
            v[j] = (iA - h * iB) / (4 * PI);
          } else {
            Q(gl, &q3w[j], &q1w[j]);
            // int lambda_j grad'(1/R) = -(lr V0 + Q3 gl) + n iA ; int lambda_j grad' R = (lr V1 + Q1 gl) - n iB
            const V3 g1 = (-1.0) * (lr * VEC(0) + q3w[j]) + iA * ns;
            const V3 gr = (lr * VEC(1) + q1w[j]) - iB * ns;
            v[j] = -(dot(nt, g1) + h * dot(nt, gr)) / (4 * PI);
          }
        }
      }
      for (int i = 0; i < nt; ++i) {
        const double ft = tk == ORC_P0 ? 1.0 : bx[i];
        for (int j = 0; j < nb; ++j) out[i * nb + j] += op.alpha * ft * v[j] * dx;
      }
      return true;
    }
  }
  return false;
}

int regular_kind(int k) {
  switch (k) {
    case ORC_MW_SL: return ORC_MW_SL_REG;
    case ORC_MW_DL: return ORC_MW_DL_REG;
    case ORC_HH_SL: return ORC_HH_SL_REG;
    case ORC_HH_DL: return ORC_HH_DL_REG;
    case ORC_HH_DLT: return ORC_HH_DLT_REG;
  }
  return k;
}

// Singularity extraction: src/quadrature/singularityextractionints.jl:4-22
bool se_block(const Op& op, int tk, int bk, const Tri& t, const Tri& s, int deg_o, int deg_i,
              cplx* out) {
  Op rop = op;
  rop.kind = regular_kind(op.kind);
  dq_block(rop, tk, bk, t, s, deg_o, deg_i, out);
  const TriRule& ro = trirule(deg_o);
  for (size_t a = 0; a < ro.w.size(); ++a) {
    double bx[3];
    V3 x = rule_point(t, ro.u[a], ro.v[a], bx);
    if (!se_singular(op, tk, bk, t, s, x, bx, ro.w[a] * t.area, out)) return false;
  }
  return true;
}

// ------------------------------------------------------------------------------------
// Sauter-Schwab rules for touching pairs (src/quadrature/sauterschwabints.jl:156-182 drives
// the un-vendored SauterSchwabQuadrature.jl).  Restated from Sauter & Schwab, Boundary
// Element Methods (2011), ch. 5: both triangles are parametrised on the reference
// triangle {0 <= x2 <= x1 <= 1} with chi(x) = A + x1 (B - A) + x2 (C - B), the shared
// vertices first and in the same order; the 4D integral is split into subregions, each
// mapped from [0,1]^4 with a Jacobian that cancels the singularity, and integrated with a
// tensor Gauss-Legendre rule of n points per direction.
//   common vertex: 2 regions, common edge: 6 regions, common face: 6 regions.
// ------------------------------------------------------------------------------------

// emits (xhat, yhat, weight) for all nodes of one region set
template <class F>
void ss_nodes(int kind, int n, F&& emit) {
  std::vector<double> gx, gw;
  gauss_legendre01(n, gx, gw);
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b)
      for (int c = 0; c < n; ++c)
        for (int d = 0; d < n; ++d) {
          double xi = gx[a], e1 = gx[b], e2 = gx[c], e3 = gx[d];
          double w = gw[a] * gw[b] * gw[c] * gw[d];
          if (kind == ORC_RULE_SS_VERT) {
            double wt = w * xi * xi * xi * e2;
            double X[2] = {xi, xi * e1}, Y[2] = {xi * e2, xi * e2 * e3};
            emit(X, Y, wt);
            emit(Y, X, wt);
          } else if (kind == ORC_RULE_SS_EDGE) {
            // x1 = xi, x2 = xi b, y1 = xi (1-a'), y2 = xi (1-a') c ; Duffy of (a',b,c) by max
            for (int sub = 0; sub < 3; ++sub) {
              double ap, bb, cc;
              if (sub == 0) { ap = e1; bb = e1 * e2; cc = e1 * e3; }
              else if (sub == 1) { bb = e1; ap = e1 * e2; cc = e1 * e3; }
              else { cc = e1; ap = e1 * e2; bb = e1 * e3; }
              double wt = w * xi * xi * xi * (1 - ap) * e1 * e1;
              double X[2] = {xi, xi * bb}, Y[2] = {xi * (1 - ap), xi * (1 - ap) * cc};
              emit(X, Y, wt);
              emit(Y, X, wt);
            }
          } else {
            // common face: x1 = xi, x2 = xi b, y1 = xi (1-a'), y2 = xi c'
            double s = e1, t = e2, u = e3;
            double wt = w * xi * xi * xi * s * (1 - s);
            {  // c' >= b
              double ap = s * t, e = s * (1 - t), b = (1 - s) * u;
              double X[2] = {xi, xi * b}, Y[2] = {xi * (1 - ap), xi * (b + e)};
              emit(X, Y, wt);
              emit(Y, X, wt);
            }
            {  // c' <= b, a' >= e'
              double ap = s, ep = s * t, cp = (1 - s) * u;
              double X[2] = {xi, xi * (cp + ep)}, Y[2] = {xi * (1 - ap), xi * cp};
              emit(X, Y, wt);
              emit(Y, X, wt);
            }
            {  // c' <= b, e' >= a'
              double ep = s, ap = s * t, cp = (1 - s) * u;
              double X[2] = {xi, xi * (cp + ep)}, Y[2] = {xi * (1 - ap), xi * cp};
              emit(X, Y, wt);
              emit(Y, X, wt);
            }
          }
        }
}

// find the vertex correspondence; returns hits and fills permutations so that the shared
// vertices come first and in the same order (the role of SauterSchwabQuadrature.reorder)
int match_vertices(const Tri& t, const Tri& s, int* pt, int* ps) {
  const double dtol = 1.0e3 * 2.220446049250313e-16;
  int hits = 0;
  int ti[3], si[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      if (norm(t.v[i] - s.v[j]) < dtol) {
        ti[hits] = i;
        si[hits] = j;
        ++hits;
      }
  int k = 0;
  for (int h = 0; h < hits; ++h) pt[k++] = ti[h];
  for (int i = 0; i < 3; ++i) {
    bool used = false;
    for (int h = 0; h < hits; ++h) used |= (ti[h] == i);
    if (!used) pt[k++] = i;
  }
  k = 0;
  for (int h = 0; h < hits; ++h) ps[k++] = si[h];
  for (int j = 0; j < 3; ++j) {
    bool used = false;
    for (int h = 0; h < hits; ++h) used |= (si[h] == j);
    if (!used) ps[k++] = j;
  }
  return hits;
}

void ss_block(const Op& op, int tk, int bk, const Tri& t, const Tri& s, int rule, int n,
              cplx* out) {
  int pt[3], ps[3];
  match_vertices(t, s, pt, ps);
  // double-layer type kernels vanish identically on a flat common face (all vectors of the
  // triple product lie in the plane); the reference evaluates rounding noise there.
  if (rule == ORC_RULE_SS_FACE &&
      (op.kind == ORC_MW_DL || op.kind == ORC_HH_DL || op.kind == ORC_HH_DLT))
    return;
  V3 A = t.v[pt[0]], B = t.v[pt[1]], C = t.v[pt[2]];
  V3 As = s.v[ps[0]], Bs = s.v[ps[1]], Cs = s.v[ps[2]];
  double jac = 4 * t.area * s.area;
  Shapes f, g;
  ss_nodes(rule, n, [&](const double* X, const double* Y, double w) {
    double bx[3], by[3], lt[3] = {1 - X[0], X[0] - X[1], X[1]}, ls[3] = {1 - Y[0], Y[0] - Y[1], Y[1]};
    for (int k = 0; k < 3; ++k) {
      bx[pt[k]] = lt[k];
      by[ps[k]] = ls[k];
    }
    V3 x = lt[0] * A + lt[1] * B + lt[2] * C;
    V3 y = ls[0] * As + ls[1] * Bs + ls[2] * Cs;
    eval_shapes(tk, t, x, bx, f);
    eval_shapes(bk, s, y, by, g);
    integrand(op, x, y, t.n, s.n, f, g, w * jac, out);
  });
}

int classify(const Op& op, const orc_qs& qs, const Tri& t, const Tri& s) {
  // src/quadrature/doublenumwiltonsauterqstrat.jl:32-69, doublenumsauterqstrat.jl:226-240
  const double dtol = 1.0e3 * 2.220446049250313e-16;
  int hits = 0;
  double dmin2 = 1e308;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      V3 d = t.v[i] - s.v[j];
      double d2 = dot(d, d);
      dmin2 = std::min(dmin2, d2);
      if (std::sqrt(d2) < dtol) ++hits;
    }
  if (qs.kind == ORC_QS_DOUBLENUM) return 0;
  if (hits > 0) return hits;
  if (qs.kind == ORC_QS_SAUTER) return 0;
  double h2 = s.area;
  double k2 = std::norm(op.gamma);
  if (std::max(dmin2 * k2, dmin2 / (16 * h2)) < 0.2 * 0.2) return -1;
  return 0;
}

void pair_block(const Op& op, const orc_qs& qs, int tk, int bk, const Tri& t, const Tri& s, cplx* z) {
  int c = classify(op, qs, t, s);
  // DoubleNumQStrat on a common face: the double-layer type kernels vanish identically there
  // (as in ss_block); the plain rule would only sum rounding noise
  if (qs.kind == ORC_QS_DOUBLENUM &&
      (op.kind == ORC_MW_DL || op.kind == ORC_MW_NXDL || op.kind == ORC_HH_DL || op.kind == ORC_HH_DLT)) {
    const double dtol = 1.0e3 * 2.220446049250313e-16;
    int hits = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) hits += norm(t.v[i] - s.v[j]) < dtol;
    if (hits == 3) return;
  }
  int outer_far = qs.outer_far, inner_far = qs.inner_far;
  if (c == 3)
    ss_block(op, tk, bk, t, s, ORC_RULE_SS_FACE, qs.ss_face, z);
  else if (c == 2)
    ss_block(op, tk, bk, t, s, ORC_RULE_SS_EDGE, qs.ss_edge, z);
  else if (c == 1)
    ss_block(op, tk, bk, t, s, ORC_RULE_SS_VERT, qs.ss_vert, z);
  else if (c == -1)
    se_block(op, tk, bk, t, s, qs.outer_near, qs.inner_near, z);
  else
    dq_block(op, tk, bk, t, s, outer_far, inner_far, z);
}

Tri mesh_tri(const orc_mesh* m, int64_t c) {
  double p[9];
  for (int k = 0; k < 3; ++k) {
    const double* v = m->verts + 3 * (int64_t)m->cells[3 * c + k];
    p[3 * k] = v[0];
    p[3 * k + 1] = v[1];
    p[3 * k + 2] = v[2];
  }
  return make_tri(p);
}

// RT shapes of `parent` on its child `ch` (src/bases/local/interpolate.jl:61-75 with the RT
// interpolation of src/bases/local/rtlocal.jl:82-111): Q[j][k] = f_j(m_k) . (t_k x n), the
// flux of parent shape j through the child's edge k (t_k the edge vector, so |t_k x n| = |e_k|,
// oriented outward).
void rt_restrict(const Tri& parent, const Tri& ch, double Q[3][3]) {
  for (int k = 0; k < 3; ++k) {
    const V3 a = ch.v[(k + 1) % 3], b = ch.v[(k + 2) % 3];
    V3 m = cross(b - a, ch.n);
    if (dot(ch.v[k] - a, m) > 0) m = -1.0 * m;
    const V3 mid = 0.5 * (a + b);
    for (int j = 0; j < 3; ++j) Q[j][k] = dot((1.0 / (2.0 * parent.area)) * (mid - parent.v[j]), m);
  }
}

// TestRefinesTrialQStrat / TrialRefinesTestQStrat (src/quadrature/strategies/
// testrefinestrialqstrat.jl:9-17, trialrefinestestqstrat.jl:9-17): a pair sharing a vertex
// integrates the coarse cell's children one by one with the wrapped strategy and maps the
// child blocks back through the restriction (rules/testrefinestrialqrule.jl:6-52,
// rules/trialrefinestestqrule.jl:6-40); every other pair uses the wrapped strategy whole.
// `children`: [coarse mesh cell][nchild][9]; split_test selects the trial-refines-test form.
void refines_block(const Op& op, const orc_qs& qs, const Tri& t, const Tri& s, int64_t coarse_cell,
                   const double* children, int nchild, int split_test, cplx* z) {
  if (classify(op, qs, t, s) <= 0) {
    pair_block(op, qs, ORC_RT, ORC_RT, t, s, z);
    return;
  }
  const Tri& parent = split_test ? t : s;
  for (int c = 0; c < nchild; ++c) {
    const Tri ch = make_tri(children + (coarse_cell * nchild + c) * 9);
    cplx b[9] = {};
    if (split_test)
      pair_block(op, qs, ORC_RT, ORC_RT, ch, s, b);
    else
      pair_block(op, qs, ORC_RT, ORC_RT, t, ch, b);
    double Q[3][3];
    rt_restrict(parent, ch, Q);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) z[i * 3 + j] += split_test ? Q[i][k] * b[k * 3 + j] : b[i * 3 + k] * Q[j][k];
  }
}

}  // namespace

extern "C" int orc_trirule(int degree, double* uv, double* w, int cap) {
  const TriRule& r = trirule(degree);
  int n = (int)r.w.size();
  if (cap < n) return -n;
  for (int i = 0; i < n; ++i) {
    uv[2 * i] = r.u[i];
    uv[2 * i + 1] = r.v[i];
    w[i] = r.w[i];
  }
  return n;
}

extern "C" int orc_gausslegendre(int n, double* x, double* w) {
  std::vector<double> gx, gw;
  gauss_legendre01(n, gx, gw);
  for (int i = 0; i < n; ++i) {
    x[i] = gx[i];
    w[i] = gw[i];
  }
  return n;
}

extern "C" int orc_cellpair(const orc_op* o, int tkind, int bkind, const double* tv, const double* bv,
                            int rule, int deg_o, int deg_i, int gl, double* out) {
  Op op = make_op(o);
  Tri t = make_tri(tv), s = make_tri(bv);
  cplx z[9] = {};
  switch (rule) {
    case ORC_RULE_DQ: dq_block(op, tkind, bkind, t, s, deg_o, deg_i, z); break;
    case ORC_RULE_SE:
      if (!se_block(op, tkind, bkind, t, s, deg_o, deg_i, z)) return -1;
      break;
    default: ss_block(op, tkind, bkind, t, s, rule, gl, z); break;
  }
  int nt = nshapes(tkind), nb = nshapes(bkind);
  for (int i = 0; i < nt * nb; ++i) {
    out[2 * i] = z[i].real();
    out[2 * i + 1] = z[i].imag();
  }
  return 0;
}

extern "C" int orc_classify(const orc_op* o, const orc_qs* qs, const double* tv, const double* bv) {
  return classify(make_op(o), *qs, make_tri(tv), make_tri(bv));
}

// Dense assembly: src/operator.jl:100-116 (assemble), 215-231 (dof splitting over threads),
// src/integralop.jl:69-116 (assemblechunk!), 146-184 (the pair loop and the scatter
// store(a*z*b, m, n)).
extern "C" int orc_assemble(const orc_op* o, const orc_qs* qs, const orc_mesh* mesh,
                            const orc_space* ts, const orc_space* bs, double* Z, int64_t ldz,
                            int64_t row_lo, int64_t row_hi, int nthreads) {
  Op op = make_op(o);
  if (row_hi < 0) row_hi = ts->nfuncs;
  if (nthreads < 1) nthreads = 1;
  const int ntk = nshapes(ts->kind), nbk = nshapes(bs->kind);
  std::vector<Tri> ttri(ts->ncells), btri(bs->ncells);
  for (int64_t c = 0; c < ts->ncells; ++c) ttri[c] = mesh_tri(mesh, ts->cells[c]);
  for (int64_t c = 0; c < bs->ncells; ++c) btri[c] = mesh_tri(mesh, bs->cells[c]);
  int64_t nrows = row_hi - row_lo;
  std::atomic<int> bad(0);
  auto worker = [&](int tid) {
    int64_t lo = row_lo + nrows * tid / nthreads, hi = row_lo + nrows * (tid + 1) / nthreads;
    if (hi <= lo) return;
    cplx z[9];
    for (int64_t p = 0; p < ts->ncells; ++p) {
      // does this test cell carry a dof in [lo,hi)?
      bool act = false;
      for (int r = 0; r < ts->nshapes && !act; ++r)
        for (int k = 0; k < ts->maxfn; ++k) {
          int64_t m = ts->ad_dof[(p * ts->nshapes + r) * ts->maxfn + k];
          if (m >= lo && m < hi) act = true;
        }
      if (!act) continue;
      for (int64_t q = 0; q < bs->ncells; ++q) {
        for (int i = 0; i < 9; ++i) z[i] = 0;
        pair_block(op, *qs, ts->kind, bs->kind, ttri[p], btri[q], z);
        for (int j = 0; j < nbk; ++j)
          for (int kb = 0; kb < bs->maxfn; ++kb) {
            int64_t n = bs->ad_dof[(q * bs->nshapes + j) * bs->maxfn + kb];
            if (n < 0) continue;
            double b = bs->ad_coeff[(q * bs->nshapes + j) * bs->maxfn + kb];
            for (int i = 0; i < ntk; ++i)
              for (int ka = 0; ka < ts->maxfn; ++ka) {
                int64_t m = ts->ad_dof[(p * ts->nshapes + i) * ts->maxfn + ka];
                if (m < lo || m >= hi) continue;
                double a = ts->ad_coeff[(p * ts->nshapes + i) * ts->maxfn + ka];
                cplx v = a * z[i * nbk + j] * b;
                double* e = Z + 2 * ((m - row_lo) + n * ldz);
                e[0] += v.real();
                e[1] += v.imag();
              }
          }
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) th.emplace_back(worker, t);
  for (auto& t : th) t.join();
  return bad.load();
}

// Dense assembly of RT x RT pairs across a refinement: the test space on `tmesh`, the trial
// space on `bmesh`, one of them the barycentric refinement of the other (operator.jl:256-262
// picks the strategy from which mesh refines which).  Layout and threading as orc_assemble.
extern "C" int orc_assemble_refines(const orc_op* o, const orc_qs* qs, const orc_mesh* tmesh,
                                    const orc_mesh* bmesh, const orc_space* ts, const orc_space* bs,
                                    const double* children, int nchild, int split_test, double* Z,
                                    int64_t ldz, int nthreads) {
  if (ts->kind != ORC_RT || bs->kind != ORC_RT || qs->kind != ORC_QS_WILTON_SAUTER) return -1;
  Op op = make_op(o);
  if (nthreads < 1) nthreads = 1;
  std::vector<Tri> ttri(ts->ncells), btri(bs->ncells);
  for (int64_t c = 0; c < ts->ncells; ++c) ttri[c] = mesh_tri(tmesh, ts->cells[c]);
  for (int64_t c = 0; c < bs->ncells; ++c) btri[c] = mesh_tri(bmesh, bs->cells[c]);
  const int64_t nrows = ts->nfuncs;
  auto worker = [&](int tid) {
    const int64_t lo = nrows * tid / nthreads, hi = nrows * (tid + 1) / nthreads;
    if (hi <= lo) return;
    for (int64_t p = 0; p < ts->ncells; ++p) {
      bool act = false;
      for (int r = 0; r < 3 && !act; ++r)
        for (int k = 0; k < ts->maxfn; ++k) {
          const int64_t m = ts->ad_dof[(p * 3 + r) * ts->maxfn + k];
          if (m >= lo && m < hi) act = true;
        }
      if (!act) continue;
      for (int64_t q = 0; q < bs->ncells; ++q) {
        cplx z[9] = {};
        refines_block(op, *qs, ttri[p], btri[q], split_test ? ts->cells[p] : bs->cells[q], children, nchild,
                      split_test, z);
        for (int j = 0; j < 3; ++j)
          for (int kb = 0; kb < bs->maxfn; ++kb) {
            const int64_t n = bs->ad_dof[(q * 3 + j) * bs->maxfn + kb];
            if (n < 0) continue;
            const double b = bs->ad_coeff[(q * 3 + j) * bs->maxfn + kb];
            for (int i = 0; i < 3; ++i)
              for (int ka = 0; ka < ts->maxfn; ++ka) {
                const int64_t m = ts->ad_dof[(p * 3 + i) * ts->maxfn + ka];
                if (m < lo || m >= hi) continue;
                const cplx v = ts->ad_coeff[(p * 3 + i) * ts->maxfn + ka] * z[i * 3 + j] * b;
                double* e = Z + 2 * (m + n * ldz);
                e[0] += v.real();
                e[1] += v.imag();
              }
          }
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) th.emplace_back(worker, t);
  for (auto& t : th) t.join();
  return 0;
}

// Identity / NCross on RT x RT (src/identityop.jl:7-24, SingleNumQStrat(6) identityop.jl:66-67;
// the local assembly loops src/localop.jl:107-155)
extern "C" int orc_assemble_local(int which, const orc_mesh* mesh, const orc_space* ts,
                                  const orc_space* bs, int degree, double cre, double cim,
                                  double* Z, int64_t ldz) {
  cplx coeff(cre, cim);
  const TriRule& r = trirule(degree);
  // map mesh cell -> active trial cell
  std::vector<int64_t> bidx(mesh->nc, -1);
  for (int64_t q = 0; q < bs->ncells; ++q) bidx[bs->cells[q]] = q;
  for (int64_t p = 0; p < ts->ncells; ++p) {
    int64_t q = bidx[ts->cells[p]];
    if (q < 0) continue;
    Tri t = mesh_tri(mesh, ts->cells[p]);
    double z[9] = {};
    Shapes f, g;
    for (size_t a = 0; a < r.w.size(); ++a) {
      double bx[3];
      V3 x = rule_point(t, r.u[a], r.v[a], bx);
      eval_shapes(ts->kind, t, x, bx, f);
      eval_shapes(bs->kind, t, x, bx, g);
      double w = r.w[a] * t.area;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          z[i * 3 + j] += w * (which == 0 ? dot(f.v[i], g.v[j]) : dot(f.v[i], cross(t.n, g.v[j])));
    }
    for (int i = 0; i < 3; ++i)
      for (int ka = 0; ka < ts->maxfn; ++ka) {
        int64_t m = ts->ad_dof[(p * 3 + i) * ts->maxfn + ka];
        if (m < 0) continue;
        double a = ts->ad_coeff[(p * 3 + i) * ts->maxfn + ka];
        for (int j = 0; j < 3; ++j)
          for (int kb = 0; kb < bs->maxfn; ++kb) {
            int64_t n = bs->ad_dof[(q * 3 + j) * bs->maxfn + kb];
            if (n < 0) continue;
            double b = bs->ad_coeff[(q * 3 + j) * bs->maxfn + kb];
            cplx v = coeff * (a * z[i * 3 + j] * b);
            Z[2 * (m + n * ldz)] += v.real();
            Z[2 * (m + n * ldz) + 1] += v.imag();
          }
      }
  }
  return 0;
}

// Excitation: src/excitation.jl:38-65 (per-cell loop), 91-115 (celltestvalues),
// 166-181 (CrossTraceMW / TangTraceMW), src/maxwell/mwexc.jl:36-42 (PlaneWaveMW),
// mwexc.jl:44-52 (curl of a plane wave), src/helmholtz3d/hh3dexc.jl (plane wave trace)
extern "C" int orc_rhs_planewave(int kind, const orc_mesh* mesh, const orc_space* ts,
                                 const double* dir, const double* pol, double gre, double gim,
                                 double are, double aim, int degree, double* b) {
  cplx gamma(gre, gim), amp(are, aim);
  V3 d = v3(dir), u = v3(pol);
  const TriRule& r = trirule(degree);
  const int nt = nshapes(ts->kind);
  for (int64_t p = 0; p < ts->ncells; ++p) {
    Tri t = mesh_tri(mesh, ts->cells[p]);
    cplx loc[3] = {};
    Shapes f;
    for (size_t a = 0; a < r.w.size(); ++a) {
      double bx[3];
      V3 x = rule_point(t, r.u[a], r.v[a], bx);
      eval_shapes(ts->kind, t, x, bx, f);
      double w = r.w[a] * t.area;
      cplx ph = amp * std::exp(-gamma * dot(d, x));
      if (kind == 2) {
        for (int i = 0; i < nt; ++i) loc[i] += w * (f.s[i] * ph);
        continue;
      }
      V3 fu = u;
      cplx fa = ph;
      if (kind == 1) {
        // H = -1/(i k) curl E with k = -i gamma:  curl E = -gamma (d x u) e^{-gamma d.x} a
        // so H = -1/(gamma) * (-gamma) (d x u) ... = (d x u) a e^{-gamma d.x} / (i k / gamma)
        cplx k = cplx(0, -1) * gamma;
        cplx pref = -1.0 / (cplx(0, 1) * k) * (-gamma);
        fu = cross(d, u);
        fa = pref * ph;
      }
      // field values F(x) = fa * fu (complex scalar times real vector)
      V3 n = t.n;
      for (int i = 0; i < nt; ++i) {
        double val;
        if (kind == 0) {
          V3 tr = cross(cross(n, fu), n);  // (n x F) x n
          val = dot(f.v[i], tr);
        } else {
          V3 tr = cross(n, fu);  // n x H
          val = dot(f.v[i], tr);
        }
        loc[i] += w * (fa * val);
      }
    }
    for (int i = 0; i < nt; ++i)
      for (int k = 0; k < ts->maxfn; ++k) {
        int64_t m = ts->ad_dof[(p * ts->nshapes + i) * ts->maxfn + k];
        if (m < 0) continue;
        double a = ts->ad_coeff[(p * ts->nshapes + i) * ts->maxfn + k];
        b[2 * m] += (a * loc[i]).real();
        b[2 * m + 1] += (a * loc[i]).imag();
      }
  }
  return 0;
}

// ------------------------------------------------------------------------------------
// Dense solve.  The reference calls LAPACK (zgetrf/zgetrs through `\`,
// src/solvers/lusolver.jl:30, src/solvers/lu.jl:40-47).  Restated: right-looking blocked
// LU with partial pivoting (same pivot choice as zgetrf: max |re|+|im| per column, first
// index on ties), threaded trailing update.
// ------------------------------------------------------------------------------------
namespace {
inline double cabs1(cplx z) { return std::fabs(z.real()) + std::fabs(z.imag()); }

template <class F>
void parallel_for(int64_t n, int nthreads, F&& f) {
  if (nthreads <= 1 || n < 64) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t) {
    int64_t lo = n * t / nthreads, hi = n * (t + 1) / nthreads;
    if (hi > lo) th.emplace_back([&, lo, hi] { f(lo, hi); });
  }
  for (auto& t : th) t.join();
}
}  // namespace

extern "C" int orc_lu_factor(int64_t n, double* Ad, int64_t lda, int64_t* ipiv, int nthreads) {
  cplx* A = reinterpret_cast<cplx*>(Ad);
  const int64_t nb = 64;
  int info = 0;
  for (int64_t k0 = 0; k0 < n; k0 += nb) {
    int64_t kb = std::min(nb, n - k0);
    // unblocked panel factorisation of columns k0..k0+kb-1 (rows k0..n-1)
    for (int64_t k = k0; k < k0 + kb; ++k) {
      int64_t p = k;
      double mx = cabs1(A[k + k * lda]);
      for (int64_t i = k + 1; i < n; ++i) {
        double v = cabs1(A[i + k * lda]);
        if (v > mx) { mx = v; p = i; }
      }
      ipiv[k] = p;
      if (mx == 0) { if (!info) info = (int)k + 1; continue; }
      if (p != k)
        for (int64_t j = 0; j < n; ++j) std::swap(A[k + j * lda], A[p + j * lda]);
      cplx inv = 1.0 / A[k + k * lda];
      for (int64_t i = k + 1; i < n; ++i) A[i + k * lda] *= inv;
      // rank-1 update inside the panel
      for (int64_t j = k + 1; j < k0 + kb; ++j) {
        cplx u = A[k + j * lda];
        if (u == cplx(0)) continue;
        for (int64_t i = k + 1; i < n; ++i) A[i + j * lda] -= A[i + k * lda] * u;
      }
    }
    int64_t j1 = k0 + kb;
    if (j1 >= n) break;
    // U12 = L11^{-1} A12
    parallel_for(n - j1, nthreads, [&](int64_t lo, int64_t hi) {
      for (int64_t j = j1 + lo; j < j1 + hi; ++j)
        for (int64_t k = k0; k < k0 + kb; ++k) {
          cplx u = A[k + j * lda];
          for (int64_t i = k + 1; i < k0 + kb; ++i) A[i + j * lda] -= A[i + k * lda] * u;
        }
    });
    // A22 -= L21 U12
    parallel_for(n - j1, nthreads, [&](int64_t lo, int64_t hi) {
      for (int64_t j = j1 + lo; j < j1 + hi; ++j)
        for (int64_t k = k0; k < k0 + kb; ++k) {
          cplx u = A[k + j * lda];
          if (u == cplx(0)) continue;
          cplx* cj = A + j * lda;
          const cplx* ck = A + k * lda;
          for (int64_t i = j1; i < n; ++i) cj[i] -= ck[i] * u;
        }
    });
  }
  return info;
}

extern "C" int orc_lu_solve(int64_t n, const double* Ad, int64_t lda, const int64_t* ipiv,
                            int64_t nrhs, double* Bd, int64_t ldb) {
  const cplx* A = reinterpret_cast<const cplx*>(Ad);
  cplx* B = reinterpret_cast<cplx*>(Bd);
  for (int64_t r = 0; r < nrhs; ++r) {
    cplx* b = B + r * ldb;
    for (int64_t k = 0; k < n; ++k)
      if (ipiv[k] != k) std::swap(b[k], b[ipiv[k]]);
    for (int64_t k = 0; k < n; ++k) {
      cplx v = b[k];
      if (v == cplx(0)) continue;
      for (int64_t i = k + 1; i < n; ++i) b[i] -= A[i + k * lda] * v;
    }
    for (int64_t k = n - 1; k >= 0; --k) {
      b[k] /= A[k + k * lda];
      cplx v = b[k];
      if (v == cplx(0)) continue;
      for (int64_t i = 0; i < k; ++i) b[i] -= A[i + k * lda] * v;
    }
  }
  return 0;
}

// Restarted GMRES with modified Gram-Schmidt and Givens rotations (the algorithm of
// IterativeSolvers.gmres!, called from src/solvers/itsolver.jl:83-125)
extern "C" int orc_gmres(int64_t n, const double* Ad, int64_t lda, const double* bd, double* xd,
                         double reltol, int restart, int maxiter, int nthreads, double* resnorm) {
  const cplx* A = reinterpret_cast<const cplx*>(Ad);
  const cplx* b = reinterpret_cast<const cplx*>(bd);
  cplx* x = reinterpret_cast<cplx*>(xd);
  auto matvec = [&](const cplx* v, cplx* y) {
    parallel_for(n, nthreads, [&](int64_t lo, int64_t hi) {
      for (int64_t i = lo; i < hi; ++i) y[i] = 0;
      for (int64_t j = 0; j < n; ++j) {
        cplx vj = v[j];
        const cplx* col = A + j * lda;
        for (int64_t i = lo; i < hi; ++i) y[i] += col[i] * vj;
      }
    });
  };
  auto nrm = [&](const cplx* v) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += std::norm(v[i]);
    return std::sqrt(s);
  };
  double bn = nrm(b);
  std::vector<cplx> r(n), w(n);
  std::vector<std::vector<cplx>> V;
  int it = 0;
  double rn = 0;
  if (restart < 1) restart = (int)std::min<int64_t>(n, 1000);
  while (true) {
    matvec(x, r.data());
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - r[i];
    rn = nrm(r.data());
    if (rn <= reltol * bn || it >= maxiter) break;
    V.assign(1, std::vector<cplx>(n));
    for (int64_t i = 0; i < n; ++i) V[0][i] = r[i] / rn;
    std::vector<cplx> H((size_t)(restart + 1) * restart, 0.0), cs(restart), sn(restart),
        g(restart + 1, 0.0);
    g[0] = rn;
    int k = 0;
    for (; k < restart && it < maxiter; ++k, ++it) {
      matvec(V[k].data(), w.data());
      for (int j = 0; j <= k; ++j) {
        cplx h = 0;
        for (int64_t i = 0; i < n; ++i) h += std::conj(V[j][i]) * w[i];
        H[j + k * (restart + 1)] = h;
        for (int64_t i = 0; i < n; ++i) w[i] -= h * V[j][i];
      }
      double hn = nrm(w.data());
      H[k + 1 + k * (restart + 1)] = hn;
      V.emplace_back(n);
      for (int64_t i = 0; i < n; ++i) V[k + 1][i] = w[i] / hn;
      for (int j = 0; j < k; ++j) {
        cplx h0 = H[j + k * (restart + 1)], h1 = H[j + 1 + k * (restart + 1)];
        H[j + k * (restart + 1)] = std::conj(cs[j]) * h0 + std::conj(sn[j]) * h1;
        H[j + 1 + k * (restart + 1)] = -sn[j] * h0 + cs[j] * h1;
      }
      cplx h0 = H[k + k * (restart + 1)], h1 = H[k + 1 + k * (restart + 1)];
      double den = std::sqrt(std::norm(h0) + std::norm(h1));
      cs[k] = h0 / den;
      sn[k] = h1 / den;
      H[k + k * (restart + 1)] = den;
      H[k + 1 + k * (restart + 1)] = 0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = std::conj(cs[k]) * g[k];
      if (std::abs(g[k + 1]) <= reltol * bn) { ++k; ++it; break; }
    }
    // back substitution
    std::vector<cplx> yv(k);
    for (int j = k - 1; j >= 0; --j) {
      cplx s = g[j];
      for (int l = j + 1; l < k; ++l) s -= H[j + l * (restart + 1)] * yv[l];
      yv[j] = s / H[j + j * (restart + 1)];
    }
    for (int j = 0; j < k; ++j)
      for (int64_t i = 0; i < n; ++i) x[i] += yv[j] * V[j][i];
  }
  *resnorm = rn / bn;
  return rn <= reltol * bn ? it : -it;
}

extern "C" int orc_farfield(const orc_mesh* mesh, const orc_space* ts, const double* ud,
                            const double* pts, int64_t npts, double gre, double gim, int degree,
                            double* ffd) {
  cplx gamma(gre, gim);
  const cplx* u = reinterpret_cast<const cplx*>(ud);
  CV3* ff = reinterpret_cast<CV3*>(ffd);
  const TriRule& r = trirule(degree);
  for (int64_t pi = 0; pi < npts; ++pi) {
    V3 yh = v3(pts + 3 * pi);
    cplx acc[3] = {};
    for (int64_t p = 0; p < ts->ncells; ++p) {
      Tri t = mesh_tri(mesh, ts->cells[p]);
      Shapes f;
      cplx loc[3][3] = {};
      for (size_t a = 0; a < r.w.size(); ++a) {
        double bx[3];
        V3 x = rule_point(t, r.u[a], r.v[a], bx);
        eval_shapes(ORC_RT, t, x, bx, f);
        double w = r.w[a] * t.area;
        cplx krn = std::exp(gamma * dot(yh, x));
        for (int i = 0; i < 3; ++i) {
          V3 tr = cross(cross(yh, f.v[i]), yh);  // (y x (krn f)) x y, krn scalar
          loc[i][0] += w * krn * tr.x;
          loc[i][1] += w * krn * tr.y;
          loc[i][2] += w * krn * tr.z;
        }
      }
      for (int i = 0; i < 3; ++i)
        for (int k = 0; k < ts->maxfn; ++k) {
          int64_t m = ts->ad_dof[(p * 3 + i) * ts->maxfn + k];
          if (m < 0) continue;
          double a = ts->ad_coeff[(p * 3 + i) * ts->maxfn + k];
          for (int c = 0; c < 3; ++c) acc[c] += loc[i][c] * a * u[m];
        }
    }
    ff[pi].x = acc[0];
    ff[pi].y = acc[1];
    ff[pi].z = acc[2];
  }
  return 0;
}
