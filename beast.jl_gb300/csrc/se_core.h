// Geometry and complex helpers of the assembly kernels, the Wilton et al. (1984) potential
// integrals and the singular part of the singularity-extraction rule (src/quadrature/
// singularityextractionints.jl:4-22; src/maxwell/wiltonints.jl:8-84;
// src/helmholtz3d/wiltonints.jl:19-378).  Host + device, so that the CPU tests run this very
// code against the oracle.
#pragma once
#include <math.h>

#include "internal.h"
#include "se_p1.h"

#if defined(__CUDACC__)
#define SEC_HD __host__ __device__ __forceinline__
#else
#define SEC_HD inline
#endif

namespace {

template <typename R>
struct V3 {
  R x, y, z;
};
template <typename R>
SEC_HD V3<R> mk(R a, R b, R c) {
  return V3<R>{a, b, c};
}
template <typename R>
SEC_HD V3<R> operator+(V3<R> a, V3<R> b) {
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename R>
SEC_HD V3<R> operator-(V3<R> a, V3<R> b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename R>
SEC_HD V3<R> operator*(R s, V3<R> a) {
  return {s * a.x, s * a.y, s * a.z};
}
template <typename R>
SEC_HD R dot(V3<R> a, V3<R> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename R>
SEC_HD V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// complex numbers as (re, im) pairs
template <typename R>
struct C2 {
  R re, im;
};
template <typename R>
SEC_HD C2<R> cmul(C2<R> a, C2<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R>
SEC_HD C2<R> cadd(C2<R> a, C2<R> b) {
  return {a.re + b.re, a.im + b.im};
}
template <typename R>
SEC_HD C2<R> csub(C2<R> a, C2<R> b) {
  return {a.re - b.re, a.im - b.im};
}
template <typename R>
SEC_HD C2<R> cscale(R s, C2<R> a) {
  return {s * a.re, s * a.im};
}
// complex vector (3 complex components)
template <typename R>
struct CV {
  C2<R> x, y, z;
};
template <typename R>
SEC_HD void cv_zero(CV<R>& a) {
  a.x = a.y = a.z = C2<R>{0, 0};
}
template <typename R>
SEC_HD void cv_axpy(C2<R> s, V3<R> v, CV<R>& acc) {  // acc += s * v
  acc.x.re += s.re * v.x; acc.x.im += s.im * v.x;
  acc.y.re += s.re * v.y; acc.y.im += s.im * v.y;
  acc.z.re += s.re * v.z; acc.z.im += s.im * v.z;
}
template <typename R>
SEC_HD C2<R> rdot(V3<R> v, const CV<R>& c) {  // v . c
  return {v.x * c.x.re + v.y * c.y.re + v.z * c.z.re, v.x * c.x.im + v.y * c.y.im + v.z * c.z.im};
}
template <typename R>
SEC_HD CV<R> rcross_cv(V3<R> a, const CV<R>& c) {  // a x c
  CV<R> r;
  r.x = {a.y * c.z.re - a.z * c.y.re, a.y * c.z.im - a.z * c.y.im};
  r.y = {a.z * c.x.re - a.x * c.z.re, a.z * c.x.im - a.x * c.z.im};
  r.z = {a.x * c.y.re - a.y * c.x.re, a.x * c.y.im - a.y * c.x.im};
  return r;
}

const double PI = 3.14159265358979323846;
const double I4PI = 0.07957747154594767;  // 1/(4 pi)

struct Geo {
  V3<double> v[3];
  V3<double> c, n;
  double area;
};
SEC_HD Geo load_geo(const double* g) {
  Geo r;
  for (int i = 0; i < 3; ++i) r.v[i] = mk(g[3 * i], g[3 * i + 1], g[3 * i + 2]);
  r.c = mk(g[9], g[10], g[11]);
  r.n = mk(g[12], g[13], g[14]);
  r.area = g[15];
  return r;
}

// Wilton et al. (1984) potential integrals over triangle s seen from x:
// S[0] = int d/R^3, S[1] = int 1/R, S[2] = int 1, S[3] = int R;
// Vm1 = int (rho'-rho)/R^3, V1 = int (rho'-rho)/R, V2 = int (rho'-rho), V3 = int (rho'-rho) R
struct Wilton {
  double S[4];
  V3<double> V[4];
  V3<double> n;
  double d;
};

SEC_HD void wilton(const Geo& s, V3<double> x, Wilton& W) {
  const double tol = 2.220446049250313e-16 * 1e3;
  V3<double> n = cross(s.v[1] - s.v[0], s.v[2] - s.v[0]);
  n = (1.0 / sqrt(dot(n, n))) * n;
  double d = dot(x - s.v[0], n);
  double D = fabs(d);
  V3<double> c = x - d * n;
  for (int k = 0; k < 4; ++k) {
    W.S[k] = 0;
    W.V[k] = mk(0.0, 0.0, 0.0);
  }
  bool inside = true;
  int nthru = 0;
  int thru[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i) {
    V3<double> a = s.v[i], b = s.v[(i + 1) % 3];
    V3<double> ab = b - a;
    double l = sqrt(dot(ab, ab));
    V3<double> t = (1.0 / l) * ab;
    V3<double> m = cross(t, n);
    double xa = dot(a - c, t), xb = dot(b - c, t);
    double p = dot(a - c, m);
    if (p < 0) inside = false;
    double w2 = p * p + d * d;
    double ra = sqrt(xa * xa + w2), rb = sqrt(xb * xb + w2);
    double lg;
    if (fabs(p) > tol) {
      lg = log((xb + rb) / (xa + ra));
      double at = atan(d * xb / (p * rb)) - atan(d * xa / (p * ra));
      W.S[0] += -at;
      W.S[1] += p * lg + d * at;
      W.S[2] += 0.5 * p * (xb - xa);
      W.S[3] += p * (xb * rb - xa * ra) / 6.0 + (0.5 * d * d + p * p / 6.0) * p * lg + d * d * d * at / 3.0;
      W.V[1] = W.V[1] + (0.5 * ((xb * rb - xa * ra) + w2 * lg)) * m;
      W.V[2] = W.V[2] + (0.5 * xb * (xb * xb / 3.0 + p * p) - 0.5 * xa * (xa * xa / 3.0 + p * p)) * m;
    } else {
      if (xa * xb < tol * tol) thru[nthru++] = i;
      if (D > tol) {
        lg = log((xb + rb) / (xa + ra));
        W.V[1] = W.V[1] + (0.5 * (xb * rb - xa * ra) + 0.5 * w2 * lg) * m;
      } else {
        lg = (xb > 0) ? log(xb / xa) : log(xa / xb);
        W.V[1] = W.V[1] + (0.5 * (xb * rb - xa * ra)) * m;
      }
      W.V[2] = W.V[2] + (xb * xb * xb / 6.0 - xa * xa * xa / 6.0) * m;
    }
    W.V[0] = W.V[0] + (-lg) * m;
    W.V[3] = W.V[3] + ((xb * rb * rb * rb - xa * ra * ra * ra) / 12.0 + w2 * (xb * rb - xa * ra) / 8.0 +
                       w2 * w2 * lg / 8.0) * m;
  }
  double sgn = D < tol ? 0.0 : (d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0));
  double alpha = 0;
  if (nthru == 0 && inside)
    alpha = 2 * PI;
  else if (nthru == 1)
    alpha = PI;
  else if (nthru == 2) {
    V3<double> e1 = s.v[(thru[0] + 1) % 3] - s.v[thru[0]];
    V3<double> e2 = s.v[(thru[1] + 1) % 3] - s.v[thru[1]];
    double ca = -dot(e1, e2) / sqrt(dot(e1, e1) * dot(e2, e2));
    alpha = acos(fmax(-1.0, fmin(1.0, ca)));
  }
  W.S[0] += alpha * sgn;
  W.S[1] += -alpha * D;
  W.S[3] += -alpha * D * D * D / 3.0;
  W.n = n;
  W.d = d;
}

// singular part at one test point x (barycentrics bx in the test cell, weight dx); returns
// false if not available
SEC_HD bool se_singular(const OpParams& op, int tk, int bk, const Geo& t, const Geo& s,
                     V3<double> x, const double* bx, double dx, C2<double>* acc) {
  Wilton W;
  wilton(s, x, W);
  V3<double> rho = x - W.d * W.n;
  C2<double> g{op.gr, op.gi};
  C2<double> g2 = cmul(g, g);
  C2<double> h = cscale(0.5, g2);
  // grad'(1/R) and grad' R integrated over the trial triangle
  V3<double> gm1 = (-1.0) * (W.V[0] - W.S[0] * W.n);
  V3<double> gR = W.V[1] - (W.d * W.S[1]) * W.n;
  C2<double> al{op.ar, op.ai}, be{op.br, op.bi};
  switch (op.kind) {
    case BEAST_MW_SL: {
      if (tk != BEAST_RT || bk != BEAST_RT) return false;
      // int G = (S1 - g S2 + g^2/2 S3) / 4pi ; int G y = (V1 + S1 rho - g (V2 + S2 rho) + g^2/2 (V3 + S3 rho)) / 4pi
      C2<double> iG = cscale(1.0 / (4 * PI), cadd(csub(C2<double>{W.S[1], 0}, cscale(W.S[2], g)),
                                                  cscale(W.S[3], h)));
      V3<double> a1 = W.V[1] + W.S[1] * rho, a2 = W.V[2] + W.S[2] * rho, a3 = W.V[3] + W.S[3] * rho;
      CV<double> iGy;
      iGy.x = cscale(1.0 / (4 * PI), cadd(csub(C2<double>{a1.x, 0}, cscale(a2.x, g)), cscale(a3.x, h)));
      iGy.y = cscale(1.0 / (4 * PI), cadd(csub(C2<double>{a1.y, 0}, cscale(a2.y, g)), cscale(a3.y, h)));
      iGy.z = cscale(1.0 / (4 * PI), cadd(csub(C2<double>{a1.z, 0}, cscale(a2.z, g)), cscale(a3.z, h)));
      double a = 1.0 / (4.0 * t.area * s.area);
      for (int i = 0; i < 3; ++i) {
        V3<double> gi = x - t.v[i];
        for (int j = 0; j < 3; ++j) {
          V3<double> b = s.v[j];
          CV<double> f;
          f.x = csub(iGy.x, cscale(b.x, iG));
          f.y = csub(iGy.y, cscale(b.y, iG));
          f.z = csub(iGy.z, cscale(b.z, iG));
          C2<double> dg = rdot(gi, f);
          C2<double> v = cadd(cscale(a, cmul(al, dg)), cscale(a * 4.0, cmul(be, iG)));
          acc[i * 3 + j] = cadd(acc[i * 3 + j], cscale(dx, v));
        }
      }
      return true;
    }
    case BEAST_MW_DL: {
      if (tk != BEAST_RT || bk != BEAST_RT) return false;
      // int grad_x G_s = -(grad'(1/R) + g^2/2 grad'R) / 4pi
      CV<double> iDG;
      iDG.x = cscale(-1.0 / (4 * PI), cadd(C2<double>{gm1.x, 0}, cscale(gR.x, h)));
      iDG.y = cscale(-1.0 / (4 * PI), cadd(C2<double>{gm1.y, 0}, cscale(gR.y, h)));
      iDG.z = cscale(-1.0 / (4 * PI), cadd(C2<double>{gm1.z, 0}, cscale(gR.z, h)));
      double a = 1.0 / (4.0 * t.area * s.area);
      for (int i = 0; i < 3; ++i) {
        V3<double> gi = x - t.v[i];
        for (int j = 0; j < 3; ++j) {
          V3<double> cr = cross(x - s.v[j], gi);
          acc[i * 3 + j] = cadd(acc[i * 3 + j], cscale(a * dx, rdot(cr, iDG)));
        }
      }
      return true;
    }
    case BEAST_HH_SL: {
      // src/helmholtz3d/wiltonints.jl:19-135: P0 or P1 on either side; a P1 trial shape's
      // integrals against 1/R and R come from the first-order potential integrals (se_p1.h),
      // a P1 test shape is the barycentric coordinate of x
      const int nt = tk == BEAST_P0 ? 1 : 3, nb = bk == BEAST_P0 ? 1 : 3;
      C2<double> iG[3];
      if (bk == BEAST_P0) {
        iG[0] = cscale(1.0 / (4 * PI), cadd(C2<double>{W.S[1], 0}, cscale(W.S[3], h)));
      } else {
        const double v[3][3] = {{s.v[0].x, s.v[0].y, s.v[0].z}, {s.v[1].x, s.v[1].y, s.v[1].z},
                                {s.v[2].x, s.v[2].y, s.v[2].z}};
        const double nn[3] = {W.n.x, W.n.y, W.n.z}, rr[3] = {rho.x, rho.y, rho.z};
        const double v1[3] = {W.V[1].x, W.V[1].y, W.V[1].z}, v3[3] = {W.V[3].x, W.V[3].y, W.V[3].z};
        double i1[3], i3[3];
        se_p1_moments(v, nn, rr, W.S[1], W.S[3], v1, v3, i1, i3);
        for (int j = 0; j < 3; ++j) iG[j] = cscale(1.0 / (4 * PI), cadd(C2<double>{i1[j], 0}, cscale(i3[j], h)));
      }
      for (int i = 0; i < nt; ++i) {
        const double ft = tk == BEAST_P0 ? 1.0 : bx[i];
        for (int j = 0; j < nb; ++j) acc[i * nb + j] = cadd(acc[i * nb + j], cscale(dx * ft, cmul(al, iG[j])));
      }
      return true;
    }
    case BEAST_HH_DL:
    case BEAST_HH_DLT: {
      // P0 or P1 test shapes (a factor: the barycentric coordinate of x).  P1 trial shapes
      // (se_p1.h): for the double layer the source normal is constant on the flat trial triangle;
      // the transposed double layer adds the in-plane second moments of rho' - rho.
      const int nt = tk == BEAST_P0 ? 1 : 3, nb = bk == BEAST_P0 ? 1 : 3;
      C2<double> v[3];
      if (bk == BEAST_P0) {
        CV<double> iDG;
        iDG.x = cscale(-1.0 / (4 * PI), cadd(C2<double>{gm1.x, 0}, cscale(gR.x, h)));
        iDG.y = cscale(-1.0 / (4 * PI), cadd(C2<double>{gm1.y, 0}, cscale(gR.y, h)));
        iDG.z = cscale(-1.0 / (4 * PI), cadd(C2<double>{gm1.z, 0}, cscale(gR.z, h)));
        if (op.kind == BEAST_HH_DL)
          v[0] = cscale(-1.0, rdot(s.n, iDG));
        else
          v[0] = rdot(t.n, iDG);
      } else {
        const double sv[3][3] = {{s.v[0].x, s.v[0].y, s.v[0].z}, {s.v[1].x, s.v[1].y, s.v[1].z},
                                 {s.v[2].x, s.v[2].y, s.v[2].z}};
        const double nn[3] = {W.n.x, W.n.y, W.n.z}, rr[3] = {rho.x, rho.y, rho.z};
        const double v0[3] = {W.V[0].x, W.V[0].y, W.V[0].z}, v1[3] = {W.V[1].x, W.V[1].y, W.V[1].z};
        double iA[3], iB[3];
        if (op.kind == BEAST_HH_DL) {
          se_p1_dl_moments(sv, nn, rr, W.d, W.S[0], W.S[1], v0, v1, iA, iB);
          for (int j = 0; j < 3; ++j) v[j] = cscale(1.0 / (4 * PI), csub(C2<double>{iA[j], 0}, cscale(iB[j], h)));
        } else {
          // -(nx . int lambda_j grad'(1/R) + h nx . int lambda_j grad' R) / (4 pi)
          const double nx[3] = {t.n.x, t.n.y, t.n.z};
          se_p1_dlt_moments(sv, nn, rr, W.d, W.S[0], W.S[1], W.S[3], v0, v1, nx, iA, iB);
          for (int j = 0; j < 3; ++j) v[j] = cscale(-1.0 / (4 * PI), cadd(C2<double>{iA[j], 0}, cscale(iB[j], h)));
        }
      }
      for (int i = 0; i < nt; ++i) {
        const double ft = tk == BEAST_P0 ? 1.0 : bx[i];
        for (int j = 0; j < nb; ++j) acc[i * nb + j] = cadd(acc[i * nb + j], cscale(dx * ft, cmul(al, v[j])));
      }
      return true;
    }
  }
  return false;
}

}  // namespace
