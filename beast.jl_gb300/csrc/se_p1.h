// Singularity extraction with P1 (barycentric) trial shapes: the integrals of the shapes against
// 1/R and R over the trial triangle, from the first-order potential integrals of Wilton et al.
// (1984).  A shape is affine in the plane, lambda_j(y) = lambda_j(rho) + grad lambda_j . (y - rho)
// with rho the projection of the observation point on the plane, so
//   int lambda_j / R = lambda_j(rho) S1 + grad lambda_j . V1,
//   int lambda_j R   = lambda_j(rho) S3 + grad lambda_j . V3,
// S1 = int 1/R, S3 = int R, V1 = int (rho' - rho)/R, V3 = int (rho' - rho) R.  (The reference
// takes these from WiltonInts84.higherorder, src/helmholtz3d/wiltonints.jl:77-135.)
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define SEP1_HD __host__ __device__ __forceinline__
#else
#define SEP1_HD inline
#endif

// v: trial vertices [3][3]; n: unit normal of (v1 - v0) x (v2 - v0); rho: projection of the
// observation point; out1[j] = int lambda_j / R, out3[j] = int lambda_j R
SEP1_HD void se_p1_moments(const double (*v)[3], const double* n, const double* rho, double S1, double S3,
                           const double* V1, const double* V3, double* out1, double* out3) {
  auto cr = [](const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  };
  double e1[3], e2[3], c[3];
  for (int k = 0; k < 3; ++k) {
    e1[k] = v[1][k] - v[0][k];
    e2[k] = v[2][k] - v[0][k];
  }
  cr(e1, e2, c);
  const double a2 = c[0] * n[0] + c[1] * n[1] + c[2] * n[2];  // twice the area
  for (int j = 0; j < 3; ++j) {
    const double* a = v[(j + 1) % 3];
    const double* b = v[(j + 2) % 3];
    double ar[3], br[3], ab[3], g[3];
    for (int k = 0; k < 3; ++k) {
      ar[k] = a[k] - rho[k];
      br[k] = b[k] - rho[k];
      ab[k] = b[k] - a[k];
    }
    cr(ar, br, c);
    const double lr = (c[0] * n[0] + c[1] * n[1] + c[2] * n[2]) / a2;  // lambda_j(rho)
    cr(n, ab, g);                                                       // 2A grad lambda_j
    out1[j] = lr * S1 + (g[0] * V1[0] + g[1] * V1[1] + g[2] * V1[2]) / a2;
    out3[j] = lr * S3 + (g[0] * V3[0] + g[1] * V3[1] + g[2] * V3[2]) / a2;
  }
}

// Double layer (normal derivative at the source, flat trial triangle): with d = n.(x - y), the
// same for every y of the triangle, n.grad_y(1/R) = d/R^3 and n.grad_y R = -d/R, so
//   outA[j] = int lambda_j d / R^3 = lambda_j(rho) S0 + d grad lambda_j . V0,
//   outB[j] = int lambda_j d / R   = d (lambda_j(rho) S1 + grad lambda_j . V1),
// S0 = int d / R^3 (the signed solid angle), V0 = int (rho' - rho) / R^3.
SEP1_HD void se_p1_dl_moments(const double (*v)[3], const double* n, const double* rho, double d, double S0,
                              double S1, const double* V0, const double* V1, double* outA, double* outB) {
  double l1[3], l3[3];
  // lambda_j(rho) and grad lambda_j . V through se_p1_moments with (S, V) = (S0, V0), (S1, V1)
  se_p1_moments(v, n, rho, S0, S1, V0, V1, l1, l3);
  // l1[j] = lambda_j(rho) S0 + g.V0 and l3[j] = lambda_j(rho) S1 + g.V1: scale the V0 part by d
  double z3[3] = {0, 0, 0}, lr0[3], lr1[3];
  se_p1_moments(v, n, rho, 1.0, 0.0, z3, z3, lr0, lr1);  // lr0[j] = lambda_j(rho)
  for (int j = 0; j < 3; ++j) {
    outA[j] = lr0[j] * S0 + d * (l1[j] - lr0[j] * S0);
    outB[j] = d * l3[j];
  }
}

// In-plane second moments over the trial triangle, u = rho' - rho (rho the projection of the
// observation point, d its signed distance from the plane):
//   Mm3 = int u u^T / R^3 = P S1 - sum_e (int_e u / R ds) m_e^T,
//   M1  = int u u^T / R   = sum_e (int_e u R ds) m_e^T - P S3,
// from d_l(u_k / R) = delta_kl / R - u_k u_l / R^3 and d_l(u_k R) = delta_kl R + u_k u_l / R
// integrated over the triangle (divergence theorem; P = I - n n^T, m_e the outward in-plane edge
// normal).  On an edge with tangent t, u = p m + s t for s from sa to sb (p = (a - rho).m), and
//   int_e u / R ds = p L m + (rb - ra) t,   int_e u R ds = p (s R + w2 L)/2 |sa..sb m + (rb^3 - ra^3)/3 t,
// with w2 = p^2 + d^2, ra, rb the distances of the edge ends and L = int_e ds / R.
SEP1_HD void se_p1_second_moments(const double (*v)[3], const double* n, const double* rho, double d, double S1,
                                  double S3, double (*Mm3)[3], double (*M1)[3]) {
  for (int k = 0; k < 3; ++k)
    for (int l = 0; l < 3; ++l) {
      const double P = (k == l ? 1.0 : 0.0) - n[k] * n[l];
      Mm3[k][l] = P * S1;
      M1[k][l] = -P * S3;
    }
  for (int e = 0; e < 3; ++e) {
    const double* a = v[e];
    const double* b = v[(e + 1) % 3];
    double t[3], m[3], len = 0;
    for (int k = 0; k < 3; ++k) {
      t[k] = b[k] - a[k];
      len += t[k] * t[k];
    }
    len = sqrt(len);
    for (int k = 0; k < 3; ++k) t[k] /= len;
    m[0] = t[1] * n[2] - t[2] * n[1];  // t x n: outward for a counter-clockwise triangle about n
    m[1] = t[2] * n[0] - t[0] * n[2];
    m[2] = t[0] * n[1] - t[1] * n[0];
    double sa = 0, sb = 0, p = 0;
    for (int k = 0; k < 3; ++k) {
      sa += (a[k] - rho[k]) * t[k];
      sb += (b[k] - rho[k]) * t[k];
      p += (a[k] - rho[k]) * m[k];
    }
    const double w2 = p * p + d * d;
    const double ra = sqrt(sa * sa + w2), rb = sqrt(sb * sb + w2);
    // L = ln((sb + rb) / (sa + ra)), in the form without cancellation
    const double L = (sa + sb >= 0) ? log((sb + rb) / (sa + ra)) : log((ra - sa) / (rb - sb));
    const double IR = 0.5 * (sb * rb - sa * ra + w2 * L);
    double f1[3], f3[3];
    for (int k = 0; k < 3; ++k) {
      f1[k] = p * L * m[k] + (rb - ra) * t[k];
      f3[k] = p * IR * m[k] + (rb * rb * rb - ra * ra * ra) / 3.0 * t[k];
    }
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) {
        Mm3[k][l] -= f1[k] * m[l];
        M1[k][l] += f3[k] * m[l];
      }
  }
}

// Transposed double layer (normal derivative at the observation point, test normal nx) with P1
// trial shapes: with grad_y(1/R) = (d n - u)/R^3 and grad_y R = (u - d n)/R,
//   int lambda_j grad_y(1/R) = -(lambda_j(rho) V0 + Mm3 grad lambda_j) + n int lambda_j d / R^3,
//   int lambda_j grad_y R    =  (lambda_j(rho) V1 + M1 grad lambda_j)  - n int lambda_j d / R,
// and outA[j], outB[j] are their components along nx.
SEP1_HD void se_p1_dlt_moments(const double (*v)[3], const double* n, const double* rho, double d, double S0,
                               double S1, double S3, const double* V0, const double* V1, const double* nx,
                               double* outA, double* outB) {
  double iA[3], iB[3], Mm3[3][3], M1[3][3], z3[3] = {0, 0, 0}, lr[3], unused[3];
  se_p1_dl_moments(v, n, rho, d, S0, S1, V0, V1, iA, iB);
  se_p1_second_moments(v, n, rho, d, S1, S3, Mm3, M1);
  se_p1_moments(v, n, rho, 1.0, 0.0, z3, z3, lr, unused);  // lr[j] = lambda_j(rho)
  double e1[3], e2[3], c[3];
  for (int k = 0; k < 3; ++k) {
    e1[k] = v[1][k] - v[0][k];
    e2[k] = v[2][k] - v[0][k];
  }
  c[0] = e1[1] * e2[2] - e1[2] * e2[1];
  c[1] = e1[2] * e2[0] - e1[0] * e2[2];
  c[2] = e1[0] * e2[1] - e1[1] * e2[0];
  const double a2 = c[0] * n[0] + c[1] * n[1] + c[2] * n[2];
  const double nxn = nx[0] * n[0] + nx[1] * n[1] + nx[2] * n[2];
  for (int j = 0; j < 3; ++j) {
    const double* a = v[(j + 1) % 3];
    const double* b = v[(j + 2) % 3];
    const double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const double g[3] = {(n[1] * ab[2] - n[2] * ab[1]) / a2, (n[2] * ab[0] - n[0] * ab[2]) / a2,
                         (n[0] * ab[1] - n[1] * ab[0]) / a2};  // grad lambda_j
    double g1 = 0, gr = 0;
    for (int k = 0; k < 3; ++k) {
      const double m3g = Mm3[k][0] * g[0] + Mm3[k][1] * g[1] + Mm3[k][2] * g[2];
      const double m1g = M1[k][0] * g[0] + M1[k][1] * g[1] + M1[k][2] * g[2];
      g1 += nx[k] * (-(lr[j] * V0[k] + m3g));
      gr += nx[k] * (lr[j] * V1[k] + m1g);
    }
    outA[j] = g1 + nxn * iA[j];
    outB[j] = gr - nxn * iB[j];
  }
}
