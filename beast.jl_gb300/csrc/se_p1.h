// Singularity extraction with P1 (barycentric) trial shapes: the integrals of the shapes against
// 1/R and R over the trial triangle, from the first-order potential integrals of Wilton et al.
// (1984).  A shape is affine in the plane, lambda_j(y) = lambda_j(rho) + grad lambda_j . (y - rho)
// with rho the projection of the observation point on the plane, so
//   int lambda_j / R = lambda_j(rho) S1 + grad lambda_j . V1,
//   int lambda_j R   = lambda_j(rho) S3 + grad lambda_j . V3,
// S1 = int 1/R, S3 = int R, V1 = int (rho' - rho)/R, V3 = int (rho' - rho) R.  (The reference
// takes these from WiltonInts84.higherorder, src/helmholtz3d/wiltonints.jl:77-135.)
#pragma once

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
