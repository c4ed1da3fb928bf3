// EFIE (MWSingleLayer3D) far-pair block of RT x RT shapes in double-float arithmetic: the
// quadrature of DoubleQuadRule (src/quadrature/doublenumints.jl:12-43) applied to the
// integrand of src/maxwell/mwops.jl:100-117,
//   z_ij = sum_a sum_b w_a w_b G(x_a - y_b) [alpha/4 (x_a - v_i).(y_b - w_j) + beta],
// reduced to moments about the cell centroids as in the FP32 / FP64 far kernels:
//   x_a = c_p + xi_a, y_b = c_q + eta_b, v_i = c_p + tau_i, w_j = c_q + sig_j,
//   M0 = sum G, V1 = sum G xi, V2 = sum G eta, M1 = sum G xi.eta (weights included),
//   z_ij = alpha/4 (M1 - sig_j.V1 - tau_i.V2 + (tau_i.sig_j) M0) + beta M0.
// Every step is a pair operation of dfloat.h, so the block is good to about 1e-11 relative
// (against ~1e-7 for the FP32 kernel) while running on the FP32 pipes.  Inputs are pairs
// (from double geometry); the caller supplies d = c_p - c_q, the rule points relative to
// their centroids and the weights.  Host and device builds round alike.
#pragma once
#include "dfloat.h"

namespace dfl {

struct cdf {
  df re, im;
};
DF_HD cdf cadd(cdf a, cdf b) { return {add(a.re, b.re), add(a.im, b.im)}; }
DF_HD cdf csub(cdf a, cdf b) { return {sub(a.re, b.re), sub(a.im, b.im)}; }
DF_HD cdf cscale(cdf a, df s) { return {mul(a.re, s), mul(a.im, s)}; }
DF_HD cdf cmul(cdf a, cdf b) {
  return {sub(mul(a.re, b.re), mul(a.im, b.im)), add(mul(a.re, b.im), mul(a.im, b.re))};
}
DF_HD df dot3(const df* a, const df* b) { return add(add(mul(a[0], b[0]), mul(a[1], b[1])), mul(a[2], b[2])); }

// out[3 i + j] = z_ij.  d[3]: c_p - c_q; tau[3][3], sig[3][3]: cell vertices minus centroid;
// xi[no][3], wo[no]: test rule points minus c_p and weights; eta[ni][3], wi[ni]: trial rule
// points minus c_q and weights; k: real wavenumber (gamma = i k); alpha, beta: operator
// coefficients.
DF_HD void efie_far_pair(const df* d, const df (*tau)[3], const df (*sig)[3], int no, const df (*xi)[3],
                         const df* wo, int ni, const df (*eta)[3], const df* wi, df k, cdf alpha, cdf beta,
                         cdf* out) {
  const df z0 = make(0.f);
  cdf M0{z0, z0}, M1{z0, z0}, V1[3], V2[3];
  for (int c = 0; c < 3; ++c) V1[c] = V2[c] = cdf{z0, z0};
  for (int a = 0; a < no; ++a) {
    df dx[3];
    for (int c = 0; c < 3; ++c) dx[c] = add(d[c], xi[a][c]);
    cdf U0{z0, z0}, U1[3];
    for (int c = 0; c < 3; ++c) U1[c] = cdf{z0, z0};
    for (int b = 0; b < ni; ++b) {
      df r[3];
      for (int c = 0; c < 3; ++c) r[c] = sub(dx[c], eta[b][c]);
      const df R = norm3(r[0], r[1], r[2]);
      cdf G;
      green(R, k, &G.re, &G.im);
      const cdf K = cscale(G, wi[b]);
      U0 = cadd(U0, K);
      for (int c = 0; c < 3; ++c) U1[c] = cadd(U1[c], cscale(K, eta[b][c]));
    }
    const cdf s0 = cscale(U0, wo[a]);
    M0 = cadd(M0, s0);
    cdf xu{z0, z0};
    for (int c = 0; c < 3; ++c) {
      V1[c] = cadd(V1[c], cscale(s0, xi[a][c]));
      const cdf u = cscale(U1[c], wo[a]);
      V2[c] = cadd(V2[c], u);
      xu = cadd(xu, cscale(u, xi[a][c]));
    }
    M1 = cadd(M1, xu);
  }
  const cdf a4{scale(alpha.re, 0.25f), scale(alpha.im, 0.25f)};
  const cdf bM0 = cmul(beta, M0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      cdf sV1{z0, z0}, tV2{z0, z0};
      for (int c = 0; c < 3; ++c) {
        sV1 = cadd(sV1, cscale(V1[c], sig[j][c]));
        tV2 = cadd(tV2, cscale(V2[c], tau[i][c]));
      }
      const cdf f = cadd(csub(csub(M1, sV1), tV2), cscale(M0, dot3(tau[i], sig[j])));
      out[3 * i + j] = cadd(cmul(a4, f), bM0);
    }
}

}  // namespace dfl
