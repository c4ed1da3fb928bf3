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

// The same block for rule sizes known at compile time (the default far rules: NO = 3 test and
// NI = 4 trial points), with the work per point pair cut down:
//   * R^2 = (A_a + Q_b) - 2 P_ab with A_a = |d + xi_a|^2 (per test point), Q_b = |eta_b|^2 -
//     2 d.eta_b (per trial point) and P_ab = xi_a.eta_b, which the M1 moment needs anyway;
//   * 1 / R from a pair reciprocal square root, R = R^2 / R, and both weights in one table,
//     wab[a][b] = w_a w_b / (4 pi) (rule constants), so that a term is wab / R exp(-i k R);
//   * sums whose terms do not cancel far below their size (dot products of small vectors, the
//     angle sum of the sine / cosine) as sloppy pair sums, the moments as running sums
//     normalised once, and products that feed a sum or another product left unnormalised;
//   * the table of sin / cos(m pi/32) read from `tab` (shared memory in the kernel);
//   * the 3 x 3 block from per-row and per-column parts: z_ij = C - S_j - T_i + (tau_i.sig_j) D
//     with C = a4 M1 + beta M0, S_j = a4 sig_j.V1, T_i = a4 tau_i.V2, D = a4 M0, a4 = alpha/4.
// eta2[b] = |eta_b|^2 (staged with the trial cell).  Matches efie_far_pair to the pair
// arithmetic's accuracy.
DF_HD cdf cadds(cdf a, cdf b) { return {adds(a.re, b.re), adds(a.im, b.im)}; }
// running complex sums, normalised once at the end (acc / norm of dfloat.h)
DF_HD void cacc(cdf& a, cdf x) {
  acc(a.re, x.re);
  acc(a.im, x.im);
}
DF_HD cdf cnorm(cdf a) { return {norm(a.re), norm(a.im)}; }
DF_HD cdf csubs(cdf a, cdf b) { return {subs(a.re, b.re), subs(a.im, b.im)}; }
// unnormalised products (mulu) for operands of sums and products
DF_HD cdf cscaleu(cdf a, df s) { return {mulu(a.re, s), mulu(a.im, s)}; }
DF_HD cdf cmulu(cdf a, cdf b) {
  return {subs(mulu(a.re, b.re), mulu(a.im, b.im)), adds(mulu(a.re, b.im), mulu(a.im, b.re))};
}
DF_HD df dot3s(const df* a, const df* b) { return adds(adds(mul(a[0], b[0]), mul(a[1], b[1])), mul(a[2], b[2])); }
DF_HD df dot3u(const df* a, const df* b) { return adds(adds(mulu(a[0], b[0]), mulu(a[1], b[1])), mulu(a[2], b[2])); }
DF_HD cdf cdot3u(const cdf* v, const df* b) {
  return cadds(cadds(cscaleu(v[0], b[0]), cscaleu(v[1], b[1])), cscaleu(v[2], b[2]));
}
// wab[a][b] = w_a w_b / (4 pi) for the fast core (the same products on host and device)
template <int NO, int NI>
DF_HD void efie_far_weights(const df* wo, const df* wi, df (*wab)[NI]) {
  const df i4pi{DF_I4PI_HI, DF_I4PI_LO};
  for (int a = 0; a < NO; ++a)
    for (int b = 0; b < NI; ++b) wab[a][b] = mul(mul(wo[a], wi[b]), i4pi);
}

template <int NO, int NI>
DF_HD void efie_far_pair_fast(const df* d, const df (*tau)[3], const df (*sig)[3], const df (*xi)[3],
                              const df (*wab)[NI], const df (*eta)[3], const df* eta2, df k, cdf alpha, cdf beta,
                              const float (*tab)[4], cdf* out) {
  // The loops stay rolled: unrolled (even over the three test points alone), the kernel comes
  // to thousands of instructions and its warps stall on instruction fetch (measured: 12.2 ms
  // fully unrolled, 9.2 ms with the test points unrolled, 7.5 ms rolled, at 5120 cells).
  const df z0 = make(0.f);
  df A[NO];
  cdf U0[NO];  // sum over b of the terms of test point a (its weight included)
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
  for (int a = 0; a < NO; ++a) {
    df dx[3];
    for (int c = 0; c < 3; ++c) dx[c] = adds(d[c], xi[a][c]);  // |d| >> |xi|: no cancellation
    A[a] = dot3u(dx, dx);
    U0[a] = cdf{z0, z0};
  }
  cdf M0{z0, z0}, M1{z0, z0}, V2[3];
  for (int c = 0; c < 3; ++c) V2[c] = cdf{z0, z0};
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
  for (int b = 0; b < NI; ++b) {
    // Q, P, R^2, 1 / R and the sine / cosine left unnormalised: their consumers are running
    // sums and pair products (the reciprocal square root's, R, k R, the amplitude, K, K P)
    df Q = mulu(d[0], eta[b][0]);
    acc(Q, mulu(d[1], eta[b][1]));
    acc(Q, mulu(d[2], eta[b][2]));
    Q = addu(eta2[b], scale(Q, -2.f));
    cdf T{z0, z0};
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
    for (int a = 0; a < NO; ++a) {
      df P = mulu(xi[a][0], eta[b][0]);
      acc(P, mulu(xi[a][1], eta[b][1]));
      acc(P, mulu(xi[a][2], eta[b][2]));
      df R2 = A[a];
      acc(R2, Q);
      acc(R2, scale(P, -2.f));
      const df iR = rsqrtu(R2);
      const df R = mulu(R2, iR);
      df sn, cs;
      sincos_tab<false>(mulu(k, R), tab, &sn, &cs);
      const df amp = mulu(iR, wab[a][b]);  // w_a w_b / (4 pi R)
      const cdf K{mulu(amp, cs), neg(mulu(amp, sn))};
      cacc(U0[a], K);
      cacc(T, K);
      cacc(M1, cscaleu(K, P));
    }
    T = cnorm(T);
    cacc(M0, T);
    for (int c = 0; c < 3; ++c) cacc(V2[c], cscaleu(T, eta[b][c]));
  }
  M0 = cnorm(M0);
  M1 = cnorm(M1);
  for (int c = 0; c < 3; ++c) V2[c] = cnorm(V2[c]);
  cdf V1[3];
  for (int c = 0; c < 3; ++c) V1[c] = cdf{z0, z0};
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
  for (int a = 0; a < NO; ++a) {
    const cdf s = cnorm(U0[a]);
    for (int c = 0; c < 3; ++c) cacc(V1[c], cscaleu(s, xi[a][c]));
  }
  for (int c = 0; c < 3; ++c) V1[c] = cnorm(V1[c]);
  const cdf a4{scale(alpha.re, 0.25f), scale(alpha.im, 0.25f)};
  const cdf C = cadds(cmulu(a4, M1), cmulu(beta, M0));
  const cdf D = cmulu(a4, M0);
  cdf S[3];
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
  for (int j = 0; j < 3; ++j) S[j] = cmulu(a4, cdot3u(V1, sig[j]));
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
  for (int i = 0; i < 3; ++i) {
    const cdf Ti = cmulu(a4, cdot3u(V2, tau[i]));
    const cdf Ci = csubs(C, Ti);
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
    for (int j = 0; j < 3; ++j) out[3 * i + j] = cadds(csubs(Ci, S[j]), cscaleu(D, dot3u(tau[i], sig[j])));
  }
}

// The same block for the balanced mode: the Green's-function values in double-float, the beta
// (divergence) term beta M0 in double-float, the alpha (vector-potential) term in FP32.  An RT
// entry sums four cell-pair blocks with signs; their beta terms cancel there to a second
// difference of the Green's function (the divergences integrate to zero) and need the
// double-float values, while their alpha terms do not cancel, so FP32 moments and an FP32
// finish (relative error ~1e-7 of the alpha term) cost the entry about what rounding it to
// FP32 would -- at a fraction of the pair sums of efie_far_pair_fast.  Same arguments.
struct cf {  // complex FP32 (host and device)
  float x, y;
};
DF_HD float f32(df a) { return add_rn(a.hi, a.lo); }
DF_HD cf cmulf(cf a, cf b) { return {fmaf(a.x, b.x, -mul_rn(a.y, b.y)), fmaf(a.x, b.y, mul_rn(a.y, b.x))}; }
template <int NO, int NI>
DF_HD void efie_far_pair_beta(const df* d, const df (*tau)[3], const df (*sig)[3], const df (*xi)[3],
                              const df (*wab)[NI], const df (*eta)[3], const df* eta2, df k, cdf alpha, cdf beta,
                              const float (*tab)[4], cdf* out) {
  // Test points outside, trial points inside: every per-test-point value (x_a - c_q, its square,
  // the U0 sum) lives in registers for one pass of the inner loop, and the trial points come
  // from the caller's shared-memory record, so nothing is indexed by a rolled loop's counter in
  // thread-local arrays.  R^2 = |d + xi_a|^2 + |eta_b|^2 - 2 (d + xi_a).eta_b.
  const df z0 = make(0.f);
  cdf M0{z0, z0};  // the beta term's moment, double-float running sum over all point pairs
  cf M1 = cf{0.f, 0.f}, V1[3], V2[3];
  for (int c = 0; c < 3; ++c) V1[c] = V2[c] = cf{0.f, 0.f};
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
  for (int a = 0; a < NO; ++a) {
    df dx[3];
    float xf[3];
    for (int c = 0; c < 3; ++c) {
      dx[c] = adds(d[c], xi[a][c]);
      xf[c] = f32(xi[a][c]);
    }
    const df A = dot3u(dx, dx);
    cf U0 = cf{0.f, 0.f};  // FP32 sum over b of the terms of test point a
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
    for (int b = 0; b < NI; ++b) {
      // R^2, 1 / R and the sine / cosine left unnormalised: their consumers are pair
      // products (the reciprocal square root's, R, k R, the amplitude and K)
      df Pd = mulu(dx[0], eta[b][0]);
      acc(Pd, mulu(dx[1], eta[b][1]));
      acc(Pd, mulu(dx[2], eta[b][2]));
      df R2 = A;
      acc(R2, eta2[b]);
      acc(R2, scale(Pd, -2.f));
      const df iR = rsqrtu(R2);
      const df R = mulu(R2, iR);
      df sn, cs;
      sincos_tab<false>(mulu(k, R), tab, &sn, &cs);
      const df amp = mulu(iR, wab[a][b]);
      const cdf K{mulu(amp, cs), neg(mulu(amp, sn))};
      cacc(M0, K);
      const float kr = f32(K.re), ki = f32(K.im);
      float ef[3];
      for (int c = 0; c < 3; ++c) ef[c] = f32(eta[b][c]);
      const float p = fmaf(xf[0], ef[0], fmaf(xf[1], ef[1], xf[2] * ef[2]));
      U0.x += kr;
      U0.y += ki;
      M1.x = fmaf(kr, p, M1.x);
      M1.y = fmaf(ki, p, M1.y);
      for (int c = 0; c < 3; ++c) {
        V2[c].x = fmaf(kr, ef[c], V2[c].x);
        V2[c].y = fmaf(ki, ef[c], V2[c].y);
      }
    }
    for (int c = 0; c < 3; ++c) {
      V1[c].x = fmaf(U0.x, xf[c], V1[c].x);
      V1[c].y = fmaf(U0.y, xf[c], V1[c].y);
    }
  }
  M0 = cnorm(M0);
  // alpha term in FP32: a4 (M1 - sig_j.V1 - tau_i.V2 + (tau_i.sig_j) M0)
  const cf a4 = cf{0.25f * f32(alpha.re), 0.25f * f32(alpha.im)};
  const cf C = cmulf(a4, M1), D = cmulf(a4, cf{f32(M0.re), f32(M0.im)});
  float ts[3][3], ss[3][3];
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) {
      ts[i][c] = f32(tau[i][c]);
      ss[i][c] = f32(sig[i][c]);
    }
  cf S[3], Tm[3];
  for (int j = 0; j < 3; ++j) {
    cf sv = cf{0.f, 0.f}, tv = cf{0.f, 0.f};
    for (int c = 0; c < 3; ++c) {
      sv.x = fmaf(ss[j][c], V1[c].x, sv.x);
      sv.y = fmaf(ss[j][c], V1[c].y, sv.y);
      tv.x = fmaf(ts[j][c], V2[c].x, tv.x);
      tv.y = fmaf(ts[j][c], V2[c].y, tv.y);
    }
    S[j] = cmulf(a4, sv);
    Tm[j] = cmulf(a4, tv);
  }
  // beta term in double-float, once per pair
  const cdf bM0 = cmulu(beta, M0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const float g = fmaf(ts[i][0], ss[j][0], fmaf(ts[i][1], ss[j][1], ts[i][2] * ss[j][2]));
      const float zr = C.x - S[j].x - Tm[i].x + g * D.x;
      const float zi = C.y - S[j].y - Tm[i].y + g * D.y;
      out[3 * i + j] = cdf{add(bM0.re, zr), add(bM0.im, zi)};
    }
}

}  // namespace dfl
