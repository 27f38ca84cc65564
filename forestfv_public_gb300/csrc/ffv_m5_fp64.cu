// Model-5 (six-equation multi-material flow with hyperelastic solids, ghost-fluid
// coupling, pressure relaxation) FP64 stage kernels.
//
// Compiled with --fmad=false and written in the operation order of the reference's C
// code (m5_*.c, state_equation.c, F_pe-free relaxation modes 1 and 3), so that the only
// rounding differences from the reference come from pow(): CUDA's and glibc's pow differ
// in the last bit for some arguments.
//
// One stage:
//   m5_recon_face   (cell, face)  MUSCL face state + face-state pressure relaxation
//                                  (m5_faceinterp_V1 / m5_reconctruct_V1 / m5_relaxationvec)
//   m5_face_flux    (cell, face)  HLLC or ghost-fluid HLLC per face or subface; a 1:1 face
//                                  is evaluated once, by the cell first in leaf order, and
//                                  the other takes its negative (the reference's flux
//                                  reuse, m5_residual.c:59-173)
//   m5_cell_update  (cell)        residual sum + non-conservative terms (m5_residual.c:175-215),
//                                  RK stage (m5_RK.c), positivity and ZEROU masks
//   compaction + m5_gfm_seq       cells whose solid fraction crosses AVF_LIM in stage 1, in
//                                  leaf order (m5_gfm.c reads earlier neighbours' new state)
//   m5_relax_cell   (cell)        cell pressure relaxation (m5_relaxation_solid.c)
//   compaction + m5_gfm_rel_seq   relaxation-crossing cells in leaf order (m5_gfm_rel.c)
#include <math.h>

#include "ffv_device.cuh"
#include "ffv_m5.cuh"
#include "ffv_m5_frame.cuh"
#include "ffv_plastic.cuh"

namespace {

// ------------------------------------------------------------------ EOS (state_equation.c)
__device__ __forceinline__ void gmat_of(const double A[9], double G[9], double &Gmag) {
  G[0] = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
  G[1] = A[0] * A[3] + A[1] * A[4] + A[2] * A[5];
  G[2] = A[0] * A[6] + A[1] * A[7] + A[2] * A[8];
  G[3] = A[3] * A[0] + A[4] * A[1] + A[5] * A[2];
  G[4] = A[3] * A[3] + A[4] * A[4] + A[5] * A[5];
  G[5] = A[3] * A[6] + A[4] * A[7] + A[5] * A[8];
  G[6] = A[6] * A[0] + A[7] * A[1] + A[8] * A[2];
  G[7] = A[6] * A[3] + A[7] * A[4] + A[8] * A[5];
  G[8] = A[6] * A[6] + A[7] * A[7] + A[8] * A[8];
  Gmag = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
         G[2] * (G[3] * G[7] - G[4] * G[6]);
}

// state_equation.c:269-317 and :217-267 (need_mu: the G_det form's extra mu != 0 test)
__device__ double elastic_energy(const double G[9], double Gmag, double mu, bool need_mu) {
  if (!(fabs(Gmag) != 0.0) || (need_mu && !(mu != 0.0))) return 0.0;
  double g13 = pow(fabs(Gmag), 1.0 / 3.0);
  if (isnan(g13)) g13 = 0.0;
  const double M1[9] = {G[0] - g13, G[1], G[2], G[3], G[4] - g13, G[5], G[6], G[7], G[8] - g13};
  double M2[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int j = 0; j < 3; ++j) M2[i * 3 + j] += M1[i * 3 + k] * M1[k * 3 + j];
  const double tr1 = M2[0] + M2[4] + M2[8];
  return mu / (4.0 * pow(fabs(Gmag), 1.0 / 6.0)) * tr1;
}

// state_equation.c:143-204, accumulated into st (and stored in ast when given)
__device__ void eos_stress_acc(double st[3][3], double avf, double pr, const double G[9],
                               double Gmag, double mu, double (*ast)[3]) {
  double s[3][3];
  if ((fabs(Gmag) != 0.0) && (mu != 0.0)) {
    double G2[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) G2[i * 3 + j] += G[i * 3 + k] * G[k * 3 + j];
    const double J1 = G[0] + G[4] + G[8], J2 = G2[0] + G2[4] + G2[8];
    const double p13 = pow(fabs(Gmag), 1.0 / 3.0);
    const double f = mu / pow(fabs(Gmag), 1.0 / 6.0);
#pragma unroll
    for (int q = 0; q < 9; q++) {
      const double ss = (q == 0 || q == 4 || q == 8) ? G2[q] - J2 / 3.0 - p13 * (G[q] - J1 / 3.0)
                                                     : G2[q] - p13 * (G[q]);
      s[q / 3][q % 3] = (q == 0 || q == 4 || q == 8) ? -avf * pr - f * (ss) : -f * (ss);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 9; q++) s[q / 3][q % 3] = (q == 0 || q == 4 || q == 8) ? -avf * pr : 0.0;
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      st[i][j] += s[i][j];
      if (ast) ast[i][j] = s[i][j];
    }
}

template <int N>
struct Sol {
  double r, u, v, w, e, ut, vt, wt, phi0, c2;
  double ra[N], avf[N], are[N], p[N];
  double A[9], st[3][3];
  double vec[K5<N>::NC];  // conservative part of the state vector (HLLC corrections)
};

// m5_facevalues.c:3-192 (from_face false: U is a cell state) and m5_facercnstr.c:3-191
// (from_face true: U is a face state); Sc is the cell-centre state whose volume fractions
// give phi.  ast (optional) receives each material's stress.
template <int N>
__device__ void make_sol(const M5Consts &k, const double *U, const double *Sc, bool from_face,
                         Sol<N> &s, double (*ast)[3][3] = nullptr) {
  using C = K5<N>;
  const double lo = k.amin / 100.0, hi = 1.0 - (k.amin / 100.0);
  s.r = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    s.r += U[i];
    s.ra[i] = U[i];
    s.vec[i] = U[i];
  }
  s.u = U[C::i1 + 0] / s.r;
  s.v = U[C::i1 + 1] / s.r;
  s.w = U[C::i1 + 2] / s.r;
  s.vec[C::i1 + 0] = U[C::i1 + 0];
  s.vec[C::i1 + 1] = U[C::i1 + 1];
  s.vec[C::i1 + 2] = U[C::i1 + 2];
  s.e = U[C::i2] / s.r;
  s.vec[C::i2] = U[C::i2];
  double at[N], ac[N], sum = 0.0;
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    at[i] = U[C::i3 + i];
    ac[i] = Sc[C::i3 + i];
    if (at[i] <= lo) at[i] = lo;
    else if (at[i] >= hi) at[i] = hi;
    if (from_face) {
      if (ac[i] >= hi) ac[i] = hi;
      else if (ac[i] <= lo) ac[i] = lo;
    } else {
      if (ac[i] <= lo) ac[i] = lo;
      else if (ac[i] >= hi) ac[i] = hi;
    }
    sum += at[i];
  }
  if (sum > hi) {
    const double dif = sum - hi;
#pragma unroll
    for (int j = 0; j < N - 1; ++j) {
      const double per = at[j] / sum;
      at[j] = at[j] - per * dif;
    }
    sum = hi;
  }
  at[N - 1] = 1.0 - sum;
  sum = 0.0;
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    s.avf[i] = at[i];
    sum += at[i];
  }
  s.avf[N - 1] = 1.0 - sum;
  // phi[0] (m5_facevalues.c:83-99): the solid fraction(s) against AVF_LIM
  if (k.nsolids == 2 && k.mu[0] != 0.0)
    s.phi0 = ((ac[0] > ac[N > 2 ? 1 : 0]) ? ac[0] : ac[N > 2 ? 1 : 0]) - k.avf_lim;
  else
    s.phi0 = ac[0] - k.avf_lim;
#pragma unroll
  for (int i = 0; i < N; ++i) s.are[i] = U[C::i4 + i];
#pragma unroll
  for (int q = 0; q < 9; q++) s.A[q] = U[C::i5 + q];
  double G[9], Gmag;
  gmat_of(s.A, G, Gmag);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) s.st[i][j] = 0.0;
  double c2 = 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const double ael = (k.mu[i] != 0.0) ? elastic_energy(G, Gmag, k.mu[i], false) : 0.0;
    const double a = from_face ? s.avf[i] : at[i];
    const double press = ((k.gamma[i] - 1.0) * (s.are[i] - ael) / a) - k.gamma[i] * k.pinf[i];
    c2 += (a / s.r) * k.gamma[i] * (press + k.pinf[i]);
    s.p[i] = press;
    eos_stress_acc(s.st, s.avf[i], press, G, Gmag, k.mu[i], ast ? ast[i] : nullptr);
  }
  s.c2 = c2;
}

// m5_bc.c (m5_bc_symmetry) / bc_reflective.c / bc_wall.c: ghost velocity
template <int F, int N>
__device__ __forceinline__ void ghost(const Sol<N> &L, int bc, Sol<N> &R) {
  R = L;
  if (bc == 1 || bc == 4 || bc == 5) {
    const double v3[3] = {L.u, L.v, L.w};
    const double ul = loc<F, 0>(v3), vl = loc<F, 1>(v3), wl = loc<F, 2>(v3);
    const double ur = -ul, vr = bc == 5 ? -vl : vl, wr = bc == 5 ? -wl : wl;
    R.u = glob<F, 0>(ur, vr, wr);
    R.v = glob<F, 1>(ur, vr, wr);
    R.w = glob<F, 2>(ur, vr, wr);
  }
}

template <int N>
struct NC {
  double unc[3], avf[N], are[N], A[9];
};

// m5_star_region.c:3-158
template <int F, int N>
__device__ unsigned star_region(const M5Consts &k, const Sol<N> &s, const Sol<N> &L,
                                const Sol<N> &R, bool leftside, double u_S, double SL, double SR,
                                double uL, double vL, double wL, double uR, double vR, double wR,
                                const double sL[3], const double sR[3], double *Us, NC<N> &nc) {
  using C = K5<N>;
  double SK, uK, vK, wK, s11K, s12K, s13K;
  if (leftside) {
    SK = SL; uK = uL; vK = vL; wK = wL; s11K = sL[0]; s12K = sL[1]; s13K = sL[2];
  } else {
    SK = SR; uK = uR; vK = vR; wK = wR; s11K = sR[0]; s12K = sR[1]; s13K = sR[2];
  }
  double ar_S[N], r_S = 0.0;
#pragma unroll
  for (int v = 0; v < N; ++v) {
    ar_S[v] = s.ra[v] * (SK - uK) / (SK - u_S);
    r_S += ar_S[v];
  }
  const double s11_S = ((uR - SR) * R.r * (sL[0]) - (uL - SL) * L.r * (sR[0]) +
                        (uL - SL) * L.r * (uR - SR) * R.r * (uR - uL)) /
                       ((uR - SR) * R.r - (uL - SL) * L.r);
  double s12_S, s13_S;
  if ((L.phi0 > 0.0) && (R.phi0 > 0.0)) {
    s12_S = ((uR - SR) * R.r * (sL[1]) - (uL - SL) * L.r * (sR[1]) +
             (uL - SL) * L.r * (uR - SR) * R.r * (vR - vL)) /
            ((uR - SR) * R.r - (uL - SL) * L.r);
    s13_S = ((uR - SR) * R.r * (sL[2]) - (uL - SL) * L.r * (sR[2]) +
             (uL - SL) * L.r * (uR - SR) * R.r * (wR - wL)) /
            ((uR - SR) * R.r - (uL - SL) * L.r);
  } else {
    s12_S = 0.0;
    s13_S = 0.0;
  }
  const double v_S = vK + (s12_S - s12K) / ((uK - SK) * s.r);
  const double w_S = wK + (s13_S - s13K) / ((uK - SK) * s.r);
  const double vel[3] = {glob<F, 0>(u_S, v_S, w_S), glob<F, 1>(u_S, v_S, w_S),
                         glob<F, 2>(u_S, v_S, w_S)};
  const double re = s.r * s.e;
  // the reference's expression, or the Rankine-Hugoniot energy jump across the S_K wave
  // (FFV_FLUX_CONSISTENT, include/ffv.h)
  const double Em_S =
      k.flux_form == FFV_FLUX_CONSISTENT
          ? (re * (uK - SK) - s11K * uK - s12K * vK - s13K * wK + s11_S * u_S + s12_S * v_S +
             s13_S * w_S) / (r_S * (u_S - SK))
          : (re * (uK - SK) + s11K * uK - s12K * vK - s13K * wK + s11_S * u_S + s12_S * v_S +
             s13_S * w_S) / (r_S * (u_S + SK));
  double Am[3][3], Al[3][3], AS[3][3], Ag[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Am[i][j] = s.A[3 * i + j];
  tens_to_local<F>(Am, Al);
#pragma unroll
  for (int j = 0; j < 3; j++) {
    AS[0][j] = (Al[0][j] * (uK - SK) - Al[1][j] * (vK - v_S) + Al[2][j] * (wK - w_S)) / (u_S - SK);
    AS[1][j] = Al[1][j];
    AS[2][j] = Al[2][j];
  }
  tens_to_global<F>(AS, Ag);
  double G[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      G[3 * i + j] = Ag[i][0] * Ag[j][0] + Ag[i][1] * Ag[j][1] + Ag[i][2] * Ag[j][2];
  const double Gmag = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
                      G[2] * (G[3] * G[7] - G[4] * G[6]);
#pragma unroll
  for (int v = 0; v < N; ++v) {
    const double rm = (s.ra[v] / s.avf[v]);
    const double rm_S = (s.ra[v] / s.avf[v]) * (uK - SK) / (u_S - SK);
    const double p_k = -s.p[v];
    const double ga = k.gamma[v], pi = k.pinf[v];
    const double p_S = (p_k + pi) * (((ga - 1.0) * rm + (ga + 1.0) * rm_S) /
                                     ((ga - 1.0) * rm_S + (ga + 1.0) * rm)) - pi;
    const double ael = elastic_energy(G, Gmag, k.mu[v], true);
    const double eel = ael / (s.avf[v] * rm_S);
    const double e_S = (p_S + ga * pi) / (rm_S * (ga + 1.0)) + eel;
    nc.are[v] = ar_S[v] * e_S;
  }
#pragma unroll
  for (int v = 0; v < N; ++v) Us[C::i0 + v] = ar_S[v];
#pragma unroll
  for (int v = 0; v < 3; ++v) Us[C::i1 + v] = r_S * vel[v];
  Us[C::i2] = r_S * Em_S;
#pragma unroll
  for (int d = 0; d < 3; d++) nc.unc[d] = vel[d];
#pragma unroll
  for (int v = 0; v < N - 1; ++v) nc.avf[v] = s.avf[v];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) nc.A[3 * i + j] = Ag[i][j];
  unsigned st = 0;
#pragma unroll
  for (int iv = 0; iv < C::NC; ++iv)
    if (isnan(Us[iv])) st |= FFV_ST_NAN;
  return st;
}

// m5_flux.c (gfm false) / m5_flux_gfm.c (gfm true), normal component along face F:
// Fn[iv] = sum_d F[iv][d] n_d with n the signed unit axis of F.
template <int F, int N>
__device__ void flux_n(const Sol<N> &s, int flag, bool gfm, bool cons, NC<N> &nc, double *Fn) {
  using C = K5<N>;
  constexpr int a = Fr<F, 0>::ax, sg = Fr<F, 0>::sg;
  const double vu = gfm ? s.ut : s.u, vv = gfm ? s.vt : s.v, vw = gfm ? s.wt : s.w;
  const double vel[3] = {vu, vv, vw};
  const double va = vel[a];
#pragma unroll
  for (int v = 0; v < N; v++) Fn[C::i0 + v] = sgn<sg>(va * s.ra[v]);
#pragma unroll
  for (int b = 0; b < 3; b++)
    Fn[C::i1 + b] = sgn<sg>((gfm || cons) ? va * vel[b] * s.r - s.st[b][a]
                                          : va * vel[b] * s.r + s.st[b][a]);
  Fn[C::i2] = sgn<sg>(s.r * s.e * va - s.st[a][0] * vu - s.st[a][1] * vv - s.st[a][2] * vw);
  if (flag == 0 || flag == 3) {
#pragma unroll
    for (int d = 0; d < 3; d++) nc.unc[d] = vel[d];
#pragma unroll
    for (int v = 0; v < N - 1; ++v) nc.avf[v] = s.avf[v];
#pragma unroll
    for (int v = 0; v < N; ++v) nc.are[v] = s.are[v];
#pragma unroll
    for (int q = 0; q < 9; q++) nc.A[q] = (gfm || cons) ? s.A[q] : -s.A[q];
  } else if (flag == 4) {  // symmetry face (m5_flux.c:58-66): the velocity is the caller's
#pragma unroll
    for (int v = 0; v < N - 1; ++v) nc.avf[v] = s.avf[v];
#pragma unroll
    for (int v = 0; v < N; ++v) nc.are[v] = s.are[v];
#pragma unroll
    for (int q = 0; q < 9; q++) nc.A[q] = s.A[q];
  }
  const double ua = nc.unc[a];
#pragma unroll
  for (int v = 0; v < N - 1; ++v) Fn[C::i3 + v] = sgn<sg>(ua * nc.avf[v]);
#pragma unroll
  for (int v = 0; v < N; ++v) Fn[C::i4 + v] = sgn<sg>(ua * nc.are[v]);
#pragma unroll
  for (int q = 0; q < 9; q++) Fn[C::i5 + q] = sgn<sg>(ua * nc.A[q]);
}

// m5_hllc.c:3-95 / m5_hllc_gfm.c:3-100 with the wave speeds, accumulated as
// m5_residual.c:155-165: ff += A (F.n + corr); unc receives the face velocity.
template <int F, int N>
__device__ unsigned hllc_acc(const M5Consts &k, Sol<N> L, Sol<N> R, int bc, bool gfm,
                             double Area, double *ff, double unc[3]) {
  using C = K5<N>;
  const double vl3[3] = {L.u, L.v, L.w}, vr3[3] = {R.u, R.v, R.w};
  const double uL = loc<F, 0>(vl3), vL = loc<F, 1>(vl3), wL = loc<F, 2>(vl3);
  double uR = loc<F, 0>(vr3), vR = loc<F, 1>(vr3), wR = loc<F, 2>(vr3);
  if (gfm) {
    vR = vL;
    wR = wL;
    L.ut = L.u;
    L.vt = L.v;
    L.wt = L.w;
    R.ut = glob<F, 0>(uR, vR, wR);
    R.vt = glob<F, 1>(uR, vR, wR);
    R.wt = glob<F, 2>(uR, vR, wR);
    R.vec[C::i1 + 0] = R.ut * R.r;
    R.vec[C::i1 + 1] = R.vt * R.r;
    R.vec[C::i1 + 2] = R.wt * R.r;
    R.vec[C::i2] = R.r * R.e;
  }
  const double ruL = L.r * uL, ruR = R.r * uR;
  const double cL = sqrt(L.c2), cR = sqrt(R.c2);
  double a = uL + cL, b = uR + cR;
  const double SR = (a > b) ? a : b;
  a = uL - cL;
  b = uR - cR;
  const double SL = (a < b) ? a : b;
  double TL[3][3], TR[3][3];
  tens_to_local<F>(L.st, TL);
  tens_to_local<F>(R.st, TR);
  const double sL[3] = {TL[0][0], TL[0][1], TL[0][2]}, sR[3] = {TR[0][0], TR[0][1], TR[0][2]};
  double u_S = ((L.r * (uL * uL) - (sL[0])) - (R.r * (uR * uR) - (sR[0])) - (SL * ruL) +
                (SR * ruR)) / (ruL - ruR - (SL * L.r) + (SR * R.r));
  unsigned st = (isnan(u_S) || isnan(SR) || isnan(SL)) ? FFV_ST_NAN_SPEED : 0u;
  if (!gfm && bc == 4) u_S = 0.0;
  NC<N> nc;
  double Fn[C::NEQ], Us[C::NC], corr[C::NC];
#pragma unroll
  for (int iv = 0; iv < C::NC; ++iv) corr[iv] = 0.0;
  const bool left_star = gfm ? (SL < 0.0 && 0.0 <= u_S) : (SL <= 0.0 && 0.0 <= u_S);
  const bool right_star = gfm ? (u_S < 0.0 && 0.0 < SR) : (u_S <= 0.0 && 0.0 <= SR);
  if (0.0 <= SL) {
    flux_n<F>(L, 0, gfm, k.flux_form == FFV_FLUX_CONSISTENT, nc, Fn);
  } else if (left_star) {
    st |= star_region<F>(k, L, L, R, true, u_S, SL, SR, uL, vL, wL, uR, vR, wR, sL, sR, Us, nc);
    flux_n<F>(L, 1, gfm, k.flux_form == FFV_FLUX_CONSISTENT, nc, Fn);
#pragma unroll
    for (int iv = 0; iv < C::NC; ++iv) corr[iv] = SL * (Us[iv] - L.vec[iv]);
  } else if (right_star) {
    st |= star_region<F>(k, R, L, R, false, u_S, SL, SR, uL, vL, wL, uR, vR, wR, sL, sR, Us, nc);
    flux_n<F>(R, 2, gfm, k.flux_form == FFV_FLUX_CONSISTENT, nc, Fn);
#pragma unroll
    for (int iv = 0; iv < C::NC; ++iv) corr[iv] = SR * (Us[iv] - R.vec[iv]);
  } else if (SR <= 0.0) {
    flux_n<F>(R, 3, gfm, k.flux_form == FFV_FLUX_CONSISTENT, nc, Fn);
  } else {
    st |= FFV_ST_NO_BRANCH;
#pragma unroll
    for (int iv = 0; iv < C::NEQ; ++iv) Fn[iv] = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) nc.unc[d] = 0.0;
  }
#pragma unroll
  for (int iv = 0; iv < C::NEQ; ++iv)
    ff[iv] += (Area) * (Fn[iv] + (iv < C::NC ? corr[iv] : 0.0));
#pragma unroll
  for (int d = 0; d < 3; d++) unc[d] = nc.unc[d];
  return st;
}

// m5_hllc.c:56-85, a symmetry face (bc 1): the mean of the physical fluxes of the cell's own
// state (m5_facevalues.c, not the reconstructed face state) and of its mirror image
// (m5_bc_symmetry: normal velocity reversed), the advected volume fractions, energies and
// deformation moving with the mean velocity, no HLLC part; accumulated as m5_residual.c:155-165
template <int F, int N>
__device__ void symmetry_acc(const Sol<N> &Lc, bool cons, double Area, double *ff, double unc[3]) {
  using C = K5<N>;
  Sol<N> Rc;
  ghost<F, N>(Lc, 1, Rc);
  NC<N> nc;
  nc.unc[0] = 0.5 * (Lc.u + Rc.u);
  nc.unc[1] = 0.5 * (Lc.v + Rc.v);
  nc.unc[2] = 0.5 * (Lc.w + Rc.w);
  double FL[C::NEQ], FR[C::NEQ];
  flux_n<F>(Lc, 4, false, cons, nc, FL);
  flux_n<F>(Rc, 4, false, cons, nc, FR);
#pragma unroll
  for (int iv = 0; iv < C::NEQ; ++iv) ff[iv] += (Area) * ((0.5 * FL[iv]) + (0.5 * FR[iv]));
#pragma unroll
  for (int d = 0; d < 3; d++) unc[d] = nc.unc[d];
}

// ------------------------------------------------------------ relaxation (m5_relaxationvec.c)
template <int N>
__device__ __forceinline__ void vf_limit_relax(const M5Consts &k, double *avf, bool elseif) {
  const double lo = k.amin / 100.0, hi = 1.0 - (k.amin / 100.0);
  double sum = 0.0;
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    if (elseif) {
      if (avf[i] <= lo) avf[i] = lo;
      else if (avf[i] >= hi) avf[i] = hi;
    } else {
      if (avf[i] <= lo) avf[i] = lo;
      if (avf[i] >= hi) avf[i] = hi;
    }
    sum += avf[i];
  }
  if (sum >= hi) {
    const double dif = sum - hi;
#pragma unroll
    for (int j = 0; j < N - 1; ++j) {
      const double per = avf[j] / sum;
      avf[j] = avf[j] - per * dif;
    }
    sum = hi;
  }
  avf[N - 1] = 1.0 - sum;
}

template <int N>
__device__ unsigned relaxationvec(const M5Consts &k, double *V) {
  using C = K5<N>;
  double ar[N], are[N], avf[N], avf0[N], A[9], G[9], Gmag;
  double rho = 0.0;
#pragma unroll
  for (int iv = 0; iv < N; ++iv) {
    ar[iv] = V[iv + C::i0];
    are[iv] = V[iv + C::i4];
    rho += ar[iv];
  }
  const double u = V[C::i1 + 0] / rho, v = V[C::i1 + 1] / rho, w = V[C::i1 + 2] / rho;
  const double rE = V[C::i2];
#pragma unroll
  for (int iv = 0; iv < N - 1; ++iv) avf[iv] = V[iv + C::i3];
  vf_limit_relax<N>(k, avf, true);
#pragma unroll
  for (int iv = 0; iv < N; ++iv) avf0[iv] = avf[iv];
#pragma unroll
  for (int q = 0; q < 9; q++) A[q] = V[q + C::i5];
  gmat_of(A, G, Gmag);
  const double eps_sml = 1.0e-12, eps_big = 1.0e-8;
  unsigned st = 0;
  if (k.prelax == 1) {
    double t0[N], p0[N];
#pragma unroll
    for (int iv = 0; iv < N; ++iv) {
      const double ael = (k.mu[iv] != 0.0) ? elastic_energy(G, Gmag, k.mu[iv], false) : 0.0;
      t0[iv] = 1.0 / (ar[iv] / avf[iv]);
      p0[iv] = ((k.gamma[iv] - 1.0) * (are[iv] - ael) / avf[iv]) - k.gamma[iv] * k.pinf[iv];
    }
    const double *ga = k.gamma, *pi = k.pinf;
    const double A_1 = (avf[0] / ga[0]) * (p0[0] + pi[0]) / ((avf[0] / ga[0]) + (avf[1] / ga[1]));
    const double A_2 = (avf[1] / ga[1]) * (p0[1] + pi[1]) / ((avf[0] / ga[0]) + (avf[1] / ga[1]));
    const double d = (A_2 - A_1 - (pi[1] - pi[0]));
    const double pe = 0.5 * (A_1 + A_2 - (pi[0] + pi[1])) + sqrt(0.25 * (d * d) + A_1 * A_2);
    if (isnan(pe)) st |= FFV_ST_NAN;
#pragma unroll
    for (int iv = 0; iv < N; ++iv) {
      const double t1 = t0[iv] * (p0[iv] + ga[iv] * pi[iv] + (ga[iv] - 1.0) * pe) /
                        (pe + ga[iv] * pi[iv] + (ga[iv] - 1.0) * pe);
      const double rm = 1.0 / t1;
      avf[iv] = ar[iv] / rm;
    }
    vf_limit_relax<N>(k, avf, false);
#pragma unroll
    for (int q = 0; q < 9; q++) A[q] = A[q] * (avf[0] / avf0[0]);
  } else {  // PRELAX 3
    double rhoKs[N], pkinit[N];
#pragma unroll
    for (int iv = 0; iv < N; ++iv) {
      if (avf[iv] < 0.0 || ar[iv] < 0.0) {
        avf[iv] = eps_sml;
        ar[iv] = eps_sml;
        are[iv] = eps_sml;
      }
      if (avf[iv] >= 1.0) avf[iv] = 1.0 - eps_sml;
    }
    bool irelax = true;
#pragma unroll
    for (int iv = 0; iv < N; ++iv)
      if (avf[iv] > 1.0 - eps_sml) irelax = false;
    if (irelax) {
      double p_relaxed = 0.0;
#pragma unroll
      for (int iv = 0; iv < N; ++iv) {
        if (avf[iv] > eps_sml) {
          const double ael = (k.mu[iv] != 0.0) ? elastic_energy(G, Gmag, k.mu[iv], false) : 0.0;
          pkinit[iv] = ((k.gamma[iv] - 1.0) * (are[iv] - ael) / avf[iv]) - k.gamma[iv] * k.pinf[iv];
          if (pkinit[iv] <= -(1.0 - eps_big) * k.pinf[iv] + eps_big)
            pkinit[iv] = -(1.0 - eps_big) * k.pinf[iv] + eps_big;
        } else {
          pkinit[iv] = 0.0;
        }
        p_relaxed += avf[iv] * pkinit[iv];
      }
      int iter = 0;
      double F = 1.0e-9, dF = 1.0e9, p_prev = NAN;
#pragma unroll
      for (int iv = 0; iv < N; ++iv) rhoKs[iv] = 0.0;
      // the reference's own iteration cap (m5_relaxationvec.c:458) bounds this loop.  An
      // iterate that repeats bitwise is a fixed point: F, dF and rhoKs repeat with it, so
      // the remaining iterations up to the cap would recompute the same values -- leaving
      // there gives exactly the reference's result (most non-converging face states of a
      // stiff two-phase interface reach such a point within a few iterations and would
      // otherwise spin to the cap).
      while ((fabs(F) > 1.0e-12) && (iter < 500)) {
        p_relaxed = p_relaxed - F / dF;
        iter = iter + 1;
#pragma unroll
        for (int iv = 0; iv < N; ++iv)
          if (p_relaxed < -(1.0 - eps_big) * k.pinf[iv] + eps_big)
            p_relaxed = -(1.0 - eps_big) * k.pinf[iv] + 1.0;
        F = -1.0;
        dF = 0.0;
#pragma unroll
        for (int iv = 0; iv < N; ++iv) {
          if (avf[iv] > eps_sml) {
            const double am = (avf[iv] > eps_sml) ? avf[iv] : eps_sml;
            rhoKs[iv] = ar[iv] / am *
                        pow((p_relaxed + k.pinf[iv]) / (pkinit[iv] + k.pinf[iv]), 1.0 / k.gamma[iv]);
            F = F + ar[iv] / rhoKs[iv];
            dF = dF - ar[iv] / (k.gamma[iv] * rhoKs[iv] * (p_relaxed + k.pinf[iv]));
          }
        }
        if (isnan(p_relaxed) || isnan(F) || isnan(dF)) {
          st |= FFV_ST_NAN;
          break;
        }
        if (p_relaxed == p_prev) break;
        p_prev = p_relaxed;
      }
#pragma unroll
      for (int iv = 0; iv < N; ++iv)
        if (avf[iv] > eps_sml) avf[iv] = ar[iv] / rhoKs[iv];
      vf_limit_relax<N>(k, avf, true);
    }
    const int i_as = ((avf[0] < avf[1]) && (k.mu[1] != 0.0)) ? 1 : 0;
    const double ratio = avf[i_as] / avf0[i_as];
#pragma unroll
    for (int q = 0; q < 9; q++) A[q] = A[q] * ratio;
  }
  double e_elast = 0.0, ael_t[N];
#pragma unroll
  for (int iv = 0; iv < N; ++iv) {
    ael_t[iv] = (k.mu[iv] != 0.0) ? elastic_energy(G, Gmag, k.mu[iv], false) : 0.0;
    const double eK = ael_t[iv] / (ar[iv]);
    const double Ys = ar[iv] / rho;
    e_elast += Ys * eK;
  }
  const double e_hyd = rE / rho - 0.5 * (u * u + v * v + w * w) - e_elast;
  double num = 0.0, den = 0.0;
#pragma unroll
  for (int iv = 0; iv < N; ++iv) {
    num += avf[iv] * k.gamma[iv] * k.pinf[iv] / (k.gamma[iv] - 1.0);
    den += avf[iv] / (k.gamma[iv] - 1.0);
  }
  const double p_relaxed = (rho * e_hyd - num) / den;
#pragma unroll
  for (int iv = 0; iv < N - 1; ++iv) {
    if (isnan(avf[iv])) st |= FFV_ST_NAN;
    V[iv + C::i3] = avf[iv];
  }
#pragma unroll
  for (int iv = 0; iv < N; iv++) {
    const double a2 = (avf[iv] * (p_relaxed + k.gamma[iv] * k.pinf[iv]) / (k.gamma[iv] - 1.0)) + ael_t[iv];
    if (isnan(a2)) st |= FFV_ST_NAN;
    V[iv + C::i4] = a2;
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) V[q + C::i5] = A[q];
  return st;
}

// avf_limit.c:3-21 on a state vector
template <int N>
__device__ __forceinline__ void avf_limit(const M5Consts &k, double *S) {
  using C = K5<N>;
  const double lo = k.amin / 100.0, hi = 1.0 - (k.amin / 100.0);
  double sum = 0.0;
#pragma unroll
  for (int v = 0; v < N - 1; ++v) {
    double a = S[C::i3 + v];
    if (a <= lo) a = lo;
    else if (a >= hi) a = hi;
    S[C::i3 + v] = a;
    sum += a;
  }
  if (sum > hi) {
    const double dif = sum - hi;
#pragma unroll
    for (int j = 0; j < N - 1; ++j) {
      const double a = S[C::i3 + j];
      S[C::i3 + j] = a - (a / sum) * dif;
    }
  }
}

template <int N>
__device__ __forceinline__ void load_state(const double *__restrict__ S, int64_t n, int64_t c,
                                           double *U) {
#pragma unroll
  for (int v = 0; v < K5<N>::NEQ; v++) U[v] = S[(int64_t)v * n + c];
}

// m5_facevalues_MUSCL.c:3-45 (iside 1): value across face f, volume fractions limited
template <int N>
__device__ void value_across(const M5Consts &k, const ffv_dmesh &m, const double *__restrict__ S,
                             int64_t c, int f, uint32_t kind, const double *Sc, double *X) {
  using C = K5<N>;
  if (kind & FFV_FK_BC) {
    // the ghost's state vector: the cell's own with the clamped volume fractions of
    // m5_facevalues.c:46-80 (the bc only changes the ghost's primitive velocity)
    const double lo = k.amin / 100.0, hi = 1.0 - (k.amin / 100.0);
#pragma unroll
    for (int i = 0; i < C::NEQ; i++) X[i] = Sc[i];
    double at[N], sum = 0.0;
#pragma unroll
    for (int i = 0; i < N - 1; ++i) {
      at[i] = Sc[C::i3 + i];
      if (at[i] <= lo) at[i] = lo;
      else if (at[i] >= hi) at[i] = hi;
      sum += at[i];
    }
    if (sum > hi) {
      const double dif = sum - hi;
#pragma unroll
      for (int j = 0; j < N - 1; ++j) {
        const double per = at[j] / sum;
        at[j] = at[j] - per * dif;
      }
    }
#pragma unroll
    for (int i = 0; i < N - 1; ++i) X[C::i3 + i] = at[i];
  } else if (kind == FFV_FK_FINER) {
    const int32_t *sg = m.sub + 4 * (int64_t)m.nbr[(int64_t)f * m.n + c];
#pragma unroll
    for (int i = 0; i < C::NEQ; i++) X[i] = 0.0;
#pragma unroll 1
    for (int q = 0; q < 4; q++) {
      const int64_t o = sg[q];
#pragma unroll
      for (int i = 0; i < C::NEQ; i++) X[i] += S[(int64_t)i * m.n + o] / 4.0;
    }
  } else {
    load_state<N>(S, m.n, m.nbr[(int64_t)f * m.n + c], X);
  }
  avf_limit<N>(k, X);
}

// ------------------------------------------------------------------------------ kernels
template <int N>
__global__ void __launch_bounds__(128) m5_recon_face(ffv_dmesh m, ffv_geom g, M5Consts k,
                                                     const double *__restrict__ S,
                                                     double *__restrict__ SF,
                                                     unsigned *__restrict__ status) {
  using C = K5<N>;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6 * m.n) return;
  const int f = (int)(t / m.n);
  const int64_t c = t - (int64_t)f * m.n;
  const int fo = fr_opp(f);
  const uint32_t info = m.info[c];
  const int l = ffv_info_level(info);
  const uint32_t kf = ffv_face_kind(info, f), ko = ffv_face_kind(info, fo);
  double Sc[C::NEQ], SL[C::NEQ], X[C::NEQ], out[C::NEQ];
  load_state<N>(S, m.n, c, Sc);
#pragma unroll
  for (int i = 0; i < C::NEQ; i++) SL[i] = Sc[i];
  avf_limit<N>(k, SL);
  value_across<N>(k, m, S, c, f, kf, Sc, X);
  double df[C::NEQ];
#pragma unroll
  for (int i = 0; i < C::NEQ; i++) df[i] = X[i] - SL[i];
  value_across<N>(k, m, S, c, fo, ko, Sc, X);
  const double dp = g.dcc[l][face_class(kf)], dm = g.dcc[l][face_class(ko)];
  const double cf = g.dcf[l][face_class(kf)];
#pragma unroll
  for (int i = 0; i < C::NEQ; i++) {
    const double db = X[i] - SL[i];
    double grad = 0.0;
    if (!(kf & FFV_FK_BC)) {
      if (fabs(df[i]) > 1e-10) {
        const double product = (-db / dm) * (df[i] / dp);
        if (product > 0.0) {
          const double lim = (i >= C::i4 && i < C::i5) ? 0.0 : 1.0;
          if (fabs(-db / dm) > fabs(df[i] / dp))
            grad = lim * (df[i] / dp);
          else
            grad = lim * (-db / dm);
        }
      }
    }
    out[i] = SL[i] + cf * grad;
  }
  // m5_reconctruct.c:144-179: volume-fraction limits of the face state
  const double lo = k.amin / 100.0;
  double avf[N], sum = 0.0;
#pragma unroll
  for (int iv = 0; iv < N - 1; ++iv) {
    avf[iv] = out[iv + C::i3];
    if (avf[iv] <= lo) avf[iv] = lo;
    else if (avf[iv] >= (1.0 - (2.0 * lo))) avf[iv] = 1.0 - (2.0 * lo);
    sum += avf[iv];
  }
  if (sum >= (1.0 - lo)) {
    const double dif = sum - (1.0 - lo);
#pragma unroll
    for (int j = 0; j < N - 1; ++j) {
      const double per = avf[j] / sum;
      avf[j] = avf[j] - per * dif;
    }
  }
#pragma unroll
  for (int iv = 0; iv < N - 1; ++iv) out[iv + C::i3] = avf[iv];
  const unsigned st = relaxationvec<N>(k, out);
#pragma unroll
  for (int i = 0; i < C::NEQ; i++) SF[((int64_t)f * C::NEQ + i) * m.n + c] = out[i];
  if (st) atomicOr(status, st);
}

template <int N>
__device__ __forceinline__ void load_face_state(const double *__restrict__ SF, int64_t n, int f,
                                                int64_t c, double *U) {
#pragma unroll
  for (int v = 0; v < K5<N>::NEQ; v++) U[v] = SF[((int64_t)f * K5<N>::NEQ + v) * n + c];
}

// face flux of cell c through face F (all subfaces), the reference's reuse included
template <int N, int F>
__device__ void face_flux(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k,
                          const double *__restrict__ S, const double *__restrict__ SF, int64_t c,
                          uint32_t info, double *ff, double uf[3], double &gfm_face,
                          unsigned &st, bool &owner) {
  using C = K5<N>;
  constexpr int FO = fr_opp(F);
  const uint32_t kind = ffv_face_kind(info, F);
  const int l = ffv_info_level(info);
  double U[C::NEQ], Sc[C::NEQ], So[C::NEQ];
#pragma unroll
  for (int iv = 0; iv < C::NEQ; iv++) ff[iv] = 0.0;
  uf[0] = uf[1] = uf[2] = 0.0;
  gfm_face = 0.0;
  Sol<N> L, R;
  load_state<N>(S, m.n, c, Sc);
  if (kind == FFV_FK_SAME && m.nbr[(int64_t)F * m.n + c] < c) {
    // 1:1 face whose neighbour comes first in leaf order: the neighbour's thread evaluates
    // it (face F^1 of the neighbour) and m5_cell_update takes the negative, as the
    // reference's flux reuse does (m5_residual.c:80-99); no ghost-fluid flag here
    owner = false;
    return;
  }
  if (kind == (FFV_FK_BC | FFV_BC_SYMMETRY)) {
    // the cell's own state, not the face state; the HLLC flux the reference computes first
    // for this face is discarded (m5_hllc.c:59-63)
    make_sol<N>(k, Sc, Sc, false, L);
    symmetry_acc<F, N>(L, k.flux_form == FFV_FLUX_CONSISTENT, g.area[l], ff, uf);
    return;
  }
  if (k.order == 2) load_face_state<N>(SF, m.n, F, c, U);
  make_sol<N>(k, k.order == 2 ? U : Sc, Sc, k.order == 2, L);
  if (kind & FFV_FK_BC) {
    const int bc = (int)(kind & 7u);
    ghost<F, N>(L, bc, R);
    const bool gfm = L.phi0 * R.phi0 < 0.0;
    if (gfm) gfm_face = 1.0;
    st |= hllc_acc<F, N>(k, L, R, bc, gfm, g.area[l], ff, uf);
    return;
  }
  const int nsub = kind == FFV_FK_FINER ? 4 : 1;
  const double A = kind == FFV_FK_FINER ? g.area[l + 1] : g.area[l];
  const int32_t *sg = kind == FFV_FK_FINER ? m.sub + 4 * (int64_t)m.nbr[(int64_t)F * m.n + c] : nullptr;
#pragma unroll 1
  for (int q = 0; q < nsub; q++) {
    const int64_t o = sg ? sg[q] : m.nbr[(int64_t)F * m.n + c];
    load_state<N>(S, m.n, o, So);
    if (k.order == 2) load_face_state<N>(SF, m.n, FO, o, U);
    make_sol<N>(k, k.order == 2 ? U : So, So, k.order == 2, R);
    const bool gfm = L.phi0 * R.phi0 < 0.0;
    if (gfm) gfm_face = 1.0;
    double un[3];
    st |= hllc_acc<F, N>(k, L, R, 0, gfm, A, ff, un);
    uf[0] = un[0] / ((double)nsub);
    uf[1] = un[1] / ((double)nsub);
    uf[2] = un[2] / ((double)nsub);
  }
}

template <int N>
__global__ void __launch_bounds__(128) m5_face_flux(ffv_dmesh m, ffv_geom g, M5Consts k,
                                                    const double *__restrict__ S,
                                                    const double *__restrict__ SF,
                                                    double *__restrict__ FF,
                                                    double *__restrict__ UF,
                                                    double *__restrict__ GF,
                                                    unsigned *__restrict__ status) {
  using C = K5<N>;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6 * m.n) return;
  const int f = (int)(t / m.n);
  const int64_t c = t - (int64_t)f * m.n;
  const uint32_t info = m.info[c];
  double ff[C::NEQ], uf[3], gf = 0.0;
  unsigned st = 0;
  bool owner = true;
  switch (f) {
    case 0: face_flux<N, 0>(m, g, k, S, SF, c, info, ff, uf, gf, st, owner); break;
    case 1: face_flux<N, 1>(m, g, k, S, SF, c, info, ff, uf, gf, st, owner); break;
    case 2: face_flux<N, 2>(m, g, k, S, SF, c, info, ff, uf, gf, st, owner); break;
    case 3: face_flux<N, 3>(m, g, k, S, SF, c, info, ff, uf, gf, st, owner); break;
    case 4: face_flux<N, 4>(m, g, k, S, SF, c, info, ff, uf, gf, st, owner); break;
    default: face_flux<N, 5>(m, g, k, S, SF, c, info, ff, uf, gf, st, owner); break;
  }
  if (owner) {
#pragma unroll
    for (int iv = 0; iv < C::NEQ; iv++) FF[((int64_t)f * C::NEQ + iv) * m.n + c] = ff[iv];
#pragma unroll
    for (int d = 0; d < 3; d++) UF[((int64_t)f * 3 + d) * m.n + c] = uf[d];
  }
  GF[(int64_t)f * m.n + c] = gf;
  if (st) atomicOr(status, st);
}

// residual sum and non-conservative terms (m5_residual.c:171-214) for face F
template <int N, int F>
__device__ __forceinline__ void nonconservative(const ffv_geom &g, const Sol<N> &Cs,
                                                const double (*ast)[3][3], uint32_t info, int l,
                                                double un, double vn, double wn, double *rhs) {
  using C = K5<N>;
  const uint32_t kind = ffv_face_kind(info, F);
  double Area_f = 0.0;
  if (kind == FFV_FK_FINER) {
#pragma unroll
    for (int q = 0; q < 4; q++) Area_f += g.area[l + 1];
  } else {
    Area_f += g.area[l];
  }
  constexpr int a = Fr<F, 0>::ax, sg = Fr<F, 0>::sg;
  // with n the signed unit axis, u_nc*nx + v_nc*ny + w_nc*nz keeps one term
  const double nn[3] = {a == 0 ? (double)sg : 0.0, a == 1 ? (double)sg : 0.0, a == 2 ? (double)sg : 0.0};
  const double nx = nn[0], ny = nn[1], nz = nn[2];
#pragma unroll
  for (int iv = 0; iv < N - 1; ++iv) {
    const double s = Cs.avf[iv];
    rhs[C::i3 + iv] += Area_f * (s * un * nx + s * vn * ny + s * wn * nz);
  }
#pragma unroll
  for (int iv = 0; iv < N; ++iv) {
    const double(*t)[3] = ast[iv];
    rhs[C::i4 + iv] += Area_f * (t[0][0] * un * nx + t[0][1] * vn * nx + t[0][2] * wn * nx +
                                 t[1][0] * un * ny + t[1][1] * vn * ny + t[1][2] * wn * ny +
                                 t[2][0] * un * nz + t[2][1] * vn * nz + t[2][2] * wn * nz);
  }
  const double *Am = Cs.A;
  const double A1 = Am[0], A2 = Am[1], A3 = Am[2], B1 = Am[3], B2 = Am[4], B3 = Am[5],
               C1 = Am[6], C2 = Am[7], C3 = Am[8];
  double *R5 = rhs + C::i5;
  R5[0] += Area_f * ((A1 * vn * ny + A1 * wn * nz) + B1 * vn * nx - C1 * wn * nx);
  R5[1] += Area_f * ((A2 * vn * ny + A2 * wn * nz) + B2 * vn * nx - C2 * wn * nx);
  R5[2] += Area_f * ((A3 * vn * ny + A3 * wn * nz) + B3 * vn * nx - C3 * wn * nx);
  R5[3] += Area_f * ((B1 * un * nx + B1 * wn * nz) + A1 * un * ny - C1 * wn * ny);
  R5[4] += Area_f * ((B2 * un * nx + B2 * wn * nz) + A2 * un * ny - C2 * wn * ny);
  R5[5] += Area_f * ((B3 * un * nx + B3 * wn * nz) + A3 * un * ny - C3 * wn * ny);
  R5[6] += Area_f * ((C1 * un * nx + C1 * vn * ny) + A1 * un * nz - B1 * vn * nz);
  R5[7] += Area_f * ((C2 * un * nx + C2 * vn * ny) + A2 * un * nz - B2 * vn * nz);
  R5[8] += Area_f * ((C3 * un * nx + C3 * vn * ny) + A3 * un * nz - B3 * vn * nz);
}

template <int N>
__device__ __forceinline__ void clamp_zerou(const M5Consts &k, double *s, const double *sn) {
  using C = K5<N>;
#pragma unroll
  for (int v = 0; v < N; v++)
    if (s[C::i0 + v] < 0.0) s[C::i0 + v] = sn[C::i0 + v];
  constexpr int e5 = C::i5;
  if (k.zerou[0]) {
    s[C::i1 + 0] = sn[C::i1 + 0];
    s[e5 + 1] = sn[e5 + 1]; s[e5 + 2] = sn[e5 + 2]; s[e5 + 3] = sn[e5 + 3]; s[e5 + 6] = sn[e5 + 6];
  }
  if (k.zerou[1]) {
    s[C::i1 + 1] = sn[C::i1 + 1];
    s[e5 + 1] = sn[e5 + 1]; s[e5 + 3] = sn[e5 + 3]; s[e5 + 5] = sn[e5 + 5]; s[e5 + 7] = sn[e5 + 7];
  }
  if (k.zerou[2]) {
    s[C::i1 + 2] = sn[C::i1 + 2];
    s[e5 + 2] = sn[e5 + 2]; s[e5 + 5] = sn[e5 + 5]; s[e5 + 6] = sn[e5 + 6]; s[e5 + 7] = sn[e5 + 7];
  }
}

// residual + RK stage (m5_RK.c): writes RHS and the new state into Snew; stage-1 cells
// whose solid fraction crosses AVF_LIM get the partial update and a flag for m5_gfm_seq
template <int N, typename TF>
__global__ void __launch_bounds__(128) m5_cell_update(ffv_dmesh m, ffv_geom g, M5Consts k,
                                                      const double *__restrict__ S,
                                                      double *__restrict__ SN,
                                                      const TF *__restrict__ FF,
                                                      const TF *__restrict__ UF,
                                                      double *__restrict__ RHS,
                                                      double *__restrict__ Snew,
                                                      uint8_t *__restrict__ flag,
                                                      const double *__restrict__ dtp, int irk,
                                                      unsigned *__restrict__ status) {
  using C = K5<N>;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  const uint32_t info = m.info[c];
  const int l = ffv_info_level(info);
  double s[C::NEQ], rhs[C::NEQ];
  load_state<N>(S, m.n, c, s);
  Sol<N> Cs;
  double ast[N][3][3];
  make_sol<N>(k, s, s, false, Cs, ast);
#pragma unroll
  for (int iv = 0; iv < C::NEQ; iv++) rhs[iv] = 0.0;
#define FACE(F)                                                                          \
  {                                                                                      \
    int64_t fc = c;                                                                      \
    int ff = F;                                                                          \
    double sg = 1.0;                                                                     \
    if (ffv_face_kind(info, F) == FFV_FK_SAME) {                                         \
      const int64_t o = m.nbr[(int64_t)F * m.n + c];                                     \
      if (o < c) {                                                                       \
        fc = o;                                                                          \
        ff = fr_opp(F);                                                                  \
        sg = -1.0;                                                                       \
      }                                                                                  \
    }                                                                                    \
    _Pragma("unroll") for (int iv = 0; iv < C::NEQ; iv++) {                              \
      const double x = (double)FF[((int64_t)ff * C::NEQ + iv) * m.n + fc];               \
      rhs[iv] += sg < 0.0 ? -x : x;                                                      \
    }                                                                                    \
    const double u0 = (double)UF[((int64_t)ff * 3 + 0) * m.n + fc];                      \
    const double u1 = (double)UF[((int64_t)ff * 3 + 1) * m.n + fc];                      \
    const double u2 = (double)UF[((int64_t)ff * 3 + 2) * m.n + fc];                      \
    nonconservative<N, F>(g, Cs, ast, info, l, sg < 0.0 ? -u0 : u0, sg < 0.0 ? -u1 : u1, \
                          sg < 0.0 ? -u2 : u2, rhs);                                     \
  }
  FACE(0) FACE(1) FACE(2) FACE(3) FACE(4) FACE(5)
#undef FACE
  // a non-positive density in the stage's input is reported (the arithmetic is untouched)
  double rho_in = 0.0;
#pragma unroll
  for (int v = 0; v < N; ++v) rho_in += s[C::i0 + v];
  unsigned st = rho_in <= 0.0 ? FFV_ST_NEG_DENSITY : 0u;
#pragma unroll
  for (int iv = 0; iv < C::NEQ; iv++) {
    if (isnan(rhs[iv])) st |= FFV_ST_NAN;
    RHS[(int64_t)iv * m.n + c] = rhs[iv];
  }
  const double dt = *dtp, V = g.vol[l];
  double sn[C::NEQ];
  if (irk == 1) {
#pragma unroll
    for (int e = 0; e < C::NEQ; e++) {
      sn[e] = s[e];
      SN[(int64_t)e * m.n + c] = s[e];
    }
  } else {
    load_state<N>(SN, m.n, c, sn);
  }
  bool gfm = false;
  if (irk == 1) {
#pragma unroll
    for (int v = 0; v < N - 1; ++v) {
      if (k.mu[v] != 0.0) {
        const int e = C::i3 + v;
        const double phi_old = s[e] - k.avf_lim;
        const double buf = (1.0 / V) * rhs[e];
        const double as_new = sn[e] + dt * buf;
        if (phi_old * (as_new - k.avf_lim) < 0.0) gfm = true;
      }
    }
    if (gfm) {
#pragma unroll
      for (int e = C::i2; e < C::NEQ; e++) s[e] = sn[e] + dt * ((1.0 / V) * rhs[e]);
    } else {
#pragma unroll
      for (int e = 0; e < C::NEQ; e++) s[e] = sn[e] + dt * ((1.0 / V) * rhs[e]);
    }
  } else if (irk == 2) {
#pragma unroll
    for (int e = 0; e < C::NEQ; e++)
      s[e] = (3.0 / 4.0) * sn[e] + (1.0 / 4.0) * s[e] + (1.0 / 4.0) * dt * rhs[e] / V;
  } else if (irk == 3) {
#pragma unroll
    for (int e = 0; e < C::NEQ; e++)
      s[e] = (1.0 / 3.0) * sn[e] + (2.0 / 3.0) * s[e] + (2.0 / 3.0) * dt * rhs[e] / V;
  } else {
#pragma unroll
    for (int e = 0; e < C::NEQ; e++)
      s[e] = (1.0 / 2.0) * sn[e] + (1.0 / 2.0) * s[e] + (1.0 / 2.0) * dt * rhs[e] / V;
  }
  if (!gfm) clamp_zerou<N>(k, s, sn);
#pragma unroll
  for (int e = 0; e < C::NEQ; e++) Snew[(int64_t)e * m.n + c] = s[e];
  flag[c] = gfm ? 1 : 0;
  if (st) atomicOr(status, st);
}

// cell pressure relaxation (m5_relaxation_solid.c:16-32); flags solid-fraction crossings
template <int N>
__global__ void __launch_bounds__(128) m5_relax_cell(int64_t n, M5Consts k,
                                                     const double *__restrict__ Sin,
                                                     double *__restrict__ Sout,
                                                     uint8_t *__restrict__ flag,
                                                     unsigned *__restrict__ status) {
  using C = K5<N>;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double s[C::NEQ];
  load_state<N>(Sin, n, c, s);
  const double phi_old = s[C::i3] - k.avf_lim;
  const unsigned st = relaxationvec<N>(k, s);
  // the plastic return where the reference's prototype would run it (m5_relaxation_solid.c:14),
  // after the relaxation so that the stored state lies on or inside the yield surface
  if (k.plastic) plastic_return<N>(k, s);
  // phi_new[0] exists in the reference only for a solid material 0 (else no trigger)
  const double phi_new = (k.mu[0] != 0.0) ? s[C::i3] - k.avf_lim : phi_old;
  flag[c] = (phi_old * phi_new < 0.0) ? 1 : 0;
#pragma unroll
  for (int e = 0; e < C::NEQ; e++) Sout[(int64_t)e * n + c] = s[e];
  if (st) atomicOr(status, st);
}

// m5_gfm.c (relax false) / m5_gfm_rel.c (relax true) for the flagged cells, one warp, in
// leaf order.  A neighbour earlier in leaf order is read from Snew (its final state of this
// pass), a later one from Sold, as the reference's in-place list walk sees them.
template <int N>
__global__ void __launch_bounds__(32) m5_gfm_seq(ffv_dmesh m, ffv_geom g, M5Consts k,
                                                 const int32_t *__restrict__ list,
                                                 const int32_t *__restrict__ count,
                                                 const double *__restrict__ Sold,
                                                 double *__restrict__ Snew,
                                                 const double *__restrict__ SN,
                                                 const double *__restrict__ RHS,
                                                 const double *__restrict__ GF,
                                                 const double *__restrict__ dtp, int relax) {
  using C = K5<N>;
  __shared__ double s_phiR[6], s_vel[6][3], s_own[C::NEQ];
  const int lane = threadIdx.x;
  const int cnt = *count;
  const double DT = *dtp;
  for (int idx = 0; idx < cnt; idx++) {
    const int64_t c = list[idx];
    const uint32_t info = m.info[c];
    const int l = ffv_info_level(info);
    if (lane == 0)
      for (int e = 0; e < C::NEQ; e++) s_own[e] = Snew[(int64_t)e * m.n + c];
    __syncwarp();
    double own[C::NEQ];
#pragma unroll
    for (int e = 0; e < C::NEQ; e++) own[e] = s_own[e];
    Sol<N> L;
    make_sol<N>(k, own, own, false, L);
    if (lane < 6) {
      const int f = lane;
      const uint32_t kind = ffv_face_kind(info, f);
      double phiR = 0.0, vr[3] = {0.0, 0.0, 0.0};
      if (GF[(int64_t)f * m.n + c] == 1.0) {
        Sol<N> R;
        if (kind & FFV_FK_BC) {
          const int bc = (int)(kind & 7u);
          switch (f) {
            case 0: ghost<0, N>(L, bc, R); break;
            case 1: ghost<1, N>(L, bc, R); break;
            case 2: ghost<2, N>(L, bc, R); break;
            case 3: ghost<3, N>(L, bc, R); break;
            case 4: ghost<4, N>(L, bc, R); break;
            default: ghost<5, N>(L, bc, R); break;
          }
        } else {
          const int64_t o = kind == FFV_FK_FINER ? m.sub[4 * (int64_t)m.nbr[(int64_t)f * m.n + c]]
                                                 : m.nbr[(int64_t)f * m.n + c];
          double so[C::NEQ];
          load_state<N>(o < c ? Snew : Sold, m.n, o, so);
          make_sol<N>(k, so, so, false, R);
        }
        phiR = R.phi0;
        vr[0] = R.u;
        vr[1] = R.v;
        vr[2] = R.w;
      }
      s_phiR[f] = phiR;
      s_vel[f][0] = vr[0];
      s_vel[f][1] = vr[1];
      s_vel[f][2] = vr[2];
    }
    __syncwarp();
    if (lane == 0) {
      double s[C::NEQ], sn[C::NEQ];
#pragma unroll
      for (int e = 0; e < C::NEQ; e++) {
        s[e] = own[e];
        sn[e] = SN[(int64_t)e * m.n + c];
      }
      const double V = g.vol[l];
      double rho_new = 0.0, ut, vt, wt;
      if (!relax) {
        for (int v = 0; v < N; ++v) rho_new += s[v] + (DT / V) * RHS[(int64_t)v * m.n + c];
        ut = s[C::i1 + 0] + (DT / V) * RHS[(int64_t)(C::i1 + 0) * m.n + c];
        vt = s[C::i1 + 1] + (DT / V) * RHS[(int64_t)(C::i1 + 1) * m.n + c];
        wt = s[C::i1 + 2] + (DT / V) * RHS[(int64_t)(C::i1 + 2) * m.n + c];
        ut = ut / rho_new;
        vt = vt / rho_new;
        wt = wt / rho_new;
      } else {
        for (int v = 0; v < N; ++v) rho_new += s[v];
        ut = s[C::i1 + 0] / rho_new;
        vt = s[C::i1 + 1] / rho_new;
        wt = s[C::i1 + 2] / rho_new;
      }
      double nxi = 0.0, nyi = 0.0, nzi = 0.0, total = 0.0, ug[6], vg[6], wg[6];
      int nint = 0;
      for (int f = 0; f < 6; f++) {
        if (GF[(int64_t)f * m.n + c] == 1.0) {
          const double phi = (L.phi0 + s_phiR[f]) / 2.0;
          const double A = g.area[ffv_face_kind(info, f) == FFV_FK_FINER ? l + 1 : l];
          const int ax = fr_n_axis(f), sg = fr_n_sign(f);
          const double nv[3] = {ax == 0 ? (double)sg : 0.0, ax == 1 ? (double)sg : 0.0,
                                ax == 2 ? (double)sg : 0.0};
          if (relax) {
            nxi += phi * A * nv[0];
            nyi += phi * A * nv[1];
            nzi += phi * A * nv[2];
          } else {
            nxi = phi * A * nv[0];
            nyi = phi * A * nv[1];
            nzi = phi * A * nv[2];
          }
          ug[nint] = s_vel[f][0];
          vg[nint] = s_vel[f][1];
          wg[nint] = s_vel[f][2];
          total += A;
          nint++;
        }
      }
      if (nint != 0) {
        const double norm = sqrt(nxi * nxi + nyi * nyi + nzi * nzi);
        nxi = -nxi / norm;
        nyi = -nyi / norm;
        nzi = -nzi / norm;
        double n1x, n1y, n1z;
        if (fabs(nzi) < 0.99) {
          n1x = nyi;
          n1y = -nxi;
          n1z = 0.0;
        } else {
          n1x = nzi;
          n1y = 0.0;
          n1z = -nxi;
        }
        const double n2x = nyi * n1z - nzi * n1y, n2y = nzi * n1x - nxi * n1z,
                     n2z = nxi * n1y - nyi * n1x;
        const double ul = ut * nxi + vt * nyi + wt * nzi;
        double vnl = 0.0, wnl = 0.0;
        int ft = 0;
        for (int f = 0; f < 6; f++) {
          if (GF[(int64_t)f * m.n + c] == 1.0) {
            const double A = g.area[ffv_face_kind(info, f) == FFV_FK_FINER ? l + 1 : l];
            const double vl = ug[ft] * n1x + vg[ft] * n1y + wg[ft] * n1z;
            const double wl = ug[ft] * n2x + vg[ft] * n2y + wg[ft] * n2z;
            vnl = vl * (A / total);
            wnl = wl * (A / total);
            ft++;
          }
        }
        const double ung = ul * nxi + vnl * n1x + wnl * n2x;
        const double vng = ul * nyi + vnl * n1y + wnl * n2y;
        const double wng = ul * nzi + vnl * n1z + wnl * n2z;
        if (!relax)
          for (int v = 0; v < N; ++v) s[v] = s[v] + (DT / V) * RHS[(int64_t)v * m.n + c];
        s[C::i1 + 0] = rho_new * ung;
        s[C::i1 + 1] = rho_new * vng;
        s[C::i1 + 2] = rho_new * wng;
        s[C::i2] -= rho_new * 0.5 * (ut * ut + vt * vt + wt * wt);
        s[C::i2] += rho_new * 0.5 * (ung * ung + vng * vng + wng * wng);
      } else if (!relax) {
        for (int v = 0; v < N; ++v) s[v] = s[v] + (DT / V) * RHS[(int64_t)v * m.n + c];
        for (int d = 0; d < 3; d++)
          s[C::i1 + d] = s[C::i1 + d] + (DT / V) * RHS[(int64_t)(C::i1 + d) * m.n + c];
      }
      if (!relax) clamp_zerou<N>(k, s, sn);
      for (int e = 0; e < C::NEQ; e++) Snew[(int64_t)e * m.n + c] = s[e];
    }
    __syncwarp();
  }
}

// ordered compaction of flag[] into list[] (leaf order kept): per-block counts, one-block
// exclusive scan, per-block ordered scatter
constexpr int CB = 1024;
__global__ void __launch_bounds__(CB) flag_count(int64_t n, const uint8_t *__restrict__ flag,
                                                 int32_t *__restrict__ bcount) {
  __shared__ int warp_sum[CB / 32];
  const int64_t c = (int64_t)blockIdx.x * CB + threadIdx.x;
  const int f = (c < n) ? flag[c] : 0;
  const unsigned b = __ballot_sync(0xffffffffu, f);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < CB / 32; w++) s += warp_sum[w];
    bcount[blockIdx.x] = s;
  }
}
__global__ void __launch_bounds__(CB) flag_scan(int nb, int32_t *__restrict__ bcount,
                                                int32_t *__restrict__ total) {
  // single block: sequential carry over chunks of CB, warp-level scans inside
  __shared__ int warp_tot[CB / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += CB) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? bcount[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) warp_tot[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      int t = warp_tot[threadIdx.x];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (threadIdx.x >= o) t += y;
      }
      warp_tot[threadIdx.x] = t;
    }
    __syncthreads();
    const int incl = x + ((threadIdx.x >> 5) ? warp_tot[(threadIdx.x >> 5) - 1] : 0);
    if (i < nb) bcount[i] = carry + incl - v;
    __syncthreads();
    if (threadIdx.x == CB - 1) carry += incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}
__global__ void __launch_bounds__(CB) flag_scatter(int64_t n, const uint8_t *__restrict__ flag,
                                                   const int32_t *__restrict__ boff,
                                                   int32_t *__restrict__ list) {
  __shared__ int warp_off[CB / 32];
  const int64_t c = (int64_t)blockIdx.x * CB + threadIdx.x;
  const int f = (c < n) ? flag[c] : 0;
  const unsigned b = __ballot_sync(0xffffffffu, f);
  if ((threadIdx.x & 31) == 0) warp_off[threadIdx.x >> 5] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < CB / 32; w++) {
      const int t = warp_off[w];
      warp_off[w] = s;
      s += t;
    }
  }
  __syncthreads();
  if (f) {
    const int r = __popc(b & ((1u << (threadIdx.x & 31)) - 1u));
    list[boff[blockIdx.x] + warp_off[threadIdx.x >> 5] + r] = (int32_t)c;
  }
}

// CFL (new, the reference has a fixed DT): dt = h / (max_a |u_a| + c), mixture sound
// speed c = sqrt(sum_k c2Y_k) as m5_wave_speeds.c:43-50 forms it
template <int N>
__global__ void m5_cfl_kernel(ffv_dmesh m, ffv_geom g, M5Consts k, const double *__restrict__ S,
                              unsigned long long *out) {
  double best = INFINITY;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < m.n;
       c += (int64_t)gridDim.x * blockDim.x) {
    double s[K5<N>::NEQ];
    load_state<N>(S, m.n, c, s);
    Sol<N> q;
    make_sol<N>(k, s, s, false, q);
    const double sp = fmax(fmax(fabs(q.u), fabs(q.v)), fabs(q.w)) + sqrt(q.c2);
    const double dt = g.h[ffv_info_level(m.info[c])] / sp;
    best = (dt < best || isnan(dt)) ? dt : best;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double other = __shfl_xor_sync(0xffffffffu, best, o);
    best = (other < best || isnan(other)) ? other : best;
  }
  if ((threadIdx.x & 31) == 0) {
    const unsigned long long bits =
        isnan(best) ? 0x7ff8000000000000ULL : (unsigned long long)__double_as_longlong(best);
    atomicMin(out, best >= 0.0 || isnan(best) ? bits : 0ULL);
  }
}

// ------------------------------------------------------------------ refinement tags
// phi[v] of a cell (m5_facevalues.c:83-99): the clamped volume fractions against AVF_LIM
// (phi[0] the larger of two solids' fractions when there are two)
template <int N>
__device__ __forceinline__ void cell_phi(const M5Consts &k, const double *__restrict__ S,
                                         int64_t n, int64_t c, double phi[2]) {
  using C = K5<N>;
  const double lo = k.amin / 100.0, hi = 1.0 - (k.amin / 100.0);
  double ac[2] = {0.0, 0.0};
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    double a = S[(int64_t)(C::i3 + i) * n + c];
    if (a <= lo) a = lo;
    else if (a >= hi) a = hi;
    ac[i] = a;
  }
  phi[0] = ac[0] - k.avf_lim;
  phi[1] = ac[1] - k.avf_lim;
  if (N > 2 && k.nsolids == 2 && k.mu[0] != 0.0)
    phi[0] = ((ac[0] > ac[1]) ? ac[0] : ac[1]) - k.avf_lim;
}

// neighbour q (< count) of cell c across face f; count 0 for boundary faces
__device__ __forceinline__ int face_neighbours(const ffv_dmesh &m, int64_t c, uint32_t info, int f,
                                               int64_t nb[4]) {
  const uint32_t kind = ffv_face_kind(info, f);
  if (kind & FFV_FK_BC) return 0;
  const int32_t s = m.nbr[(int64_t)f * m.n + c];
  if (kind == FFV_FK_FINER) {
#pragma unroll
    for (int q = 0; q < 4; q++) nb[q] = m.sub[4 * (int64_t)s + q];
    return 4;
  }
  nb[0] = s;
  return 1;
}

// interface_location.c:17-46: SI = 1 where phi changes sign across a face (the face loop
// stops after the first face that shows a change)
template <int N>
__global__ void __launch_bounds__(128) m5_si_first(ffv_dmesh m, M5Consts k,
                                                   const double *__restrict__ S,
                                                   int32_t *__restrict__ SI) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  const uint32_t info = m.info[c];
  double pl[2], pr[2];
  cell_phi<N>(k, S, m.n, c, pl);
  int si0 = 0, si1 = 0;
  bool hit = false;
  for (int f = 0; f < 6 && !hit; f++) {
    int64_t nb[4];
    const int cnt = face_neighbours(m, c, info, f, nb);
    for (int q = 0; q < cnt; q++) {
      cell_phi<N>(k, S, m.n, nb[q], pr);
      for (int v = 0; v < N - 1; ++v)
        if (pl[v] * pr[v] < 0.0) {
          if (v == 0) si0 = 1;
          else si1 = 1;
          hit = true;
        }
    }
  }
  SI[c] = si0;
  SI[m.n + c] = si1;
}

// interface_location.c:52-80: layer lvl next to layer lvl - 1.  The reference updates in
// place in leaf order, but a cell only reads neighbours' lvl - 1 entries and only writes
// lvl into entries that were 0, so reading the previous layer's copy gives the same result.
__global__ void __launch_bounds__(128) m5_si_layer(ffv_dmesh m, int lvl,
                                                   const int32_t *__restrict__ SIin,
                                                   int32_t *__restrict__ SIout) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  const uint32_t info = m.info[c];
  int s[2] = {SIin[c], SIin[m.n + c]};
  bool hit = false;
  for (int f = 0; f < 6 && !hit; f++) {
    int64_t nb[4];
    const int cnt = face_neighbours(m, c, info, f, nb);
    for (int q = 0; q < cnt; q++)
      for (int v = 0; v < 2; ++v)
        if (SIin[(int64_t)v * m.n + nb[q]] == lvl - 1 && s[v] == 0) {
          s[v] = lvl;
          hit = true;
        }
  }
  SIout[c] = s[0];
  SIout[m.n + c] = s[1];
}

// relative jump |x_nb - x| / max(|x_nb|, |x|) (criterionsplt.c:83-89), 0 below 1e-8
__device__ __forceinline__ double rel_jump(double x_cur, double x_nb) {
  const double eps = 1.0e-8;
  if ((fabs(x_nb) > eps) || (fabs(x_cur) > eps)) {
    const double a = fabs(x_nb), b = fabs(x_cur);
    return fabs(x_nb - x_cur) / ((a > b) ? a : b);
  }
  return 0.0;
}

// each cell's alpha-weighted pressure sum_k alpha_k p_k and density, from the reference's cell
// primitives (make_sol of the cell state): computed once per cell here, read by every
// neighbour's criterion below (the same doubles the per-neighbour evaluation gave)
template <int N>
__global__ void __launch_bounds__(128) m5_tag_prims(int64_t n, M5Consts k,
                                                    const double *__restrict__ S,
                                                    double *__restrict__ pr) {
  using C = K5<N>;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double s[C::NEQ];
  load_state<N>(S, n, c, s);
  Sol<N> q;
  make_sol<N>(k, s, s, false, q);
  double p = 0.0;
#pragma unroll
  for (int iv = 0; iv < N; ++iv) p += q.avf[iv] * q.p[iv];
  pr[c] = p;
  pr[n + c] = q.r;
}

// criterionsplt.c:3-140 per cell: the uniform level, the gradient criterion over every
// sub-neighbour and the interface layers
__global__ void __launch_bounds__(128) m5_tag_split(ffv_dmesh m, ffv_m5_tagc t,
                                                    const double *__restrict__ pr,
                                                    const int32_t *__restrict__ SI,
                                                    int32_t *__restrict__ split) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  int level = 1;
  if (t.uniform == 1) level = level > t.lvl_uniform ? level : t.lvl_uniform;
  if (t.prs == 1 || t.rho == 1 || t.vel == 1) {
    const uint32_t info = m.info[c];
    const double pL = pr[c], rL = pr[m.n + c];
    double gp = 0.0, gr = 0.0, gv = 0.0;
    for (int f = 0; f < 6; f++) {
      int64_t nb[4];
      const int cnt = face_neighbours(m, c, info, f, nb);
      for (int q = 0; q < cnt; q++) {
        if (t.prs == 1) {
          const double g = rel_jump(pL, pr[nb[q]]);
          gp = (g > gp) ? g : gp;
        }
        double grho = 0.0;
        if (t.rho == 1) {
          grho = rel_jump(rL, pr[m.n + nb[q]]);
          gr = (grho > gr) ? grho : gr;
        }
        // the reference's velocity criterion takes the density jump (criterionsplt.c:120)
        if (t.vel == 1) gv = (grho > gv) ? grho : gv;
      }
    }
    int lt = 1;
    if (t.prs == 1 && fabs(gp) >= t.thr_prs) lt = t.lvl_prs;
    if (t.rho == 1 && fabs(gr) >= t.thr_rho) lt = t.lvl_rho;
    if (t.vel == 1 && fabs(gv) >= t.thr_vel) lt = t.lvl_vel;
    level = level > lt ? level : lt;
  }
  if (t.inter0 != 0) {
    for (int v = 0; v < 2; ++v) {
      const int si = SI[(int64_t)v * m.n + c];
      if (si >= 1 && si < t.lrs0) level = level > t.lvl0 ? level : t.lvl0;
      if (si >= t.lrs0 && si < t.lrs1) level = level > t.lvl1 ? level : t.lvl1;
    }
  }
  split[c] = level;
}

// exported fields (FP64): rho, u, v, w, sum_k alpha_k p_k, alpha_k, p_k, von Mises stress
// of the reference's cell primitives (make_sol of the cell state)
template <int N>
__global__ void __launch_bounds__(128) m5_export_fields(int64_t n, M5Consts k,
                                                        const double *__restrict__ S,
                                                        double *__restrict__ F) {
  using C = K5<N>;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double s[C::NEQ];
  load_state<N>(S, n, c, s);
  Sol<N> q;
  make_sol<N>(k, s, s, false, q);
  double p = 0.0;
#pragma unroll
  for (int iv = 0; iv < N; ++iv) p += q.avf[iv] * q.p[iv];
  const double tr = (q.st[0][0] + q.st[1][1] + q.st[2][2]) / 3.0;
  double j2 = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const double d = q.st[i][j] - (i == j ? tr : 0.0);
      j2 += d * d;
    }
  F[c] = q.r;
  F[n + c] = -q.u;  // the state holds the negated momentum in this node layout
  F[2 * n + c] = -q.v;
  F[3 * n + c] = -q.w;
  F[4 * n + c] = p;
#pragma unroll
  for (int iv = 0; iv < N; ++iv) {
    F[(int64_t)(5 + iv) * n + c] = q.avf[iv];
    F[(int64_t)(5 + N + iv) * n + c] = q.p[iv];
  }
  F[(int64_t)(5 + 2 * N) * n + c] = sqrt(1.5 * j2);
}

// merged cells of a mesh adaptation (map < 0): the reference's relaxation of the merged
// state (merge.c:52-57)
template <int N>
__global__ void __launch_bounds__(128) m5_relax_merged(int64_t n, M5Consts k,
                                                       const int64_t *__restrict__ map,
                                                       double *__restrict__ S) {
  using C = K5<N>;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n || map[c] >= 0) return;
  double s[C::NEQ];
  load_state<N>(S, n, c, s);
  relaxationvec<N>(k, s);
#pragma unroll
  for (int e = 0; e < C::NEQ; e++) S[(int64_t)e * n + c] = s[e];
}

}  // namespace

void ffv_m5_relax_merged(int64_t n, const M5Consts &k, const int64_t *map, double *S,
                         cudaStream_t st) {
  const unsigned gc = (unsigned)((n + 127) / 128);
  if (k.nmat == 2) m5_relax_merged<2><<<gc, 128, 0, st>>>(n, k, map, S);
  else m5_relax_merged<3><<<gc, 128, 0, st>>>(n, k, map, S);
}

void ffv_m5_export_fields(int64_t n, const M5Consts &k, const double *S, double *F,
                          cudaStream_t st) {
  const unsigned gc = (unsigned)((n + 127) / 128);
  if (k.nmat == 2) m5_export_fields<2><<<gc, 128, 0, st>>>(n, k, S, F);
  else m5_export_fields<3><<<gc, 128, 0, st>>>(n, k, S, F);
}

void ffv_m5_tags(const ffv_dmesh &m, const M5Consts &k, const ffv_m5_tagc &t, const double *S,
                 int32_t *SI, int32_t *SItmp, int32_t *split, double *pr, cudaStream_t st) {
  const unsigned gc = (unsigned)((m.n + 127) / 128);
  if (t.inter0 != 0) {
    if (k.nmat == 2) m5_si_first<2><<<gc, 128, 0, st>>>(m, k, S, SI);
    else m5_si_first<3><<<gc, 128, 0, st>>>(m, k, S, SI);
    for (int lvl = 2; lvl < t.si_max; lvl++) {
      cudaMemcpyAsync(SItmp, SI, sizeof(int32_t) * 2 * m.n, cudaMemcpyDeviceToDevice, st);
      m5_si_layer<<<gc, 128, 0, st>>>(m, lvl, SItmp, SI);
    }
  } else {
    cudaMemsetAsync(SI, 0, sizeof(int32_t) * 2 * m.n, st);
  }
  if (t.prs == 1 || t.rho == 1 || t.vel == 1) {
    if (k.nmat == 2) m5_tag_prims<2><<<gc, 128, 0, st>>>(m.n, k, S, pr);
    else m5_tag_prims<3><<<gc, 128, 0, st>>>(m.n, k, S, pr);
  }
  m5_tag_split<<<gc, 128, 0, st>>>(m, t, pr, SI, split);
}

void ffv_m5_cfl(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                unsigned long long *d_out, cudaStream_t st) {
  if (k.nmat == 2) m5_cfl_kernel<2><<<152 * 4, 128, 0, st>>>(m, g, k, S, d_out);
  else m5_cfl_kernel<3><<<152 * 4, 128, 0, st>>>(m, g, k, S, d_out);
}

int ffv_m5_neq(int nmat) { return 3 * nmat + 12; }

// kernel names in launch order, for ffv_profile_stage
static const char *k_names[] = {"m5_recon_face", "m5_face_flux",  "m5_cell_update",
                                "flag_count",    "flag_scan",     "flag_scatter",
                                "m5_gfm_seq",    "m5_relax_cell", "flag_count",
                                "flag_scan",     "flag_scatter",  "m5_gfm_seq(relax)"};

struct Rec {
  cudaEvent_t *ev;
  int i;
  const char **names;
  cudaStream_t st;
  void operator()(const char *name) {
    if (ev) {
      names[i] = name;
      cudaEventRecord(ev[++i], st);
    }
  }
};

template <int N>
static void stage_impl(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k,
                       const ffv_m5_bufs &b, int irk, cudaStream_t st, cudaEvent_t *ev,
                       const char **names) {
  const int tpb = 128;
  const unsigned gf = (unsigned)((6 * m.n + tpb - 1) / tpb), gc = (unsigned)((m.n + tpb - 1) / tpb);
  const unsigned nb = (unsigned)((m.n + CB - 1) / CB);
  Rec rec{ev, 0, names, st};
  if (ev) cudaEventRecord(ev[0], st);
  const bool f32 = k.precision == FFV_FP32_FLUX;
  // the FP32 form keeps its face states and fluxes in the same buffers, as floats
  float *SFf = (float *)b.SF, *FFf = (float *)b.FF, *UFf = (float *)b.UF;
  if (k.order == 2) {
    if (f32) {
      // the FP32 copy of the state lives in RHS, which m5_cell_update writes later
      ffv_m5f_shadow(m.n, k, b.S, (float *)b.RHS, st);
      rec("m5f_shadow");
      ffv_m5f_recon(m, g, k, b.S, (float *)b.RHS, SFf, b.status, st);
    } else {
      m5_recon_face<N><<<gf, tpb, 0, st>>>(m, g, k, b.S, b.SF, b.status);
    }
    rec(f32 ? "m5f_recon_face" : k_names[0]);
  }
  if (f32)
    ffv_m5f_flux(m, g, k, b.S, k.order == 2 ? (const float *)b.RHS : nullptr, SFf, FFf, UFf, b.GF,
                 b.status, st);
  else m5_face_flux<N><<<gf, tpb, 0, st>>>(m, g, k, b.S, b.SF, b.FF, b.UF, b.GF, b.status);
  rec(f32 ? "m5f_face_flux" : k_names[1]);
  if (f32)
    ffv_m5f_cell_update(m, g, k, b.S, b.SN, FFf, UFf, b.RHS, b.Snew, b.flag, b.dt, irk, b.status,
                        st);
  else
    m5_cell_update<N, double><<<gc, tpb, 0, st>>>(m, g, k, b.S, b.SN, b.FF, b.UF, b.RHS, b.Snew,
                                                  b.flag, b.dt, irk, b.status);
  rec(f32 ? "m5f_cell_update" : k_names[2]);
  if (irk == 1) {
    flag_count<<<nb, CB, 0, st>>>(m.n, b.flag, b.bcount);
    rec(k_names[3]);
    flag_scan<<<1, CB, 0, st>>>((int)nb, b.bcount, b.count);
    rec(k_names[4]);
    flag_scatter<<<nb, CB, 0, st>>>(m.n, b.flag, b.bcount, b.list);
    rec(k_names[5]);
    m5_gfm_seq<N><<<1, 32, 0, st>>>(m, g, k, b.list, b.count, b.S, b.Snew, b.SN, b.RHS, b.GF,
                                    b.dt, 0);
    rec(k_names[6]);
  }
  if (f32) ffv_m5f_relax_cell(m.n, k, b.Snew, b.S, b.flag, b.status, st);
  else m5_relax_cell<N><<<gc, tpb, 0, st>>>(m.n, k, b.Snew, b.S, b.flag, b.status);
  rec(f32 ? "m5f_relax_cell" : k_names[7]);
  flag_count<<<nb, CB, 0, st>>>(m.n, b.flag, b.bcount);
  rec(k_names[8]);
  flag_scan<<<1, CB, 0, st>>>((int)nb, b.bcount, b.count);
  rec(k_names[9]);
  flag_scatter<<<nb, CB, 0, st>>>(m.n, b.flag, b.bcount, b.list);
  rec(k_names[10]);
  // relaxed states are in S; a later neighbour is still unrelaxed (Snew)
  m5_gfm_seq<N><<<1, 32, 0, st>>>(m, g, k, b.list, b.count, b.Snew, b.S, b.SN, b.RHS, b.GF,
                                  b.dt, 1);
  rec(k_names[11]);
}

void ffv_m5_fp64_stage(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k,
                       const ffv_m5_bufs &b, int irk, cudaStream_t st, cudaEvent_t *ev,
                       const char **names) {
  if (k.nmat == 2) stage_impl<2>(m, g, k, b, irk, st, ev, names);
  else stage_impl<3>(m, g, k, b, irk, st, ev, names);
}

int ffv_m5_launches_per_stage(const M5Consts &k, int irk) {
  const int recon = k.order == 2 ? (k.precision == FFV_FP32_FLUX ? 2 : 1) : 0;
  return recon + 2 + (irk == 1 ? 4 : 0) + 1 + 4;
}
