// Model-5 FP32-flux form: face reconstruction, wave speeds, star states and HLLC /
// ghost-fluid HLLC fluxes in FP32; double-float (FP32 pairs, ffv_df.cuh) where cancellation
// needs more than FP32, FP64 only for the RK state and the residual sums.
//
// The algorithm is the FP64 form's (ffv_m5_fp64.cu, itself the reference's m5_* code), with
// these precision choices:
//   * MUSCL slopes and limiter in FP32 on an FP32 copy of the state.  The "critical" slots
//     -- volume fractions, internal energies, total energy, which the stiffened-gas
//     pressure recovery divides and cancels -- are carried as double-float pairs (the low
//     parts written by m5f_shadow once per cell and stage): their face values are the pair
//     plus the FP32 slope correction, their slopes the pairs' differences.
//   * Pressure relaxation of a face or cell state: each material's initial pressure
//     p_k = (gamma_k - 1)(alpha rho e_k - e_el) / alpha_k - gamma_k p_inf_k (a difference
//     of two ~1e9 numbers for a liquid with p_inf 6e8, divided by alpha_k that can be
//     1e-8) and the final energy-consistent equilibrium pressure and internal energies in
//     double-float; the Newton iteration on the equilibrium pressure in between in FP32 (it
//     only has to locate the volume fractions).  GB300 runs FP64 at 1/64 of the FP32 rate,
//     and FP64<->FP32 conversions share that pipe: double-float keeps this work on the FP32
//     pipe.
//   * The face record handed to the flux kernel holds the face state in FP32 plus each
//     material's recovered pressure (rounded once to FP32) and the last material's volume
//     fraction (1 - sum formed on the pairs: in FP32 that difference would lose a 1e-6
//     fraction next to 1).
//   * The deformation tensor A is carried as its deviation D = A - I wherever it is FP32
//     (copy of the state, face records, face states): the elastic stress and energy are
//     formed from E = A A^T - I = D + D^T + D D^T, exact to FP32 relative to the strain.
//   * Wave speeds, star region, physical flux, HLLC and its ghost-fluid variant: FP32.
//     Face fluxes are stored as FP32 and summed into the FP64 cell residual by
//     m5f_cell_update; the RK state stays FP64.
// Compiled with FMA contraction (no bit-exactness goal here: the error against the FP64
// form is measured instead).
#include <math.h>

#include "ffv_cvt.cuh"
#include "ffv_device.cuh"
#include "ffv_m5.cuh"
#include "ffv_m5_frame.cuh"
#include "ffv_plastic.cuh"

namespace {

// face record: [neq conserved | nmat pressures | last volume fraction]
template <int N>
struct RecL {
  static constexpr int NEQ = K5<N>::NEQ, P = NEQ, AL = NEQ + N, SIZE = NEQ + N + 1;
};

// ------------------------------------------------------------------ EOS in FP32
// The FP32 form carries the deformation tensor as its deviation D = A - I from the identity
// (the FP32 copy of the state, the face records, the face states).  The solid's stress is
// mu times the strain, ~1e-3 beside the identity: G = A A^T formed from an FP32 A would carry
// the ~6e-8 rounding of entries near 1 into every stress (mu * 1e-7, tens of kPa for a metal),
// while E = G - I = D + D^T + D D^T keeps FP32 precision relative to the strain itself.
// The reference's G-form expressions (state_equation.c:143-204, 269-317) are rewritten
// exactly in E:  |G| - 1 = tr E + (sum of E's principal 2x2 minors) + det E,
// tr((G - |G|^(1/3) I)^2) = tr((E - g I)^2) and the stress deviator
// G^2 - tr(G^2)/3 I - |G|^(1/3) (G - tr G/3 I) = (1 - g) dev E + dev(E^2), g = |G|^(1/3) - 1.
struct StrainF {
  float E[6];    // G - I (symmetric): E00, E11, E22, E01, E02, E12
  float g;       // |G|^(1/3) - 1
  float ig16;    // |G|^(-1/6)
  float tr2;     // tr((E - g I)^2)
  float dev[6];  // (1 - g) dev E + dev(E^2), by stress_deviator_f
  bool solid;    // |G| != 0 (a fluid cell carries A = 0: no elastic stress)
};

// slot of E_ij in StrainF::E
__host__ __device__ constexpr int esym(int i, int j) {
  return i == j ? i : (i + j == 1 ? 3 : (i + j == 2 ? 4 : 5));
}

// E, |G|^(1/3) - 1, |G|^(-1/6) and tr((E - g I)^2) of a deviation D: the material-independent
// parts of every material's elastic energy (the materials differ by their shear modulus only)
__device__ __forceinline__ void strain_f(const float D[9], StrainF &s) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++)
      s.E[esym(i, j)] = D[3 * i + j] + D[3 * j + i] +
                        (D[3 * i] * D[3 * j] + D[3 * i + 1] * D[3 * j + 1] + D[3 * i + 2] * D[3 * j + 2]);
  const float e00 = s.E[0], e11 = s.E[1], e22 = s.E[2], e01 = s.E[3], e02 = s.E[4], e12 = s.E[5];
  const float m2 = (e00 * e11 - e01 * e01) + (e00 * e22 - e02 * e02) + (e11 * e22 - e12 * e12);
  const float dE = e00 * (e11 * e22 - e12 * e12) - e01 * (e01 * e22 - e12 * e02) +
                   e02 * (e01 * e12 - e11 * e02);
  const float x = (e00 + e11 + e22) + m2 + dE;  // |G| - 1
  s.solid = (1.0f + x) != 0.0f;
  float g16;
  if (fabsf(x) <= 0.03125f) {
    // (1 + x)^(1/3) - 1 by its binomial series to x^5 (coefficients 1/3, -1/9, 5/81,
    // -10/243, 22/729); the first omitted term is below 2e-9 of the sum for |x| <= 1/32
    s.g = x * (1.0f / 3.0f + x * (-1.0f / 9.0f + x * (5.0f / 81.0f + x * (-10.0f / 243.0f + x * (22.0f / 729.0f)))));
    g16 = sqrtf(1.0f + s.g);
  } else {
    const float g13 = cbrtf(fabsf(1.0f + x));
    s.g = g13 - 1.0f;
    g16 = sqrtf(g13);
  }
  s.ig16 = 1.0f / g16;
  const float d0 = e00 - s.g, d1 = e11 - s.g, d2 = e22 - s.g;
  s.tr2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.0f * (e01 * e01 + e02 * e02 + e12 * e12);
}

// the stress deviator's material-independent factor (1 - g) dev E + dev(E^2) into s.dev
__device__ __forceinline__ void stress_deviator_f(StrainF &s) {
  const float *E = s.E;
  float E2[6];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++)
      E2[esym(i, j)] = E[esym(i, 0)] * E[esym(0, j)] + E[esym(i, 1)] * E[esym(1, j)] +
                       E[esym(i, 2)] * E[esym(2, j)];
  const float J1 = (E[0] + E[1] + E[2]) * (1.0f / 3.0f), J2 = (E2[0] + E2[1] + E2[2]) * (1.0f / 3.0f);
  const float a = 1.0f - s.g;
#pragma unroll
  for (int q = 0; q < 6; q++) s.dev[q] = q < 3 ? a * (E[q] - J1) + (E2[q] - J2) : a * E[q] + E2[q];
}

// e_el = mu / (4 |G|^(1/6)) tr((G - |G|^(1/3) I)^2)   (state_equation.c:269-317)
__device__ __forceinline__ float elastic_energy_f(const StrainF &s, float mu) {
  if (!s.solid || !(mu != 0.0f)) return 0.0f;
  return (0.25f * mu) * s.ig16 * s.tr2;
}

// material stress -alpha p I - mu/|G|^(1/6) ((1 - g) dev E + dev(E^2)), accumulated into st
// (state_equation.c:143-204 in the E form; s.dev from stress_deviator_f)
__device__ __forceinline__ void eos_stress_f(float st[3][3], float avf, float pr, const StrainF &e,
                                             float mu, float (*ast)[3]) {
  float s[6];
  if (e.solid && (mu != 0.0f)) {
    const float f = mu * e.ig16;
#pragma unroll
    for (int q = 0; q < 6; q++) s[q] = q < 3 ? -avf * pr - f * e.dev[q] : -f * e.dev[q];
  } else {
#pragma unroll
    for (int q = 0; q < 6; q++) s[q] = q < 3 ? -avf * pr : 0.0f;
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      st[i][j] += s[esym(i, j)];
      if (ast) ast[i][j] = s[esym(i, j)];
    }
}

// D of an FP64 deformation tensor: A - I formed in FP64, then rounded
__device__ __forceinline__ float dev_of(const double *A, int q) {
  return f32_of_f64(A[q] - ((q == 0 || q == 4 || q == 8) ? 1.0 : 0.0));
}

// A of a deviation, for the advection of A (there relative FP32 precision of A is enough)
__device__ __forceinline__ float full_of(const float *D, int q) {
  return D[q] + ((q == 0 || q == 4 || q == 8) ? 1.0f : 0.0f);
}

template <int N>
struct SolF {
  float r, u, v, w, e, ut, vt, wt, c2;
  float phi0;
  float ra[N], avf[N], are[N], p[N];
  float D[9], st[3][3];  // D = A - I
  float vec[K5<N>::NC];
};

// primitive state of a face record (m5_facercnstr.c:3-191 with the pressures given)
template <int N>
__device__ void make_sol_f(const M5Consts &k, const float *U, float phi0, SolF<N> &s) {
  using C = K5<N>;
  using RL = RecL<N>;
  s.r = 0.0f;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    s.r += U[i];
    s.ra[i] = U[i];
    s.vec[i] = U[i];
  }
  const float ir = 1.0f / s.r;
  s.u = U[C::i1 + 0] * ir;
  s.v = U[C::i1 + 1] * ir;
  s.w = U[C::i1 + 2] * ir;
#pragma unroll
  for (int d = 0; d < 3; d++) s.vec[C::i1 + d] = U[C::i1 + d];
  s.e = U[C::i2] * ir;
  s.vec[C::i2] = U[C::i2];
#pragma unroll
  for (int i = 0; i < N - 1; ++i) s.avf[i] = U[C::i3 + i];
  s.avf[N - 1] = U[RL::AL];
  s.phi0 = phi0;
#pragma unroll
  for (int i = 0; i < N; ++i) s.are[i] = U[C::i4 + i];
#pragma unroll
  for (int q = 0; q < 9; q++) s.D[q] = U[C::i5 + q];
  StrainF sE;
  strain_f(s.D, sE);
  stress_deviator_f(sE);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) s.st[i][j] = 0.0f;
  float c2 = 0.0f;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const float press = U[RL::P + i];
    s.p[i] = press;
    c2 += (s.avf[i] * ir) * k.gamma_f[i] * (press + k.pinf_f[i]);
    eos_stress_f(s.st, s.avf[i], press, sE, k.mu_f[i], nullptr);
  }
  s.c2 = c2;
}

// phi[0] of a cell (m5_facevalues.c:83-99): the solid fraction(s) against AVF_LIM, FP64
template <int N>
__device__ __forceinline__ double cell_phi0(const M5Consts &k, const double *__restrict__ S,
                                            int64_t n, int64_t c) {
  using C = K5<N>;
  const double lo = k.amin / 100.0, hi = 1.0 - (k.amin / 100.0);
  double ac[N > 2 ? 2 : 1];
#pragma unroll
  for (int i = 0; i < (N > 2 ? 2 : 1); ++i) {
    double a = S[(int64_t)(C::i3 + i) * n + c];
    if (a >= hi) a = hi;
    else if (a <= lo) a = lo;
    ac[i] = a;
  }
  if (N > 2 && k.nsolids == 2 && k.mu[0] != 0.0)
    return ((ac[0] > ac[N > 2 ? 1 : 0]) ? ac[0] : ac[N > 2 ? 1 : 0]) - k.avf_lim;
  return ac[0] - k.avf_lim;
}

// the same from the FP32 copy of the state (order 2: the reconstruction made it); only the
// sign of phi0 is used (which side of AVF_LIM a cell is on)
template <int N>
__device__ __forceinline__ float cell_phi0_f(const M5Consts &k, const float *__restrict__ Sf,
                                             int64_t n, int64_t c) {
  using C = K5<N>;
  float ac[N > 2 ? 2 : 1];
#pragma unroll
  for (int i = 0; i < (N > 2 ? 2 : 1); ++i) {
    float a = Sf[(int64_t)(C::i3 + i) * n + c];
    if (a >= k.ahi_f) a = k.ahi_f;
    else if (a <= k.alo_f) a = k.alo_f;
    ac[i] = a;
  }
  const float lim = k.avf_lim_f;
  if (N > 2 && k.phi_pair)
    return ((ac[0] > ac[N > 2 ? 1 : 0]) ? ac[0] : ac[N > 2 ? 1 : 0]) - lim;
  return ac[0] - lim;
}

template <int F, int N>
__device__ __forceinline__ void ghost_f(const SolF<N> &L, int bc, SolF<N> &R) {
  R = L;
  if (bc == 1 || bc == 4 || bc == 5) {
    const float v3[3] = {L.u, L.v, L.w};
    const float ul = loc<F, 0>(v3), vl = loc<F, 1>(v3), wl = loc<F, 2>(v3);
    const float ur = -ul, vr = bc == 5 ? -vl : vl, wr = bc == 5 ? -wl : wl;
    R.u = glob<F, 0>(ur, vr, wr);
    R.v = glob<F, 1>(ur, vr, wr);
    R.w = glob<F, 2>(ur, vr, wr);
  }
}

template <int N>
struct NCf {
  float unc[3], avf[N], are[N], A[9];  // A itself (advected), not its deviation
};

// m5_star_region.c:3-158 in FP32.  dU receives the jump U*_K - U_K of the conservative
// variables (what the HLLC correction S_K (U*_K - U_K) needs).  With the consistent flux
// form the jumps of the partial densities and of the total energy are formed as differences,
// never as U*_K minus U_K: the solid's total energy is ~5e10 J/m^3 (p_inf 3.2e10), whose FP32
// ulp (4096) would otherwise enter every face's energy flux as noise even at rest.
template <int F, int N>
__device__ unsigned star_region_f(const M5Consts &k, const SolF<N> &s, float rL, float rR,
                                  bool both_solid, bool leftside, float u_S, float SL, float SR,
                                  float uL, float vL, float wL, float uR, float vR, float wR,
                                  const float sL[3], const float sR[3], float *dU, NCf<N> &nc) {
  using C = K5<N>;
  float SK, uK, vK, wK, s11K, s12K, s13K;
  if (leftside) {
    SK = SL; uK = uL; vK = vL; wK = wL; s11K = sL[0]; s12K = sL[1]; s13K = sL[2];
  } else {
    SK = SR; uK = uR; vK = vR; wK = wR; s11K = sR[0]; s12K = sR[1]; s13K = sR[2];
  }
  const float q = (SK - uK) / (SK - u_S);
  float ar_S[N], r_S = 0.0f;
#pragma unroll
  for (int v = 0; v < N; ++v) {
    ar_S[v] = s.ra[v] * q;
    r_S += ar_S[v];
  }
  const float mR = (uR - SR) * rR, mL = (uL - SL) * rL;
  const float iden = 1.0f / (mR - mL);
  const float s11_S = (mR * sL[0] - mL * sR[0] + mL * mR * (uR - uL)) * iden;
  float s12_S = 0.0f, s13_S = 0.0f;
  if (both_solid) {
    s12_S = (mR * sL[1] - mL * sR[1] + mL * mR * (vR - vL)) * iden;
    s13_S = (mR * sL[2] - mL * sR[2] + mL * mR * (wR - wL)) * iden;
  }
  const float ik = 1.0f / ((uK - SK) * s.r);
  const float v_S = vK + (s12_S - s12K) * ik;
  const float w_S = wK + (s13_S - s13K) * ik;
  const float vel[3] = {glob<F, 0>(u_S, v_S, w_S), glob<F, 1>(u_S, v_S, w_S),
                        glob<F, 2>(u_S, v_S, w_S)};
  const float re = s.r * s.e;
  const float Em_S =
      k.flux_form == FFV_FLUX_CONSISTENT
          ? (re * (uK - SK) - s11K * uK - s12K * vK - s13K * wK + s11_S * u_S + s12_S * v_S +
             s13_S * w_S) / (r_S * (u_S - SK))
          : (re * (uK - SK) + s11K * uK - s12K * vK - s13K * wK + s11_S * u_S + s12_S * v_S +
             s13_S * w_S) / (r_S * (u_S + SK));
  // the star deformation, row 0 in the face frame
  //   A*_0j = (A_0j (uK - SK) - A_1j (vK - v*) + A_2j (wK - w*)) / (u* - SK),
  // rows 1 and 2 unchanged; on D = A - I the identity's share of row 0 is the jump
  // (uK - u*) / (u* - SK), formed as that difference
  float Dm[3][3], Dl[3][3], DS[3][3], Dg[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) Dm[i][j] = s.D[3 * i + j];
  tens_to_local<F>(Dm, Dl);
  const float ius = 1.0f / (u_S - SK);
#pragma unroll
  for (int j = 0; j < 3; j++) {
    DS[0][j] = ((j == 0 ? uK - u_S : 0.0f) + Dl[0][j] * (uK - SK) -
                ((j == 1 ? 1.0f : 0.0f) + Dl[1][j]) * (vK - v_S) +
                ((j == 2 ? 1.0f : 0.0f) + Dl[2][j]) * (wK - w_S)) * ius;
    DS[1][j] = Dl[1][j];
    DS[2][j] = Dl[2][j];
  }
  tens_to_global<F>(DS, Dg);
  StrainF sE;
  strain_f(&Dg[0][0], sE);
#pragma unroll
  for (int v = 0; v < N; ++v) {
    const float rm = s.ra[v] / s.avf[v];
    const float rm_S = rm * (uK - SK) * ius;
    const float ga = k.gamma_f[v], pi = k.pinf_f[v];
    // the reference takes p_k = -p_hydro here (m5_star_region.c:122)
    const float p_S = (-s.p[v] + pi) * (((ga - 1.0f) * rm + (ga + 1.0f) * rm_S) /
                                       ((ga - 1.0f) * rm_S + (ga + 1.0f) * rm)) - pi;
    const float ael = elastic_energy_f(sE, k.mu_f[v]);
    const float eel = ael / (s.avf[v] * rm_S);
    const float e_S = (p_S + ga * pi) / (rm_S * (ga + 1.0f)) + eel;
    nc.are[v] = ar_S[v] * e_S;
  }
  if (k.flux_form == FFV_FLUX_CONSISTENT) {
    const float iw = 1.0f / (SK - u_S);
#pragma unroll
    for (int v = 0; v < N; ++v) dU[C::i0 + v] = s.ra[v] * (u_S - uK) * iw;
    dU[C::i2] = (re * (uK - u_S) - s11K * uK - s12K * vK - s13K * wK + s11_S * u_S + s12_S * v_S +
                 s13_S * w_S) / (u_S - SK);
  } else {
#pragma unroll
    for (int v = 0; v < N; ++v) dU[C::i0 + v] = ar_S[v] - s.vec[C::i0 + v];
    dU[C::i2] = r_S * Em_S - s.vec[C::i2];
  }
#pragma unroll
  for (int v = 0; v < 3; ++v) dU[C::i1 + v] = r_S * vel[v] - s.vec[C::i1 + v];
#pragma unroll
  for (int d = 0; d < 3; d++) nc.unc[d] = vel[d];
#pragma unroll
  for (int v = 0; v < N - 1; ++v) nc.avf[v] = s.avf[v];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) nc.A[3 * i + j] = Dg[i][j] + (i == j ? 1.0f : 0.0f);
  unsigned st = 0;
#pragma unroll
  for (int iv = 0; iv < C::NC; ++iv)
    if (isnan(dU[iv])) st |= FFV_ST_NAN;
  return st;
}

// m5_flux.c / m5_flux_gfm.c normal component along face F, FP32
template <int F, int N>
__device__ void flux_n_f(const SolF<N> &s, int flag, bool gfm, bool cons, NCf<N> &nc, float *Fn) {
  using C = K5<N>;
  constexpr int a = Fr<F, 0>::ax, sg = Fr<F, 0>::sg;
  const float vu = gfm ? s.ut : s.u, vv = gfm ? s.vt : s.v, vw = gfm ? s.wt : s.w;
  const float vel[3] = {vu, vv, vw};
  const float va = vel[a];
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
    for (int q = 0; q < 9; q++) nc.A[q] = (gfm || cons) ? full_of(s.D, q) : -full_of(s.D, q);
  } else if (flag == 4) {  // symmetry face (m5_flux.c:58-66): the velocity is the caller's
#pragma unroll
    for (int v = 0; v < N - 1; ++v) nc.avf[v] = s.avf[v];
#pragma unroll
    for (int v = 0; v < N; ++v) nc.are[v] = s.are[v];
#pragma unroll
    for (int q = 0; q < 9; q++) nc.A[q] = full_of(s.D, q);
  }
  const float ua = nc.unc[a];
#pragma unroll
  for (int v = 0; v < N - 1; ++v) Fn[C::i3 + v] = sgn<sg>(ua * nc.avf[v]);
#pragma unroll
  for (int v = 0; v < N; ++v) Fn[C::i4 + v] = sgn<sg>(ua * nc.are[v]);
#pragma unroll
  for (int q = 0; q < 9; q++) Fn[C::i5 + q] = sgn<sg>(ua * nc.A[q]);
}

// K = a ? A : B, field by field (selects: the states stay in registers)
template <int N>
__device__ __forceinline__ void select_sol(bool a, const SolF<N> &A, const SolF<N> &B, SolF<N> &K) {
  K.r = a ? A.r : B.r;
  K.u = a ? A.u : B.u;
  K.v = a ? A.v : B.v;
  K.w = a ? A.w : B.w;
  K.e = a ? A.e : B.e;
  K.ut = a ? A.ut : B.ut;
  K.vt = a ? A.vt : B.vt;
  K.wt = a ? A.wt : B.wt;
  K.c2 = a ? A.c2 : B.c2;
  K.phi0 = a ? A.phi0 : B.phi0;
#pragma unroll
  for (int i = 0; i < N; i++) {
    K.ra[i] = a ? A.ra[i] : B.ra[i];
    K.avf[i] = a ? A.avf[i] : B.avf[i];
    K.are[i] = a ? A.are[i] : B.are[i];
    K.p[i] = a ? A.p[i] : B.p[i];
  }
#pragma unroll
  for (int q = 0; q < 9; q++) K.D[q] = a ? A.D[q] : B.D[q];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) K.st[i][j] = a ? A.st[i][j] : B.st[i][j];
#pragma unroll
  for (int q = 0; q < K5<N>::NC; q++) K.vec[q] = a ? A.vec[q] : B.vec[q];
}

// m5_hllc.c:3-95 / m5_hllc_gfm.c:3-100 in FP32: ff += A (F.n + corr).  The solver's four
// branches share one star-region and one physical-flux evaluation on the state of the
// contact's upwind side (one inlined copy of each: the kernel is large enough for the
// instruction cache to matter)
template <int F, int N>
__device__ unsigned hllc_acc_f(const M5Consts &k, SolF<N> L, SolF<N> R, int bc, bool gfm,
                               float Area, float *ff, float unc[3]) {
  using C = K5<N>;
  const float vl3[3] = {L.u, L.v, L.w}, vr3[3] = {R.u, R.v, R.w};
  const float uL = loc<F, 0>(vl3), vL = loc<F, 1>(vl3), wL = loc<F, 2>(vl3);
  float uR = loc<F, 0>(vr3), vR = loc<F, 1>(vr3), wR = loc<F, 2>(vr3);
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
  const float ruL = L.r * uL, ruR = R.r * uR;
  const float cL = sqrtf(L.c2), cR = sqrtf(R.c2);
  const float SR = fmaxf(uL + cL, uR + cR);
  const float SL = fminf(uL - cL, uR - cR);
  float TL[3][3], TR[3][3];
  tens_to_local<F>(L.st, TL);
  tens_to_local<F>(R.st, TR);
  const float sL[3] = {TL[0][0], TL[0][1], TL[0][2]}, sR[3] = {TR[0][0], TR[0][1], TR[0][2]};
  float u_S = ((L.r * (uL * uL) - sL[0]) - (R.r * (uR * uR) - sR[0]) - (SL * ruL) + (SR * ruR)) /
              (ruL - ruR - (SL * L.r) + (SR * R.r));
  unsigned st = (isnan(u_S) || isnan(SR) || isnan(SL)) ? FFV_ST_NAN_SPEED : 0u;
  if (!gfm && bc == 4) u_S = 0.0f;
  NCf<N> nc;
  float Fn[C::NEQ], dU[C::NC], corr[C::NC];
#pragma unroll
  for (int iv = 0; iv < C::NC; ++iv) corr[iv] = 0.0f;
  const bool left_star = gfm ? (SL < 0.0f && 0.0f <= u_S) : (SL <= 0.0f && 0.0f <= u_S);
  const bool right_star = gfm ? (u_S < 0.0f && 0.0f < SR) : (u_S <= 0.0f && 0.0f <= SR);
  // 0: supersonic from the left, 1: left star state, 2: right star state, 3: supersonic
  // from the right
  const int branch = (0.0f <= SL) ? 0 : left_star ? 1 : right_star ? 2 : (SR <= 0.0f) ? 3 : -1;
  if (branch < 0) {
    st |= FFV_ST_NO_BRANCH;
#pragma unroll
    for (int iv = 0; iv < C::NEQ; ++iv) Fn[iv] = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; d++) nc.unc[d] = 0.0f;
  } else {
    const bool left = branch <= 1;
    SolF<N> K;
    select_sol<N>(left, L, R, K);
    if (branch == 1 || branch == 2) {
      st |= star_region_f<F>(k, K, L.r, R.r, (L.phi0 > 0.0f) && (R.phi0 > 0.0f), left, u_S, SL,
                             SR, uL, vL, wL, uR, vR, wR, sL, sR, dU, nc);
      const float SK = left ? SL : SR;
#pragma unroll
      for (int iv = 0; iv < C::NC; ++iv) corr[iv] = SK * dU[iv];
    }
    flux_n_f<F>(K, branch, gfm, k.flux_form == FFV_FLUX_CONSISTENT, nc, Fn);
  }
#pragma unroll
  for (int iv = 0; iv < C::NEQ; ++iv) ff[iv] += Area * (Fn[iv] + (iv < C::NC ? corr[iv] : 0.0f));
#pragma unroll
  for (int d = 0; d < 3; d++) unc[d] = nc.unc[d];
  return st;
}

// m5_hllc.c:56-85 in FP32, a symmetry face: the mean of the physical fluxes of the cell's own
// state and of its mirror image, advected terms moving with the mean velocity, no HLLC part
template <int F, int N>
__device__ void symmetry_acc_f(const SolF<N> &Lc, bool cons, float Area, float *ff, float unc[3]) {
  using C = K5<N>;
  SolF<N> Rc;
  ghost_f<F, N>(Lc, 1, Rc);
  NCf<N> nc;
  nc.unc[0] = 0.5f * (Lc.u + Rc.u);
  nc.unc[1] = 0.5f * (Lc.v + Rc.v);
  nc.unc[2] = 0.5f * (Lc.w + Rc.w);
  float FL[C::NEQ], FR[C::NEQ];
  flux_n_f<F>(Lc, 4, false, cons, nc, FL);
  flux_n_f<F>(Rc, 4, false, cons, nc, FR);
#pragma unroll
  for (int iv = 0; iv < C::NEQ; ++iv) ff[iv] += Area * ((0.5f * FL[iv]) + (0.5f * FR[iv]));
#pragma unroll
  for (int d = 0; d < 3; d++) unc[d] = nc.unc[d];
}

// face record of a state V (FP64): conserved variables (the deformation as D = A - I), the
// volume fractions as the FP64 form's make_sol clamps them, and each material's pressure
// recovered in FP64
template <int N>
__device__ void write_record(const M5Consts &k, const double *V, const double *press, float *out,
                             int64_t stride) {
  using C = K5<N>;
  using RL = RecL<N>;
  const double lo = k.amin / 100.0, hi = 1.0 - (k.amin / 100.0);
  double at[N], sum = 0.0;
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    at[i] = V[C::i3 + i];
    if (at[i] <= lo) at[i] = lo;
    else if (at[i] >= hi) at[i] = hi;
    sum += at[i];
  }
  if (sum > hi) {
    const double dif = sum - hi;
#pragma unroll
    for (int j = 0; j < N - 1; ++j) at[j] = at[j] - (at[j] / sum) * dif;
    sum = hi;
  }
  at[N - 1] = 1.0 - sum;
#pragma unroll
  for (int i = 0; i < C::i5; i++) out[i * stride] = f32_of_f64(V[i]);
#pragma unroll
  for (int q = 0; q < 9; q++) out[(C::i5 + q) * stride] = dev_of(V + C::i5, q);
#pragma unroll
  for (int i = 0; i < N - 1; ++i) out[(C::i3 + i) * stride] = (float)at[i];
  out[RL::AL * stride] = (float)at[N - 1];
  if (press) {
#pragma unroll
    for (int i = 0; i < N; ++i) out[(RL::P + i) * stride] = (float)press[i];
  } else {
    float D[9];
#pragma unroll
    for (int q = 0; q < 9; q++) D[q] = dev_of(V + C::i5, q);
    StrainF sE;
    strain_f(D, sE);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const double ael = (double)elastic_energy_f(sE, k.mu_f[i]);
      const double p = ((k.gamma[i] - 1.0) * (V[C::i4 + i] - ael) / at[i]) - k.gamma[i] * k.pinf[i];
      out[(RL::P + i) * stride] = (float)p;
    }
  }
}

template <int N>
__device__ __forceinline__ void load_state(const double *__restrict__ S, int64_t n, int64_t c,
                                           double *U) {
#pragma unroll
  for (int v = 0; v < K5<N>::NEQ; v++) U[v] = S[(int64_t)v * n + c];
}

// ------------------------------------------------------------ FP32 face reconstruction
// A face state is held as an FP32 copy of every variable plus FP64 values of its
// "critical" slots -- the volume fractions, the materials' internal energies and the total
// energy, which enter the stiffened-gas pressure recovery: j < N-1 is alpha_j, then
// (alpha rho e)_0..N-1, then E.
template <int N>
__device__ __forceinline__ constexpr int crit_slot(int j) {
  return j < N - 1 ? K5<N>::i3 + j : (j < 2 * N - 1 ? K5<N>::i4 + (j - (N - 1)) : K5<N>::i2);
}

// avf_limit.c:3-21 on an FP32 state
template <int N>
__device__ __forceinline__ void avf_limit_f(const M5Consts &k, float *S) {
  using C = K5<N>;
  const float lo = k.alo_f, hi = k.ahi_f;
  float sum = 0.0f;
#pragma unroll
  for (int v = 0; v < N - 1; ++v) {
    float a = S[C::i3 + v];
    if (a <= lo) a = lo;
    else if (a >= hi) a = hi;
    S[C::i3 + v] = a;
    sum += a;
  }
  if (sum > hi) {
    const float dif = sum - hi;
#pragma unroll
    for (int j = 0; j < N - 1; ++j) S[C::i3 + j] -= (S[C::i3 + j] / sum) * dif;
  }
}

// m5_facevalues_MUSCL.c:3-45 (iside 1) on the FP32 copy of the state
template <int N>
__device__ void value_across_f(const M5Consts &k, const ffv_dmesh &m, const float *__restrict__ Sf,
                               int64_t c, int f, uint32_t kind, const float *sc, float *X) {
  using C = K5<N>;
  if (kind & FFV_FK_BC) {
#pragma unroll
    for (int i = 0; i < C::NEQ; i++) X[i] = sc[i];
  } else if (kind == FFV_FK_FINER) {
    const int32_t *sg = m.sub + 4 * (int64_t)m.nbr[(int64_t)f * m.n + c];
#pragma unroll
    for (int i = 0; i < C::NEQ; i++) X[i] = 0.0f;
#pragma unroll 1
    for (int q = 0; q < 4; q++) {
      const int64_t o = sg[q];
#pragma unroll
      for (int i = 0; i < C::NEQ; i++) X[i] += Sf[(int64_t)i * m.n + o];
    }
#pragma unroll
    for (int i = 0; i < C::NEQ; i++) X[i] *= 0.25f;
  } else {
    const int64_t o = m.nbr[(int64_t)f * m.n + c];
#pragma unroll
    for (int i = 0; i < C::NEQ; i++) X[i] = Sf[(int64_t)i * m.n + o];
  }
  avf_limit_f<N>(k, X);
}

// the critical slots of cell o as double-float pairs: hi from the FP32 copy, lo from
// Sflo [2N][n] (written with it by m5f_shadow)
template <int N>
__device__ __forceinline__ void crit_load(const float *__restrict__ Sf, const float *__restrict__ Sflo,
                                          int64_t n, int64_t o, df *X) {
#pragma unroll
  for (int j = 0; j < 2 * N; j++) X[j] = df{Sf[(int64_t)crit_slot<N>(j) * n + o], Sflo[(int64_t)j * n + o]};
}

// avf_limit.c:3-21 on the double-float volume fractions X[0..N-2]
template <int N>
__device__ __forceinline__ void avf_limit_df(const M5Consts &k, df *X) {
  df sum = df_make(0.0f);
#pragma unroll
  for (int j = 0; j < N - 1; ++j) {
    df a = X[j];
    if (df_le(a, k.alo_d)) a = k.alo_d;
    else if (df_le(k.ahi_d, a)) a = k.ahi_d;
    X[j] = a;
    sum = df_add(sum, a);
  }
  if (df_lt(k.ahi_d, sum)) {
    const df dif = df_sub(sum, k.ahi_d);
#pragma unroll
    for (int j = 0; j < N - 1; ++j) X[j] = df_sub(X[j], df_mul(df_div(X[j], sum), dif));
  }
}

// the critical slots across face f (neighbour, mean of four finer, or the cell itself at
// a boundary), volume fractions limited as avf_limit does: their slopes are differences of
// nearly equal numbers (a liquid fraction 1 - 1e-6, an energy of 1e9), which the FP32 copy
// alone cannot resolve
template <int N>
__device__ void crit_across_df(const M5Consts &k, const ffv_dmesh &m, const float *__restrict__ Sf,
                               const float *__restrict__ Sflo, int64_t c, int f, uint32_t kind,
                               const df *own, df *X) {
  constexpr int NCR = 2 * N;
  if (kind & FFV_FK_BC) {
#pragma unroll
    for (int j = 0; j < NCR; j++) X[j] = own[j];
    return;
  }
  if (kind == FFV_FK_FINER) {
    const int32_t *sg = m.sub + 4 * (int64_t)m.nbr[(int64_t)f * m.n + c];
    crit_load<N>(Sf, Sflo, m.n, sg[0], X);
#pragma unroll 1
    for (int q = 1; q < 4; q++) {
      df Y[NCR];
      crit_load<N>(Sf, Sflo, m.n, sg[q], Y);
#pragma unroll
      for (int j = 0; j < NCR; j++) X[j] = df_add(X[j], Y[j]);
    }
#pragma unroll
    for (int j = 0; j < NCR; j++) X[j] = df{X[j].hi * 0.25f, X[j].lo * 0.25f};
  } else {
    crit_load<N>(Sf, Sflo, m.n, m.nbr[(int64_t)f * m.n + c], X);
  }
  avf_limit_df<N>(k, X);
}

// the volume-fraction limits of m5_relaxationvec.c in double-float: the N-1 fractions
// clamped (else-if or two ifs as the reference's two call sites have it), renormalised when
// their sum reaches 1 - lo, the last fraction 1 - sum
template <int N>
__device__ __forceinline__ void vf_limit_relax_df(const M5Consts &k, df *avf, bool elseif) {
  df sum = df_make(0.0f);
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    if (elseif) {
      if (df_le(avf[i], k.alo_d)) avf[i] = k.alo_d;
      else if (df_le(k.ahi_d, avf[i])) avf[i] = k.ahi_d;
    } else {
      if (df_le(avf[i], k.alo_d)) avf[i] = k.alo_d;
      if (df_le(k.ahi_d, avf[i])) avf[i] = k.ahi_d;
    }
    sum = df_add(sum, avf[i]);
  }
  if (df_le(k.ahi_d, sum)) {
    const df dif = df_sub(sum, k.ahi_d);
#pragma unroll
    for (int j = 0; j < N - 1; ++j) avf[j] = df_sub(avf[j], df_mul(df_div(avf[j], sum), dif));
    sum = k.ahi_d;
  }
  avf[N - 1] = df_sub(df_make(1.0f), sum);
}

// m5_relaxationvec.c on a face state: FP32 partial densities, momentum and deformation
// deviation D = A - I in v, the critical slots in cr as double-float pairs; the pressure recovery and the
// energy-consistent equilibrium in double-float, the Newton iteration in FP32 (below).
// PRELAX 1 (the two-material closed form) converts to FP64 and back.
template <int N>
__device__ unsigned relax_face_df(const M5Consts &k, float *v, df *cr, float &p_out,
                                  df *ratio_out = nullptr) {
  using C = K5<N>;
  df ar[N], are[N], avf[N], avf0[N];
  float ael[N];
  float rf = 0.0f;
#pragma unroll
  for (int iv = 0; iv < N; ++iv) {
    rf += v[C::i0 + iv];
    ar[iv] = df_make(v[C::i0 + iv]);
    are[iv] = cr[N - 1 + iv];
  }
  const df rE = cr[2 * N - 1];
  const float mx = v[C::i1], my = v[C::i1 + 1], mz = v[C::i1 + 2];
  const float ke = 0.5f * (mx * mx + my * my + mz * mz) / rf;
#pragma unroll
  for (int iv = 0; iv < N - 1; ++iv) avf[iv] = cr[iv];
  vf_limit_relax_df<N>(k, avf, true);
#pragma unroll
  for (int iv = 0; iv < N; ++iv) avf0[iv] = avf[iv];
  {
    StrainF sE;
    strain_f(v + C::i5, sE);
#pragma unroll
    for (int iv = 0; iv < N; ++iv) ael[iv] = elastic_energy_f(sE, k.mu_f[iv]);
  }
  unsigned st = 0;
  df ratio = df_make(1.0f);
  if (N == 2 && k.prelax == 1) {  // closed form for two materials (only), in FP64
    double a[N], t0[N], p0[N];
#pragma unroll
    for (int iv = 0; iv < N; ++iv) {
      a[iv] = (double)avf[iv].hi + (double)avf[iv].lo;
      t0[iv] = a[iv] / (double)ar[iv].hi;
      p0[iv] = ((k.gamma[iv] - 1.0) * (((double)are[iv].hi + (double)are[iv].lo) - (double)ael[iv]) /
                a[iv]) - k.gpi[iv];
    }
    const double *ga = k.gamma, *pi = k.pinf;
    const double w0 = a[0] / ga[0], w1 = a[1] / ga[1];
    const double A_1 = w0 * (p0[0] + pi[0]) / (w0 + w1);
    const double A_2 = w1 * (p0[1] + pi[1]) / (w0 + w1);
    const double d = (A_2 - A_1 - (pi[1] - pi[0]));
    const double pe = 0.5 * (A_1 + A_2 - (pi[0] + pi[1])) + sqrt(0.25 * (d * d) + A_1 * A_2);
    if (isnan(pe)) st |= FFV_ST_NAN;
#pragma unroll
    for (int iv = 0; iv < N; ++iv)
      avf[iv] = df_from_double((double)ar[iv].hi * t0[iv] * (p0[iv] + k.gpi[iv] + (ga[iv] - 1.0) * pe) /
                               (pe + k.gpi[iv] + (ga[iv] - 1.0) * pe));
    vf_limit_relax_df<N>(k, avf, false);
    ratio = df_div(avf[0], avf0[0]);
  } else {  // PRELAX 3
#pragma unroll
    for (int iv = 0; iv < N; ++iv) {
      if (avf[iv].hi < 0.0f || ar[iv].hi < 0.0f) {
        avf[iv] = k.eps_d;
        ar[iv] = k.eps_d;
        are[iv] = k.eps_d;
      }
      if (!df_lt(avf[iv], df_make(1.0f))) avf[iv] = k.oneeps_d;
    }
    bool irelax = true;
#pragma unroll
    for (int iv = 0; iv < N; ++iv)
      if (df_lt(k.oneeps_d, avf[iv])) irelax = false;
    if (irelax) {
      df sum0 = df_make(-1.0f);
      float p0 = 0.0f;  // the Newton iteration's start, FP32 is enough
      float a0[N], pkf[N], pif[N], b0[N], ig[N], e[N], plo[N], preset[N];
      bool live[N];
#pragma unroll
      for (int iv = 0; iv < N; ++iv) {
        df pk = df_make(0.0f);
        live[iv] = df_lt(k.eps_d, avf[iv]);
        if (live[iv]) {
          pk = df_sub(df_div(df_mul(k.gm1_d[iv], df_sub(are[iv], df_make(ael[iv]))), avf[iv]),
                      k.gpi_d[iv]);
          if (df_le(pk, k.floor_d[iv])) pk = k.floor_d[iv];
          sum0 = df_add(sum0, avf[iv]);
        }
        a0[iv] = df_to_float(avf[iv]);
        pkf[iv] = df_to_float(pk);
        p0 += a0[iv] * pkf[iv];
        pif[iv] = k.pinf_f[iv];
        // at a material's pressure floor pk + p_inf is a few Pa beside 6e8: the sum in
        // double-float, its reciprocal in FP32
        b0[iv] = 1.0f / df_to_float(df_add(pk, k.pinf_d[iv]));
        ig[iv] = k.igam_f[iv];
        plo[iv] = k.plo_f[iv];
        preset[iv] = k.preset_f[iv];
        e[iv] = 0.0f;
      }
      // Newton on sum_k alpha_k(p) = 1 along each material's isentrope,
      // alpha_k(p) = alpha_k0 ((p + pi_k) / (pk_k + pi_k))^(-1/gamma_k), in FP32.  The sum
      // is formed in delta form, F = (sum_k alpha_k0 - 1) + sum_k alpha_k0 e_k with
      // e_k = expm1(-log1p(x_k) / gamma_k), x_k = (p - pk_k) / (pk_k + pi_k), so that every
      // term keeps FP32 precision relative to its own size: summing alpha_k(p) - 1 directly
      // would resolve a 1e-6 volume fraction next to 1 - 1e-6 only to ~6e-8, which
      // p_inf = 6e8 turns into ~200 Pa.  The iterate settles within a few steps; the cap
      // bounds the loop.  Near equilibrium (|x| <= 1/32, most faces away from shocks and
      // interfaces) e_k is the binomial series of (1 + x)^a - 1, a = -1/gamma, to x^7 in
      // Horner form: its first omitted term is below 1e-9 of e_k for gamma >= 1.
      const float F0 = df_to_float(sum0);
      float pf = p0, F = 0.0f, dF = 1.0f, prev1 = NAN, prev2 = NAN;
#pragma unroll 1
      for (int iter = 0; iter < 64; iter++) {
        const float step = F / dF;
        if (iter > 0 && !(fabsf(step) > 1.0e-7f * fabsf(pf))) break;
        pf = pf - step;
#pragma unroll
        for (int iv = 0; iv < N; ++iv)
          if (pf < plo[iv]) pf = preset[iv];
        if (pf == prev1 || pf == prev2) break;
        F = F0;
        dF = 0.0f;
#pragma unroll
        for (int iv = 0; iv < N; ++iv) {
          if (live[iv]) {
            const float x = (pf - pkf[iv]) * b0[iv];
            const float opx = x > -0.5f ? 1.0f + x : fmaxf((pf + pif[iv]) * b0[iv], 1.0e-30f);
            if (fabsf(x) <= 0.03125f) {
              const float *cb = k.bin_f[iv];
              float t = fmaf(cb[5] * x, 1.0f, 1.0f);
              t = fmaf(cb[4] * x, t, 1.0f);
              t = fmaf(cb[3] * x, t, 1.0f);
              t = fmaf(cb[2] * x, t, 1.0f);
              t = fmaf(cb[1] * x, t, 1.0f);
              t = fmaf(cb[0] * x, t, 1.0f);
              e[iv] = (-ig[iv] * x) * t;
            } else {
              const float lx = x > -0.5f ? log1pf(x) : logf(opx);
              e[iv] = expm1f(-lx * ig[iv]);
            }
            F += a0[iv] * e[iv];
            // the derivative only steers the iteration: a fast quotient is enough
            dF -= __fdividef(a0[iv] * (1.0f + e[iv]) * ig[iv] * b0[iv], opx);
          }
        }
        if (isnan(pf) || isnan(F) || isnan(dF)) {
          st |= FFV_ST_NAN;
          break;
        }
        prev2 = prev1;
        prev1 = pf;
      }
#pragma unroll
      for (int iv = 0; iv < N; ++iv)
        if (live[iv]) avf[iv] = df_add(avf[iv], df_mul_f(avf[iv], e[iv]));
      vf_limit_relax_df<N>(k, avf, true);
    }
    const int i_as = (df_lt(avf[0], avf[1]) && (k.mu[1] != 0.0)) ? 1 : 0;
    ratio = df_div(avf[i_as], avf0[i_as]);
  }
  df num = df_make(0.0f), den = df_make(0.0f);
  float sael = 0.0f;
#pragma unroll
  for (int iv = 0; iv < N; ++iv) {
    num = df_add(num, df_mul(avf[iv], k.gpg_d[iv]));
    den = df_add(den, df_mul(avf[iv], k.ig1_d[iv]));
    sael += ael[iv];
  }
  const df p = df_div(df_sub(df_add_f(df_add_f(rE, -ke), -sael), num), den);
#pragma unroll
  for (int iv = 0; iv < N - 1; ++iv) {
    if (df_isnan(avf[iv])) st |= FFV_ST_NAN;
    cr[iv] = avf[iv];
  }
#pragma unroll
  for (int iv = 0; iv < N; iv++) {
    const df a2 = df_add_f(df_mul(df_mul(avf[iv], df_add(p, k.gpi_d[iv])), k.ig1_d[iv]), ael[iv]);
    if (df_isnan(a2)) st |= FFV_ST_NAN;
    cr[N - 1 + iv] = a2;
  }
  // A <- ratio A, i.e. D <- ratio D + (ratio - 1) I
  const float rf32 = df_to_float(ratio), rm1 = df_to_float(df_add_f(ratio, -1.0f));
#pragma unroll
  for (int q = 0; q < 9; ++q) v[C::i5 + q] = rf32 * v[C::i5 + q] + ((q == 0 || q == 4 || q == 8) ? rm1 : 0.0f);
  p_out = df_to_float(p);
  if (ratio_out) *ratio_out = ratio;
  return st;
}

// m5_relaxationvec.c's PRELAX 1 / 3 on an FP64 cell state V: the values it reads converted
// once to double-float pairs, the pressure recovery and the energy-consistent equilibrium
// in double-float, the Newton iteration in FP32 (as relax_face_df), the results converted
// back to FP64.
template <int N>
__device__ unsigned relax_cell_df(const M5Consts &k, double *V) {
  using C = K5<N>;
  // relax_face_df's inputs: the FP32 partial densities, momentum and deformation deviation,
  // and the critical slots as pairs
  float v[C::NEQ];
#pragma unroll
  for (int i = 0; i < C::i5; i++) v[i] = f32_of_f64(V[i]);
#pragma unroll
  for (int q = 0; q < 9; q++) v[C::i5 + q] = dev_of(V + C::i5, q);
  df cr[2 * N];
#pragma unroll
  for (int j = 0; j < 2 * N; j++) cr[j] = df_from_double(V[crit_slot<N>(j)]);
  // relax_face_df takes the kinetic energy from FP32 momentum and partial densities; for a
  // cell the partial densities enter the Newton iteration and the recovery as FP32 values,
  // their sum is the density of the kinetic energy
  float p_eq;
  df ratio;
  const unsigned st = relax_face_df<N>(k, v, cr, p_eq, &ratio);
#pragma unroll
  for (int iv = 0; iv < N - 1; ++iv) V[C::i3 + iv] = f64_of_f32(cr[iv].hi) + f64_of_f32(cr[iv].lo);
#pragma unroll
  for (int iv = 0; iv < N; ++iv)
    V[C::i4 + iv] = f64_of_f32(cr[N - 1 + iv].hi) + f64_of_f32(cr[N - 1 + iv].lo);
  const double r = f64_of_f32(ratio.hi) + f64_of_f32(ratio.lo);
#pragma unroll
  for (int q = 0; q < 9; ++q) V[C::i5 + q] = V[C::i5 + q] * r;
  return st;
}

// ------------------------------------------------------------------------------ kernels
// FP32 copy of the state for the reconstruction (made once per cell per stage) -- the
// deformation as its deviation D = A - I -- and the low parts of the critical slots'
// double-float pairs: Sflo[j][c] = S - (double)(float)S
template <int N>
__global__ void __launch_bounds__(256) m5f_shadow(int64_t n, const double *__restrict__ S,
                                                  float *__restrict__ Sf, float *__restrict__ Sflo) {
  using C = K5<N>;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int v = 0; v < C::NEQ; v++) {
      const double x = S[(int64_t)v * n + c] -
                       ((v == C::i5 || v == C::i5 + 4 || v == C::i5 + 8) ? 1.0 : 0.0);
      const float h = (float)x;  // hardware conversions: this kernel is bound by memory
      Sf[(int64_t)v * n + c] = h;
#pragma unroll
      for (int j = 0; j < 2 * N; j++)
        if (crit_slot<N>(j) == v) Sflo[(int64_t)j * n + c] = (float)(x - (double)h);
    }
  }
}

// 7 blocks of 128 threads per SM (72 registers): the kernel is bound by latency and
// instruction issue; measured on the wall configuration, 6 blocks (80 registers) 4.4 % and
// 5 blocks (96 registers) 7 % slower
template <int N>
__global__ void __launch_bounds__(128, 7) m5f_recon_face(ffv_dmesh m, ffv_geom g, M5Consts k,
                                                      const float *__restrict__ Sf,
                                                      const float *__restrict__ Sflo,
                                                      float *__restrict__ SF,
                                                      unsigned *__restrict__ status) {
  using C = K5<N>;
  using RL = RecL<N>;
  constexpr int NCR = 2 * N;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6 * m.n) return;
  const int f = (int)(t / m.n);
  const int64_t c = t - (int64_t)f * m.n;
  const int fo = fr_opp(f);
  const uint32_t info = m.info[c];
  const int l = ffv_info_level(info);
  const uint32_t kf = ffv_face_kind(info, f), ko = ffv_face_kind(info, fo);
  float sl[C::NEQ], x[C::NEQ], df_[C::NEQ];
#pragma unroll
  for (int i = 0; i < C::NEQ; i++) sl[i] = Sf[(int64_t)i * m.n + c];
  avf_limit_f<N>(k, sl);
  // the critical slots of the cell (volume fractions limited as avf_limit does)
  df cr[NCR];
  crit_load<N>(Sf, Sflo, m.n, c, cr);
  avf_limit_df<N>(k, cr);
  // the differences across face f (side 0) and across the opposite face (side 1), unrolled:
  // both neighbours' loads are in flight together, and with the two sides' arrays resolved
  // at compile time the 80 registers spill less (measured: 11 % faster than one rolled copy)
  float db_[C::NEQ];
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const int fs = side ? fo : f;
    const uint32_t ks = side ? ko : kf;
    value_across_f<N>(k, m, Sf, c, fs, ks, sl, x);
    // the critical slots' differences in double-float, rounded to FP32
    df xc[NCR];
    crit_across_df<N>(k, m, Sf, Sflo, c, fs, ks, cr, xc);
#pragma unroll
    for (int i = 0; i < C::NEQ; i++) x[i] -= sl[i];
#pragma unroll
    for (int j = 0; j < NCR; j++) x[crit_slot<N>(j)] = df_to_float(df_sub(xc[j], cr[j]));
#pragma unroll
    for (int i = 0; i < C::NEQ; i++) {
      if (side == 0) df_[i] = x[i];
      else db_[i] = x[i];
    }
  }
  const float idp = g.idcc_f[l][face_class(kf)];
  const float idm = g.idcc_f[l][face_class(ko)];
  const float cf = g.dcf_f[l][face_class(kf)];
  float corr[C::NEQ];
#pragma unroll
  for (int i = 0; i < C::NEQ; i++) {
    const float db = db_[i];
    float grad = 0.0f;
    if (!(kf & FFV_FK_BC) && fabsf(df_[i]) > 1e-10f && !(i >= C::i4 && i < C::i5)) {
      const float sf = df_[i] * idp, sb = -db * idm;
      if (sb * sf > 0.0f) grad = (fabsf(sb) > fabsf(sf)) ? sf : sb;
    }
    corr[i] = cf * grad;
    sl[i] += corr[i];  // the face value of the FP32 copy
  }
#pragma unroll
  for (int j = 0; j < NCR; j++) cr[j] = df_add_f(cr[j], corr[crit_slot<N>(j)]);
  // m5_reconctruct.c:144-179: volume-fraction limits of the face state
  {
    df sum = df_make(0.0f);
#pragma unroll
    for (int iv = 0; iv < N - 1; ++iv) {
      df a = cr[iv];
      if (df_le(a, k.alo_d)) a = k.alo_d;
      else if (df_le(k.a2lo_d, a)) a = k.a2lo_d;
      cr[iv] = a;
      sum = df_add(sum, a);
    }
    if (df_le(k.ahi_d, sum)) {
      const df dif = df_sub(sum, k.ahi_d);
#pragma unroll
      for (int j = 0; j < N - 1; ++j) cr[j] = df_sub(cr[j], df_mul(df_div(cr[j], sum), dif));
    }
  }
  float p_eq;
  const unsigned st = relax_face_df<N>(k, sl, cr, p_eq);
  // the face record: FP32 state with the critical slots rounded from their pairs, the
  // volume fractions as make_sol limits them, the equilibrium pressure for every material
  df at[N];
  df sum = df_make(0.0f);
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    at[i] = cr[i];
    if (df_le(at[i], k.alo_d)) at[i] = k.alo_d;
    else if (df_le(k.ahi_d, at[i])) at[i] = k.ahi_d;
    sum = df_add(sum, at[i]);
  }
  if (df_lt(k.ahi_d, sum)) {
    const df dif = df_sub(sum, k.ahi_d);
#pragma unroll
    for (int j = 0; j < N - 1; ++j) at[j] = df_sub(at[j], df_mul(df_div(at[j], sum), dif));
    sum = k.ahi_d;
  }
  at[N - 1] = df_sub(df_make(1.0f), sum);
  float *out = SF + (int64_t)f * RL::SIZE * m.n + c;
#pragma unroll
  for (int j = N - 1; j < NCR; j++) sl[crit_slot<N>(j)] = df_to_float(cr[j]);
#pragma unroll
  for (int i = 0; i < N - 1; ++i) sl[C::i3 + i] = df_to_float(at[i]);
#pragma unroll
  for (int i = 0; i < C::NEQ; i++) out[(int64_t)i * m.n] = sl[i];
  out[(int64_t)RL::AL * m.n] = df_to_float(at[N - 1]);
#pragma unroll
  for (int i = 0; i < N; ++i) out[(int64_t)(RL::P + i) * m.n] = p_eq;
  if (st) atomicOr(status, st);
}

template <int N>
__device__ __forceinline__ void load_record(const float *__restrict__ SF, int64_t n, int f,
                                            int64_t c, float *U) {
  using RL = RecL<N>;
#pragma unroll
  for (int v = 0; v < RL::SIZE; v++) U[v] = SF[((int64_t)f * RL::SIZE + v) * n + c];
}

// order 1: the record of a cell state
template <int N>
__device__ __forceinline__ void record_of_cell(const M5Consts &k, const double *__restrict__ S,
                                               int64_t n, int64_t c, float *U) {
  double V[K5<N>::NEQ];
  load_state<N>(S, n, c, V);
  write_record<N>(k, V, nullptr, U, 1);
}

template <int N, int F>
__device__ void face_flux_f(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k,
                            const double *__restrict__ S, const float *__restrict__ Sf,
                            const float *__restrict__ SF, int64_t c, uint32_t info, float *ff,
                            float uf[3], double &gfm_face, unsigned &st, bool &owner) {
  using C = K5<N>;
  using RL = RecL<N>;
  constexpr int FO = fr_opp(F);
  const uint32_t kind = ffv_face_kind(info, F);
  const int l = ffv_info_level(info);
#pragma unroll
  for (int iv = 0; iv < C::NEQ; iv++) ff[iv] = 0.0f;
  uf[0] = uf[1] = uf[2] = 0.0f;
  gfm_face = 0.0;
  if (kind == FFV_FK_SAME && m.nbr[(int64_t)F * m.n + c] < c) {
    owner = false;  // evaluated by the neighbour (flux reuse, m5_residual.c:80-99)
    return;
  }
  float U[RL::SIZE];
  SolF<N> L, R;
  if (kind == (FFV_FK_BC | FFV_BC_SYMMETRY)) {  // the cell's own state (m5_hllc.c:59-63)
    record_of_cell<N>(k, S, m.n, c, U);
    make_sol_f<N>(k, U, 0.0f, L);
    symmetry_acc_f<F, N>(L, k.flux_form == FFV_FLUX_CONSISTENT, g.area_f[l], ff, uf);
    return;
  }
  if (k.order == 2) load_record<N>(SF, m.n, F, c, U);
  else record_of_cell<N>(k, S, m.n, c, U);
  make_sol_f<N>(k, U, Sf ? cell_phi0_f<N>(k, Sf, m.n, c) : (float)cell_phi0<N>(k, S, m.n, c), L);
  // one solver call site for the boundary (the ghost state) and the interior faces (the
  // neighbour's record, or each of four finer neighbours' in turn; the face velocity is the
  // last subface's divided by four, m5_residual.c:163-165)
  const bool bnd = (kind & FFV_FK_BC) != 0;
  const int bc = bnd ? (int)(kind & 7u) : 0;
  const int nsub = kind == FFV_FK_FINER ? 4 : 1;
  const float A = kind == FFV_FK_FINER ? g.area_f[l + 1] : g.area_f[l];
  const int32_t *sg = kind == FFV_FK_FINER ? m.sub + 4 * (int64_t)m.nbr[(int64_t)F * m.n + c] : nullptr;
  const float inv = 1.0f / (float)nsub;
#pragma unroll 1
  for (int q = 0; q < nsub; q++) {
    if (bnd) {
      ghost_f<F, N>(L, bc, R);
    } else {
      const int64_t o = sg ? sg[q] : m.nbr[(int64_t)F * m.n + c];
      if (k.order == 2) load_record<N>(SF, m.n, FO, o, U);
      else record_of_cell<N>(k, S, m.n, o, U);
      make_sol_f<N>(k, U, Sf ? cell_phi0_f<N>(k, Sf, m.n, o) : (float)cell_phi0<N>(k, S, m.n, o), R);
    }
    const bool gfm = L.phi0 * R.phi0 < 0.0f;
    if (gfm) gfm_face = 1.0;
    float un[3];
    st |= hllc_acc_f<F, N>(k, L, R, bc, gfm, A, ff, un);
    uf[0] = un[0] * inv;
    uf[1] = un[1] * inv;
    uf[2] = un[2] * inv;
  }
}

// 4 blocks of 128 threads per SM (128 registers instead of 164): 6 % faster despite a few
// hundred bytes of spill
template <int N>
__global__ void __launch_bounds__(128, 4) m5f_face_flux(ffv_dmesh m, ffv_geom g, M5Consts k,
                                                     const double *__restrict__ S,
                                                     const float *__restrict__ Sf,
                                                     const float *__restrict__ SF,
                                                     float *__restrict__ FF,
                                                     float *__restrict__ UF,
                                                     double *__restrict__ GF,
                                                     unsigned *__restrict__ status) {
  using C = K5<N>;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6 * m.n) return;
  const int f = (int)(t / m.n);
  const int64_t c = t - (int64_t)f * m.n;
  const uint32_t info = m.info[c];
  float ff[C::NEQ], uf[3];
  double gf = 0.0;
  unsigned st = 0;
  bool owner = true;
  switch (f) {
    case 0: face_flux_f<N, 0>(m, g, k, S, Sf, SF, c, info, ff, uf, gf, st, owner); break;
    case 1: face_flux_f<N, 1>(m, g, k, S, Sf, SF, c, info, ff, uf, gf, st, owner); break;
    case 2: face_flux_f<N, 2>(m, g, k, S, Sf, SF, c, info, ff, uf, gf, st, owner); break;
    case 3: face_flux_f<N, 3>(m, g, k, S, Sf, SF, c, info, ff, uf, gf, st, owner); break;
    case 4: face_flux_f<N, 4>(m, g, k, S, Sf, SF, c, info, ff, uf, gf, st, owner); break;
    default: face_flux_f<N, 5>(m, g, k, S, Sf, SF, c, info, ff, uf, gf, st, owner); break;
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

// ZEROU masks and positivity (m5_RK.c), as the FP64 form's clamp_zerou
template <int N>
__device__ __forceinline__ void clamp_zerou_d(const M5Consts &k, double *s, const double *sn) {
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

// m5_cell_update of the FP32-flux form: the face fluxes of the partial densities, momentum,
// energy, volume fractions and internal energies are summed exactly, as double-float pairs
// (the energy fluxes of opposite faces cancel to ~1e-12 of their size: identical fluxes of a
// quiet region must cancel exactly), those of the deformation in FP32; the
// non-conservative terms (m5_residual.c:175-215) are formed in FP32 from the cell's volume
// fractions, deformation and material stresses (pressures recovered in double-float) and
// added to the pairs.  The residual is then rounded once to FP32 -- an error of 6e-8 of the
// residual, below the FP32 face fluxes' own rounding of 6e-8 of each flux -- so that the FP64
// pipe (1/64 of the FP32 rate on GB300) only carries the RK stage: a conversion and one or
// three fused multiply-adds per variable.  The RK stage, positivity, ZEROU and the stage-1
// ghost-fluid trigger as in the FP64 form.  RHS receives the entries the ghost-fluid fix
// reads (partial densities and momentum).
// three blocks of 128 threads per SM (at most 170 registers)
template <int N>
__global__ void __launch_bounds__(128, 3) m5f_cell_update(ffv_dmesh m, ffv_geom g, M5Consts k,
                                                       const double *__restrict__ S,
                                                       double *__restrict__ SN,
                                                       const float *__restrict__ FF,
                                                       const float *__restrict__ UF,
                                                       double *__restrict__ RHS,
                                                       double *__restrict__ Snew,
                                                       uint8_t *__restrict__ flag,
                                                       const double *__restrict__ dtp, int irk,
                                                       unsigned *__restrict__ status) {
  using C = K5<N>;
  constexpr int NA = C::i5;  // residual entries summed in FP64: all but the deformation
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  const uint32_t info = m.info[c];
  const int l = ffv_info_level(info);
  double s[C::NEQ];
  load_state<N>(S, m.n, c, s);
  // the cell's volume fractions (make_sol, cell form: clamped to [amin/100, 1 - amin/100],
  // renormalised when their sum exceeds the upper bound) as double-float pairs, and the
  // material stresses
  df at[N], asum = df_make(0.0f);
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    df a = df_from_double(s[C::i3 + i]);
    if (df_le(a, k.alo_d)) a = k.alo_d;
    else if (df_le(k.ahi_d, a)) a = k.ahi_d;
    at[i] = a;
    asum = df_add(asum, a);
  }
  if (df_lt(k.ahi_d, asum)) {
    const df dif = df_sub(asum, k.ahi_d);
#pragma unroll
    for (int j = 0; j < N - 1; ++j) at[j] = df_sub(at[j], df_mul(df_div(at[j], asum), dif));
    asum = k.ahi_d;
  }
  at[N - 1] = df_sub(df_make(1.0f), asum);
  float A[9], D[9], avf[N], ast[N][3][3], st_all[3][3];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    D[q] = dev_of(s + C::i5, q);
    A[q] = full_of(D, q);
  }
  StrainF sE;
  strain_f(D, sE);
  stress_deviator_f(sE);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) st_all[i][j] = 0.0f;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    // the material pressure only enters the FP32 stress: recovered in double-float
    const float ael = elastic_energy_f(sE, k.mu_f[i]);
    const df a_d = at[i];
    const df p = df_sub(df_div(df_mul(k.gm1_d[i], df_add_f(df_from_double(s[C::i4 + i]), -ael)), a_d),
                        k.gpi_d[i]);
    avf[i] = a_d.hi;
    eos_stress_f(st_all, avf[i], df_to_float(p), sE, k.mu_f[i], ast[i]);
  }
  df rhs[NA];
  float rhsA[9], nc[N - 1 + N + 9];
#pragma unroll
  for (int iv = 0; iv < NA; iv++) rhs[iv] = df_make(0.0f);
#pragma unroll
  for (int q = 0; q < 9; q++) rhsA[q] = 0.0f;
#pragma unroll
  for (int q = 0; q < N - 1 + N + 9; q++) nc[q] = 0.0f;
#pragma unroll
  for (int F = 0; F < 6; F++) {
    int64_t fc = c;
    int ff = F;
    float sg = 1.0f;
    const uint32_t kind = ffv_face_kind(info, F);
    if (kind == FFV_FK_SAME) {
      const int64_t o = m.nbr[(int64_t)F * m.n + c];
      if (o < c) {
        fc = o;
        ff = fr_opp(F);
        sg = -1.0f;
      }
    }
#pragma unroll
    for (int iv = 0; iv < NA; iv++) rhs[iv] = df_add_f(rhs[iv], sg * FF[((int64_t)ff * C::NEQ + iv) * m.n + fc]);
#pragma unroll
    for (int q = 0; q < 9; q++) rhsA[q] += sg * FF[((int64_t)ff * C::NEQ + C::i5 + q) * m.n + fc];
    const float un = sg * UF[((int64_t)ff * 3 + 0) * m.n + fc];
    const float vn = sg * UF[((int64_t)ff * 3 + 1) * m.n + fc];
    const float wn = sg * UF[((int64_t)ff * 3 + 2) * m.n + fc];
    const float Af = kind == FFV_FK_FINER ? g.area4_fine_f[l] : g.area_f[l];
    const int ax = fr_n_axis(F);
    const float nn[3] = {ax == 0 ? (float)fr_n_sign(F) : 0.0f, ax == 1 ? (float)fr_n_sign(F) : 0.0f,
                         ax == 2 ? (float)fr_n_sign(F) : 0.0f};
    const float nx = nn[0], ny = nn[1], nz = nn[2];
#pragma unroll
    for (int iv = 0; iv < N - 1; ++iv) nc[iv] += Af * (avf[iv] * un * nx + avf[iv] * vn * ny + avf[iv] * wn * nz);
#pragma unroll
    for (int iv = 0; iv < N; ++iv) {
      const float(*t)[3] = ast[iv];
      nc[N - 1 + iv] += Af * (t[0][0] * un * nx + t[0][1] * vn * nx + t[0][2] * wn * nx +
                              t[1][0] * un * ny + t[1][1] * vn * ny + t[1][2] * wn * ny +
                              t[2][0] * un * nz + t[2][1] * vn * nz + t[2][2] * wn * nz);
    }
    const float A1 = A[0], A2 = A[1], A3 = A[2], B1 = A[3], B2 = A[4], B3 = A[5], C1 = A[6], C2 = A[7],
                C3 = A[8];
    float *R5 = nc + (2 * N - 1);
    R5[0] += Af * ((A1 * vn * ny + A1 * wn * nz) + B1 * vn * nx - C1 * wn * nx);
    R5[1] += Af * ((A2 * vn * ny + A2 * wn * nz) + B2 * vn * nx - C2 * wn * nx);
    R5[2] += Af * ((A3 * vn * ny + A3 * wn * nz) + B3 * vn * nx - C3 * wn * nx);
    R5[3] += Af * ((B1 * un * nx + B1 * wn * nz) + A1 * un * ny - C1 * wn * ny);
    R5[4] += Af * ((B2 * un * nx + B2 * wn * nz) + A2 * un * ny - C2 * wn * ny);
    R5[5] += Af * ((B3 * un * nx + B3 * wn * nz) + A3 * un * ny - C3 * wn * ny);
    R5[6] += Af * ((C1 * un * nx + C1 * vn * ny) + A1 * un * nz - B1 * vn * nz);
    R5[7] += Af * ((C2 * un * nx + C2 * vn * ny) + A2 * un * nz - B2 * vn * nz);
    R5[8] += Af * ((C3 * un * nx + C3 * vn * ny) + A3 * un * nz - B3 * vn * nz);
  }
#pragma unroll
  for (int iv = 0; iv < N - 1; iv++) rhs[C::i3 + iv] = df_add_f(rhs[C::i3 + iv], nc[iv]);
#pragma unroll
  for (int iv = 0; iv < N; iv++) rhs[C::i4 + iv] = df_add_f(rhs[C::i4 + iv], nc[N - 1 + iv]);
  float r[C::NEQ];
#pragma unroll
  for (int iv = 0; iv < NA; iv++) r[iv] = df_to_float(rhs[iv]);
#pragma unroll
  for (int q = 0; q < 9; q++) r[C::i5 + q] = rhsA[q] + nc[2 * N - 1 + q];
  // a non-positive density in the stage's input is reported (the arithmetic is untouched)
  double rho_in = 0.0;
#pragma unroll
  for (int v = 0; v < N; ++v) rho_in += s[C::i0 + v];
  unsigned st = rho_in <= 0.0 ? FFV_ST_NEG_DENSITY : 0u;
  double rd[C::NEQ];
#pragma unroll
  for (int iv = 0; iv < C::NEQ; iv++) {
    if (isnan(r[iv])) st |= FFV_ST_NAN;
    rd[iv] = f64_of_f32(r[iv]);
  }
#pragma unroll
  for (int iv = 0; iv < C::i2; iv++) RHS[(int64_t)iv * m.n + c] = rd[iv];
  const double dtiV = *dtp * g.inv_vol[l];
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
        const double as_new = fma(dtiV, rd[e], sn[e]);
        if (phi_old * (as_new - k.avf_lim) < 0.0) gfm = true;
      }
    }
#pragma unroll
    for (int e = 0; e < C::NEQ; e++)
      if (!gfm || e >= C::i2) s[e] = fma(dtiV, rd[e], sn[e]);
  } else {
    const double a = irk == 2 ? 3.0 / 4.0 : (irk == 3 ? 1.0 / 3.0 : 1.0 / 2.0);
    const double b = 1.0 - a;
#pragma unroll
    for (int e = 0; e < C::NEQ; e++) s[e] = fma(a, sn[e], b * fma(dtiV, rd[e], s[e]));
  }
  if (!gfm) clamp_zerou_d<N>(k, s, sn);
#pragma unroll
  for (int e = 0; e < C::NEQ; e++) Snew[(int64_t)e * m.n + c] = s[e];
  flag[c] = gfm ? 1 : 0;
  if (st) atomicOr(status, st);
}

// 6 blocks of 128 threads per SM (80 registers): 10 % faster than 4 blocks at 124 registers
template <int N>
__global__ void __launch_bounds__(128, 6) m5f_relax_cell(int64_t n, M5Consts k,
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
  const unsigned st = relax_cell_df<N>(k, s);
  if (k.plastic) plastic_return<N>(k, s);  // as the FP64 form: FP64 return after relaxation
  const double phi_new = (k.mu[0] != 0.0) ? s[C::i3] - k.avf_lim : phi_old;
  flag[c] = (phi_old * phi_new < 0.0) ? 1 : 0;
#pragma unroll
  for (int e = 0; e < C::NEQ; e++) Sout[(int64_t)e * n + c] = s[e];
  if (st) atomicOr(status, st);
}

// the indicator's five per-cell fields (log rho, log p, alpha_0, |u|, von Mises stress) in
// FP32 from the FP64 state: the volume fractions, internal energies and each material's
// pressure recovery in double-float (the mixture pressure sum_k alpha_k p_k cancels
// (gamma_k - 1) alpha rho e_k against alpha_k gamma_k p_inf_k), the stress deviator in FP32
template <int N>
__global__ void __launch_bounds__(128) m5f_indicator_fields(int64_t n, M5Consts k,
                                                            const double *__restrict__ S,
                                                            float *__restrict__ F) {
  using C = K5<N>;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  float r = 0.0f;
#pragma unroll
  for (int iv = 0; iv < N; ++iv) r += f32_of_f64(S[(int64_t)(C::i0 + iv) * n + c]);
  const float mx = f32_of_f64(S[(int64_t)C::i1 * n + c]), my = f32_of_f64(S[(int64_t)(C::i1 + 1) * n + c]),
              mz = f32_of_f64(S[(int64_t)(C::i1 + 2) * n + c]);
  df at[N];
#pragma unroll
  for (int i = 0; i < N - 1; ++i) at[i] = df_from_double(S[(int64_t)(C::i3 + i) * n + c]);
  avf_limit_df<N>(k, at);
  df sum = df_make(0.0f);
#pragma unroll
  for (int i = 0; i < N - 1; ++i) sum = df_add(sum, at[i]);
  at[N - 1] = df_sub(df_make(1.0f), sum);
  float D[9];
#pragma unroll
  for (int q = 0; q < 9; q++)
    D[q] = f32_of_f64(S[(int64_t)(C::i5 + q) * n + c] - ((q == 0 || q == 4 || q == 8) ? 1.0 : 0.0));
  StrainF sE;
  strain_f(D, sE);
  stress_deviator_f(sE);
  float st[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
  df p = df_make(0.0f);
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const float ael = elastic_energy_f(sE, k.mu_f[i]);
    const df pk = df_sub(df_div(df_mul(k.gm1_d[i], df_add_f(df_from_double(S[(int64_t)(C::i4 + i) * n + c]), -ael)),
                                at[i]),
                         k.gpi_d[i]);
    p = df_add(p, df_mul(at[i], pk));
    // the von Mises stress depends on the deviator only, to which -alpha_k p_k I adds
    // nothing: the elastic part alone (in FP32 the isotropic terms, up to ~1e10 for a nearly
    // absent material, would round away the deviator)
    eos_stress_f(st, 0.0f, 0.0f, sE, k.mu_f[i], nullptr);
  }
  const float tr = (st[0][0] + st[1][1] + st[2][2]) * (1.0f / 3.0f);
  float j2 = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const float d = st[i][j] - (i == j ? tr : 0.0f);
      j2 += d * d;
    }
  const float pf = df_to_float(p);
  F[c] = logf(fmaxf(r, 1e-30f));
  F[n + c] = logf(fmaxf(pf, 1.0f));
  F[2 * n + c] = df_to_float(at[0]);
  F[3 * n + c] = sqrtf(mx * mx + my * my + mz * mz) / r;
  F[4 * n + c] = sqrtf(1.5f * j2);
}

}  // namespace

void ffv_m5f_shadow(int64_t n, const M5Consts &k, const double *S, float *Sf, cudaStream_t st) {
  float *Sflo = Sf + (int64_t)ffv_m5_neq(k.nmat) * n;
  if (k.nmat == 2) m5f_shadow<2><<<152 * 8, 256, 0, st>>>(n, S, Sf, Sflo);
  else m5f_shadow<3><<<152 * 8, 256, 0, st>>>(n, S, Sf, Sflo);
}

void ffv_m5f_recon(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                   const float *Sf, float *SFf, unsigned *status, cudaStream_t st) {
  (void)S;
  const float *Sflo = Sf + (int64_t)ffv_m5_neq(k.nmat) * m.n;
  const unsigned blocks = (unsigned)((6 * m.n + 127) / 128);
  if (k.nmat == 2) m5f_recon_face<2><<<blocks, 128, 0, st>>>(m, g, k, Sf, Sflo, SFf, status);
  else m5f_recon_face<3><<<blocks, 128, 0, st>>>(m, g, k, Sf, Sflo, SFf, status);
}

void ffv_m5f_flux(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                  const float *Sf, const float *SFf, float *FFf, float *UFf, double *GF,
                  unsigned *status,
                  cudaStream_t st) {
  const unsigned blocks = (unsigned)((6 * m.n + 127) / 128);
  if (k.nmat == 2) m5f_face_flux<2><<<blocks, 128, 0, st>>>(m, g, k, S, Sf, SFf, FFf, UFf, GF, status);
  else m5f_face_flux<3><<<blocks, 128, 0, st>>>(m, g, k, S, Sf, SFf, FFf, UFf, GF, status);
}

void ffv_m5f_cell_update(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                         double *SN, const float *FFf, const float *UFf, double *RHS,
                         double *Snew, uint8_t *flag, const double *dt, int irk, unsigned *status,
                         cudaStream_t st) {
  const unsigned blocks = (unsigned)((m.n + 127) / 128);
  if (k.nmat == 2)
    m5f_cell_update<2><<<blocks, 128, 0, st>>>(m, g, k, S, SN, FFf, UFf, RHS, Snew, flag, dt, irk, status);
  else
    m5f_cell_update<3><<<blocks, 128, 0, st>>>(m, g, k, S, SN, FFf, UFf, RHS, Snew, flag, dt, irk, status);
}

void ffv_m5f_indicator_fields(int64_t n, const M5Consts &k, const double *S, float *F,
                              cudaStream_t st) {
  const unsigned blocks = (unsigned)((n + 127) / 128);
  if (k.nmat == 2) m5f_indicator_fields<2><<<blocks, 128, 0, st>>>(n, k, S, F);
  else m5f_indicator_fields<3><<<blocks, 128, 0, st>>>(n, k, S, F);
}

void ffv_m5f_relax_cell(int64_t n, const M5Consts &k, const double *Sin, double *Sout,
                        uint8_t *flag, unsigned *status, cudaStream_t st) {
  const unsigned blocks = (unsigned)((n + 127) / 128);
  if (k.nmat == 2) m5f_relax_cell<2><<<blocks, 128, 0, st>>>(n, k, Sin, Sout, flag, status);
  else m5f_relax_cell<3><<<blocks, 128, 0, st>>>(n, k, Sin, Sout, flag, status);
}
