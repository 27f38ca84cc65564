// Model-0 (Euler, stiffened gas) FP64 stage kernels.
//
// Compiled with --fmad=false: every multiply and add rounds separately, in the operation
// order of the reference's C code, so results are bit-identical to the reference
// (m0_*.c) on Cartesian forests.  Face frames are axis-aligned there, so the rotations of
// m0_wave_speeds.c:16-28 / m0_star_region.c:27-30 reduce to picking a component with a
// sign; that is exact (the other terms are products with 0.0).
//
// Per stage two kernels run:
//   m0_recon    grad_scheme -> m0_faceinterp_V1 (m0_faceinterp.c:59-88): limited face
//               states SF of all six faces of every cell;
//   m0_flux_rk  RHS -> m0_residual (m0_residual.c:7-141) fused with the RK stage update
//               (RK.c:3-53).  Each cell gathers its own faces (no atomics); a 1:1 face
//               whose neighbour comes first in leaf order is evaluated from that
//               neighbour's side and negated, which is what the reference's flux reuse
//               (m0_residual.c:112-129) yields.
#include <math.h>

#include "ffv_device.cuh"

namespace {

constexpr int NV = 5;

struct Sol {
  double r, u, v, w, e, p, c;
  double vec[NV];
};

// m0_facercnstr.c:29-43: face state vector -> primitive state
__device__ __forceinline__ void to_sol(const double U[NV], double gamma, double pinf, Sol &s) {
  s.r = U[0];
  s.u = U[1] / s.r;
  s.v = U[2] / s.r;
  s.w = U[3] / s.r;
#pragma unroll
  for (int i = 0; i < NV; i++) s.vec[i] = U[i];
  s.e = U[4];
  double ei = (s.e / s.r) - 0.5 * (s.u * s.u + s.v * s.v + s.w * s.w);
  s.p = s.r * (gamma - 1.0) * ei - gamma * pinf;
  s.c = sqrt(gamma * (s.p + pinf) / s.r);
}

template <int A>
__device__ __forceinline__ double vc(const Sol &s) {
  return A == 0 ? s.u : (A == 1 ? s.v : s.w);
}
template <int S>
__device__ __forceinline__ double sgn(double x) {
  return S > 0 ? x : -x;
}
// components of the velocity in the frame of face F (m0_wave_speeds.c:21-35)
template <int F> __device__ __forceinline__ double rot_n(const Sol &s) { return sgn<fr_n_sign(F)>(vc<fr_n_axis(F)>(s)); }
template <int F> __device__ __forceinline__ double rot_t1(const Sol &s) { return sgn<fr_t1_sign(F)>(vc<fr_t1_axis(F)>(s)); }
template <int F> __device__ __forceinline__ double rot_t2(const Sol &s) { return sgn<fr_t2_sign(F)>(vc<fr_t2_axis(F)>(s)); }
// global component A of a*n + b*t1 + c*t2 (m0_star_region.c:27-29, bc_reflective.c:26-28)
template <int F, int A>
__device__ __forceinline__ double unrot(double a, double b, double c) {
  return fr_n_axis(F) == A ? sgn<fr_n_sign(F)>(a)
                           : (fr_t1_axis(F) == A ? sgn<fr_t1_sign(F)>(b) : sgn<fr_t2_sign(F)>(c));
}

// m0_bc.c:3-31: ghost state of a boundary face; only the velocity changes
// (bc_reflective.c for 1 and 4, bc_wall.c for 5).
template <int F>
__device__ __forceinline__ void ghost(const Sol &L, int bc, Sol &R) {
  R = L;
  if (bc == 1 || bc == 4 || bc == 5) {
    double ul = rot_n<F>(L), vl = rot_t1<F>(L), wl = rot_t2<F>(L);
    double ur = -ul, vr = bc == 5 ? -vl : vl, wr = bc == 5 ? -wl : wl;
    R.u = unrot<F, 0>(ur, vr, wr);
    R.v = unrot<F, 1>(ur, vr, wr);
    R.w = unrot<F, 2>(ur, vr, wr);
  }
}

// m0_flux.c:3-28, normal component along face F: sum_d F[i][d] n_d
template <int F>
__device__ __forceinline__ void flux_n(const Sol &s, double Fn[NV]) {
  constexpr int a = fr_n_axis(F);
  const double va = vc<a>(s);
  Fn[0] = sgn<fr_n_sign(F)>(va * s.r);
  Fn[1] = sgn<fr_n_sign(F)>(a == 0 ? s.r * s.u * s.u + s.p : s.r * s.u * va);
  Fn[2] = sgn<fr_n_sign(F)>(a == 1 ? s.r * s.v * s.v + s.p : s.r * s.v * va);
  Fn[3] = sgn<fr_n_sign(F)>(a == 2 ? s.r * s.w * s.w + s.p : s.r * s.w * va);
  Fn[4] = sgn<fr_n_sign(F)>(va * (s.e + s.p));
}

// m0_star_region.c:3-31
template <int F>
__device__ __forceinline__ void star(const Sol &s, double S_S, double SK, double uK, double vK,
                                     double wK, double Us[NV]) {
  double const_S = s.r * (SK - uK) / (SK - S_S);
  Us[0] = const_S;
  Us[1] = const_S * unrot<F, 0>(S_S, vK, wK);
  Us[2] = const_S * unrot<F, 1>(S_S, vK, wK);
  Us[3] = const_S * unrot<F, 2>(S_S, vK, wK);
  Us[4] = const_S * ((s.e / s.r) + (S_S - uK) * (S_S + (s.p / (s.r * (SK - uK)))));
}

// m0_hllc.c:3-59 with m0_wave_speeds.c:3-135, accumulated as m0_residual.c:178-184:
// ff[i] += -(A) * (F.n + HLLC correction).  Returns status bits.
template <int F>
__device__ __forceinline__ unsigned hllc_acc(const Sol &L, const Sol &R, bool bc4, double A,
                                             double ff[NV]) {
  double uL = rot_n<F>(L), vL = rot_t1<F>(L), wL = rot_t2<F>(L);
  double uR = rot_n<F>(R), vR = rot_t1<F>(R), wR = rot_t2<F>(R);
  double ruL = L.r * uL, ruR = R.r * uR;
  double a = uL + L.c, b = uR + R.c;
  double SR = (a > b) ? a : b;
  a = uL - L.c;
  b = uR - R.c;
  double SL = (a < b) ? a : b;
  // s11 of the rotated stress tensor p I is p (rotate_vectors.c:73-106, unit normal)
  double S_S = ((L.r * (uL * uL) + L.p) - (R.r * (uR * uR) + R.p) - (SL * ruL) + (SR * ruR)) /
               (ruL - ruR - (SL * L.r) + (SR * R.r));
  unsigned st = isnan(S_S) ? FFV_ST_NAN_SPEED : 0u;
  if (bc4) S_S = 0.0;
  double Fn[NV], corr[NV] = {0.0, 0.0, 0.0, 0.0, 0.0}, Us[NV];
  if (0.0 <= SL) {
    flux_n<F>(L, Fn);
  } else if (SL <= 0.0 && 0.0 <= S_S) {
    star<F>(L, S_S, SL, uL, vL, wL, Us);
    flux_n<F>(L, Fn);
#pragma unroll
    for (int i = 0; i < NV; i++) corr[i] = SL * (Us[i] - L.vec[i]);
  } else if (S_S <= 0.0 && 0.0 <= SR) {
    star<F>(R, S_S, SR, uR, vR, wR, Us);
    flux_n<F>(R, Fn);
#pragma unroll
    for (int i = 0; i < NV; i++) corr[i] = SR * (Us[i] - R.vec[i]);
  } else if (SR <= 0.0) {
    flux_n<F>(R, Fn);
  } else {
    st |= FFV_ST_NO_BRANCH;
#pragma unroll
    for (int i = 0; i < NV; i++) Fn[i] = 0.0;
  }
#pragma unroll
  for (int i = 0; i < NV; i++) ff[i] += -(A) * (Fn[i] + corr[i]);
  return st;
}

// Face-state access: ORDER 2 reads SF[f][v][c]; ORDER 1 reads a stage-start copy of S.
template <int ORDER>
__device__ __forceinline__ void load_face(const double *__restrict__ FS, int64_t n, int f,
                                          int64_t c, double U[NV]) {
#pragma unroll
  for (int v = 0; v < NV; v++)
    U[v] = ORDER == 2 ? FS[((int64_t)f * NV + v) * n + c] : FS[(int64_t)v * n + c];
}

template <int ORDER, int F>
__device__ __forceinline__ unsigned face_residual(const ffv_dmesh &m, const ffv_geom &g,
                                                  const double *__restrict__ FS, int64_t c,
                                                  uint32_t info, int l, double gamma,
                                                  double pinf, double rhs[NV]) {
  constexpr int FO = fr_opp(F);
  const uint32_t kind = ffv_face_kind(info, F);
  double ff[NV] = {0.0, 0.0, 0.0, 0.0, 0.0};
  unsigned st = 0;
  double U[NV];
  Sol L, R;
  if (kind == FFV_FK_SAME) {
    const int64_t o = m.nbr[(int64_t)F * m.n + c];
    if (o < c) {
      // the neighbour came first in leaf order: it evaluated this face with its own
      // state on the left and its own frame; this cell takes the negative (reuse)
      double t[NV] = {0.0, 0.0, 0.0, 0.0, 0.0};
      load_face<ORDER>(FS, m.n, FO, o, U);
      to_sol(U, gamma, pinf, L);
      load_face<ORDER>(FS, m.n, F, c, U);
      to_sol(U, gamma, pinf, R);
      st |= hllc_acc<FO>(L, R, false, g.area[l], t);
#pragma unroll
      for (int i = 0; i < NV; i++) ff[i] = -t[i];
    } else {
      load_face<ORDER>(FS, m.n, F, c, U);
      to_sol(U, gamma, pinf, L);
      load_face<ORDER>(FS, m.n, FO, o, U);
      to_sol(U, gamma, pinf, R);
      st |= hllc_acc<F>(L, R, false, g.area[l], ff);
    }
  } else {
    load_face<ORDER>(FS, m.n, F, c, U);
    to_sol(U, gamma, pinf, L);
    if (kind == FFV_FK_COARSER) {
      const int64_t o = m.nbr[(int64_t)F * m.n + c];
      load_face<ORDER>(FS, m.n, FO, o, U);
      to_sol(U, gamma, pinf, R);
      st |= hllc_acc<F>(L, R, false, g.area[l], ff);
    } else if (kind == FFV_FK_FINER) {
      const int32_t *sg = m.sub + 4 * (int64_t)m.nbr[(int64_t)F * m.n + c];
#pragma unroll 1
      for (int k = 0; k < 4; k++) {
        load_face<ORDER>(FS, m.n, FO, sg[k], U);
        to_sol(U, gamma, pinf, R);
        st |= hllc_acc<F>(L, R, false, g.area[l + 1], ff);
      }
    } else {
      const int bc = (int)(kind & 7u);
      ghost<F>(L, bc, R);
      st |= hllc_acc<F>(L, R, bc == 4, g.area[l], ff);
    }
  }
#pragma unroll
  for (int i = 0; i < NV; i++) rhs[i] += ff[i];
  return st;
}

template <int ORDER>
__global__ void __launch_bounds__(128) m0_flux_rk(ffv_dmesh m, ffv_geom g,
                                                  const double *__restrict__ FS,
                                                  double *__restrict__ S,
                                                  double *__restrict__ SN,
                                                  const double *__restrict__ dtp, double gamma,
                                                  double pinf, int irk,
                                                  unsigned *__restrict__ status) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  const uint32_t info = m.info[c];
  const int l = ffv_info_level(info);
  double rhs[NV] = {0.0, 0.0, 0.0, 0.0, 0.0};
  // a non-positive density in the stage's input (the reference runs on into a NaN sound
  // speed there); the status word reports it, the arithmetic is untouched
  unsigned st = S[c] <= 0.0 ? FFV_ST_NEG_DENSITY : 0u;
  st |= face_residual<ORDER, 0>(m, g, FS, c, info, l, gamma, pinf, rhs);
  st |= face_residual<ORDER, 1>(m, g, FS, c, info, l, gamma, pinf, rhs);
  st |= face_residual<ORDER, 2>(m, g, FS, c, info, l, gamma, pinf, rhs);
  st |= face_residual<ORDER, 3>(m, g, FS, c, info, l, gamma, pinf, rhs);
  st |= face_residual<ORDER, 4>(m, g, FS, c, info, l, gamma, pinf, rhs);
  st |= face_residual<ORDER, 5>(m, g, FS, c, info, l, gamma, pinf, rhs);
#pragma unroll
  for (int i = 0; i < NV; i++)
    if (isnan(rhs[i])) st |= FFV_ST_NAN;
  // RK.c:21-45 (stage 1 also performs RK(0): SN = S, RK.c:17-20)
  const double dt = *dtp, V = g.vol[l], iV = g.inv_vol[l];
#pragma unroll
  for (int e = 0; e < NV; e++) {
    const int64_t k = (int64_t)e * m.n + c;
    const double s = S[k];
    double out;
    if (irk == 1) {
      SN[k] = s;
      out = s - dt * iV * rhs[e];
    } else {
      const double sn = SN[k];
      if (irk == 2)
        out = (3.0 / 4.0) * sn + (1.0 / 4.0) * s - (1.0 / 4.0) * dt * rhs[e] / V;
      else if (irk == 3)
        out = (1.0 / 3.0) * sn + (2.0 / 3.0) * s - (2.0 / 3.0) * dt * rhs[e] / V;
      else
        out = (1.0 / 2.0) * sn + (1.0 / 2.0) * s - (1.0 / 2.0) * dt * rhs[e] / V;
    }
    S[k] = out;
    if (e == 0 && out <= 0.0) st |= FFV_ST_NEG_DENSITY;
  }
  if (st) atomicOr(status, st);
}

// m0_facevalues_MUSCL.c:3-56 (iside 1): value across face F
template <int F>
__device__ __forceinline__ void across(const ffv_dmesh &m, const double *__restrict__ S,
                                       int64_t c, uint32_t info, const double Sc[NV],
                                       double out[NV]) {
  const uint32_t kind = ffv_face_kind(info, F);
  if (kind & FFV_FK_BC) {
#pragma unroll
    for (int v = 0; v < NV; v++) out[v] = Sc[v];
  } else if (kind == FFV_FK_FINER) {
    const int32_t *sg = m.sub + 4 * (int64_t)m.nbr[(int64_t)F * m.n + c];
    const int64_t s0 = sg[0], s1 = sg[1], s2 = sg[2], s3 = sg[3];
#pragma unroll
    for (int v = 0; v < NV; v++) {
      const double *Sv = S + (int64_t)v * m.n;
      double a = 0.0;
      a += Sv[s0] / 4.0;
      a += Sv[s1] / 4.0;
      a += Sv[s2] / 4.0;
      a += Sv[s3] / 4.0;
      out[v] = a;
    }
  } else {
    const int64_t o = m.nbr[(int64_t)F * m.n + c];
#pragma unroll
    for (int v = 0; v < NV; v++) out[v] = S[(int64_t)v * m.n + o];
  }
}

// m0_deltavalues.c:23-57 + m0_reconctruct.c:160-207 for face F
template <int F>
__device__ __forceinline__ void recon_face(const ffv_geom &g, int64_t n, int64_t c,
                                           uint32_t info, int l, const double Sc[NV],
                                           const double (&X)[6][NV], double *__restrict__ SF) {
  constexpr int FO = fr_opp(F);
  const uint32_t kf = ffv_face_kind(info, F), ko = ffv_face_kind(info, FO);
  const double dp = g.dcc[l][face_class(kf)], dm = g.dcc[l][face_class(ko)];
  const double cf = g.dcf[l][face_class(kf)];
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const double df = X[F][v] - Sc[v], db = X[FO][v] - Sc[v];
    double grad = 0.0;
    if (!(kf & FFV_FK_BC)) {
      if (fabs(df) > 1e-10) {
        const double product = (-db / dm) * (df / dp);
        if (product > 0.0) {
          if (fabs(db / dm) > fabs(df / dp))
            grad = 1.0 * df / dp;
          else
            grad = -1.0 * db / dm;
        }
      }
    }
    SF[((int64_t)F * NV + v) * n + c] = Sc[v] + cf * grad;
  }
}

__global__ void __launch_bounds__(128) m0_recon(ffv_dmesh m, ffv_geom g,
                                                const double *__restrict__ S,
                                                double *__restrict__ SF) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  const uint32_t info = m.info[c];
  const int l = ffv_info_level(info);
  double Sc[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) Sc[v] = S[(int64_t)v * m.n + c];
  double X[6][NV];
  across<0>(m, S, c, info, Sc, X[0]);
  across<1>(m, S, c, info, Sc, X[1]);
  across<2>(m, S, c, info, Sc, X[2]);
  across<3>(m, S, c, info, Sc, X[3]);
  across<4>(m, S, c, info, Sc, X[4]);
  across<5>(m, S, c, info, Sc, X[5]);
  recon_face<0>(g, m.n, c, info, l, Sc, X, SF);
  recon_face<1>(g, m.n, c, info, l, Sc, X, SF);
  recon_face<2>(g, m.n, c, info, l, Sc, X, SF);
  recon_face<3>(g, m.n, c, info, l, Sc, X, SF);
  recon_face<4>(g, m.n, c, info, l, Sc, X, SF);
  recon_face<5>(g, m.n, c, info, l, Sc, X, SF);
}

__global__ void m0_copy_state(int64_t count, const double *__restrict__ S, double *__restrict__ D) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    D[i] = S[i];
}

}  // namespace

int ffv_m0_launches_per_stage(int order) { return 2; (void)order; }

const char *ffv_m0_fp64_kernel_name(int order, int i) {
  static const char *o2[2] = {"m0_recon", "m0_flux_rk<2>"};
  static const char *o1[2] = {"m0_copy_state", "m0_flux_rk<1>"};
  if (i < 0 || i > 1) return "";
  return order == 2 ? o2[i] : o1[i];
}

void ffv_m0_fp64_stage(const ffv_dmesh &m, const ffv_geom &g, const ffv_m0_bufs &b,
                       const ffv_m0_consts &k, int irk, cudaStream_t st, cudaEvent_t *ev) {
  const int tpb = 128;
  const unsigned blocks = (unsigned)((m.n + tpb - 1) / tpb);
  if (ev) cudaEventRecord(ev[0], st);
  if (k.order == 2)
    m0_recon<<<blocks, tpb, 0, st>>>(m, g, b.S, b.SF);
  else
    m0_copy_state<<<1024, 256, 0, st>>>(NV * m.n, b.S, b.SF);
  if (ev) cudaEventRecord(ev[1], st);
  if (k.order == 2)
    m0_flux_rk<2><<<blocks, tpb, 0, st>>>(m, g, b.SF, b.S, b.SN, b.dt, k.gamma, k.pinf, irk,
                                          b.status);
  else
    m0_flux_rk<1><<<blocks, tpb, 0, st>>>(m, g, b.SF, b.S, b.SN, b.dt, k.gamma, k.pinf, irk,
                                          b.status);
  if (ev) cudaEventRecord(ev[2], st);
}
