/*
 * Model-5 (Saurel six-equation multi-material flow with hyperelastic solids, ghost-fluid
 * coupling) restatement of the reference's explicit FV step.
 * TEST INFRASTRUCTURE ONLY: the oracle for the CUDA path; see ffv_oracle.h.
 *
 * Each function names the reference function it restates and keeps its operation order.
 * The reference updates leaves in place in list order inside m5_RK (with m5_gfm) and
 * m5_relaxation_solid (with m5_gfm_rel), and those two read neighbour states; this
 * restatement keeps that order, so a leaf sees its earlier neighbours' new values.
 *
 * State layout (m5_input.c:134-176), N materials:
 *   [ alpha_k rho_k (N) | rho u, rho v, rho w | E | alpha_k (N-1) | alpha_k rho_k e_k (N) | A (9) ]
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ffv_oracle.h"

#define MAXN 4
#define MAXNEQ (3 * MAXN + 12)

typedef struct cfg {
  int N, neq, ncons, i0, i1, i2, i3, i4, i5, order, rk_steps, prelax, nsolids;
  int zerou[3];
  int flux_form;
  int plastic;
  double gamma[MAXN], pinf[MAXN], mu[MAXN], yield[MAXN], amin, avf_lim, dt;
  double lim[MAXNEQ];
} cfg;

typedef struct sol {
  double r, u, v, w, e;          /* e = E / rho */
  double ut, vt, wt;             /* u_temp.. of the ghost-fluid path */
  double ra[MAXN], Y[MAXN], avf[MAXN + 1], phi[MAXN], are[MAXN], c2Y[MAXN], p[MAXN];
  double A[9], st[3][3], ast[MAXN][3][3];
  double vec[MAXNEQ];
} sol;

typedef struct geo {
  double n[3], t1[3], t2[3];
} geo;

/* star-region outputs that m5_flux reads through run->u_nc / avf_S / are_S / Amat_S */
typedef struct ncs {
  double unc[3], avf[MAXN], are[MAXN], A[9];
} ncs;

static geo face_geo(const ffvo_mesh *m, int64_t c, int f) {
  const double *q = m->nrm + 54 * c + 9 * f;
  geo g;
  for (int k = 0; k < 3; k++) {
    g.n[k] = q[k];
    g.t1[k] = q[3 + k];
    g.t2[k] = q[6 + k];
  }
  return g;
}

/* ------------------------------------------------------------ EOS (state_equation.c) */

static void gmat_of(const double A[9], double G[9], double *Gmag) {
  G[0] = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
  G[1] = A[0] * A[3] + A[1] * A[4] + A[2] * A[5];
  G[2] = A[0] * A[6] + A[1] * A[7] + A[2] * A[8];
  G[3] = A[3] * A[0] + A[4] * A[1] + A[5] * A[2];
  G[4] = A[3] * A[3] + A[4] * A[4] + A[5] * A[5];
  G[5] = A[3] * A[6] + A[4] * A[7] + A[5] * A[8];
  G[6] = A[6] * A[0] + A[7] * A[1] + A[8] * A[2];
  G[7] = A[6] * A[3] + A[7] * A[4] + A[8] * A[5];
  G[8] = A[6] * A[6] + A[7] * A[7] + A[8] * A[8];
  *Gmag = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
          G[2] * (G[3] * G[7] - G[4] * G[6]);
}

/* state_equation.c:269-317 (m5_elastic_energy_solid_V2) and :217-267 (the G_det form,
 * which additionally requires mu != 0) */
static double elastic_energy(const double G[9], double Gmag, double mu, int need_mu) {
  if (!(fabs(Gmag) != 0.0) || (need_mu && !(mu != 0.0))) return 0.0;
  double g13 = pow(fabs(Gmag), 1.0 / 3.0);
  if (isnan(g13)) g13 = 0.0;
  double M1[9] = {G[0] - g13, G[1], G[2], G[3], G[4] - g13, G[5], G[6], G[7], G[8] - g13};
  double M2[9] = {0};
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j) M2[i * 3 + j] += M1[i * 3 + k] * M1[k * 3 + j];
  double tr1 = M2[0] + M2[4] + M2[8];
  return mu / (4.0 * pow(fabs(Gmag), 1.0 / 6.0)) * tr1;
}

/* state_equation.c:143-204 (m5_eos_stress_V2) */
static void eos_stress(double s[3][3], double avf, double pr, const double G[9], double Gmag,
                       double mu) {
  if ((fabs(Gmag) != 0.0) && (mu != 0.0)) {
    double G2[9] = {0}, ss[9];
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 3; ++j) G2[i * 3 + j] += G[i * 3 + k] * G[k * 3 + j];
    double J1 = G[0] + G[4] + G[8], J2 = G2[0] + G2[4] + G2[8];
    double p13 = pow(fabs(Gmag), 1.0 / 3.0);
    for (int k = 0; k < 9; k++) {
      if (k == 0 || k == 4 || k == 8)
        ss[k] = G2[k] - J2 / 3.0 - p13 * (G[k] - J1 / 3.0);
      else
        ss[k] = G2[k] - p13 * (G[k]);
    }
    double f = mu / pow(fabs(Gmag), 1.0 / 6.0);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        s[i][j] = (i == j) ? -avf * pr - f * (ss[3 * i + j]) : -f * (ss[3 * i + j]);
  } else {
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) s[i][j] = (i == j) ? -avf * pr : 0.0;
  }
}

/* ------------------------------------------------- face / cell states (m5_facevalues.c,
 * m5_facercnstr.c).  U is the state vector the primitives come from (cell S or face SF),
 * Sc the cell-centre state whose volume fractions define phi. */
static void make_sol(const cfg *k, const double *U, const double *Sc, int from_face, sol *s) {
  const int N = k->N, n1 = N - 1;
  const double lo = k->amin / 100.0, hi = 1.0 - (k->amin / 100.0);
  s->r = 0.0;
  for (int i = 0; i < N; ++i) {
    s->r += U[i];
    s->ra[i] = U[i];
    s->vec[i] = U[i];
  }
  for (int i = 0; i < N; ++i) s->Y[i] = s->ra[i] / s->r;
  s->u = U[k->i1 + 0] / s->r;
  s->v = U[k->i1 + 1] / s->r;
  s->w = U[k->i1 + 2] / s->r;
  for (int d = 0; d < 3; d++) s->vec[k->i1 + d] = U[k->i1 + d];
  s->e = U[k->i2] / s->r;
  s->vec[k->i2] = U[k->i2];
  double at[MAXN + 1], ac[MAXN + 1] = {0}, sum = 0.0;
  for (int i = 0; i < n1; ++i) {
    at[i] = U[k->i3 + i];
    ac[i] = Sc[k->i3 + i];
  }
  for (int i = 0; i < n1; ++i) {
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
    double dif = sum - hi;
    for (int j = 0; j < n1; ++j) {
      double per = at[j] / sum;
      at[j] = at[j] - per * dif;
    }
    sum = hi;
  }
  at[n1] = 1.0 - sum;
  sum = 0.0;
  for (int i = 0; i < n1; ++i) {
    s->avf[i] = at[i];
    s->vec[k->i3 + i] = at[i];
    sum += at[i];
  }
  s->avf[n1] = 1.0 - sum;
  for (int i = 0; i < n1; ++i) s->phi[i] = ac[i] - k->avf_lim;
  if (k->nsolids == 1) s->phi[0] = ac[0] - k->avf_lim;
  else if (k->nsolids == 2) s->phi[0] = ((ac[0] > ac[1]) ? ac[0] : ac[1]) - k->avf_lim;
  for (int i = 0; i < n1; ++i)
    if (k->mu[i] == 0.0) s->phi[i] = ac[i] - k->avf_lim;
  for (int i = 0; i < N; ++i) {
    s->are[i] = U[k->i4 + i];
    s->vec[k->i4 + i] = U[k->i4 + i];
  }
  for (int q = 0; q < 9; q++) {
    s->A[q] = U[k->i5 + q];
    s->vec[k->i5 + q] = U[k->i5 + q];
  }
  double G[9], Gmag;
  gmat_of(s->A, G, &Gmag);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) s->st[i][j] = 0.0;
  for (int i = 0; i < N; ++i) {
    double ael = (k->mu[i] != 0.0) ? elastic_energy(G, Gmag, k->mu[i], 0) : 0.0;
    /* m5_facevalues divides by the clamped fraction, m5_facercnstr by the stored one */
    double a = from_face ? s->avf[i] : at[i];
    double press = ((k->gamma[i] - 1.0) * (s->are[i] - ael) / a) - k->gamma[i] * k->pinf[i];
    s->c2Y[i] = (a / s->r) * k->gamma[i] * (press + k->pinf[i]);
    s->p[i] = press;
    eos_stress(s->ast[i], s->avf[i], s->p[i], G, Gmag, k->mu[i]);
    for (int p = 0; p < 3; p++)
      for (int q = 0; q < 3; q++) s->st[p][q] += s->ast[i][p][q];
  }
}

/* m5_bc.c:3-31: only the velocity of the ghost changes (m5_bc.c:51-82 m5_bc_symmetry,
 * bc_reflective.c, bc_wall.c) */
static int apply_bc(int bc, const geo *g, const sol *L, sol *R) {
  if (bc == 1 || bc == 4 || bc == 5) {
    double u = L->u, v = L->v, w = L->w;
    double ul = u * g->n[0] + v * g->n[1] + w * g->n[2];
    double vl = u * g->t1[0] + v * g->t1[1] + w * g->t1[2];
    double wl = u * g->t2[0] + v * g->t2[1] + w * g->t2[2];
    double ur = -ul, vr = (bc == 5) ? -vl : vl, wr = (bc == 5) ? -wl : wl;
    R->u = ur * g->n[0] + vr * g->t1[0] + wr * g->t2[0];
    R->v = ur * g->n[1] + vr * g->t1[1] + wr * g->t2[1];
    R->w = ur * g->n[2] + vr * g->t1[2] + wr * g->t2[2];
    return 0;
  }
  if (bc == 2 || bc == 3) return 0;  /* outlet; inlet has no model-5 state (m5_bc.c:35-48) */
  return 9;
}

/* rotate_vectors.c:73-106: R T R^T for R with rows r0, r1, r2 (full loops) */
static void rotate_tensor(double out[3][3], const double T[3][3], const double R[3][3]) {
  double M1[3][3] = {{0}}, M2[3][3] = {{0}};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) M1[i][j] += R[i][k] * T[k][j];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) M2[i][j] += M1[i][k] * R[j][k];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) out[i][j] = M2[i][j];
}

static void frame_rows(const geo *g, double R[3][3]) {
  for (int k = 0; k < 3; k++) {
    R[0][k] = g->n[k];
    R[1][k] = g->t1[k];
    R[2][k] = g->t2[k];
  }
}

/* m5_star_region.c:3-158 */
static int star_region(const cfg *k, const geo *g, const sol *s, const sol *L, const sol *R,
                       int flag, double u_S, double SL, double SR, double uL, double vL,
                       double wL, double uR, double vR, double wR, const double sL[3],
                       const double sR[3], double *Us, ncs *nc) {
  const int N = k->N;
  double SK, uK, vK, wK, s11K, s12K, s13K;
  if (flag == 1) {
    SK = SL; uK = uL; vK = vL; wK = wL; s11K = sL[0]; s12K = sL[1]; s13K = sL[2];
  } else {
    SK = SR; uK = uR; vK = vR; wK = wR; s11K = sR[0]; s12K = sR[1]; s13K = sR[2];
  }
  double ar_S[MAXN], r_S = 0.0;
  for (int v = 0; v < N; ++v) {
    ar_S[v] = s->ra[v] * (SK - uK) / (SK - u_S);
    r_S += ar_S[v];
  }
  double s11_S = ((uR - SR) * R->r * (sL[0]) - (uL - SL) * L->r * (sR[0]) +
                  (uL - SL) * L->r * (uR - SR) * R->r * (uR - uL)) /
                 ((uR - SR) * R->r - (uL - SL) * L->r);
  double s12_S, s13_S;
  if ((L->phi[0] > 0.0) && (R->phi[0] > 0.0)) {
    s12_S = ((uR - SR) * R->r * (sL[1]) - (uL - SL) * L->r * (sR[1]) +
             (uL - SL) * L->r * (uR - SR) * R->r * (vR - vL)) /
            ((uR - SR) * R->r - (uL - SL) * L->r);
    s13_S = ((uR - SR) * R->r * (sL[2]) - (uL - SL) * L->r * (sR[2]) +
             (uL - SL) * L->r * (uR - SR) * R->r * (wR - wL)) /
            ((uR - SR) * R->r - (uL - SL) * L->r);
  } else {
    s12_S = 0.0;
    s13_S = 0.0;
  }
  double v_S = vK + (s12_S - s12K) / ((uK - SK) * s->r);
  double w_S = wK + (s13_S - s13K) / ((uK - SK) * s->r);
  double vel[3];
  for (int d = 0; d < 3; d++) vel[d] = u_S * g->n[d] + v_S * g->t1[d] + w_S * g->t2[d];
  double re = s->r * s->e;
  double Em_S;
  if (k->flux_form) {
    /* energy jump across the S_K wave, S_K (U*_K - U_K) = F*_K - F_K, with the normal energy
       flux rho E u - sigma_n . u: (rho E)* (u* - S_K) = rho E (u_K - S_K) - sigma_K . u_K +
       sigma* . u* */
    Em_S = (re * (uK - SK) - s11K * uK - s12K * vK - s13K * wK + s11_S * u_S + s12_S * v_S +
            s13_S * w_S) / (r_S * (u_S - SK));
  } else {
    Em_S = (re * (uK - SK) + s11K * uK - s12K * vK - s13K * wK + s11_S * u_S + s12_S * v_S +
            s13_S * w_S) / (r_S * (u_S + SK));
  }
  double Rm[3][3], Rt[3][3], Am[3][3], Al[3][3], AS[3][3], Ag[3][3];
  frame_rows(g, Rm);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      Rt[i][j] = Rm[j][i];
      Am[i][j] = s->A[3 * i + j];
    }
  rotate_tensor(Al, Am, Rm);
  for (int j = 0; j < 3; j++)
    AS[0][j] = (Al[0][j] * (uK - SK) - Al[1][j] * (vK - v_S) + Al[2][j] * (wK - w_S)) / (u_S - SK);
  for (int j = 0; j < 3; j++) {
    AS[1][j] = Al[1][j];
    AS[2][j] = Al[2][j];
  }
  rotate_tensor(Ag, AS, Rt);
  double G[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      G[3 * i + j] = Ag[i][0] * Ag[j][0] + Ag[i][1] * Ag[j][1] + Ag[i][2] * Ag[j][2];
  double Gmag = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
                G[2] * (G[3] * G[7] - G[4] * G[6]);
  double e_S[MAXN];
  for (int v = 0; v < N; ++v) {
    double rm = (s->ra[v] / s->avf[v]);
    double rm_S = (s->ra[v] / s->avf[v]) * (uK - SK) / (u_S - SK);
    double p_k = -s->p[v];
    double ga = k->gamma[v], pi = k->pinf[v];
    double p_S = (p_k + pi) * (((ga - 1.0) * rm + (ga + 1.0) * rm_S) /
                               ((ga - 1.0) * rm_S + (ga + 1.0) * rm)) - pi;
    double ael = elastic_energy(G, Gmag, k->mu[v], 1);
    double eel = ael / (s->avf[v] * rm_S);
    e_S[v] = (p_S + ga * pi) / (rm_S * (ga + 1.0)) + eel;
  }
  for (int v = 0; v < N; ++v) Us[k->i0 + v] = ar_S[v];
  for (int v = 0; v < 3; ++v) Us[k->i1 + v] = r_S * vel[v];
  Us[k->i2] = r_S * Em_S;
  for (int d = 0; d < 3; d++) nc->unc[d] = vel[d];
  for (int v = 0; v < N - 1; ++v) nc->avf[v] = s->avf[v];
  for (int v = 0; v < N; ++v) nc->are[v] = ar_S[v] * e_S[v];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) nc->A[3 * i + j] = Ag[i][j];
  for (int iv = 0; iv < k->ncons; ++iv)
    if (isnan(Us[iv])) return 5;
  return 0;
}

/* m5_flux.c:3-96 (gfm = 0) and m5_flux_gfm.c:3-87 (gfm = 1): physical flux tensor */
static void phys_flux(const cfg *k, const sol *s, int flag, int gfm, ncs *nc, double F[][3]) {
  const int N = k->N;
  const double vu = gfm ? s->ut : s->u, vv = gfm ? s->vt : s->v, vw = gfm ? s->wt : s->w;
  const double vel[3] = {vu, vv, vw};
  for (int v = 0; v < N; v++)
    for (int d = 0; d < 3; d++) F[k->i0 + v][d] = vel[d] * s->ra[v];
  for (int a = 0; a < 3; a++)
    for (int d = 0; d < 3; d++)
      F[k->i1 + a][d] = (gfm || k->flux_form) ? vel[d] * vel[a] * s->r - s->st[a][d]
                                              : vel[d] * vel[a] * s->r + s->st[a][d];
  for (int d = 0; d < 3; d++)
    F[k->i2][d] = s->r * s->e * vel[d] - s->st[d][0] * vu - s->st[d][1] * vv - s->st[d][2] * vw;
  if (flag == 0 || flag == 3) {
    for (int d = 0; d < 3; d++) nc->unc[d] = vel[d];
    for (int v = 0; v < N - 1; ++v) nc->avf[v] = s->avf[v];
    for (int v = 0; v < N; ++v) nc->are[v] = s->are[v];
    for (int q = 0; q < 9; q++) nc->A[q] = (gfm || k->flux_form) ? s->A[q] : -s->A[q];
  } else if (flag == 4) { /* symmetry face: the caller gives the velocity */
    for (int v = 0; v < N - 1; ++v) nc->avf[v] = s->avf[v];
    for (int v = 0; v < N; ++v) nc->are[v] = s->are[v];
    for (int q = 0; q < 9; q++) nc->A[q] = s->A[q];
  }
  for (int v = 0; v < N - 1; ++v)
    for (int d = 0; d < 3; d++) F[k->i3 + v][d] = nc->unc[d] * nc->avf[v];
  for (int v = 0; v < N; ++v)
    for (int d = 0; d < 3; d++) F[k->i4 + v][d] = nc->unc[d] * nc->are[v];
  for (int q = 0; q < 9; q++)
    for (int d = 0; d < 3; d++) F[k->i5 + q][d] = nc->unc[d] * nc->A[q];
}

static void s1row(const sol *s, const double R[3][3], double out[3]) {
  double T[3][3];
  rotate_tensor(T, s->st, R);
  out[0] = T[0][0];
  out[1] = T[0][1];
  out[2] = T[0][2];
}

/* m5_hllc.c:3-95 with m5_wave_speeds.c:3-131 (gfm = 0), m5_hllc_gfm.c:3-100 with
 * m5_wave_speeds_gfm.c (gfm = 1).  Fills F (physical flux), corr (HLLC correction) and
 * the face velocity u_nc. */
static int hllc(const cfg *k, const geo *g, sol *L, sol *R, int bc, int gfm, double F[][3],
                double *corr, double unc[3]) {
  const int N = k->N;
  double Rm[3][3];
  frame_rows(g, Rm);
  double uL = L->u * g->n[0] + L->v * g->n[1] + L->w * g->n[2];
  double vL = L->u * g->t1[0] + L->v * g->t1[1] + L->w * g->t1[2];
  double wL = L->u * g->t2[0] + L->v * g->t2[1] + L->w * g->t2[2];
  double uR = R->u * g->n[0] + R->v * g->n[1] + R->w * g->n[2];
  double vR = R->u * g->t1[0] + R->v * g->t1[1] + R->w * g->t1[2];
  double wR = R->u * g->t2[0] + R->v * g->t2[1] + R->w * g->t2[2];
  if (gfm) {
    vR = vL;
    wR = wL;
    L->ut = L->u;
    L->vt = L->v;
    L->wt = L->w;
    R->ut = uR * g->n[0] + vR * g->t1[0] + wR * g->t2[0];
    R->vt = uR * g->n[1] + vR * g->t1[1] + wR * g->t2[1];
    R->wt = uR * g->n[2] + vR * g->t1[2] + wR * g->t2[2];
    R->vec[k->i1 + 0] = R->ut * R->r;
    R->vec[k->i1 + 1] = R->vt * R->r;
    R->vec[k->i1 + 2] = R->wt * R->r;
    R->vec[k->i2] = R->r * R->e;
  }
  double ruL = L->r * uL, ruR = R->r * uR;
  double c2L = 0.0, c2R = 0.0;
  for (int iv = 0; iv < N; ++iv) {
    c2L += L->c2Y[iv];
    c2R += R->c2Y[iv];
  }
  double cL = sqrt(c2L), cR = sqrt(c2R);
  double a = uL + cL, b = uR + cR;
  double SR = (a > b) ? a : b;
  a = uL - cL;
  b = uR - cR;
  double SL = (a < b) ? a : b;
  double sL[3], sR[3];
  s1row(L, Rm, sL);
  s1row(R, Rm, sR);
  double u_S = ((L->r * (uL * uL) - (sL[0])) - (R->r * (uR * uR) - (sR[0])) - (SL * ruL) +
                (SR * ruR)) / (ruL - ruR - (SL * L->r) + (SR * R->r));
  if (isnan(u_S) || isnan(SR) || isnan(SL)) return 2;
  if (!gfm && bc == 4) u_S = 0.0;
  for (int iv = 0; iv < k->neq; ++iv) corr[iv] = 0.0;
  ncs nc;
  double Us[MAXNEQ];
  int err = 0;
  int left_star = gfm ? (SL < 0.0 && 0.0 <= u_S) : (SL <= 0.0 && 0.0 <= u_S);
  int right_star = gfm ? (u_S < 0.0 && 0.0 < SR) : (u_S <= 0.0 && 0.0 <= SR);
  if (0.0 <= SL) {
    phys_flux(k, L, 0, gfm, &nc, F);
  } else if (left_star) {
    err = star_region(k, g, L, L, R, 1, u_S, SL, SR, uL, vL, wL, uR, vR, wR, sL, sR, Us, &nc);
    phys_flux(k, L, 1, gfm, &nc, F);
    for (int iv = 0; iv < k->ncons; ++iv) corr[iv] = SL * (Us[iv] - L->vec[iv]);
  } else if (right_star) {
    err = star_region(k, g, R, L, R, 2, u_S, SL, SR, uL, vL, wL, uR, vR, wR, sL, sR, Us, &nc);
    phys_flux(k, R, 2, gfm, &nc, F);
    for (int iv = 0; iv < k->ncons; ++iv) corr[iv] = SR * (Us[iv] - R->vec[iv]);
  } else if (SR <= 0.0) {
    phys_flux(k, R, 3, gfm, &nc, F);
  } else {
    return 3;
  }
  if (err) return err;
  for (int iv = 0; iv < k->neq; ++iv)
    if (isnan(corr[iv])) return 4;
  for (int d = 0; d < 3; d++) unc[d] = nc.unc[d];
  return 0;
}

/* ------------------------------------------------ pressure relaxation (m5_relaxationvec.c) */
static void vf_limit_relax(const cfg *k, double *avf, int elseif) {
  const int n1 = k->N - 1;
  const double lo = k->amin / 100.0, hi = 1.0 - (k->amin / 100.0);
  double sum = 0.0;
  for (int i = 0; i < n1; ++i) {
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
    double dif = sum - hi;
    for (int j = 0; j < n1; ++j) {
      double per = avf[j] / sum;
      avf[j] = avf[j] - per * dif;
    }
    sum = hi;
  }
  avf[n1] = 1.0 - sum;
}

static int relaxationvec(const cfg *k, double *V) {
  const int N = k->N;
  double ar[MAXN], are[MAXN], avf[MAXN + 1], avf0[MAXN + 1], A[9], G[9], Gmag;
  double rho = 0.0;
  for (int iv = 0; iv < N; ++iv) {
    ar[iv] = V[iv + k->i0];
    are[iv] = V[iv + k->i4];
    rho += ar[iv];
  }
  double u = V[k->i1 + 0] / rho, v = V[k->i1 + 1] / rho, w = V[k->i1 + 2] / rho;
  double rE = V[k->i2];
  for (int iv = 0; iv < N - 1; ++iv) avf[iv] = V[iv + k->i3];
  vf_limit_relax(k, avf, 1);
  double sum0 = 0.0;
  for (int iv = 0; iv < N - 1; ++iv) sum0 += avf[iv];
  for (int iv = 0; iv < N - 1; ++iv) avf0[iv] = avf[iv];
  avf0[N - 1] = avf[N - 1];
  (void)sum0;
  for (int q = 0; q < 9; q++) A[q] = V[q + k->i5];
  gmat_of(A, G, &Gmag);
  double ael_t[MAXN] = {0}, p_relaxed;
  const double eps_sml = 1.0e-12, eps_big = 1.0e-8;
  if (k->prelax == 1) {
    double t0[MAXN], p0[MAXN];
    for (int iv = 0; iv < N; ++iv) {
      double ael = (k->mu[iv] != 0.0) ? elastic_energy(G, Gmag, k->mu[iv], 0) : 0.0;
      t0[iv] = 1.0 / (ar[iv] / avf[iv]);
      p0[iv] = ((k->gamma[iv] - 1.0) * (are[iv] - ael) / avf[iv]) - k->gamma[iv] * k->pinf[iv];
    }
    const double *ga = k->gamma, *pi = k->pinf;
    double A_1 = (avf[0] / ga[0]) * (p0[0] + pi[0]) / ((avf[0] / ga[0]) + (avf[1] / ga[1]));
    double A_2 = (avf[1] / ga[1]) * (p0[1] + pi[1]) / ((avf[0] / ga[0]) + (avf[1] / ga[1]));
    double d = (A_2 - A_1 - (pi[1] - pi[0]));
    double pe = 0.5 * (A_1 + A_2 - (pi[0] + pi[1])) + sqrt(0.25 * (d * d) + A_1 * A_2);
    if (isnan(pe)) return 6;
    for (int iv = 0; iv < N; ++iv) {
      double t1 = t0[iv] * (p0[iv] + ga[iv] * pi[iv] + (ga[iv] - 1.0) * pe) /
                  (pe + ga[iv] * pi[iv] + (ga[iv] - 1.0) * pe);
      double rm = 1.0 / t1;
      avf[iv] = ar[iv] / rm;
    }
    vf_limit_relax(k, avf, 0);
    for (int q = 0; q < 9; q++) A[q] = A[q] * (avf[0] / avf0[0]);
  } else if (k->prelax == 3) {
    double rhoKs[MAXN], pkinit[MAXN];
    for (int iv = 0; iv < N; ++iv) {
      if (avf[iv] < 0.0 || ar[iv] < 0.0) {
        avf[iv] = eps_sml;
        ar[iv] = eps_sml;
        are[iv] = eps_sml;
      }
      if (avf[iv] >= 1.0) avf[iv] = 1.0 - eps_sml;
    }
    int irelax = 1;
    for (int iv = 0; iv < N; ++iv)
      if (avf[iv] > 1.0 - eps_sml) irelax = 0;
    if (irelax) {
      p_relaxed = 0.0;
      for (int iv = 0; iv < N; ++iv) {
        if (avf[iv] > eps_sml) {
          double ael = (k->mu[iv] != 0.0) ? elastic_energy(G, Gmag, k->mu[iv], 0) : 0.0;
          pkinit[iv] = ((k->gamma[iv] - 1.0) * (are[iv] - ael) / avf[iv]) -
                       k->gamma[iv] * k->pinf[iv];
          if (pkinit[iv] <= -(1.0 - eps_big) * k->pinf[iv] + eps_big)
            pkinit[iv] = -(1.0 - eps_big) * k->pinf[iv] + eps_big;
        } else {
          pkinit[iv] = 0.0;
        }
        p_relaxed += avf[iv] * pkinit[iv];
      }
      int iter = 0;
      double F = 1.0e-9, dF = 1.0e9;
      for (int iv = 0; iv < N; ++iv) rhoKs[iv] = 0.0;
      while ((fabs(F) > 1.0e-12) && (iter < 500)) {
        p_relaxed = p_relaxed - F / dF;
        iter = iter + 1;
        for (int iv = 0; iv < N; ++iv)
          if (p_relaxed < -(1.0 - eps_big) * k->pinf[iv] + eps_big)
            p_relaxed = -(1.0 - eps_big) * k->pinf[iv] + 1.0;
        F = -1.0;
        dF = 0.0;
        for (int iv = 0; iv < N; ++iv) {
          if (avf[iv] > eps_sml) {
            double am = (avf[iv] > eps_sml) ? avf[iv] : eps_sml;
            rhoKs[iv] = ar[iv] / am *
                        pow((p_relaxed + k->pinf[iv]) / (pkinit[iv] + k->pinf[iv]),
                            1.0 / k->gamma[iv]);
            F = F + ar[iv] / rhoKs[iv];
            dF = dF - ar[iv] / (k->gamma[iv] * rhoKs[iv] * (p_relaxed + k->pinf[iv]));
          }
        }
        if (isnan(p_relaxed) || isnan(F) || isnan(dF)) return 7;
      }
      for (int iv = 0; iv < N; ++iv)
        if (avf[iv] > eps_sml) avf[iv] = ar[iv] / rhoKs[iv];
      vf_limit_relax(k, avf, 1);
    }
    int i_as = 0;
    if ((avf[0] < avf[1]) && (k->mu[1] != 0.0)) i_as = 1;
    for (int q = 0; q < 9; q++) A[q] = A[q] * (avf[i_as] / avf0[i_as]);
  } else {
    return 8;
  }
  double e_elast = 0.0;
  for (int iv = 0; iv < N; ++iv) {
    ael_t[iv] = (k->mu[iv] != 0.0) ? elastic_energy(G, Gmag, k->mu[iv], 0) : 0.0;
    double eK = ael_t[iv] / (ar[iv]);
    double Ys = ar[iv] / rho;
    e_elast += Ys * eK;
  }
  double e_hyd = rE / rho - 0.5 * (u * u + v * v + w * w) - e_elast;
  double num = 0.0, den = 0.0;
  for (int iv = 0; iv < N; ++iv) {
    num += avf[iv] * k->gamma[iv] * k->pinf[iv] / (k->gamma[iv] - 1.0);
    den += avf[iv] / (k->gamma[iv] - 1.0);
  }
  p_relaxed = (rho * e_hyd - num) / den;
  for (int iv = 0; iv < N; ++iv)
    are[iv] = (avf[iv] * (p_relaxed + k->gamma[iv] * k->pinf[iv]) / (k->gamma[iv] - 1.0)) +
              ael_t[iv];
  for (int iv = 0; iv < N - 1; ++iv) {
    if (isnan(avf[iv])) return 7;
    V[iv + k->i3] = avf[iv];
  }
  for (int iv = 0; iv < N; iv++) {
    if (isnan(are[iv])) return 7;
    V[iv + k->i4] = are[iv];
  }
  for (int q = 0; q < 9; ++q) V[q + k->i5] = A[q];
  return 0;
}

/* ------------------------------------------- MUSCL face states (m5_faceinterp_V1 etc.) */

/* avf_limit.c:3-21 */
static void avf_limit(const cfg *k, double *S) {
  const int n = k->N - 1;
  const double lo = k->amin / 100.0, hi = 1.0 - (k->amin / 100.0);
  double sum = 0.0;
  for (int v = 0; v < n; ++v) {
    double *a = S + k->i3 + v;
    if (*a <= lo) *a = lo;
    else if (*a >= hi) *a = hi;
    sum += *a;
  }
  if (sum > hi) {
    double dif = sum - hi;
    for (int j = 0; j < n; ++j) {
      double *a = S + k->i3 + j;
      *a -= (*a / sum) * dif;
    }
  }
}

static const int fcopp[6] = {2, 3, 0, 1, 5, 4};

/* m5_facevalues_MUSCL.c:3-45 (iside 1) */
static void value_across(const cfg *k, const ffvo_mesh *m, const double *S, int64_t c, int f,
                         double *out) {
  const int neq = k->neq;
  int64_t r = 6 * c + f;
  if (m->bc[r] != 0) {
    sol s;
    make_sol(k, S + neq * c, S + neq * c, 0, &s);
    for (int i = 0; i < neq; i++) out[i] = s.vec[i];
  } else if (m->nn[r] == 1) {
    const double *o = S + neq * m->nb[4 * r];
    for (int i = 0; i < neq; i++) out[i] = o[i];
  } else {
    int nn = m->nn[r];
    for (int i = 0; i < neq; i++) out[i] = 0.0;
    for (int q = 0; q < nn; q++) {
      const double *o = S + neq * m->nb[4 * r + q];
      for (int i = 0; i < neq; i++) out[i] += o[i] / ((double)nn);
    }
  }
  avf_limit(k, out);
}

/* m5_faceinterp.c:59-88, m5_deltavalues.c:23-56, m5_reconctruct.c:96-191 */
static int face_interp(const cfg *k, const ffvo_mesh *m, const double *S, double *SF) {
  const int neq = k->neq, n1 = k->N - 1;
  const double lo = k->amin / 100.0;
  for (int64_t c = 0; c < m->n; c++) {
    double SLc[MAXNEQ];
    for (int i = 0; i < neq; i++) SLc[i] = S[neq * c + i];
    avf_limit(k, SLc);
    for (int f = 0; f < 6; f++) {
      int fo = fcopp[f];
      double X[MAXNEQ], df[MAXNEQ], db[MAXNEQ];
      value_across(k, m, S, c, f, X);
      for (int i = 0; i < neq; i++) df[i] = X[i] - SLc[i];
      value_across(k, m, S, c, fo, X);
      for (int i = 0; i < neq; i++) db[i] = X[i] - SLc[i];
      double dp = m->dist_cc[6 * c + f], dm = m->dist_cc[6 * c + fo], cf = m->dist_cf[6 * c + f];
      double *out = SF + (6 * c + f) * neq;
      for (int i = 0; i < neq; i++) {
        double grad = 0.0;
        if (m->bc[6 * c + f] == 0) {
          if (fabs(df[i]) > 1e-10) {
            double product = (-db[i] / dm) * (df[i] / dp);
            if (product > 0.0) {
              if (fabs(-db[i] / dm) > fabs(df[i] / dp))
                grad = k->lim[i] * (df[i] / dp);
              else
                grad = k->lim[i] * (-db[i] / dm);
            } else {
              grad = 0.0;
            }
          }
        }
        out[i] = SLc[i] + cf * grad;
      }
      double avf[MAXN + 1], sum = 0.0;
      for (int iv = 0; iv < n1; ++iv) {
        avf[iv] = out[iv + k->i3];
        if (avf[iv] <= lo) avf[iv] = lo;
        else if (avf[iv] >= (1.0 - (2.0 * lo))) avf[iv] = 1.0 - (2.0 * lo);
        sum += avf[iv];
      }
      if (sum >= (1.0 - lo)) {
        double dif = sum - (1.0 - lo);
        for (int j = 0; j < n1; ++j) {
          double per = avf[j] / sum;
          avf[j] = avf[j] - per * dif;
        }
      }
      for (int iv = 0; iv < n1; ++iv) out[iv + k->i3] = avf[iv];
      int err = relaxationvec(k, out);
      if (err) return err;
    }
  }
  return 0;
}

/* ------------------------------------------------------------ residual (m5_residual.c) */
typedef struct work {
  double *SF, *flux_face, *u_face, *gfm_face, *RHS, *SN;
  int32_t *flag;
} work;

static int residual(const cfg *k, const ffvo_mesh *m, const double *S, work *W) {
  const int neq = k->neq, N = k->N;
  for (int64_t c = 0; c < m->n; c++) {
    const double *Sc = S + neq * c;
    double *rhs = W->RHS + neq * c;
    for (int iv = 0; iv < neq; iv++) rhs[iv] = 0.0;
    sol C;
    make_sol(k, Sc, Sc, 0, &C);
    const double *Am = C.A;
    for (int f = 0; f < 6; f++) {
      int64_t r = 6 * c + f;
      double *ff = W->flux_face + r * neq, *uf = W->u_face + 3 * r;
      for (int iv = 0; iv < neq; iv++) ff[iv] = 0.0;
      W->gfm_face[r] = 0.0;
      uf[0] = uf[1] = uf[2] = 0.0;
      int compute = 1, nneig = 1;
      if (m->bc[r] == 0) {
        if (m->nn[r] == 1) {
          int64_t o = m->nb[4 * r];
          int fo = m->neigfc[r];
          if (m->nn[6 * o + fo] == 1) {
            int si_c = m->si ? m->si[c] : 0;
            if (si_c == 0) {
              if (W->flag[r] == 1) {
                const double *of = W->flux_face + (6 * o + fo) * neq;
                const double *ou = W->u_face + 3 * (6 * o + fo);
                uf[0] = -ou[0];
                uf[1] = -ou[1];
                uf[2] = -ou[2];
                for (int iv = 0; iv < neq; iv++) ff[iv] = -of[iv];
                compute = 0;
              } else {
                W->flag[6 * o + fo] = 1;
              }
            }
          }
        } else {
          nneig = m->nn[r];
        }
      }
      double Area_f = 0.0;
      for (int q = 0; q < nneig; ++q) Area_f += m->area[4 * r + q];
      geo g = face_geo(m, c, f);
      if (compute && m->bc[r] == 1) {
        /* m5_hllc.c:56-85: the HLLC flux of a symmetry face is replaced by the mean of the
         * physical fluxes of the cell state (m5_facevalues.c, imode 0) and of its mirror
         * image, no correction term */
        sol L, R;
        make_sol(k, Sc, Sc, 0, &L);
        R = L;
        apply_bc(1, &g, &L, &R);
        ncs nc;
        nc.unc[0] = 0.5 * (L.u + R.u);
        nc.unc[1] = 0.5 * (L.v + R.v);
        nc.unc[2] = 0.5 * (L.w + R.w);
        double FL[MAXNEQ][3], FR[MAXNEQ][3], F[MAXNEQ][3];
        phys_flux(k, &L, 4, 0, &nc, FL);
        phys_flux(k, &R, 4, 0, &nc, FR);
        for (int iv = 0; iv < neq; ++iv)
          for (int d = 0; d < 3; d++) F[iv][d] = (0.0 + 0.5 * FL[iv][d]) + 0.5 * FR[iv][d];
        double A = m->area[4 * r];
        for (int iv = 0; iv < neq; ++iv)
          ff[iv] += (A) * ((F[iv][0] * g.n[0] + F[iv][1] * g.n[1] + F[iv][2] * g.n[2]) + 0.0);
        uf[0] = nc.unc[0];
        uf[1] = nc.unc[1];
        uf[2] = nc.unc[2];
      } else if (compute) {
        sol L;
        if (k->order == 2) make_sol(k, W->SF + r * neq, Sc, 1, &L);
        else make_sol(k, Sc, Sc, 0, &L);
        for (int q = 0; q < nneig; ++q) {
          sol R, Lq = L;
          if (m->bc[r] == 0) {
            int64_t o = m->nb[4 * r + q];
            int fo = m->neigfc[r];
            if (k->order == 2) make_sol(k, W->SF + (6 * o + fo) * neq, S + neq * o, 1, &R);
            else make_sol(k, S + neq * o, S + neq * o, 0, &R);
          } else {
            R = L;
            int e = apply_bc(m->bc[r], &g, &L, &R);
            if (e) return e;
          }
          double F[MAXNEQ][3], corr[MAXNEQ], unc[3];
          int gfm = 0;
          if (Lq.phi[0] * R.phi[0] < 0.0) {
            W->gfm_face[r] = 1.0;
            gfm = 1;
          }
          int err = hllc(k, &g, &Lq, &R, m->bc[r], gfm, F, corr, unc);
          if (err) return err;
          double A = m->area[4 * r + q];
          for (int iv = 0; iv < neq; ++iv)
            ff[iv] += (A) * ((F[iv][0] * g.n[0] + F[iv][1] * g.n[1] + F[iv][2] * g.n[2]) + corr[iv]);
          uf[0] = unc[0] / ((double)nneig);
          uf[1] = unc[1] / ((double)nneig);
          uf[2] = unc[2] / ((double)nneig);
        }
      }
      for (int iv = 0; iv < neq; ++iv) rhs[iv] += ff[iv];
      /* m5_residual.c:178-214: non-conservative terms with the face velocity */
      const double un = uf[0], vn = uf[1], wn = uf[2], nx = g.n[0], ny = g.n[1], nz = g.n[2];
      for (int iv = 0; iv < N - 1; ++iv) {
        const double s = C.avf[iv];
        rhs[k->i3 + iv] += Area_f * (s * un * nx + s * vn * ny + s * wn * nz);
      }
      for (int iv = 0; iv < N; ++iv) {
        const double(*t)[3] = C.ast[iv];
        rhs[k->i4 + iv] += Area_f * (t[0][0] * un * nx + t[0][1] * vn * nx + t[0][2] * wn * nx +
                                     t[1][0] * un * ny + t[1][1] * vn * ny + t[1][2] * wn * ny +
                                     t[2][0] * un * nz + t[2][1] * vn * nz + t[2][2] * wn * nz);
      }
      const double A1 = Am[0], A2 = Am[1], A3 = Am[2], B1 = Am[3], B2 = Am[4], B3 = Am[5],
                   C1 = Am[6], C2 = Am[7], C3 = Am[8];
      double *R5 = rhs + k->i5;
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
    for (int iv = 0; iv < neq; iv++)
      if (isnan(rhs[iv])) return 1;
  }
  return 0;
}

/* ---------------------------------------------- ghost-fluid velocity fix (m5_gfm*.c) */
static long g_gfm_calls[2];
long ffvo_m5_gfm_calls(int relax) { return g_gfm_calls[relax ? 1 : 0]; }

static void gfm_fix(const cfg *k, const ffvo_mesh *m, double *S, const work *W, int64_t c,
                    int relax) {
  const int neq = k->neq, N = k->N;
  double *Sc = S + neq * c;
  const double *rhs = W->RHS + neq * c;
  const double V = m->vol[c], DT = k->dt;
  double rho_new = 0.0, ut, vt, wt;
  g_gfm_calls[relax ? 1 : 0]++;
  if (!relax) {
    for (int v = 0; v < N; ++v) rho_new += Sc[v] + (DT / V) * rhs[v];
    ut = Sc[k->i1 + 0] + (DT / V) * rhs[k->i1 + 0];
    vt = Sc[k->i1 + 1] + (DT / V) * rhs[k->i1 + 1];
    wt = Sc[k->i1 + 2] + (DT / V) * rhs[k->i1 + 2];
    ut = ut / rho_new;
    vt = vt / rho_new;
    wt = wt / rho_new;
  } else {
    for (int v = 0; v < N; ++v) rho_new += Sc[v];
    ut = Sc[k->i1 + 0] / rho_new;
    vt = Sc[k->i1 + 1] / rho_new;
    wt = Sc[k->i1 + 2] / rho_new;
  }
  double nxi = 0.0, nyi = 0.0, nzi = 0.0, total = 0.0;
  double ug[6], vg[6], wg[6];
  int nint = 0;
  for (int f = 0; f < 6; f++) {
    int64_t r = 6 * c + f;
    sol L, R;
    make_sol(k, Sc, Sc, 0, &L);
    geo g = face_geo(m, c, f);
    if (m->bc[r] == 0) {
      const double *So = S + neq * m->nb[4 * r];
      make_sol(k, So, So, 0, &R);
    } else {
      R = L;
      apply_bc(m->bc[r], &g, &L, &R);
    }
    if (W->gfm_face[r] == 1.0) {
      double phi = (L.phi[0] + R.phi[0]) / 2.0;
      double A = m->area[4 * r];
      if (relax) {
        nxi += phi * A * g.n[0];
        nyi += phi * A * g.n[1];
        nzi += phi * A * g.n[2];
      } else {
        nxi = phi * A * g.n[0];
        nyi = phi * A * g.n[1];
        nzi = phi * A * g.n[2];
      }
      ug[nint] = R.u;
      vg[nint] = R.v;
      wg[nint] = R.w;
      total += A;
      nint++;
    }
  }
  if (nint != 0) {
    double norm = sqrt(nxi * nxi + nyi * nyi + nzi * nzi);
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
    double n2x = nyi * n1z - nzi * n1y, n2y = nzi * n1x - nxi * n1z, n2z = nxi * n1y - nyi * n1x;
    double ul = ut * nxi + vt * nyi + wt * nzi;
    double vl[6], wl[6];
    for (int q = 0; q < nint; q++) {
      vl[q] = ug[q] * n1x + vg[q] * n1y + wg[q] * n1z;
      wl[q] = ug[q] * n2x + vg[q] * n2y + wg[q] * n2z;
    }
    double unl = ul, vnl = 0.0, wnl = 0.0;
    int ft = 0;
    for (int f = 0; f < 6; f++) {
      int64_t r = 6 * c + f;
      if (W->gfm_face[r] == 1.0) {
        vnl = vl[ft] * (m->area[4 * r] / total);
        wnl = wl[ft] * (m->area[4 * r] / total);
        ft++;
      }
    }
    double ung = unl * nxi + vnl * n1x + wnl * n2x;
    double vng = unl * nyi + vnl * n1y + wnl * n2y;
    double wng = unl * nzi + vnl * n1z + wnl * n2z;
    if (!relax)
      for (int v = 0; v < N; ++v) Sc[v] = Sc[v] + (DT / V) * rhs[v];
    Sc[k->i1 + 0] = rho_new * ung;
    Sc[k->i1 + 1] = rho_new * vng;
    Sc[k->i1 + 2] = rho_new * wng;
    Sc[k->i2] -= rho_new * 0.5 * (ut * ut + vt * vt + wt * wt);
    Sc[k->i2] += rho_new * 0.5 * (ung * ung + vng * vng + wng * wng);
  } else if (!relax) {
    for (int v = 0; v < N; ++v) Sc[v] = Sc[v] + (DT / V) * rhs[v];
    for (int d = 0; d < 3; d++) Sc[k->i1 + d] = Sc[k->i1 + d] + (DT / V) * rhs[k->i1 + d];
  }
}

/* m5_RK.c:3-127 */
static void rk_update(const cfg *k, const ffvo_mesh *m, double *S, const work *W, int irk) {
  const int neq = k->neq, N = k->N;
  const double DT = k->dt;
  for (int64_t c = 0; c < m->n; c++) {
    double *s = S + neq * c, *sn = W->SN + neq * c;
    const double *rhs = W->RHS + neq * c, V = m->vol[c];
    double phi_old[MAXN];
    for (int v = 0; v < N - 1; ++v) phi_old[v] = s[k->i3 + v] - k->avf_lim;
    switch (irk) {
      case 0:
        for (int e = 0; e < neq; e++) sn[e] = s[e];
        break;
      case 1: {
        int flag = 0;
        for (int v = 0; v < N - 1; ++v) {
          if (k->mu[v] != 0.0) {
            int e = k->i3 + v;
            double buf = (1.0 / V) * rhs[e];
            double as_new = sn[e] + DT * buf;
            if (phi_old[v] * (as_new - k->avf_lim) < 0.0) flag = 1;
          }
        }
        if (flag) {
          for (int e = k->i2; e < neq; e++) s[e] = sn[e] + DT * ((1.0 / V) * rhs[e]);
          gfm_fix(k, m, S, W, c, 0);
        } else {
          for (int e = 0; e < neq; e++) s[e] = sn[e] + DT * ((1.0 / V) * rhs[e]);
        }
        break;
      }
      case 2:
        for (int e = 0; e < neq; e++)
          s[e] = (3.0 / 4.0) * sn[e] + (1.0 / 4.0) * s[e] + (1.0 / 4.0) * DT * rhs[e] / V;
        break;
      case 3:
        for (int e = 0; e < neq; e++)
          s[e] = (1.0 / 3.0) * sn[e] + (2.0 / 3.0) * s[e] + (2.0 / 3.0) * DT * rhs[e] / V;
        break;
      case 4:
        for (int e = 0; e < neq; e++)
          s[e] = (1.0 / 2.0) * sn[e] + (1.0 / 2.0) * s[e] + (1.0 / 2.0) * DT * rhs[e] / V;
        break;
    }
    for (int v = 0; v < N; v++)
      if (s[k->i0 + v] < 0.0) s[k->i0 + v] = sn[k->i0 + v];
    const int e5 = k->i5;
    if (k->zerou[0]) {
      s[k->i1 + 0] = sn[k->i1 + 0];
      s[e5 + 1] = sn[e5 + 1]; s[e5 + 2] = sn[e5 + 2]; s[e5 + 3] = sn[e5 + 3]; s[e5 + 6] = sn[e5 + 6];
    }
    if (k->zerou[1]) {
      s[k->i1 + 1] = sn[k->i1 + 1];
      s[e5 + 1] = sn[e5 + 1]; s[e5 + 3] = sn[e5 + 3]; s[e5 + 5] = sn[e5 + 5]; s[e5 + 7] = sn[e5 + 7];
    }
    if (k->zerou[2]) {
      s[k->i1 + 2] = sn[k->i1 + 2];
      s[e5 + 2] = sn[e5 + 2]; s[e5 + 5] = sn[e5 + 5]; s[e5 + 6] = sn[e5 + 6]; s[e5 + 7] = sn[e5 + 7];
    }
  }
}

/* m5_relaxation_solid.c:3-40.  phi_new is set there only for solid materials; for a fluid
 * material 0 the reference reads it uninitialised -- here it keeps phi_old (no trigger). */
/* ------------------------------------------------------------ radial-return plasticity */
/* Eigen-decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations (Golub & Van
 * Loan, Matrix Computations, sec. 8.5): G = Q diag(lam) Q^T, Q's columns the eigenvectors. */
static void jacobi3(const double G[9], double lam[3], double Q[9]) {
  double a[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      a[i][j] = G[3 * i + j];
      Q[3 * i + j] = (i == j) ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 32; sweep++) {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    const double dg = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (!(off > 1e-32 * dg)) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (a[p][q] == 0.0) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < 3; r++) { /* a <- a J (columns p, q) */
          const double arp = a[r][p], arq = a[r][q];
          a[r][p] = c * arp - s * arq;
          a[r][q] = s * arp + c * arq;
        }
        for (int r = 0; r < 3; r++) { /* a <- J^T a (rows p, q) */
          const double apr = a[p][r], aqr = a[q][r];
          a[p][r] = c * apr - s * aqr;
          a[q][r] = s * apr + c * aqr;
        }
        for (int r = 0; r < 3; r++) { /* Q <- Q J */
          const double qp = Q[3 * r + p], qq = Q[3 * r + q];
          Q[3 * r + p] = c * qp - s * qq;
          Q[3 * r + q] = s * qp + c * qq;
        }
      }
  }
  for (int i = 0; i < 3; i++) lam[i] = a[i][i];
}

/* von Mises stress of the hyperelastic deviator (state_equation.c:143-204, the mu term) for
 * principal values g_i = exp(2 (m + beta d_i)) of G: s_i = -mu |G|^(-1/6) (t_i - mean t),
 * t_i = g_i^2 - |G|^(1/3) g_i, |G| = exp(6 m) */
static double vm_principal(double mu, double m, const double d[3], double beta) {
  const double g13 = exp(2.0 * m), g16 = exp(m);
  double t[3];
  for (int i = 0; i < 3; i++) {
    const double g = exp(2.0 * (m + beta * d[i]));
    t[i] = g * g - g13 * g;
  }
  const double tm = (t[0] + t[1] + t[2]) / 3.0;
  double j = 0.0;
  for (int i = 0; i < 3; i++) {
    const double s = -mu / g16 * (t[i] - tm);
    j += s * s;
  }
  return sqrt(1.5 * j);
}

/* J2 radial return of a cell's deformation tensor A (no counterpart in the reference):
 * with G = A A^T = Q diag(lam) Q^T, the Hencky strain h_i = ln(lam_i) / 2 splits into its
 * mean m (volume, kept) and deviator d_i; where a solid's von Mises stress exceeds its
 * yield stress, the deviator is scaled by the largest beta in [0, 1] (60 bisection steps)
 * whose stress lies on or inside the yield surface, A <- Q diag(exp((beta - 1) d_i)) Q^T A.
 * The total energy and the materials' alpha rho e are kept: the elastic energy released is
 * dissipated into the materials' internal energy (the pressure recovery subtracts e_el from
 * alpha rho e).  Returns 1 when A changed. */
static int plastic_return(const cfg *k, double *s) {
  double *A = s + k->i5, G[9], Gmag, lam[3], Q[9];
  gmat_of(A, G, &Gmag);
  jacobi3(G, lam, Q);
  if (!(lam[0] > 0.0 && lam[1] > 0.0 && lam[2] > 0.0)) return 0;
  double h[3], d[3];
  for (int i = 0; i < 3; i++) h[i] = 0.5 * log(lam[i]);
  const double m = (h[0] + h[1] + h[2]) / 3.0;
  for (int i = 0; i < 3; i++) d[i] = h[i] - m;
  double beta = 1.0;
  for (int v = 0; v < k->N; v++) {
    if (k->mu[v] == 0.0 || !(k->yield[v] > 0.0)) continue;
    if (vm_principal(k->mu[v], m, d, beta) <= k->yield[v]) continue;
    double lo = 0.0, hi = beta;
    for (int it = 0; it < 60; it++) {
      const double mid = 0.5 * (lo + hi);
      if (vm_principal(k->mu[v], m, d, mid) <= k->yield[v]) lo = mid;
      else hi = mid;
    }
    beta = lo;
  }
  if (beta == 1.0) return 0;
  double M[9], An[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double x = 0.0;
      for (int q = 0; q < 3; q++) x += Q[3 * i + q] * exp((beta - 1.0) * d[q]) * Q[3 * j + q];
      M[3 * i + j] = x;
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      An[3 * i + j] = M[3 * i + 0] * A[0 + j] + M[3 * i + 1] * A[3 + j] + M[3 * i + 2] * A[6 + j];
  for (int q = 0; q < 9; q++) A[q] = An[q];
  return 1;
}

static int relaxation_solid(const cfg *k, const ffvo_mesh *m, double *S, const work *W) {
  const int neq = k->neq, N = k->N;
  for (int64_t c = 0; c < m->n; c++) {
    double *s = S + neq * c;
    double phi_old[MAXN], phi_new[MAXN];
    for (int iv = 0; iv < N - 1; ++iv) phi_old[iv] = s[k->i3 + iv] - k->avf_lim;
    int err = relaxationvec(k, s);
    if (err) return err;
    /* the plastic step of the reference's prototype (m5_relaxation_solid.c:14 runs it per
       leaf in this loop), after the relaxation so that the stored state lies on or inside
       the yield surface (the relaxation scales A by the solid-fraction ratio) */
    if (k->plastic) plastic_return(k, s);
    for (int iv = 0; iv < N - 1; ++iv)
      phi_new[iv] = (k->mu[iv] != 0.0) ? s[k->i3 + iv] - k->avf_lim : phi_old[iv];
    if (phi_old[0] * phi_new[0] < 0.0) gfm_fix(k, m, S, W, c, 1);
  }
  return 0;
}

static int make_cfg(const ffvo_m5_params *p, double dt, cfg *k) {
  memset(k, 0, sizeof(*k));
  const int N = p->nmat;
  if (N < 2 || N > MAXN) return 10;
  k->N = N;
  k->neq = 3 * N + 12;
  k->ncons = N + 4;
  k->i0 = 0;
  k->i1 = N;
  k->i2 = N + 3;
  k->i3 = N + 4;
  k->i4 = 2 * N + 3;
  k->i5 = 3 * N + 3;
  k->order = p->order;
  k->rk_steps = p->rk_steps;
  k->prelax = p->prelax;
  k->flux_form = p->flux_form;
  if (k->flux_form != 0 && k->flux_form != 1) return 10;
  for (int d = 0; d < 3; d++) k->zerou[d] = p->zerou[d];
  for (int i = 0; i < N; i++) {
    k->gamma[i] = p->gamma[i];
    k->pinf[i] = p->pinf[i];
    k->mu[i] = p->mu[i];
    k->yield[i] = p->yield[i];
    if (p->mu[i] != 0.0) k->nsolids++;
    if (p->mu[i] != 0.0 && p->yield[i] > 0.0) k->plastic = 1;
  }
  if (k->nsolids > 2) return 10;
  k->amin = p->amin;
  k->avf_lim = p->avf_lim;
  k->dt = dt;
  for (int i = 0; i < k->neq; i++) k->lim[i] = (i >= k->i4 && i < k->i5) ? 0.0 : 1.0;
  return 0;
}

int ffvo_m5_advance(const ffvo_mesh *m, const ffvo_m5_params *p, double *S, double dt,
                    int nsteps) {
  cfg k;
  int err = make_cfg(p, dt, &k);
  if (err) return err;
  const int64_t n = m->n;
  const int neq = k.neq;
  work W;
  W.SF = (double *)calloc((size_t)n * 6 * neq, sizeof(double));
  W.flux_face = (double *)calloc((size_t)n * 6 * neq, sizeof(double));
  W.u_face = (double *)calloc((size_t)n * 6 * 3, sizeof(double));
  W.gfm_face = (double *)calloc((size_t)n * 6, sizeof(double));
  W.RHS = (double *)calloc((size_t)n * neq, sizeof(double));
  W.SN = (double *)calloc((size_t)n * neq, sizeof(double));
  W.flag = (int32_t *)calloc((size_t)n * 6, sizeof(int32_t));
  if (!W.SF || !W.flux_face || !W.u_face || !W.gfm_face || !W.RHS || !W.SN || !W.flag) {
    err = -1;
    goto out;
  }
  for (int step = 0; step < nsteps && !err; step++) {
    memset(W.flag, 0, sizeof(int32_t) * 6 * n);
    rk_update(&k, m, S, &W, 0);
    for (int irk = 1; irk <= k.rk_steps && !err; irk++) {
      if (k.order == 2) err = face_interp(&k, m, S, W.SF);
      if (!err) err = residual(&k, m, S, &W);
      if (!err) {
        memset(W.flag, 0, sizeof(int32_t) * 6 * n);
        rk_update(&k, m, S, &W, irk);
        err = relaxation_solid(&k, m, S, &W);
      }
    }
  }
out:
  free(W.SF);
  free(W.flux_face);
  free(W.u_face);
  free(W.gfm_face);
  free(W.RHS);
  free(W.SN);
  free(W.flag);
  return err;
}
