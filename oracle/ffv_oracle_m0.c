/*
 * Model-0 (Euler, stiffened gas) restatement of the reference's explicit FV step.
 * TEST INFRASTRUCTURE ONLY: the oracle for the CUDA path; see ffv_oracle.h.
 *
 * Each function names the reference function it restates and keeps its operation order,
 * so that compiled with -ffp-contract=off it reproduces the reference's doubles exactly.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ffv_oracle.h"

#define NEQ0 5

typedef struct sol {
  double r, u, v, w, e, e_internal, p, c;
  double vec[NEQ0];
} sol;

typedef struct geo {
  double nx, ny, nz, mx, my, mz, lx, ly, lz;
} geo;

static geo face_geo(const ffvo_mesh *m, int64_t c, int f) {
  const double *q = m->nrm + 54 * c + 9 * f;
  geo g = {q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8]};
  return g;
}

/* m0_facercnstr.c:3-56 (ORDER 2) and m0_facevalues.c:3-48 (ORDER 1): state vector ->
 * primitive face state with stiffened-gas pressure and sound speed. */
static void state_to_sol(const double *U, double gamma, double pinf, sol *s) {
  s->r = U[0];
  s->u = U[1] / s->r;
  s->v = U[2] / s->r;
  s->w = U[3] / s->r;
  for (int i = 0; i < NEQ0; i++) s->vec[i] = U[i];
  s->e = U[4];
  s->e_internal = (s->e / s->r) - 0.5 * (s->u * s->u + s->v * s->v + s->w * s->w);
  s->p = s->r * (gamma - 1.0) * s->e_internal - gamma * pinf;
  s->c = sqrt(gamma * (s->p + pinf) / s->r);
}

/* m0_bc.c:3-31 with bc_reflective.c:3-29 (bc 1, 4) and bc_wall.c:3-28 (bc 5): only the
 * primitive velocity of the ghost state changes; its state vector stays the interior's. */
static void apply_bc(int bc, const geo *g, const sol *L, sol *R) {
  if (bc == 1 || bc == 4 || bc == 5) {
    double u = L->u, v = L->v, w = L->w;
    double ul = u * g->nx + v * g->ny + w * g->nz;
    double vl = u * g->mx + v * g->my + w * g->mz;
    double wl = u * g->lx + v * g->ly + w * g->lz;
    double ur = -ul, vr = (bc == 5) ? -vl : vl, wr = (bc == 5) ? -wl : wl;
    R->u = ur * g->nx + vr * g->mx + wr * g->lx;
    R->v = ur * g->ny + vr * g->my + wr * g->ly;
    R->w = ur * g->nz + vr * g->mz + wr * g->lz;
  }
}

/* rotate_vectors.c:73-106 (rotate_tensor), entry [0][0] of R st R^T for st = p I. */
static double rotated_s11(double p, const geo *g) {
  const double st[3][3] = {{p, 0.0, 0.0}, {0.0, p, 0.0}, {0.0, 0.0, p}};
  const double vec0[3] = {g->nx, g->ny, g->nz};
  const double vecT0[3] = {g->nx, g->ny, g->nz};
  double m1[3] = {0.0, 0.0, 0.0};
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 3; k++) m1[j] += vec0[k] * st[k][j];
  double s = 0.0;
  for (int k = 0; k < 3; k++) s += m1[k] * vecT0[k];
  return s;
}

/* m0_flux.c:3-28: physical flux tensor, column d = direction x/y/z. */
static void phys_flux(const sol *s, double F[NEQ0][3]) {
  F[0][0] = s->u * s->r;
  F[0][1] = s->v * s->r;
  F[0][2] = s->w * s->r;
  F[1][0] = s->r * s->u * s->u + s->p;
  F[1][1] = s->r * s->u * s->v + 0.0;
  F[1][2] = s->r * s->u * s->w + 0.0;
  F[2][0] = s->r * s->v * s->u + 0.0;
  F[2][1] = s->r * s->v * s->v + s->p;
  F[2][2] = s->r * s->v * s->w + 0.0;
  F[3][0] = s->r * s->w * s->u + 0.0;
  F[3][1] = s->r * s->w * s->v + 0.0;
  F[3][2] = s->r * s->w * s->w + s->p;
  F[4][0] = s->u * (s->e + s->p);
  F[4][1] = s->v * (s->e + s->p);
  F[4][2] = s->w * (s->e + s->p);
}

/* m0_star_region.c:3-31: HLLC star state of side K. */
static void star_state(const sol *s, const geo *g, double S_S, double SK, double uK, double vK,
                       double wK, double Us[NEQ0]) {
  double const_S = s->r * (SK - uK) / (SK - S_S);
  double u = S_S, v = vK, w = wK;
  Us[0] = const_S;
  Us[1] = const_S * (u * g->nx + v * g->mx + w * g->lx);
  Us[2] = const_S * (u * g->ny + v * g->my + w * g->ly);
  Us[3] = const_S * (u * g->nz + v * g->mz + w * g->lz);
  Us[4] = const_S * ((s->e / s->r) + (S_S - uK) * (S_S + (s->p / (s->r * (SK - uK)))));
}

/* m0_hllc.c:3-59 with m0_wave_speeds.c:3-76: fills F (physical flux of the upwind side)
 * and corr (the HLLC star correction).  Returns nonzero where the reference exits. */
static int hllc(const sol *L, const sol *R, const geo *g, int bc, double F[NEQ0][3],
                double corr[NEQ0]) {
  double uL = L->u * g->nx + L->v * g->ny + L->w * g->nz;
  double vL = L->u * g->mx + L->v * g->my + L->w * g->mz;
  double wL = L->u * g->lx + L->v * g->ly + L->w * g->lz;
  double uR = R->u * g->nx + R->v * g->ny + R->w * g->nz;
  double vR = R->u * g->mx + R->v * g->my + R->w * g->mz;
  double wR = R->u * g->lx + R->v * g->ly + R->w * g->lz;
  double ruL = L->r * uL, ruR = R->r * uR;
  double cL = L->c, cR = R->c;
  double a = uL + cL, b = uR + cR;
  double SR = (a > b) ? a : b;
  a = uL - cL;
  b = uR - cR;
  double SL = (a < b) ? a : b;
  double s11L = rotated_s11(L->p, g), s11R = rotated_s11(R->p, g);
  double S_S = ((L->r * (uL * uL) + s11L) - (R->r * (uR * uR) + s11R) - (SL * ruL) + (SR * ruR)) /
               (ruL - ruR - (SL * L->r) + (SR * R->r));
  if (isnan(S_S)) return 2;
  for (int i = 0; i < NEQ0; i++) corr[i] = 0.0;
  if (bc == 4) S_S = 0.0;
  double Us[NEQ0];
  if (0.0 <= SL) {
    phys_flux(L, F);
  } else if (SL <= 0.0 && 0.0 <= S_S) {
    star_state(L, g, S_S, SL, uL, vL, wL, Us);
    phys_flux(L, F);
    for (int i = 0; i < NEQ0; i++) corr[i] = SL * (Us[i] - L->vec[i]);
  } else if (S_S <= 0.0 && 0.0 <= SR) {
    star_state(R, g, S_S, SR, uR, vR, wR, Us);
    phys_flux(R, F);
    for (int i = 0; i < NEQ0; i++) corr[i] = SR * (Us[i] - R->vec[i]);
  } else if (SR <= 0.0) {
    phys_flux(R, F);
  } else {
    return 3;
  }
  for (int i = 0; i < NEQ0; i++)
    if (isnan(corr[i])) return 4;
  return 0;
}

/* m0_facevalues_MUSCL.c:3-56 (iside 1): value across face f -- the neighbour, the mean of
 * the finer neighbours, or on a boundary the interior value (m0_facevalues + m0_bc change
 * only the ghost's velocity, not its state vector). */
static void value_across(const ffvo_mesh *m, const double *S, int64_t c, int f, double *out) {
  int64_t r = 6 * c + f;
  if (m->bc[r] != 0) {
    for (int i = 0; i < NEQ0; i++) out[i] = S[NEQ0 * c + i];
    return;
  }
  int nn = m->nn[r];
  if (nn == 1) {
    const double *o = S + NEQ0 * m->nb[4 * r];
    for (int i = 0; i < NEQ0; i++) out[i] = o[i];
  } else {
    for (int i = 0; i < NEQ0; i++) out[i] = 0.0;
    for (int k = 0; k < nn; k++) {
      const double *o = S + NEQ0 * m->nb[4 * r + k];
      for (int i = 0; i < NEQ0; i++) out[i] += o[i] / ((double)nn);
    }
  }
}

/* hex opposite face, operatetp.c:268-279 (fcopp) */
static const int fcopp[6] = {2, 3, 0, 1, 5, 4};

/* m0_faceinterp.c:59-88 with m0_deltavalues.c:23-57 and m0_reconctruct.c:160-207 (PRIMTV 0,
 * g_limitedvars = 1, m0_input.c:55-60): limited face states SF[c][f][:]. */
static void face_interp(const ffvo_mesh *m, const double *S, double *SF) {
  const double gate = pow(10.0, -10.0);
  for (int64_t c = 0; c < m->n; c++) {
    const double *SL = S + NEQ0 * c;
    for (int f = 0; f < 6; f++) {
      int fo = fcopp[f];
      double R[NEQ0], df[NEQ0], db[NEQ0];
      value_across(m, S, c, f, R);
      for (int i = 0; i < NEQ0; i++) df[i] = R[i] - SL[i];
      value_across(m, S, c, fo, R);
      for (int i = 0; i < NEQ0; i++) db[i] = R[i] - SL[i];
      double dp = m->dist_cc[6 * c + f], dm = m->dist_cc[6 * c + fo], cf = m->dist_cf[6 * c + f];
      double *out = SF + (6 * c + f) * NEQ0;
      for (int i = 0; i < NEQ0; i++) {
        double grad = 0.0;
        if (m->bc[6 * c + f] == 0) {
          if (fabs(df[i]) > gate) {
            double product = (-db[i] / dm) * (df[i] / dp);
            if (product > 0.0) {
              if (fabs(db[i] / dm) > fabs(df[i] / dp))
                grad = 1.0 * df[i] / dp;
              else
                grad = -1.0 * db[i] / dm;
            } else {
              grad = 0.0;
            }
          }
        }
        out[i] = SL[i] + cf * grad;
      }
    }
  }
}

/* m0_residual.c:7-141: face loop with flux reuse across 1:1 faces, RHS[c] = sum of faces. */
static int residual(const ffvo_mesh *m, const ffvo_params *p, const double *S, const double *SF,
                    double *flux_face, int32_t *flag, double *RHS) {
  for (int64_t c = 0; c < m->n; c++) {
    double *rhs = RHS + NEQ0 * c;
    for (int i = 0; i < NEQ0; i++) rhs[i] = 0.0;
    for (int f = 0; f < 6; f++) {
      int64_t r = 6 * c + f;
      int compute = 1, nneig = 1;
      double *ff = flux_face + r * NEQ0;
      if (m->bc[r] == 0) {
        if (m->nn[r] == 1) {
          int64_t o = m->nb[4 * r];
          int fo = m->neigfc[r];
          if (m->nn[6 * o + fo] == 1) {
            int si_c = m->si ? m->si[c] : 0;
            if (si_c == 0) {
              if (flag[r] == 1) {
                const double *of = flux_face + (6 * o + fo) * NEQ0;
                for (int i = 0; i < NEQ0; i++) ff[i] = -of[i];
                compute = 0;
              } else {
                flag[6 * o + fo] = 1;
              }
            }
          }
        } else {
          nneig = m->nn[r];
        }
      }
      if (compute) {
        for (int i = 0; i < NEQ0; i++) ff[i] = 0.0;
        const double *UL = (p->order == 2) ? SF + r * NEQ0 : S + NEQ0 * c;
        sol L;
        state_to_sol(UL, p->gamma, p->pinf, &L);
        geo g = face_geo(m, c, f);
        for (int k = 0; k < nneig; k++) {
          sol R;
          if (m->bc[r] == 0) {
            int64_t o = m->nb[4 * r + k];
            int fo = m->neigfc[r];
            const double *UR = (p->order == 2) ? SF + (6 * o + fo) * NEQ0 : S + NEQ0 * o;
            state_to_sol(UR, p->gamma, p->pinf, &R);
          } else {
            state_to_sol(UL, p->gamma, p->pinf, &R);
            apply_bc(m->bc[r], &g, &L, &R);
          }
          double F[NEQ0][3], corr[NEQ0];
          int err = hllc(&L, &R, &g, m->bc[r], F, corr);
          if (err) return err;
          double A = m->area[4 * r + k];
          for (int i = 0; i < NEQ0; i++)
            ff[i] += -(A) * ((F[i][0] * g.nx + F[i][1] * g.ny + F[i][2] * g.nz) + corr[i]);
        }
      }
      for (int i = 0; i < NEQ0; i++) rhs[i] += ff[i];
    }
    for (int i = 0; i < NEQ0; i++)
      if (isnan(rhs[i])) return 1;
  }
  return 0;
}

/* RK.c:3-53: stage combinations (stage k of a step uses case k). */
static void rk_update(const ffvo_mesh *m, double *S, double *SN, const double *RHS, int irk,
                      double dt) {
  for (int64_t c = 0; c < m->n; c++) {
    double V = m->vol[c];
    for (int e = 0; e < NEQ0; e++) {
      double *s = S + NEQ0 * c + e, sn = SN[NEQ0 * c + e], rhs = RHS[NEQ0 * c + e];
      switch (irk) {
        case 0: SN[NEQ0 * c + e] = *s; break;
        case 1: *s = sn - dt * (1.0 / V) * rhs; break;
        case 2: *s = (3.0 / 4.0) * sn + (1.0 / 4.0) * *s - (1.0 / 4.0) * dt * rhs / V; break;
        case 3: *s = (1.0 / 3.0) * sn + (2.0 / 3.0) * *s - (2.0 / 3.0) * dt * rhs / V; break;
        case 4: *s = (1.0 / 2.0) * sn + (1.0 / 2.0) * *s - (1.0 / 2.0) * dt * rhs / V; break;
        default: break;
      }
    }
  }
}

int ffvo_m0_stage(const ffvo_mesh *m, const ffvo_params *p, double *S, double *SN,
                  double *work, int irk, double dt) {
  int64_t n = m->n;
  double *SF = work;                       /* n*6*5 */
  double *flux_face = SF + n * 6 * NEQ0;   /* n*6*5 */
  double *RHS = flux_face + n * 6 * NEQ0;  /* n*5 */
  int32_t *flag = (int32_t *)(RHS + n * NEQ0);  /* n*6 */
  memset(flag, 0, sizeof(int32_t) * 6 * n);  /* RK.c:11-13 resets flux_flag each stage */
  if (irk == 0) {
    rk_update(m, S, SN, RHS, 0, dt);
    return 0;
  }
  if (p->order == 2) face_interp(m, S, SF);
  int err = residual(m, p, S, SF, flux_face, flag, RHS);
  if (err) return err;
  rk_update(m, S, SN, RHS, irk, dt);
  return 0;
}

int ffvo_m0_advance(const ffvo_mesh *m, const ffvo_params *p, double *S, double dt,
                    int nsteps) {
  int64_t n = m->n;
  double *SN = (double *)calloc((size_t)n * NEQ0, sizeof(double));
  double *work = (double *)calloc((size_t)n * (6 * NEQ0 * 2 + NEQ0 + 6), sizeof(double));
  if (!SN || !work) {
    free(SN);
    free(work);
    return -1;
  }
  int err = 0;
  for (int step = 0; step < nsteps && !err; step++) {
    err = ffvo_m0_stage(m, p, S, SN, work, 0, dt);
    for (int irk = 1; irk <= p->rk_steps && !err; irk++)
      err = ffvo_m0_stage(m, p, S, SN, work, irk, dt);
  }
  free(SN);
  free(work);
  return err;
}
