/*
 * CPU restatement of the reference's explicit finite-volume step (TEST INFRASTRUCTURE).
 *
 * This is the oracle that the CUDA path is checked against.  It restates, on flat
 * arrays, the algorithm of the reference's own C code, function by function, with the
 * same floating-point operation order; it is pinned against the reference itself
 * (oracle/_ref, built from the reference's sources by oracle/ref/Makefile) by the tests
 * under tests/.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it.  It is never part of the product path.
 *
 * Geometry is taken in the reference's own per-leaf form (general hex geometry, no
 * Cartesian shortcuts), one row per cell face, six rows per cell.
 */
#ifndef FFV_ORACLE_H
#define FFV_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ffvo_mesh {
  int64_t n;
  const int32_t *bc;        /* [6n] fc[f].bc                                  */
  const int32_t *nn;        /* [6n] lfc_neigs[f] (0 on boundary faces)        */
  const int32_t *neigfc;    /* [6n] neigfc[f]                                 */
  const int32_t *nb;        /* [24n] neigtr[f][k] as cell index, -1 unused     */
  const double *area;       /* [24n] Area[f][k]                               */
  const double *nrm;        /* [54n] nx ny nz, nxt1 nyt1 nzt1, nxt2 nyt2 nzt2 */
  const double *dist_cf;    /* [6n]                                           */
  const double *dist_cc;    /* [6n]                                           */
  const double *vol;        /* [n]  signed Vol                                */
  const int32_t *si;        /* [n]  SI[0] (interface-layer index), may be NULL */
} ffvo_mesh;

typedef struct ffvo_params {
  int32_t order;     /* ORDER 1 or 2 */
  int32_t rk_steps;  /* RK_STEPS */
  double gamma;      /* MATERGAMA[0] */
  double pinf;       /* MATERPINF[0] */
} ffvo_params;

/* Model 0: advance S (AoS, [n][5]) by nsteps steps of size dt, as loop.c:12-21 ->
 * advancetimeexplicit.c:9-24 do.  Returns 0, or a nonzero code where the reference
 * would print and exit (NaN residual, no HLLC branch taken). */
int ffvo_m0_advance(const ffvo_mesh *m, const ffvo_params *p, double *S, double dt,
                    int nsteps);

/* Model 0, one stage (irk as RK(irk)); SN, SF, RHS, flux buffers are caller-owned
 * scratch: SN [n*5], work [n*6*5*2 + n*5 + n*6]. */
int ffvo_m0_stage(const ffvo_mesh *m, const ffvo_params *p, double *S, double *SN,
                  double *work, int irk, double dt);

/* Model 5 (m5_*): N materials, NEQ = 3N + 12. */
typedef struct ffvo_m5_params {
  int32_t nmat;      /* NMATERIALS (2..4) */
  int32_t order;     /* ORDER */
  int32_t rk_steps;  /* RK_STEPS */
  int32_t prelax;    /* PRELAX: 1 (two materials, closed form) or 3 (iterative) */
  int32_t zerou[3];  /* ZEROU0..2 */
  int32_t flux_form;   /* 0: the reference's m5 flux, as written; 1: the consistent flux (a
                          deviation): the Rankine-Hugoniot star-state energy in place of
                          m5_star_region.c:59, and m5_flux.c's momentum flux and left/right
                          deformation flux with m5_flux_gfm.c's signs (rho u u - sigma, +A) */
  double gamma[4], pinf[4], mu[4];  /* MATERGAMA, MATERPINF, MATERMUSH */
  double amin;       /* AMIN */
  double avf_lim;    /* AVF_LIM */
  double yield[4];   /* von Mises yield stress per material, 0 = none (no reference
                        counterpart: the reference's plastic step is only prototyped,
                        strdata.h:809, and its call commented out, m5_relaxation_solid.c:14) */
} ffvo_m5_params;

/* Advance S (AoS, [n][3N+12]) by nsteps steps of size dt (loop.c:12-21 ->
 * advancetimeexplicit.c:9-24 with m5_RK and m5_relaxation_solid).  Returns 0 or the
 * code of the check where the reference would print and exit. */
int ffvo_m5_advance(const ffvo_mesh *m, const ffvo_m5_params *p, double *S, double dt,
                    int nsteps);

/* Number of ghost-fluid velocity fixes run so far (m5_gfm: relax 0, m5_gfm_rel: 1), so
 * that tests can show a case exercises them. */
long ffvo_m5_gfm_calls(int relax);

#ifdef __cplusplus
}
#endif
#endif
