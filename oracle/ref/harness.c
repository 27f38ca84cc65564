/*
 * Oracle harness around the reference solver's own C sources (test infrastructure).
 *
 * The reference is linked unchanged except for these hooks, all installed with
 * `ld --wrap` so that no reference source is edited or copied:
 *
 *   malloc              pads and zeroes every allocation.  The reference writes past
 *                       three of its own buffers (memallocation.c:22 `sol->vec` holds
 *                       NMATERIALS doubles but m0_facevalues.c:20-26 writes NEQ of them;
 *                       leafallocation.c:42-47 `flux_flag` holds 4 ints, indexed to 5;
 *                       filenames.c:7-13 sizes names with sizeof(int)+4).  Padding keeps
 *                       those writes inside owned memory; zeroing makes reads of
 *                       uninitialised memory repeatable.
 *   leafallocation      also allocates `el->u_face` (6 x 3 doubles), which leafallocation.c
 *                       never allocates although m5_residual.c:67-69,163-165 writes it and
 *                       leafdeallocation.c:26-29 frees it (a split crashes without it).
 *   m0_init_domain      initial conditions from a small text file `<case>.ic` written by
 *                       the Python side (oracle/refcase.py), evaluated at leaf centroids
 *                       through the reference's own m0_init_S (init_S.c:3-16).
 *   criterionsplt       optional geometric refinement target read from `<case>.rf`, so
 *                       that parity meshes can carry 2:1 hanging faces; without the file
 *                       the reference's own criterion runs.
 *   m0_input            model 0's input reader (m0_input.c:14-20) skips 31 header lines of
 *                       `<case>.ct` but inputset.c:31-125 defines 35; the wrapper points it
 *                       at `<case>.m0ct`, a file laid out the way m0_input expects.
 *   loop                dumps the leaf list (topology, geometry, state) before and after
 *                       the reference's time loop (loop.c:3-41) and times the loop; with
 *                       a `<case>.tag` file it then runs the reference's own refinement
 *                       tagging on the final state (interface_location, criterionsplt,
 *                       criterionsmth) and dumps the tags.
 *
 * The dump format is read by oracle/refcase.py (read_dump).
 */
#include "strdata.h"
#include <stdint.h>

/* inputset.c:47-56 reads these four names that strdata.h never declares; the build
 * force-includes oracle/ref/ref_decls.h into that one file, and they live here. */
double NDFI_DIST_SOLID_0, NDFI_DIST_SOLID_1, NDFI_DIST_SOLID_2, NDFI_DIST_SOLID_3;

/* ------------------------------------------------------------------ malloc padding */
void *__real_malloc(size_t n);
void *__wrap_malloc(size_t n) {
  const size_t pad = 1024;
  void *p = __real_malloc(n + pad);
  if (p) memset(p, 0, n + pad);
  return p;
}

/* ------------------------------------------------------------------ u_face */
void __real_leafallocation(struct RUN *run, struct BRANCH *crnt);
void __wrap_leafallocation(struct RUN *run, struct BRANCH *crnt) {
  __real_leafallocation(run, crnt);
  crnt->el->u_face = __wrap_malloc(6 * sizeof(double *));
  for (int f = 0; f < 6; f++) crnt->el->u_face[f] = __wrap_malloc(3 * sizeof(double));
}

/* ------------------------------------------------------------------ case files */
static FILE *open_case_file(struct RUN *run, const char *ext) {
  char path[4096];
  snprintf(path, sizeof path, "%s%s", run->con->casename, ext);
  return fopen(path, "r");
}

/* ------------------------------------------------------------------ model-0 input */
void __real_m0_input(struct RUN *run);
void __wrap_m0_input(struct RUN *run) {
  char path[4096];
  char *saved = run->con->filecon;
  snprintf(path, sizeof path, "%s.m0ct", run->con->casename);
  run->con->filecon = path;
  __real_m0_input(run);
  run->con->filecon = saved;
}

/* ------------------------------------------------------------------ initial state */
/* IC kinds (first token of <case>.ic):
 *   split  axis x0   rhoL uL vL wL pL   rhoR uR vR wR pR
 *   sphere cx cy cz r   rhoI uI vI wI pI   rhoO uO vO wO pO
 *   wave   rho0 u0 v0 w0 p0  amp  kx ky kz   (smooth 3-D perturbation of every field) */
void m0_init_S(struct RUN *run, struct BRANCH *crnt, double rho, double u, double v,
               double w, double p);
void __real_m0_init_domain(struct RUN *run);
void __wrap_m0_init_domain(struct RUN *run) {
  FILE *fp = open_case_file(run, ".ic");
  if (!fp) { __real_m0_init_domain(run); return; }
  char kind[64];
  if (fscanf(fp, "%63s", kind) != 1) { fprintf(stderr, "harness: bad .ic\n"); exit(3); }
  double a[16] = {0};
  int na = 0;
  while (na < 16 && fscanf(fp, "%lf", &a[na]) == 1) na++;
  fclose(fp);
  for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) {
    double x[3] = {c->cl->xc, c->cl->yc, c->cl->zc};
    for (int iv = 0; iv < NEQ; iv++) c->el->S[iv] = 0.0;
    if (!strcmp(kind, "split")) {
      int ax = (int)a[0];
      const double *s = (x[ax] < a[1]) ? &a[2] : &a[7];
      m0_init_S(run, c, s[0], s[1], s[2], s[3], s[4]);
    } else if (!strcmp(kind, "sphere")) {
      double d2 = (x[0] - a[0]) * (x[0] - a[0]) + (x[1] - a[1]) * (x[1] - a[1]) +
                  (x[2] - a[2]) * (x[2] - a[2]);
      const double *s = (d2 < a[3] * a[3]) ? &a[4] : &a[9];
      m0_init_S(run, c, s[0], s[1], s[2], s[3], s[4]);
    } else if (!strcmp(kind, "wave")) {
      double ph = 2.0 * M_PI * (a[6] * x[0] + a[7] * x[1] + a[8] * x[2]);
      double s1 = sin(ph), c1 = cos(ph), s2 = sin(2.0 * ph + 0.3);
      m0_init_S(run, c, a[0] * (1.0 + a[5] * s1), a[1] + a[5] * c1, a[2] + a[5] * s2,
                a[3] - a[5] * s1 * c1, a[4] * (1.0 + a[5] * c1));
    } else {
      fprintf(stderr, "harness: unknown ic kind %s\n", kind);
      exit(3);
    }
  }
}

/* ------------------------------------------------------------------ refinement target */
/* <case>.rf:  sphere cx cy cz r level_inside level_outside
 *             box x0 y0 z0 x1 y1 z1 level_inside level_outside */
void __real_criterionsplt(struct RUN *run);
static int g_real_criterion = 0; /* set while the harness runs the reference's adaptation */
void __wrap_criterionsplt(struct RUN *run) {
  FILE *fp = g_real_criterion ? NULL : open_case_file(run, ".rf");
  if (!fp) { __real_criterionsplt(run); return; }
  char kind[64];
  double a[8] = {0};
  int na = 0;
  if (fscanf(fp, "%63s", kind) != 1) { fprintf(stderr, "harness: bad .rf\n"); exit(3); }
  while (na < 8 && fscanf(fp, "%lf", &a[na]) == 1) na++;
  fclose(fp);
  for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) {
    double x = c->cl->xc, y = c->cl->yc, z = c->cl->zc;
    int inside;
    int lin, lout;
    if (!strcmp(kind, "sphere")) {
      inside = (x - a[0]) * (x - a[0]) + (y - a[1]) * (y - a[1]) + (z - a[2]) * (z - a[2]) <
               a[3] * a[3];
      lin = (int)a[4]; lout = (int)a[5];
    } else {
      inside = x > a[0] && y > a[1] && z > a[2] && x < a[3] && y < a[4] && z < a[5];
      lin = (int)a[6]; lout = (int)a[7];
    }
    c->split = inside ? lin : lout;
  }
}

void __real_criterionsplt(struct RUN *run);

/* ------------------------------------------------------------------ dump */
static void put_i32(FILE *f, int32_t v) { fwrite(&v, 4, 1, f); }
static void put_f64(FILE *f, double v) { fwrite(&v, 8, 1, f); }

static void dump(struct RUN *run, const char *tag, double loop_seconds, int64_t steps) {
  char path[4096];
  snprintf(path, sizeof path, "%s.%s.bin", run->con->runname, tag);
  FILE *f = fopen(path, "wb");
  if (!f) { fprintf(stderr, "harness: cannot write %s\n", path); exit(3); }
  int32_t n = 0;
  for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) c->el->gnum = n++;
  fwrite("FFVD", 1, 4, f);
  put_i32(f, 1);           /* version */
  put_i32(f, MODEL);
  put_i32(f, NEQ);
  put_i32(f, n);
  put_f64(f, loop_seconds);
  fwrite(&steps, 8, 1, f);
  for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) {
    put_i32(f, c->root);
    put_i32(f, c->level);
    for (int l = 0; l < 16; l++) put_i32(f, l <= c->level ? c->adrs[l] : -1);
    put_f64(f, c->cl->xc); put_f64(f, c->cl->yc); put_f64(f, c->cl->zc);
    put_f64(f, c->cl->Vol);
    put_i32(f, c->el->SI[0]); put_i32(f, c->el->SI[1]);
    for (int fc = 0; fc < 6; fc++) {
      int nn = c->lfc_neigs[fc];
      put_i32(f, c->cl->fc[fc].bc);
      put_i32(f, nn);
      put_i32(f, c->nsfc[fc]);
      put_i32(f, c->neigfc[fc]);
      for (int k = 0; k < 4; k++) {
        int idx = -1;
        if (c->cl->fc[fc].bc == 0 && k < nn && c->neigtr[fc][k] && c->neigtr[fc][k]->root != -1)
          idx = c->neigtr[fc][k]->el->gnum;
        put_i32(f, idx);
      }
      for (int k = 0; k < 4; k++) put_f64(f, k < c->nsfc[fc] ? c->cl->Area[fc][k] : 0.0);
      put_f64(f, c->cl->nx[fc]);   put_f64(f, c->cl->ny[fc]);   put_f64(f, c->cl->nz[fc]);
      put_f64(f, c->cl->nxt1[fc]); put_f64(f, c->cl->nyt1[fc]); put_f64(f, c->cl->nzt1[fc]);
      put_f64(f, c->cl->nxt2[fc]); put_f64(f, c->cl->nyt2[fc]); put_f64(f, c->cl->nzt2[fc]);
      put_f64(f, c->cl->dist_cf[fc]);
      put_f64(f, c->cl->dist_cc[fc]);
    }
    for (int iv = 0; iv < NEQ; iv++) put_f64(f, c->el->S[iv]);
  }
  fclose(f);
}

/* <case>.tag: one line per tag pass, the refinement criteria in the input file's terms
 *   uniform lvl  prs lvl thr  rho lvl thr  vel lvl thr  inter0 lvl lrs  inter1 lvl lrs
 * They are set right before each pass (the mesh generation at start-up keeps the .ct
 * values), with the derived globals formed as inputset.c:106 and m5_input.c:50-57 form
 * them.  Every pass starts from the same final state (interface_location and
 * criterionsplt recompute SI and split for every leaf).  Output <run>.tags.bin: "FFVT",
 * npass, n, then per pass and leaf SI[0], SI[1], the split level criterionsplt gives and
 * the split level after criterionsmth. */
/* set the reference's criterion globals from one .tag/.adapt line (values as the input
 * file gives them), deriving the rest as inputset.c:106 and m5_input.c:50-57 do */
static int set_criteria(FILE *fp) {
  int u, lu, pr, lp, rh, lr, ve, lv, i0, l0, r0, i1, l1, r1;
  double tp, tr, tv;
  if (fscanf(fp, "%d %d %d %d %lf %d %d %lf %d %d %lf %d %d %d %d %d %d", &u, &lu, &pr, &lp, &tp,
             &rh, &lr, &tr, &ve, &lv, &tv, &i0, &l0, &r0, &i1, &l1, &r1) != 17)
    return 0;
  CRT_UNIFORM = u; CRT_LVL_UNIFORM = lu;
  CRT_GEO_AREA = 0; CRT_LVL_GEO_AREA = 0;
  CRT_GRAD_PRS = pr; CRT_LVL_GRAD_PRS = lp; CRT_GRAD_PRS_THR = tp;
  CRT_GRAD_RHO = rh; CRT_LVL_GRAD_RHO = lr; CRT_GRAD_RHO_THR = tr;
  CRT_GRAD_VEL = ve; CRT_LVL_GRAD_VEL = lv; CRT_GRAD_VEL_THR = tv;
  CRT_ADAPT_INTER_0 = i0; CRT_LVL_ADAPT_INTER_0 = l0; CRT_LRS_ADAPT_INTER_0 = r0;
  CRT_ADAPT_INTER_1 = i1; CRT_LVL_ADAPT_INTER_1 = l1; CRT_LRS_ADAPT_INTER_1 = r0 + r1;
  ADAPT_INTER_MAX = 0;
  if (i0 == 1 && i1 == 1) ADAPT_INTER_MAX = CRT_LRS_ADAPT_INTER_0 + CRT_LRS_ADAPT_INTER_1;
  if (i0 == 1 && i1 == 0) ADAPT_INTER_MAX = CRT_LRS_ADAPT_INTER_0;
  LEVEL = max(max(max(max(lu, 0), lp), lr), lv);
  LEVEL = max(max(LEVEL, l0), l1);
  return 1;
}

/* <case>.adapt: one criterion line; after the loop (and the tag passes) the reference's own
 * meshadaptation (meshadaptation.c:3-46: LEVEL+1 passes of criterionsplt, criterionsmth,
 * refineh, restructtopo, meshproperties, interface_location) runs on the final state and
 * the adapted leaf list is dumped as <run>.adapt.bin */
static void adapt_pass(struct RUN *run) {
  FILE *fp = open_case_file(run, ".adapt");
  if (!fp) return;
  int ok = set_criteria(fp);
  fclose(fp);
  if (!ok) { fprintf(stderr, "harness: bad .adapt\n"); exit(3); }
  for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) c->el->SI[0] = c->el->SI[1] = 0;
  if (CRT_ADAPT_INTER_0 != 0) interface_location(run);
  g_real_criterion = 1;
  meshadaptation(run);
  g_real_criterion = 0;
  dump(run, "adapt", 0.0, 0);
}

static void tag_pass(struct RUN *run) {
  FILE *fp = open_case_file(run, ".tag");
  if (!fp) return;
  int32_t n = 0;
  for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) n++;
  int32_t *out = NULL, npass = 0;
  int u, lu, pr, lp, rh, lr, ve, lv, i0, l0, r0, i1, l1, r1;
  double tp, tr, tv;
  while (fscanf(fp, "%d %d %d %d %lf %d %d %lf %d %d %lf %d %d %d %d %d %d", &u, &lu, &pr, &lp,
                &tp, &rh, &lr, &tr, &ve, &lv, &tv, &i0, &l0, &r0, &i1, &l1, &r1) == 17) {
    CRT_UNIFORM = u; CRT_LVL_UNIFORM = lu;
    CRT_GEO_AREA = 0; CRT_LVL_GEO_AREA = 0;
    CRT_GRAD_PRS = pr; CRT_LVL_GRAD_PRS = lp; CRT_GRAD_PRS_THR = tp;
    CRT_GRAD_RHO = rh; CRT_LVL_GRAD_RHO = lr; CRT_GRAD_RHO_THR = tr;
    CRT_GRAD_VEL = ve; CRT_LVL_GRAD_VEL = lv; CRT_GRAD_VEL_THR = tv;
    CRT_ADAPT_INTER_0 = i0; CRT_LVL_ADAPT_INTER_0 = l0; CRT_LRS_ADAPT_INTER_0 = r0;
    CRT_ADAPT_INTER_1 = i1; CRT_LVL_ADAPT_INTER_1 = l1; CRT_LRS_ADAPT_INTER_1 = r0 + r1;
    ADAPT_INTER_MAX = 0;
    if (i0 == 1 && i1 == 1) ADAPT_INTER_MAX = CRT_LRS_ADAPT_INTER_0 + CRT_LRS_ADAPT_INTER_1;
    if (i0 == 1 && i1 == 0) ADAPT_INTER_MAX = CRT_LRS_ADAPT_INTER_0;
    LEVEL = max(max(max(max(lu, 0), lp), lr), lv);
    LEVEL = max(max(LEVEL, l0), l1);
    for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) c->el->SI[0] = c->el->SI[1] = 0;
    if (CRT_ADAPT_INTER_0 != 0) interface_location(run);
    __real_criterionsplt(run);
    out = realloc(out, sizeof(int32_t) * 4 * (size_t)n * (size_t)(npass + 1));
    int32_t *o = out + (size_t)4 * n * npass, i = 0;
    for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt, i++) {
      o[4 * i + 0] = c->el->SI[0];
      o[4 * i + 1] = c->el->SI[1];
      o[4 * i + 2] = c->split;
    }
    criterionsmth(run);
    i = 0;
    for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt, i++) o[4 * i + 3] = c->split;
    npass++;
  }
  fclose(fp);
  char path[4096];
  snprintf(path, sizeof path, "%s.tags.bin", run->con->runname);
  FILE *f = fopen(path, "wb");
  if (!f) { fprintf(stderr, "harness: cannot write %s\n", path); exit(3); }
  fwrite("FFVT", 1, 4, f);
  put_i32(f, npass);
  put_i32(f, n);
  if (npass) fwrite(out, sizeof(int32_t), (size_t)4 * n * npass, f);
  fclose(f);
  free(out);
}

void __real_loop(struct RUN *run);
void __wrap_loop(struct RUN *run) {
  dump(run, "init", 0.0, 0);
  double t0 = MPI_Wtime();
  __real_loop(run);
  double t1 = MPI_Wtime();
  dump(run, "final", t1 - t0, (int64_t)NSTEP + 1);
  /* <case>.restart present: the reference's own restart file of the final state
   * (restart_save.c, restart%08d.dat in the working directory) */
  FILE *rf = open_case_file(run, ".restart");
  if (rf) {
    fclose(rf);
    restart_save(run);
  }
  tag_pass(run);
  adapt_pass(run);
}

/* m5_init_domain.c does not compile as published; this replacement assigns each leaf one
 * material by geometric regions read from <case>.ic and fills its state with the
 * reference's own m5_init_S (init_S.c:205-266):
 *   m5 default_mat nregions  then per region one of
 *      sphere cx cy cz r mat       |   below axis x0 mat   |   above axis x0 mat
 * The first region that contains the leaf centroid wins. */
void m5_init_S(struct RUN *run, struct BRANCH *crnt, int mat);
void m5_init_domain(struct RUN *run) {
  FILE *fp = open_case_file(run, ".ic");
  if (!fp) { fprintf(stderr, "harness: model 5 needs <case>.ic\n"); exit(3); }
  char kind[64];
  int defmat = 0, nreg = 0;
  if (fscanf(fp, "%63s %d %d", kind, &defmat, &nreg) != 3 || strcmp(kind, "m5")) {
    fprintf(stderr, "harness: bad model-5 .ic\n"); exit(3);
  }
  char rk[16][16];
  double ra[16][6];
  int rm[16];
  for (int i = 0; i < nreg && i < 16; i++) {
    if (fscanf(fp, "%15s", rk[i]) != 1) exit(3);
    int np = !strcmp(rk[i], "sphere") ? 4 : 2;
    for (int j = 0; j < np; j++) if (fscanf(fp, "%lf", &ra[i][j]) != 1) exit(3);
    if (fscanf(fp, "%d", &rm[i]) != 1) exit(3);
  }
  fclose(fp);
  for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) {
    double x[3] = {c->cl->xc, c->cl->yc, c->cl->zc};
    int mat = defmat;
    for (int i = 0; i < nreg; i++) {
      int in;
      if (!strcmp(rk[i], "sphere")) {
        double d2 = (x[0] - ra[i][0]) * (x[0] - ra[i][0]) + (x[1] - ra[i][1]) * (x[1] - ra[i][1]) +
                    (x[2] - ra[i][2]) * (x[2] - ra[i][2]);
        in = d2 < ra[i][3] * ra[i][3];
      } else if (!strcmp(rk[i], "below")) {
        in = x[(int)ra[i][0]] < ra[i][1];
      } else {
        in = x[(int)ra[i][0]] > ra[i][1];
      }
      if (in) { mat = rm[i]; break; }
    }
    for (int iv = 0; iv < NEQ; iv++) c->el->S[iv] = 0.0;
    m5_init_S(run, c, mat);
  }
  /* optional <case>.mix: axis lo hi mat_a alpha_a mat_b p u v w -- cells whose centroid
   * lies in [lo, hi) along axis hold a two-material mixture at pressure p, velocity
   * (u,v,w), the remaining materials at AMIN, deformation A = I (so no elastic energy) */
  fp = open_case_file(run, ".mix");
  if (!fp) return;
  double mx[10];
  int nm = 0;
  while (nm < 10 && fscanf(fp, "%lf", &mx[nm]) == 1) nm++;
  fclose(fp);
  if (nm != 10) { fprintf(stderr, "harness: bad .mix\n"); exit(3); }
  int ax = (int)mx[0], ma = (int)mx[3], mb = (int)mx[5];
  for (struct BRANCH *c = run->topo->locl; c; c = c->lnxt) {
    double x[3] = {c->cl->xc, c->cl->yc, c->cl->zc};
    if (!(x[ax] >= mx[1] && x[ax] < mx[2])) continue;
    double a[10], rho = 0.0, E = 0.0;
    for (int k = 0; k < NMATERIALS; k++) a[k] = AMIN;
    a[ma] = mx[4];
    a[mb] = 1.0 - mx[4] - (double)(NMATERIALS - 2) * AMIN;
    for (int k = 0; k < NMATERIALS; k++) {
      double ar = a[k] * MATERRINI[k];
      double are = a[k] * (mx[6] + MATERGAMA[k] * MATERPINF[k]) / (MATERGAMA[k] - 1.0);
      c->el->S[eqtypi[0] + k] = ar;
      c->el->S[eqtypi[4] + k] = are;
      rho += ar;
      E += are;
    }
    for (int k = 0; k < NMATERIALS - 1; k++) c->el->S[eqtypi[3] + k] = a[k];
    c->el->S[eqtypi[1] + 0] = rho * mx[7];
    c->el->S[eqtypi[1] + 1] = rho * mx[8];
    c->el->S[eqtypi[1] + 2] = rho * mx[9];
    c->el->S[eqtypi[2]] = E + 0.5 * rho * (mx[7] * mx[7] + mx[8] * mx[8] + mx[9] * mx[9]);
    for (int q = 0; q < 9; q++) c->el->S[eqtypi[5] + q] = (q % 4 == 0) ? 1.0 : 0.0;
  }
}
