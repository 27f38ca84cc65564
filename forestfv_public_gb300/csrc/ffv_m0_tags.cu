// Model-0 refinement criterion and indicator fields (an extension: the reference's
// gradient criterion has no model-0 branch -- criterion_grad, criterionsplt.c:64-70, calls
// the model's face-value routine only for models 1-5 and otherwise reads whatever face
// values a previous routine left).  Here it takes the same relative jumps
// (criterionsplt.c:74-110) of the cell states of a cell and each of its face neighbours,
// with the pressure of the stiffened-gas law as m0_facercnstr.c:29 forms it.
#include <math.h>

#include "ffv_device.cuh"
#include "ffv_m5.cuh"

namespace {

__device__ __forceinline__ void m0_prim(const double *__restrict__ S, int64_t n, int64_t c,
                                        double gamma, double pinf, double &r, double &p,
                                        double &umag) {
  r = S[c];
  const double u = S[n + c] / r, v = S[2 * n + c] / r, w = S[3 * n + c] / r;
  const double e_int = S[4 * n + c] / r - 0.5 * (u * u + v * v + w * w);
  p = r * (gamma - 1.0) * e_int - gamma * pinf;
  umag = sqrt(u * u + v * v + w * w);
}

__device__ __forceinline__ double jump(double x_cur, double x_nb) {
  const double eps = 1.0e-8;
  if ((fabs(x_nb) > eps) || (fabs(x_cur) > eps)) {
    const double a = fabs(x_nb), b = fabs(x_cur);
    return fabs(x_nb - x_cur) / ((a > b) ? a : b);
  }
  return 0.0;
}

__global__ void __launch_bounds__(128) m0_tag_split(ffv_dmesh m, double gamma, double pinf,
                                                    ffv_m5_tagc t, const double *__restrict__ S,
                                                    int32_t *__restrict__ split) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.n) return;
  int level = 1;
  if (t.uniform == 1) level = level > t.lvl_uniform ? level : t.lvl_uniform;
  if (t.prs == 1 || t.rho == 1 || t.vel == 1) {
    const uint32_t info = m.info[c];
    double rL, pL, uL;
    m0_prim(S, m.n, c, gamma, pinf, rL, pL, uL);
    double gp = 0.0, gr = 0.0, gv = 0.0;
    for (int f = 0; f < 6; f++) {
      const uint32_t kind = ffv_face_kind(info, f);
      if (kind & FFV_FK_BC) continue;
      const int32_t s = m.nbr[(int64_t)f * m.n + c];
      const int cnt = kind == FFV_FK_FINER ? 4 : 1;
      for (int q = 0; q < cnt; q++) {
        const int64_t o = kind == FFV_FK_FINER ? m.sub[4 * (int64_t)s + q] : s;
        double rR, pR, uR;
        m0_prim(S, m.n, o, gamma, pinf, rR, pR, uR);
        const double a = jump(pL, pR), b = jump(rL, rR);
        gp = (a > gp) ? a : gp;
        gr = (b > gr) ? b : gr;
        gv = (b > gv) ? b : gv;  // the density jump, as the reference's velocity criterion
      }
    }
    int lt = 1;
    if (t.prs == 1 && fabs(gp) >= t.thr_prs) lt = t.lvl_prs;
    if (t.rho == 1 && fabs(gr) >= t.thr_rho) lt = t.lvl_rho;
    if (t.vel == 1 && fabs(gv) >= t.thr_vel) lt = t.lvl_vel;
    level = level > lt ? level : lt;
  }
  split[c] = level;
}

__global__ void __launch_bounds__(128) m0_indicator_fields(int64_t n, double gamma, double pinf,
                                                           const double *__restrict__ S,
                                                           float *__restrict__ F) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double r, p, um;
  m0_prim(S, n, c, gamma, pinf, r, p, um);
  F[c] = (float)log(r > 1e-300 ? r : 1e-300);
  F[n + c] = (float)log(p > 1e-30 ? p : 1e-30);
  F[2 * n + c] = 1.0f;
  F[3 * n + c] = (float)um;
  F[4 * n + c] = 0.0f;
}

__global__ void __launch_bounds__(128) m0_export_fields(int64_t n, double gamma, double pinf,
                                                        const double *__restrict__ S,
                                                        double *__restrict__ F) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double r, p, um;
  m0_prim(S, n, c, gamma, pinf, r, p, um);
  F[c] = r;
  F[n + c] = -S[n + c] / r;  // the state holds the negated momentum in this node layout
  F[2 * n + c] = -S[2 * n + c] / r;
  F[3 * n + c] = -S[3 * n + c] / r;
  F[4 * n + c] = p;
}

}  // namespace

void ffv_m0_export_fields(int64_t n, double gamma, double pinf, const double *S, double *F,
                          cudaStream_t st) {
  m0_export_fields<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, gamma, pinf, S, F);
}

void ffv_m0_tags(const ffv_dmesh &m, double gamma, double pinf, const ffv_m5_tagc &t,
                 const double *S, int32_t *split, cudaStream_t st) {
  m0_tag_split<<<(unsigned)((m.n + 127) / 128), 128, 0, st>>>(m, gamma, pinf, t, S, split);
}

void ffv_m0_indicator_fields(int64_t n, double gamma, double pinf, const double *S, float *F,
                             cudaStream_t st) {
  m0_indicator_fields<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, gamma, pinf, S, F);
}
