// Model-5 launch interface (ffv_m5_fp64.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ffv_device.cuh"
#include "ffv_df.cuh"

struct M5Consts {
  int nmat, order, prelax, nsolids;
  int precision;  // FFV_FP64 or FFV_FP32_FLUX
  int flux_form;  // FFV_FLUX_REFERENCE or FFV_FLUX_CONSISTENT
  int zerou[3];
  double gamma[FFV_MAX_MATERIALS], pinf[FFV_MAX_MATERIALS], mu[FFV_MAX_MATERIALS];
  double amin, avf_lim;
  double yield[FFV_MAX_MATERIALS];  // von Mises yield stress per material, 0 = none
  int plastic;                      // a solid material has a yield stress
  // per material, for the FP32-flux form: gamma p_inf, 1 / (gamma - 1),
  // gamma p_inf / (gamma - 1), 1 / gamma
  double gpi[FFV_MAX_MATERIALS], ig1[FFV_MAX_MATERIALS], gpg[FFV_MAX_MATERIALS],
      igam[FFV_MAX_MATERIALS];
  // the same in FP32: p_inf, 1 / gamma, mu, gamma, the relaxation's pressure floor and reset
  // value, AMIN / 100 and 1 - AMIN / 100
  float pinf_f[FFV_MAX_MATERIALS], igam_f[FFV_MAX_MATERIALS], mu_f[FFV_MAX_MATERIALS],
      gamma_f[FFV_MAX_MATERIALS], plo_f[FFV_MAX_MATERIALS], preset_f[FFV_MAX_MATERIALS];
  float alo_f, ahi_f;
  // AVF_LIM in FP32, and whether phi0 takes the larger of two solid fractions (two solids,
  // the first one elastic): the FP32-flux form's phi0 needs no FP64 instruction
  float avf_lim_f;
  int phi_pair;
  // (a - j) / (j + 1), j = 1..6, a = -1 / gamma: the FP32 Newton iteration's binomial series
  float bin_f[FFV_MAX_MATERIALS][6];
  // double-float pairs for the FP32-flux form's pressure recovery: gamma - 1, gamma p_inf,
  // 1 / (gamma - 1), gamma p_inf / (gamma - 1), p_inf, the relaxation's pressure floor; and
  // AMIN / 100, 1 - AMIN / 100, 1 - 2 AMIN / 100, 1e-12, 1 - 1e-12
  df gm1_d[FFV_MAX_MATERIALS], gpi_d[FFV_MAX_MATERIALS], ig1_d[FFV_MAX_MATERIALS],
      gpg_d[FFV_MAX_MATERIALS], pinf_d[FFV_MAX_MATERIALS], floor_d[FFV_MAX_MATERIALS];
  df alo_d, ahi_d, a2lo_d, eps_d, oneeps_d;
};

struct ffv_m5_bufs {
  double *S, *SN, *Snew, *SF, *FF, *UF, *GF, *RHS, *dt;
  uint8_t *flag;
  int32_t *list, *bcount, *count;
  unsigned int *status;
};

int ffv_m5_neq(int nmat);
// ev (nullable): an event before the first and after every kernel; names[i] receives
// kernel i's name
void ffv_m5_fp64_stage(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k,
                       const ffv_m5_bufs &b, int irk, cudaStream_t st, cudaEvent_t *ev,
                       const char **names);
int ffv_m5_launches_per_stage(const M5Consts &k, int irk);

// FP32-flux form (ffv_m5_fp32.cu): face states and face fluxes in FP32.
//   Sf:  [neq][n] float copy of the state, made by ffv_m5f_shadow (scratch)
//   SFf: [6][neq + nmat + 1][n] float -- the reconstructed, relaxed face state followed by
//        each material's pressure, recovered in FP64, and the last volume fraction
//   FFf: [6][neq][n] float face fluxes (area-weighted), UFf: [6][3][n] float face velocity
void ffv_m5f_shadow(int64_t n, const M5Consts &k, const double *S, float *Sf, cudaStream_t st);
void ffv_m5f_recon(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                   const float *Sf, float *SFf, unsigned *status, cudaStream_t st);
// Sf: the FP32 copy of the state (order 2), or nullptr (order 1: phi0 from S)
void ffv_m5f_flux(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                  const float *Sf, const float *SFf, float *FFf, float *UFf, double *GF,
                  unsigned *status, cudaStream_t st);
// residual + RK stage of the FP32-flux form (the face fluxes of all but the deformation
// summed in FP64)
void ffv_m5f_cell_update(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                         double *SN, const float *FFf, const float *UFf, double *RHS,
                         double *Snew, uint8_t *flag, const double *dt, int irk, unsigned *status,
                         cudaStream_t st);
// the indicator's fields of a model-5 state, F [5][n] float (log rho, log p, alpha_0, |u|,
// von Mises stress; FP32 with double-float pressure recovery; ffv_mlp.cu gathers them)
void ffv_m5f_indicator_fields(int64_t n, const M5Consts &k, const double *S, float *F,
                              cudaStream_t st);
// cell pressure relaxation: the Newton iteration in FP32, the pressure recovery and the
// energy-consistent pressure and internal energies in double-float
void ffv_m5f_relax_cell(int64_t n, const M5Consts &k, const double *Sin, double *Sout,
                        uint8_t *flag, unsigned *status, cudaStream_t st);
void ffv_m5_cfl(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                unsigned long long *d_out, cudaStream_t st);

// refinement criteria (criterionsplt.c, interface_location.c) with the derived values the
// reference forms from its input (m5_input.c:50-57): lrs1 = lrs0 + lrs1 as given,
// si_max = ADAPT_INTER_MAX
struct ffv_m5_tagc {
  int uniform, lvl_uniform, prs, lvl_prs, rho, lvl_rho, vel, lvl_vel;
  int inter0, lvl0, lrs0, inter1, lvl1, lrs1, si_max;
  double thr_prs, thr_rho, thr_vel;
};
// SI [2][n] (interface layers), SItmp scratch of the same size, split [n]
// pr: scratch [2][n] doubles (each cell's mixture pressure and density, made once)
void ffv_m5_tags(const ffv_dmesh &m, const M5Consts &k, const ffv_m5_tagc &t, const double *S,
                 int32_t *SI, int32_t *SItmp, int32_t *split, double *pr, cudaStream_t st);

// exported per-leaf fields, F [nf][n] double (ffv_export_fields)
void ffv_m5_export_fields(int64_t n, const M5Consts &k, const double *S, double *F,
                          cudaStream_t st);
void ffv_m0_export_fields(int64_t n, double gamma, double pinf, const double *S, double *F,
                          cudaStream_t st);

// model 0 (ffv_m0_tags.cu): the relative-jump criterion on cell states and the indicator
// fields (log rho, log p, 1, |u|, 0)
void ffv_m0_tags(const ffv_dmesh &m, double gamma, double pinf, const ffv_m5_tagc &t,
                 const double *S, int32_t *split, cudaStream_t st);
void ffv_m0_indicator_fields(int64_t n, double gamma, double pinf, const double *S, float *F,
                             cudaStream_t st);

// the reference's FP64 relaxation of the cells a mesh adaptation merged (map < 0)
void ffv_m5_relax_merged(int64_t n, const M5Consts &k, const int64_t *map, double *S,
                         cudaStream_t st);
