// Model-5 launch interface (ffv_m5_fp64.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ffv_device.cuh"

struct M5Consts {
  int nmat, order, prelax, nsolids;
  int zerou[3];
  double gamma[FFV_MAX_MATERIALS], pinf[FFV_MAX_MATERIALS], mu[FFV_MAX_MATERIALS];
  double amin, avf_lim;
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
void ffv_m5_cfl(const ffv_dmesh &m, const ffv_geom &g, const M5Consts &k, const double *S,
                unsigned long long *d_out, cudaStream_t st);
