// Device-side definitions shared by the kernels and the launch layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ffv_internal.h"

// bits of the device status word (OR-ed by kernels, read by the host after a step)
#define FFV_ST_NAN 1u         // non-finite residual (m0_residual.c:127-135)
#define FFV_ST_NO_BRANCH 2u   // no HLLC branch taken (m0_hllc.c:48-51)
#define FFV_ST_NAN_SPEED 4u   // NaN contact speed (m0_wave_speeds.c:124-133)
#define FFV_ST_NEG_DENSITY 8u

// Face frames of the Cartesian forest (n, t1, t2 of face f as axis and sign).  These are
// the values the reference's normalvector.c / tagvector.c give for the hex node layout
// of ffv_internal.h; the mesh builder recomputes them from the reference's formulas and
// refuses a mesh whose frames differ (ffv_check_frames).
__host__ __device__ constexpr int fr_n_axis(int f) { return f == 0 ? 0 : f == 1 ? 1 : f == 2 ? 0 : f == 3 ? 1 : 2; }
__host__ __device__ constexpr int fr_n_sign(int f) { return (f == 0 || f == 3 || f == 4) ? 1 : -1; }
__host__ __device__ constexpr int fr_t1_axis(int f) { return f == 0 ? 1 : f == 1 ? 2 : f == 2 ? 2 : f == 3 ? 0 : f == 4 ? 1 : 0; }
__host__ __device__ constexpr int fr_t1_sign(int f) { return (f == 3 || f == 5) ? -1 : 1; }
__host__ __device__ constexpr int fr_t2_axis(int f) { return f == 0 ? 2 : f == 1 ? 0 : f == 2 ? 1 : f == 3 ? 2 : f == 4 ? 0 : 1; }
__host__ __device__ constexpr int fr_t2_sign(int f) { return (f == 1 || f == 4) ? -1 : 1; }
__host__ __device__ constexpr int fr_opp(int f) { return f == 0 ? 2 : f == 1 ? 3 : f == 2 ? 0 : f == 3 ? 1 : f == 4 ? 5 : 4; }

// Per-level geometry, passed by value to the kernels (lands in the constant bank).
struct ffv_geom {
  double vol[FFV_MAX_LEVEL + 2];
  double inv_vol[FFV_MAX_LEVEL + 2];   // 1.0 / vol, as RK.c:25 evaluates it
  double area[FFV_MAX_LEVEL + 2];
  double h[FFV_MAX_LEVEL + 2];
  double dcf[FFV_MAX_LEVEL + 2][4];    // by face class: same, coarser, finer, boundary
  double dcc[FFV_MAX_LEVEL + 2][4];
  // FP32 forms for the FP32-flux reconstruction: dcf and 1 / dcc (inf at a boundary)
  float dcf_f[FFV_MAX_LEVEL + 2][4];
  float idcc_f[FFV_MAX_LEVEL + 2][4];
  // FP32 face areas of the FP32-flux form: a level's own, and 4 x the next finer level's
  // (the four sub-faces of a face towards finer neighbours)
  float area_f[FFV_MAX_LEVEL + 2];
  float area4_fine_f[FFV_MAX_LEVEL + 2];
};

__device__ __forceinline__ int face_class(uint32_t kind) { return (kind & FFV_FK_BC) ? 3 : (int)kind; }

// device-side views of the mesh tables
struct ffv_dmesh {
  int64_t n;
  const uint32_t *__restrict__ info;  // [n]
  const int32_t *__restrict__ nbr;    // [6][n] (face-major)
  const int32_t *__restrict__ sub;    // [4 nsub]
};

// host-side helpers implemented in ffv_api.cu
int ffv_check_frames(const ffv_mesh *m);
void ffv_fill_geom(const ffv_mesh *m, ffv_geom *g);

// model-0 FP64 launchers (ffv_m0_fp64.cu)
struct ffv_m0_bufs {
  double *S, *SN, *SF, *dt;  // S, SN: [5][n]; SF: [6][5][n]; dt: device scalar
  unsigned int *status;
};
struct ffv_m0_consts {
  double gamma, pinf;
  int order;
};
// ev (nullable): events recorded before the first and after every kernel of the stage
void ffv_m0_fp64_stage(const ffv_dmesh &m, const ffv_geom &g, const ffv_m0_bufs &b,
                       const ffv_m0_consts &k, int irk, cudaStream_t st, cudaEvent_t *ev);
const char *ffv_m0_fp64_kernel_name(int order, int i);
int ffv_m0_launches_per_stage(int order);
void ffv_m0_cfl(const ffv_dmesh &m, const ffv_geom &g, const double *S,
                const ffv_m0_consts &k, unsigned long long *d_out, cudaStream_t st);
