// C ABI implementation: device context, table upload, state transfer, stage / step
// launches (one CUDA graph per time step), CFL reduction, device status word.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <new>

#include "ffv_device.cuh"
#include "ffv_m5.cuh"

struct ffv_ctx {
  ffv_params p;
  int device;
  cudaStream_t stream;
  int64_t n;
  int32_t neq;
  int have_mesh, have_state;
  ffv_dmesh dm;
  ffv_geom geom;
  // device buffers
  uint32_t *d_info;
  int32_t *d_nbr, *d_sub;
  double *d_S, *d_SN, *d_SF, *d_dt;
  // model 5 only
  double *d_Snew, *d_FF, *d_UF, *d_GF, *d_RHS;
  uint8_t *d_flag;
  int32_t *d_list, *d_bcount, *d_count;
  M5Consts m5;
  // refinement tags
  int32_t *d_SI, *d_SItmp, *d_split;
  double *d_tagpr;  // per-cell mixture pressure and density for the criterion [2][n]
  // cells and subface groups the mesh buffers are allocated for (a new mesh that fits reuses
  // them: a regrid then allocates nothing)
  int64_t cap, cap_nsub;
  unsigned int *d_status;
  unsigned long long *d_red;
  // pinned host scalars
  unsigned int *h_status;
  unsigned long long *h_red;
  const char *knames[16];  // kernel names of the last profiled stage
  // one captured time step
  cudaGraphExec_t graph;
  int graph_valid;
};

namespace {

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? FFV_OK : FFV_ERR_CUDA; }

#define CK(x)                                  \
  do {                                         \
    cudaError_t e_ = (x);                      \
    if (e_ != cudaSuccess) return FFV_ERR_CUDA; \
  } while (0)

void free_mesh_buffers(ffv_ctx *c) {
  cudaFree(c->d_info);
  cudaFree(c->d_nbr);
  cudaFree(c->d_sub);
  cudaFree(c->d_S);
  cudaFree(c->d_SN);
  cudaFree(c->d_SF);
  cudaFree(c->d_Snew);
  cudaFree(c->d_FF);
  cudaFree(c->d_UF);
  cudaFree(c->d_GF);
  cudaFree(c->d_RHS);
  cudaFree(c->d_flag);
  cudaFree(c->d_list);
  cudaFree(c->d_bcount);
  cudaFree(c->d_count);
  cudaFree(c->d_SI);
  cudaFree(c->d_SItmp);
  cudaFree(c->d_split);
  cudaFree(c->d_tagpr);
  c->d_SI = c->d_SItmp = c->d_split = nullptr;
  c->d_tagpr = nullptr;
  c->d_info = nullptr;
  c->d_nbr = c->d_sub = nullptr;
  c->d_S = c->d_SN = c->d_SF = nullptr;
  c->d_Snew = c->d_FF = c->d_UF = c->d_GF = c->d_RHS = nullptr;
  c->d_flag = nullptr;
  c->d_list = c->d_bcount = c->d_count = nullptr;
  c->cap = c->cap_nsub = 0;
  if (c->graph_valid) cudaGraphExecDestroy(c->graph);
  c->graph_valid = 0;
  c->have_mesh = c->have_state = 0;
}

// the mesh buffers for c->cap cells and c->cap_nsub subface groups
int alloc_mesh_buffers(ffv_ctx *c) {
  const int64_t n = c->cap;
  const size_t nsub = (size_t)c->cap_nsub;
  if (cudaMalloc(&c->d_info, sizeof(uint32_t) * n) != cudaSuccess ||
      cudaMalloc(&c->d_nbr, sizeof(int32_t) * 6 * n) != cudaSuccess ||
      cudaMalloc(&c->d_sub, sizeof(int32_t) * 4 * nsub) != cudaSuccess ||
      cudaMalloc(&c->d_S, sizeof(double) * c->neq * n) != cudaSuccess ||
      cudaMalloc(&c->d_SN, sizeof(double) * c->neq * n) != cudaSuccess ||
      cudaMalloc(&c->d_SF, sizeof(double) * 6 * c->neq * n) != cudaSuccess) {
    free_mesh_buffers(c);
    return FFV_ERR_NOMEM;
  }
  if (c->p.model == 5) {
    const int64_t nb = (n + 1023) / 1024;
    if (cudaMalloc(&c->d_Snew, sizeof(double) * c->neq * n) != cudaSuccess ||
        cudaMalloc(&c->d_FF, sizeof(double) * 6 * c->neq * n) != cudaSuccess ||
        cudaMalloc(&c->d_UF, sizeof(double) * 18 * n) != cudaSuccess ||
        cudaMalloc(&c->d_GF, sizeof(double) * 6 * n) != cudaSuccess ||
        cudaMalloc(&c->d_RHS, sizeof(double) * c->neq * n) != cudaSuccess ||
        cudaMalloc(&c->d_flag, n) != cudaSuccess ||
        cudaMalloc(&c->d_list, sizeof(int32_t) * n) != cudaSuccess ||
        cudaMalloc(&c->d_bcount, sizeof(int32_t) * nb) != cudaSuccess ||
        cudaMalloc(&c->d_count, sizeof(int32_t)) != cudaSuccess) {
      free_mesh_buffers(c);
      return FFV_ERR_NOMEM;
    }
  }
  return FFV_OK;
}

// a non-positive density is reported before the NaN it leads to (a negative density gives a
// NaN sound speed within the same stage)
unsigned status_to_err(unsigned st) {
  if (st & FFV_ST_NEG_DENSITY) return FFV_ERR_NEG_DENSITY;
  if (st & (FFV_ST_NAN | FFV_ST_NAN_SPEED | FFV_ST_NO_BRANCH)) return FFV_ERR_NAN;
  return FFV_OK;
}

int neq_of(const ffv_params &p) { return p.model == 0 ? 5 : ffv_m5_neq(p.nmaterials); }

int launch_stage(ffv_ctx *c, int irk, cudaEvent_t *ev = nullptr) {
  ffv_m0_bufs b{c->d_S, c->d_SN, c->d_SF, c->d_dt, c->d_status};
  ffv_m0_consts k{c->p.gamma[0], c->p.pinf[0], c->p.order};
  if (irk == 0) {
    CK(cudaMemcpyAsync(c->d_SN, c->d_S, sizeof(double) * c->neq * c->n, cudaMemcpyDeviceToDevice,
                       c->stream));
    return FFV_OK;
  }
  if (c->p.model == 5) {
    ffv_m5_bufs mb{c->d_S,   c->d_SN,   c->d_Snew, c->d_SF,     c->d_FF,    c->d_UF,
                   c->d_GF,  c->d_RHS,  c->d_dt,   c->d_flag,   c->d_list,  c->d_bcount,
                   c->d_count, c->d_status};
    ffv_m5_fp64_stage(c->dm, c->geom, c->m5, mb, irk, c->stream, ev, c->knames);
    return cuda_rc(cudaGetLastError());
  }
  ffv_m0_fp64_stage(c->dm, c->geom, b, k, irk, c->stream, ev);
  return cuda_rc(cudaGetLastError());
}

__global__ void set_scalar(double *dst, double v) { *dst = v; }

int queue_dt(ffv_ctx *c, double dt) {
  set_scalar<<<1, 1, 0, c->stream>>>(c->d_dt, dt);
  return cuda_rc(cudaGetLastError());
}

int build_graph(ffv_ctx *c) {
  if (c->graph_valid) return FFV_OK;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int rc = FFV_OK;
  for (int irk = 1; irk <= c->p.rk_steps && rc == FFV_OK; irk++) rc = launch_stage(c, irk);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (rc != FFV_OK) return rc;
  CK(e);
  e = cudaGraphInstantiate(&c->graph, g, 0);
  cudaGraphDestroy(g);
  CK(e);
  c->graph_valid = 1;
  return FFV_OK;
}

// CFL: dt = cfl * min over cells of h / max_a(|u_a| + c)  (no reference counterpart:
// the reference runs with a fixed DT, inputset.c:69)
__global__ void m0_cfl_kernel(ffv_dmesh m, ffv_geom g, const double *__restrict__ S,
                              double gamma, double pinf, unsigned long long *out) {
  double best = INFINITY;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < m.n;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int l = ffv_info_level(m.info[c]);
    const double r = S[c], u = S[m.n + c] / r, v = S[2 * m.n + c] / r, w = S[3 * m.n + c] / r;
    const double e = S[4 * m.n + c];
    const double p = r * (gamma - 1.0) * ((e / r) - 0.5 * (u * u + v * v + w * w)) - gamma * pinf;
    const double a = sqrt(gamma * (p + pinf) / r);
    const double s = fmax(fmax(fabs(u), fabs(v)), fabs(w)) + a;
    const double dt = g.h[l] / s;
    best = (dt < best || isnan(dt)) ? dt : best;
  }
  for (int o = 16; o > 0; o >>= 1) {
    double other = __shfl_xor_sync(0xffffffffu, best, o);
    best = (other < best || isnan(other)) ? other : best;
  }
  if ((threadIdx.x & 31) == 0) {
    // non-negative doubles order like their bit patterns; NaN maps above +inf
    unsigned long long bits = isnan(best) ? 0x7ff8000000000000ULL
                                          : (unsigned long long)__double_as_longlong(best);
    if (isnan(best) || best >= 0.0) atomicMin(out, bits);
    else atomicMin(out, 0ULL);
  }
}

}  // namespace

void ffv_m0_cfl(const ffv_dmesh &m, const ffv_geom &g, const double *S, const ffv_m0_consts &k,
                unsigned long long *d_out, cudaStream_t st) {
  int blocks = 152 * 4;
  m0_cfl_kernel<<<blocks, 256, 0, st>>>(m, g, S, k.gamma, k.pinf, d_out);
}

int ffv_check_frames(const ffv_mesh *m) {
  for (int f = 0; f < 6; f++) {
    const ffv_face_frame &fr = m->frame[f];
    if (fr.n_axis != fr_n_axis(f) || fr.n_sign != fr_n_sign(f) || fr.t1_axis != fr_t1_axis(f) ||
        fr.t1_sign != fr_t1_sign(f) || fr.t2_axis != fr_t2_axis(f) || fr.t2_sign != fr_t2_sign(f))
      return FFV_ERR_TABLE;
  }
  return FFV_OK;
}

void ffv_fill_geom(const ffv_mesh *m, ffv_geom *g) {
  memset(g, 0, sizeof(*g));
  for (int l = 1; l <= FFV_MAX_LEVEL + 1; l++) {
    const double h = m->geom[l].h;
    g->vol[l] = m->geom[l].vol;
    g->inv_vol[l] = 1.0 / m->geom[l].vol;
    g->area[l] = m->geom[l].area;
    g->h[l] = h;
    // distance.c:120-167, by face class (see ffv_mesh.cpp face_dist)
    g->dcf[l][0] = 0.5 * h;
    g->dcc[l][0] = h;
    const double hp = l > 1 ? m->geom[l - 1].h : 0.0;
    g->dcf[l][1] = 0.25 * hp;
    g->dcc[l][1] = 0.25 * hp + 0.5 * hp;
    g->dcf[l][2] = 0.5 * h;
    g->dcc[l][2] = 0.5 * h + 0.25 * h;
    g->dcf[l][3] = 0.0;
    g->dcc[l][3] = 0.0;
    for (int q = 0; q < 4; q++) {
      g->dcf_f[l][q] = (float)g->dcf[l][q];
      g->idcc_f[l][q] = (float)(1.0 / g->dcc[l][q]);
    }
    g->area_f[l] = (float)g->area[l];
  }
  for (int l = 1; l <= FFV_MAX_LEVEL; l++) g->area4_fine_f[l] = (float)(4.0 * g->area[l + 1]);
}

// a read-only view of a context for the indicator (ffv_mlp.cu)
int ffv_ctx_view(ffv_ctx *c, int *device, cudaStream_t *st, ffv_dmesh *dm, const double **S,
                 const M5Consts **k, int *model, double *gamma0, double *pinf0) {
  if (!c) return FFV_ERR_ARG;
  if (!c->have_state) return FFV_ERR_STATE;
  *device = c->device;
  *st = c->stream;
  *dm = c->dm;
  *S = c->d_S;
  *k = &c->m5;
  *model = c->p.model;
  *gamma0 = c->p.gamma[0];
  *pinf0 = c->p.pinf[0];
  return FFV_OK;
}

// the context's RK copy [neq][cap] and face-state buffer [6 neq][cap] (both idle between
// steps) and the capacity the mesh buffers are allocated for, for a regrid's state remap
// (ffv_adapt.cu)
int ffv_ctx_scratch(ffv_ctx *c, double **d_SN, double **d_SF, int64_t *cap, int64_t *cap_nsub) {
  if (!c || !c->have_mesh) return FFV_ERR_STATE;
  *d_SN = c->d_SN;
  *d_SF = c->d_SF;
  *cap = c->cap;
  *cap_nsub = c->cap_nsub;
  return FFV_OK;
}

// the context's state for ffv_adapt (ffv_adapt.cu)
int ffv_ctx_adapt_view(ffv_ctx *c, int *device, cudaStream_t *st, int64_t *n, int *neq,
                       double **d_S, int *model, const M5Consts **k) {
  if (!c) return FFV_ERR_ARG;
  if (!c->have_state) return FFV_ERR_STATE;
  *device = c->device;
  *st = c->stream;
  *n = c->n;
  *neq = c->neq;
  *d_S = c->d_S;
  *model = c->p.model;
  *k = &c->m5;
  return FFV_OK;
}

int ffv_ctx_mark_state(ffv_ctx *c) {
  if (!c || !c->have_mesh) return FFV_ERR_STATE;
  c->have_state = 1;
  return FFV_OK;
}

extern "C" {

const char *ffv_error_string(int code) {
  switch (code) {
    case FFV_OK: return "ok";
    case FFV_ERR_ARG: return "invalid argument";
    case FFV_ERR_CUDA: return "CUDA runtime error";
    case FFV_ERR_TABLE: return "mesh description rejected";
    case FFV_ERR_BALANCE: return "2:1 balance violated";
    case FFV_ERR_NAN: return "non-finite residual or state on the device";
    case FFV_ERR_NEG_DENSITY: return "non-positive density on the device";
    case FFV_ERR_TIMEOUT: return "bounded device wait ran out";
    case FFV_ERR_UNSUPPORTED: return "unsupported option";
    case FFV_ERR_NOMEM: return "out of memory";
    case FFV_ERR_STATE: return "call out of order";
    case FFV_ERR_TOO_LARGE: return "mesh larger than the no-allocation scratch";
    case FFV_ERR_IO: return "file cannot be read or written, or is corrupt";
    default: return "unknown error";
  }
}

int ffv_create(ffv_ctx **out, const ffv_params *p, int device) {
  if (!out || !p) return FFV_ERR_ARG;
  *out = nullptr;
  if (p->model != 0 && p->model != 5) return FFV_ERR_UNSUPPORTED;
  if (p->model == 5) {
    if (p->nmaterials < 2 || p->nmaterials > 3) return FFV_ERR_UNSUPPORTED;
    // PRELAX 2 reads relaxation arrays the reference never fills (F_pe.c:24 reads run->ar_R,
    // run->t0_m, run->p0_m; m5_relaxationvec.c fills local arrays of the same names)
    if (!(p->prelax == 3 || (p->prelax == 1 && p->nmaterials == 2))) return FFV_ERR_UNSUPPORTED;
    int nsol = 0;
    for (int i = 0; i < p->nmaterials; i++) nsol += p->mu[i] != 0.0;
    if (nsol > 2) return FFV_ERR_UNSUPPORTED;
  }
  if (p->order != 1 && p->order != 2) return FFV_ERR_ARG;
  if (p->rk_steps < 1 || p->rk_steps > 4) return FFV_ERR_ARG;
  if (p->precision != FFV_FP64 && p->precision != FFV_FP32_FLUX) return FFV_ERR_ARG;
  if (p->precision != FFV_FP64 && p->model != 5) return FFV_ERR_UNSUPPORTED;
  if (p->flux_form != FFV_FLUX_REFERENCE && p->flux_form != FFV_FLUX_CONSISTENT) return FFV_ERR_ARG;
  if (p->flux_form != FFV_FLUX_REFERENCE && p->model != 5) return FFV_ERR_UNSUPPORTED;
  for (int i = 0; i < FFV_MAX_MATERIALS; i++)
    if (p->yield[i] < 0.0 || p->yield[i] != p->yield[i]) return FFV_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0)
    return FFV_ERR_CUDA;
  CK(cudaSetDevice(device));
  ffv_ctx *c = new (std::nothrow) ffv_ctx();
  if (!c) return FFV_ERR_NOMEM;
  memset(c, 0, sizeof(*c));
  c->p = *p;
  c->device = device;
  c->neq = neq_of(*p);
  if (p->model == 5) {
    M5Consts &k = c->m5;
    k.nmat = p->nmaterials;
    k.order = p->order;
    k.prelax = p->prelax;
    k.precision = p->precision;
    k.flux_form = p->flux_form;
    k.nsolids = 0;
    for (int d = 0; d < 3; d++) k.zerou[d] = p->zerou[d];
    for (int i = 0; i < FFV_MAX_MATERIALS; i++) {
      k.gamma[i] = p->gamma[i];
      k.pinf[i] = p->pinf[i];
      k.mu[i] = p->mu[i];
      if (i < p->nmaterials && p->mu[i] != 0.0) k.nsolids++;
    }
    k.amin = p->amin;
    k.avf_lim = p->avf_lim;
    k.plastic = 0;
    for (int i = 0; i < FFV_MAX_MATERIALS; i++) {
      k.yield[i] = (i < p->nmaterials && p->mu[i] != 0.0 && p->yield[i] > 0.0) ? p->yield[i] : 0.0;
      if (k.yield[i] > 0.0) k.plastic = 1;
    }
    for (int i = 0; i < FFV_MAX_MATERIALS; i++) {
      const double gm1 = p->gamma[i] - 1.0;
      k.gpi[i] = p->gamma[i] * p->pinf[i];
      k.ig1[i] = gm1 != 0.0 ? 1.0 / gm1 : 0.0;
      k.gpg[i] = k.gpi[i] * k.ig1[i];
      k.igam[i] = p->gamma[i] != 0.0 ? 1.0 / p->gamma[i] : 0.0;
      k.pinf_f[i] = (float)p->pinf[i];
      k.igam_f[i] = (float)k.igam[i];
      k.mu_f[i] = (float)p->mu[i];
      k.gamma_f[i] = (float)p->gamma[i];
      // m5_relaxationvec.c's floor -(1 - 1e-8) p_inf + 1e-8 and reset value
      k.plo_f[i] = (float)(-(1.0 - 1.0e-8) * p->pinf[i] + 1.0e-8);
      k.preset_f[i] = (float)(-(1.0 - 1.0e-8) * p->pinf[i] + 1.0);
      // binomial series of (1 + x)^a - 1, a = -1 / gamma: ratios (a - j) / (j + 1) of its terms
      for (int j = 1; j <= 6; j++) k.bin_f[i][j - 1] = (float)((-k.igam[i] - j) / (j + 1.0));
      k.gm1_d[i] = df_from_double(gm1);
      k.gpi_d[i] = df_from_double(k.gpi[i]);
      k.ig1_d[i] = df_from_double(k.ig1[i]);
      k.gpg_d[i] = df_from_double(k.gpg[i]);
      k.pinf_d[i] = df_from_double(p->pinf[i]);
      k.floor_d[i] = df_from_double(-(1.0 - 1.0e-8) * p->pinf[i] + 1.0e-8);
    }
    k.alo_f = (float)(p->amin / 100.0);
    k.ahi_f = (float)(1.0 - (p->amin / 100.0));
    k.avf_lim_f = (float)k.avf_lim;
    k.phi_pair = (k.nsolids == 2 && k.mu[0] != 0.0) ? 1 : 0;
    k.alo_d = df_from_double(p->amin / 100.0);
    k.ahi_d = df_from_double(1.0 - (p->amin / 100.0));
    k.a2lo_d = df_from_double(1.0 - (2.0 * (p->amin / 100.0)));
    k.eps_d = df_from_double(1.0e-12);
    k.oneeps_d = df_from_double(1.0 - 1.0e-12);
  }
  int rc = FFV_OK;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->d_dt, sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->d_status, sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&c->d_red, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&c->h_status, sizeof(unsigned)) != cudaSuccess ||
      cudaMallocHost(&c->h_red, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(c->d_status, 0, sizeof(unsigned)) != cudaSuccess)
    rc = FFV_ERR_CUDA;
  if (rc != FFV_OK) {
    ffv_destroy(c);
    return rc;
  }
  *out = c;
  return FFV_OK;
}

int ffv_destroy(ffv_ctx *c) {
  if (!c) return FFV_ERR_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_mesh_buffers(c);
  cudaFree(c->d_dt);
  cudaFree(c->d_status);
  cudaFree(c->d_red);
  cudaFreeHost(c->h_status);
  cudaFreeHost(c->h_red);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return FFV_OK;
}

int ffv_set_mesh(ffv_ctx *c, const ffv_mesh *m) {
  if (!c || !m) return FFV_ERR_ARG;
  int rc = ffv_check_frames(m);
  if (rc != FFV_OK) return rc;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  const int64_t n_mesh = m->n;
  const int64_t nsub_mesh = m->nsub > 0 ? m->nsub : 1;
  if (c->d_info && n_mesh <= c->cap && nsub_mesh <= c->cap_nsub) {
    // the buffers fit: keep them, drop what belonged to the previous mesh
    if (c->graph_valid) cudaGraphExecDestroy(c->graph);
    c->graph_valid = 0;
    c->have_state = 0;
  } else {
    free_mesh_buffers(c);
    // 25 % headroom so that meshes grown by a regrid still fit
    c->cap = n_mesh + n_mesh / 4 + 1024;
    c->cap_nsub = nsub_mesh + nsub_mesh / 4 + 1024;
    rc = alloc_mesh_buffers(c);
    if (rc != FFV_OK) return rc;
  }
  const int64_t n = n_mesh;
  // neighbour slots face-major on the device ([6][n]) for coalesced loads
  int32_t *nbr_t = (int32_t *)malloc(sizeof(int32_t) * 6 * n);
  if (!nbr_t) {
    free_mesh_buffers(c);
    return FFV_ERR_NOMEM;
  }
  parallel_chunks(n, host_threads(), [&](int, int64_t a, int64_t b) {
    for (int64_t i = a; i < b; i++)
      for (int f = 0; f < 6; f++) nbr_t[(int64_t)f * n + i] = m->nbr[6 * i + f];
  });
  cudaError_t e = cudaMemcpy(c->d_info, m->info, sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->d_nbr, nbr_t, sizeof(int32_t) * 6 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && m->nsub > 0)
    e = cudaMemcpy(c->d_sub, m->sub, sizeof(int32_t) * 4 * m->nsub, cudaMemcpyHostToDevice);
  free(nbr_t);
  if (e != cudaSuccess) {
    free_mesh_buffers(c);
    return FFV_ERR_CUDA;
  }
  c->n = n;
  c->dm = ffv_dmesh{n, c->d_info, c->d_nbr, c->d_sub};
  ffv_fill_geom(m, &c->geom);
  c->have_mesh = 1;
  return FFV_OK;
}

int ffv_upload_state(ffv_ctx *c, const double *S, int64_t ncells, int32_t neq) {
  if (!c || !S) return FFV_ERR_ARG;
  if (!c->have_mesh) return FFV_ERR_STATE;
  if (ncells != c->n || neq != c->neq) return FFV_ERR_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(c->d_S, S, sizeof(double) * neq * ncells, cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaMemcpyAsync(c->d_SN, c->d_S, sizeof(double) * neq * ncells, cudaMemcpyDeviceToDevice,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->have_state = 1;
  return FFV_OK;
}

int ffv_download_state(ffv_ctx *c, double *S, int64_t ncells, int32_t neq) {
  if (!c || !S) return FFV_ERR_ARG;
  if (!c->have_state) return FFV_ERR_STATE;
  if (ncells != c->n || neq != c->neq) return FFV_ERR_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(S, c->d_S, sizeof(double) * neq * ncells, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return FFV_OK;
}

int ffv_stage(ffv_ctx *c, int32_t irk, double dt) {
  if (!c) return FFV_ERR_ARG;
  if (!c->have_state) return FFV_ERR_STATE;
  if (irk < 0 || irk > 4) return FFV_ERR_ARG;
  CK(cudaSetDevice(c->device));
  int rc = queue_dt(c, dt);
  if (rc != FFV_OK) return rc;
  return launch_stage(c, irk);
}

int ffv_sync(ffv_ctx *c) {
  if (!c) return FFV_ERR_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return (int)status_to_err(*c->h_status);
}

int ffv_step_async(ffv_ctx *c, double dt, int32_t nsteps) {
  if (!c || nsteps < 0) return FFV_ERR_ARG;
  if (!c->have_state) return FFV_ERR_STATE;
  CK(cudaSetDevice(c->device));
  int rc = build_graph(c);
  if (rc != FFV_OK) return rc;
  rc = queue_dt(c, dt);
  if (rc != FFV_OK) return rc;
  for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(c->graph, c->stream));
  return FFV_OK;
}

int ffv_step(ffv_ctx *c, double dt, int32_t nsteps) {
  int rc = ffv_step_async(c, dt, nsteps);
  if (rc != FFV_OK) return rc;
  return ffv_sync(c);
}

int ffv_cfl_dt(ffv_ctx *c, double cfl, double *dt_out) {
  if (!c || !dt_out || !(cfl > 0.0)) return FFV_ERR_ARG;
  if (!c->have_state) return FFV_ERR_STATE;
  CK(cudaSetDevice(c->device));
  CK(cudaMemsetAsync(c->d_red, 0xff, sizeof(unsigned long long), c->stream));
  if (c->p.model == 5) {
    ffv_m5_cfl(c->dm, c->geom, c->m5, c->d_S, c->d_red, c->stream);
  } else {
    ffv_m0_consts k{c->p.gamma[0], c->p.pinf[0], c->p.order};
    ffv_m0_cfl(c->dm, c->geom, c->d_S, k, c->d_red, c->stream);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c->h_red, c->d_red, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double m;
  memcpy(&m, c->h_red, sizeof(double));
  if (!(m > 0.0) || isnan(m)) return FFV_ERR_NAN;
  *dt_out = cfl * m;
  return FFV_OK;
}

}  // extern "C"

namespace {

constexpr int kSumBlocks = 152 * 4, kSumThreads = 256;

// block b's partial of sum_c |V_c| S[v][c] over its grid-stride cells, for every variable:
// a fixed assignment of cells to threads and a fixed reduction tree, so the sums are
// reproducible bit for bit
__global__ void __launch_bounds__(kSumThreads) sum_partials(ffv_dmesh m, ffv_geom g, int neq,
                                                            const double *__restrict__ S,
                                                            double *__restrict__ part) {
  __shared__ double red[kSumThreads];
  for (int v = 0; v < neq; v++) {
    double acc = 0.0;
    for (int64_t c = (int64_t)blockIdx.x * kSumThreads + threadIdx.x; c < m.n;
         c += (int64_t)gridDim.x * kSumThreads)
      acc += fabs(g.vol[ffv_info_level(m.info[c])]) * S[(int64_t)v * m.n + c];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kSumThreads / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[(int64_t)v * gridDim.x + blockIdx.x] = red[0];
    __syncthreads();
  }
}

// one block per variable: the partials in a fixed order
__global__ void __launch_bounds__(kSumThreads) sum_final(int nparts, const double *__restrict__ part,
                                                         double *__restrict__ out) {
  __shared__ double red[kSumThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += kSumThreads) acc += part[(int64_t)blockIdx.x * nparts + i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = kSumThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

}  // namespace

extern "C" {

int ffv_conservation_sums(ffv_ctx *c, double *sums) {
  if (!c || !sums) return FFV_ERR_ARG;
  if (!c->have_state) return FFV_ERR_STATE;
  CK(cudaSetDevice(c->device));
  double *d_part = nullptr;
  CK(cudaMalloc(&d_part, sizeof(double) * ((size_t)kSumBlocks + 1) * c->neq));
  double *d_out = d_part + (size_t)kSumBlocks * c->neq;
  sum_partials<<<kSumBlocks, kSumThreads, 0, c->stream>>>(c->dm, c->geom, c->neq, c->d_S, d_part);
  sum_final<<<c->neq, kSumThreads, 0, c->stream>>>(kSumBlocks, d_part, d_out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sums, d_out, sizeof(double) * c->neq, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_part);
  return cuda_rc(e);
}

int ffv_state_device_ptr(ffv_ctx *c, double **d_S) {
  if (!c || !d_S) return FFV_ERR_ARG;
  if (!c->have_mesh) return FFV_ERR_STATE;
  *d_S = c->d_S;
  return FFV_OK;
}

int ffv_profile_stage(ffv_ctx *c, int32_t irk, double dt, float *ms, int32_t max_kernels,
                      int32_t *nkernels) {
  if (!c || !ms || !nkernels || irk < 1 || irk > 4) return FFV_ERR_ARG;
  if (!c->have_state) return FFV_ERR_STATE;
  const int nk = c->p.model == 5 ? ffv_m5_launches_per_stage(c->m5, irk)
                                 : ffv_m0_launches_per_stage(c->p.order);
  if (max_kernels < nk) return FFV_ERR_ARG;
  CK(cudaSetDevice(c->device));
  cudaEvent_t ev[17];
  for (int i = 0; i <= nk; i++) CK(cudaEventCreate(&ev[i]));
  int rc = queue_dt(c, dt);
  if (rc == FFV_OK) rc = launch_stage(c, irk, ev);
  if (rc == FFV_OK && cudaEventSynchronize(ev[nk]) != cudaSuccess) rc = FFV_ERR_CUDA;
  for (int i = 0; i < nk && rc == FFV_OK; i++)
    if (cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]) != cudaSuccess) rc = FFV_ERR_CUDA;
  for (int i = 0; i <= nk; i++) cudaEventDestroy(ev[i]);
  *nkernels = nk;
  return rc;
}

const char *ffv_stage_kernel_name(const ffv_ctx *c, int32_t i) {
  if (c && c->p.model == 5) return (i >= 0 && i < 16 && c->knames[i]) ? c->knames[i] : "";
  return c ? ffv_m0_fp64_kernel_name(c->p.order, i) : "";
}

int ffv_stream(ffv_ctx *c, void **stream) {
  if (!c || !stream) return FFV_ERR_ARG;
  *stream = (void *)c->stream;
  return FFV_OK;
}

}  // extern "C"

namespace {

// the device half of ffv_tags: SI layers and the raw target level of every leaf into
// c->d_split; *level_max receives the reference's LEVEL
int tags_device(ffv_ctx *c, const ffv_mesh *m, const ffv_tag_params *p, int32_t *level_max) {
  if (!c->have_state) return FFV_ERR_STATE;
  if (m->n != c->n) return FFV_ERR_ARG;
  if (p->inter0 == 0 && p->inter1 == 1) return FFV_ERR_ARG;  // m5_input.c:52 exits there
  if (p->grad_vel == 1 && p->grad_rho != 1) return FFV_ERR_UNSUPPORTED;
  if (c->p.model != 5 && p->inter0) return FFV_ERR_UNSUPPORTED;  // no volume fractions
  ffv_m5_tagc t;
  t.uniform = p->uniform; t.lvl_uniform = p->lvl_uniform;
  t.prs = p->grad_prs; t.lvl_prs = p->lvl_prs; t.thr_prs = p->thr_prs;
  t.rho = p->grad_rho; t.lvl_rho = p->lvl_rho; t.thr_rho = p->thr_rho;
  t.vel = p->grad_vel; t.lvl_vel = p->lvl_vel; t.thr_vel = p->thr_vel;
  t.inter0 = p->inter0; t.lvl0 = p->lvl_inter0; t.lrs0 = p->lrs_inter0;
  t.inter1 = p->inter1; t.lvl1 = p->lvl_inter1; t.lrs1 = p->lrs_inter0 + p->lrs_inter1;
  t.si_max = 0;
  if (p->inter0 == 1 && p->inter1 == 1) t.si_max = t.lrs0 + t.lrs1;
  if (p->inter0 == 1 && p->inter1 == 0) t.si_max = t.lrs0;
  // inputset.c:106, m5_input.c:53
  int32_t lmax = p->lvl_uniform;
  for (int32_t l : {p->lvl_prs, p->lvl_rho, p->lvl_vel, p->lvl_inter0, p->lvl_inter1})
    lmax = lmax > l ? lmax : l;
  *level_max = lmax;
  CK(cudaSetDevice(c->device));
  const int64_t n = c->n;
  if (!c->d_split) {  // sized for the mesh buffers' capacity, kept while meshes fit
    const int64_t cap = c->cap;
    if (cudaMalloc(&c->d_SI, sizeof(int32_t) * 2 * cap) != cudaSuccess ||
        cudaMalloc(&c->d_SItmp, sizeof(int32_t) * 2 * cap) != cudaSuccess ||
        cudaMalloc(&c->d_split, sizeof(int32_t) * cap) != cudaSuccess ||
        cudaMalloc(&c->d_tagpr, sizeof(double) * 2 * cap) != cudaSuccess) {
      cudaFree(c->d_SI);
      cudaFree(c->d_SItmp);
      cudaFree(c->d_split);
      cudaFree(c->d_tagpr);
      c->d_SI = c->d_SItmp = c->d_split = nullptr;
      c->d_tagpr = nullptr;
      return FFV_ERR_NOMEM;
    }
  }
  if (c->p.model == 5) {
    ffv_m5_tags(c->dm, c->m5, t, c->d_S, c->d_SI, c->d_SItmp, c->d_split, c->d_tagpr, c->stream);
  } else {
    ffv_m0_tags(c->dm, c->p.gamma[0], c->p.pinf[0], t, c->d_S, c->d_split, c->stream);
    CK(cudaMemsetAsync(c->d_SI, 0, sizeof(int32_t) * 2 * n, c->stream));
  }
  CK(cudaGetLastError());
  return FFV_OK;
}

// leaves whose target level is above their level (warp sums, one atomic per warp)
__global__ void count_finer(int64_t n, const uint32_t *__restrict__ info,
                            const int32_t *__restrict__ split, unsigned long long *count) {
  unsigned long long k = 0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    k += split[c] > (int32_t)ffv_info_level(info[c]) ? 1ull : 0ull;
  for (int o = 16; o > 0; o >>= 1) k += __shfl_down_sync(0xffffffffu, k, o);
  if ((threadIdx.x & 31) == 0 && k) atomicAdd(count, k);
}

}  // namespace

extern "C" {

int ffv_tags(ffv_ctx *c, const ffv_mesh *m, const ffv_tag_params *p, int32_t *split,
             int32_t *split_raw, int32_t *si) {
  if (!c || !m || !p || !split) return FFV_ERR_ARG;
  int32_t level_max;
  int rc = tags_device(c, m, p, &level_max);
  if (rc != FFV_OK) return rc;
  const int64_t n = c->n;
  CK(cudaMemcpyAsync(split, c->d_split, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
  if (si)
    CK(cudaMemcpyAsync(si, c->d_SI, sizeof(int32_t) * 2 * n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (split_raw) memcpy(split_raw, split, sizeof(int32_t) * n);
  return ffv_tags_smooth(m, level_max, split);
}

int ffv_export_fields(ffv_ctx *c, double *F_dev, int32_t *nf) {
  if (!c || !nf) return FFV_ERR_ARG;
  *nf = c->p.model == 5 ? 5 + 2 * c->p.nmaterials + 1 : 5;
  if (!F_dev) return FFV_OK;
  if (!c->have_state) return FFV_ERR_STATE;
  CK(cudaSetDevice(c->device));
  if (c->p.model == 5) ffv_m5_export_fields(c->n, c->m5, c->d_S, F_dev, c->stream);
  else ffv_m0_export_fields(c->n, c->p.gamma[0], c->p.pinf[0], c->d_S, F_dev, c->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return FFV_OK;
}

int ffv_tags_raw(ffv_ctx *c, const ffv_mesh *m, const ffv_tag_params *p, int32_t *split_raw,
                 int32_t *si) {
  if (!c || !m || !p || !split_raw) return FFV_ERR_ARG;
  int32_t level_max;
  int rc = tags_device(c, m, p, &level_max);
  if (rc != FFV_OK) return rc;
  const int64_t n = c->n;
  CK(cudaMemcpyAsync(split_raw, c->d_split, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                     c->stream));
  if (si)
    CK(cudaMemcpyAsync(si, c->d_SI, sizeof(int32_t) * 2 * n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return FFV_OK;
}

int ffv_tags_missed(ffv_ctx *c, const ffv_mesh *m, const ffv_tag_params *p, int64_t *missed) {
  if (!c || !m || !p || !missed) return FFV_ERR_ARG;
  int32_t level_max;
  int rc = tags_device(c, m, p, &level_max);
  if (rc != FFV_OK) return rc;
  CK(cudaMemsetAsync(c->d_red, 0, sizeof(unsigned long long), c->stream));
  count_finer<<<152 * 4, 256, 0, c->stream>>>(c->n, c->d_info, c->d_split, c->d_red);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c->h_red, c->d_red, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *missed = (int64_t)*c->h_red;
  return FFV_OK;
}

int ffv_launches_per_step(const ffv_ctx *c, int32_t *n) {
  if (!c || !n) return FFV_ERR_ARG;
  if (c->p.model == 5) {
    int t = 0;
    for (int irk = 1; irk <= c->p.rk_steps; irk++) t += ffv_m5_launches_per_stage(c->m5, irk);
    *n = t;
  } else {
    *n = c->p.rk_steps * ffv_m0_launches_per_stage(c->p.order);
  }
  return FFV_OK;
}

}  // extern "C"
