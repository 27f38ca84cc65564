// ffv_step_noalloc: the model-0 FP64 time step for callers that cannot allocate device
// memory.
//
// Who needs it: code that is handed device buffers but does not own the device's memory,
// e.g. a solver plugin inside a host application or framework that does all allocation
// itself (its own arena or caching allocator, a fixed memory budget), or a loop that must
// not call cudaMalloc/cudaFree because they synchronise the whole device.  ffv_create /
// ffv_set_mesh allocate the face tables, the RK copy and the face states with cudaMalloc;
// this entry point instead keeps them in one fixed, file-scope device array below and
// allocates nothing, neither on the device nor on the host.
//
// The array is part of this library's device image: every GPU that loads the library holds
// its FFV_NOALLOC_SCRATCH_BYTES until the process exits.  All calls on a device share it and
// it keeps the contents of the last call; every call rewrites the tables it reads and clears
// the status word before its first kernel.  Calls whose work overlaps on the GPU (different
// streams, or different host threads without ordering) race on the array.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it together with the id of the
// device's current CUDA context; a later call in another context (after cudaDeviceReset, or
// a reset of the primary context, reloads the module, possibly at another address) looks
// the address up again.  With lazy module loading (CUDA_MODULE_LOADING=LAZY, the default)
// that first lookup is also what loads this library's module on the device and reserves the
// array, so it can fail for lack of device memory (FFV_ERR_CUDA).  A caller with a fixed
// memory budget makes its first call -- or sets CUDA_MODULE_LOADING=EAGER -- before it takes
// the rest of the device's memory, and outside any stream capture on that device.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "ffv_device.cuh"
#include "ffv.h"

namespace {

constexpr int64_t kMaxCells = FFV_NOALLOC_MAX_CELLS;
// a 4-subface group is one coarse face with four finer neighbours; each finer cell face
// is in at most one group, so a mesh of n cells has at most 6n/4 groups
constexpr int64_t kMaxSub = (6 * kMaxCells) / 4;
constexpr int kMaxDevices = 64;

constexpr size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }
// layout of the array (every region starts on a 256-byte boundary)
constexpr size_t kOffSF = 0;                                                   // [6][5][n] f64
constexpr size_t kOffSN = up256(kOffSF + sizeof(double) * 30 * kMaxCells);     // [5][n] f64
constexpr size_t kOffInfo = up256(kOffSN + sizeof(double) * 5 * kMaxCells);    // [n] u32
constexpr size_t kOffNbr = up256(kOffInfo + sizeof(uint32_t) * kMaxCells);     // [6][n] i32
constexpr size_t kOffSub = up256(kOffNbr + sizeof(int32_t) * 6 * kMaxCells);   // [4 nsub] i32
constexpr size_t kOffDt = up256(kOffSub + sizeof(int32_t) * 4 * kMaxSub);      // f64
constexpr size_t kOffStatus = kOffDt + 256;                                    // u32
constexpr size_t kBytes = kOffStatus + 256;
static_assert(kBytes == FFV_NOALLOC_SCRATCH_BYTES, "ffv.h states the scratch size");
// the cell-major neighbour table is staged in the face-state region before the stage
// kernels overwrite it
static_assert(sizeof(int32_t) * 6 * kMaxCells <= kOffSN - kOffSF, "staging fits");

static __device__ __align__(256) unsigned char ffv_noalloc_scratch[kBytes];

std::mutex g_mu;
// device address of the array per device, and the id of the context it was looked up in
unsigned char *g_base[kMaxDevices];
unsigned long long g_ctx[kMaxDevices];

// [n][6] -> [6][n], the device layout of the neighbour slots
__global__ void noalloc_nbr_face_major(const int32_t *__restrict__ raw, int32_t *__restrict__ out,
                                       int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 6 * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / 6, f = i - 6 * c;
    out[f * n + c] = raw[i];
  }
}

__global__ void noalloc_begin(double *dt_slot, double dt, unsigned *status) {
  *dt_slot = dt;
  *status = 0u;
}

// id of the current context (cuCtxGetId through the runtime's driver entry point, so that the
// library needs no link against the driver library); false when it cannot be had
bool current_context_id(unsigned long long *id) {
  static PFN_cuCtxGetId_v12000 fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return (PFN_cuCtxGetId_v12000)f;
  }();
  return fn && fn(nullptr, id) == CUDA_SUCCESS;
}

int base_for_current_device(unsigned char **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return FFV_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return FFV_ERR_UNSUPPORTED;
  // makes the device's primary context current (the runtime creates it here if needed)
  if (cudaSetDevice(dev) != cudaSuccess) return FFV_ERR_CUDA;
  unsigned long long ctx = 0;
  const bool have_ctx = current_context_id(&ctx);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_base[dev] || !have_ctx || g_ctx[dev] != ctx) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, ffv_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      g_base[dev] = nullptr;
      return FFV_ERR_CUDA;
    }
    g_base[dev] = (unsigned char *)p;
    g_ctx[dev] = have_ctx ? ctx : 0;
  }
  *out = g_base[dev];
  return FFV_OK;
}

}  // namespace

extern "C" int ffv_step_noalloc(const ffv_mesh *m, const ffv_params *p, double *d_S, double dt,
                                int32_t nsteps, void *stream) {
  if (!m || !p || !d_S || nsteps < 0) return FFV_ERR_ARG;
  if (p->model != 0 || p->precision != FFV_FP64) return FFV_ERR_UNSUPPORTED;
  if (p->order != 1 && p->order != 2) return FFV_ERR_ARG;
  if (p->rk_steps < 1 || p->rk_steps > 4) return FFV_ERR_ARG;
  const int64_t n = m->n;
  if (n > kMaxCells || (int64_t)m->nsub > kMaxSub) return FFV_ERR_TOO_LARGE;
  if (n < 1) return FFV_ERR_ARG;
  int rc = ffv_check_frames(m);
  if (rc != FFV_OK) return rc;
  // the state must be device memory of the current device
  int dev = -1;
  cudaPointerAttributes attr;
  if (cudaGetDevice(&dev) != cudaSuccess) return FFV_ERR_CUDA;
  if (cudaPointerGetAttributes(&attr, d_S) != cudaSuccess) {
    cudaGetLastError();
    return FFV_ERR_ARG;
  }
  if ((attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) ||
      attr.device != dev)
    return FFV_ERR_ARG;

  unsigned char *base = nullptr;
  rc = base_for_current_device(&base);
  if (rc != FFV_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  double *SF = (double *)(base + kOffSF);
  double *SN = (double *)(base + kOffSN);
  uint32_t *info = (uint32_t *)(base + kOffInfo);
  int32_t *nbr = (int32_t *)(base + kOffNbr);
  int32_t *sub = (int32_t *)(base + kOffSub);
  double *d_dt = (double *)(base + kOffDt);
  unsigned *status = (unsigned *)(base + kOffStatus);

  // tables of this mesh (stream-ordered after any earlier call on the same stream)
  if (cudaMemcpyAsync(info, m->info, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(SF, m->nbr, sizeof(int32_t) * 6 * n, cudaMemcpyHostToDevice, st) !=
          cudaSuccess ||
      (m->nsub > 0 && cudaMemcpyAsync(sub, m->sub, sizeof(int32_t) * 4 * m->nsub,
                                      cudaMemcpyHostToDevice, st) != cudaSuccess))
    return FFV_ERR_CUDA;
  noalloc_nbr_face_major<<<152 * 4, 256, 0, st>>>((const int32_t *)SF, nbr, n);
  noalloc_begin<<<1, 1, 0, st>>>(d_dt, dt, status);
  if (cudaGetLastError() != cudaSuccess) return FFV_ERR_CUDA;

  ffv_geom g;
  ffv_fill_geom(m, &g);
  const ffv_dmesh dm{n, info, nbr, sub};
  const ffv_m0_bufs b{d_S, SN, SF, d_dt, status};
  const ffv_m0_consts k{p->gamma[0], p->pinf[0], p->order};
  // stage 1 also performs RK(0) (SN = S), as in ffv_step
  for (int s = 0; s < nsteps; s++)
    for (int irk = 1; irk <= p->rk_steps; irk++) ffv_m0_fp64_stage(dm, g, b, k, irk, st, nullptr);
  if (cudaGetLastError() != cudaSuccess) return FFV_ERR_CUDA;

  unsigned h_status = 0;
  if (cudaMemcpyAsync(&h_status, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return FFV_ERR_CUDA;
  if (h_status & FFV_ST_NEG_DENSITY) return FFV_ERR_NEG_DENSITY;
  if (h_status & (FFV_ST_NAN | FFV_ST_NAN_SPEED | FFV_ST_NO_BRANCH)) return FFV_ERR_NAN;
  return FFV_OK;
}
