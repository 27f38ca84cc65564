// Learned refinement indicator: a 135-64-64-1 perceptron (GELU, GELU, sigmoid) over the
// 27-cell stencil of five per-cell fields, trained on the GPU with AdamW.
//
// Inputs: for every cell, the fields log rho, log p, alpha_0, |u| and the von Mises stress
// of the 27 cells reached by steps of -1/0/+1 along x, then y, then z across faces (a
// boundary face keeps the cell, a face with four finer neighbours takes the first of them),
// normalised per field by a stored mean and standard deviation: 135 BF16 values, padded to
// 144 with zeros.  Output: the probability that the plain criterion will ask for a finer
// level within the prediction horizon.
//
// Arithmetic: BF16 operands, FP32 accumulation on the tensor cores.  Inference (features,
// both layers and the marks in one kernel, mlp_infer_tc): a CTA builds the feature rows of
// 128 cells in shared memory and one thread issues tcgen05.mma (M = 128, N = 64) for each
// layer, the accumulators in tensor memory.  Training: warp-level mma.sync m16n8k16
// (16 samples per warp); the backward pass recomputes the forward pass of its tile, forms
// the weight gradients as (16-sample) tensor-core products into shared-memory FP32
// accumulators and adds them to the global gradient once per block.
// Where a tensor-core product needs an operand the forward pass holds in FP32 (the hidden
// activations, the pre-activation gradients) it is rounded to BF16; the CPU restatement
// (oracle/mlp.py) rounds at the same points.
#include <cuda_bf16.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ffv.h"
#include "ffv_device.cuh"
#include "ffv_m5.cuh"
#include "ffv_tc.cuh"

namespace {

constexpr int NIN = 135, KIN = 144, NH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH;
constexpr int OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
static_assert(NPARAM == FFV_MLP_NPARAM, "parameter count");
constexpr int SX = 152;  // shared row stride (bf16) of 144-wide tiles: conflict-free fragments
constexpr int SH = 72;   // shared row stride (bf16) of 64-wide tiles
constexpr int WARPS = 4, TPB = 32 * WARPS;

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t ld32(const bf16 *p) { return *reinterpret_cast<const uint32_t *>(p); }
__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
__device__ __forceinline__ void mma16816(float c[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// GELU (exact, erf form) and its derivative
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// ------------------------------------------------------------------------- features
// the cells across faces fneg and fpos of cell e: a boundary face keeps the cell, a face
// with four finer neighbours takes the first of them
__device__ __forceinline__ void face_steps(const ffv_dmesh &m, int32_t e, int fneg, int fpos,
                                           int32_t &en, int32_t &ep) {
  const uint32_t info = m.info[e];
  const uint32_t kn = ffv_face_kind(info, fneg), kp = ffv_face_kind(info, fpos);
  en = e;
  ep = e;
  if (!(kn & FFV_FK_BC)) {
    const int32_t s = m.nbr[(int64_t)fneg * m.n + e];
    en = kn == FFV_FK_FINER ? m.sub[4 * (int64_t)s] : s;
  }
  if (!(kp & FFV_FK_BC)) {
    const int32_t s = m.nbr[(int64_t)fpos * m.n + e];
    ep = kp == FFV_FK_FINER ? m.sub[4 * (int64_t)s] : s;
  }
}

// the 27 stencil cells of c, o = (dx + 1) + 3 (dy + 1) + 9 (dz + 1): the step along x, then
// along y, then along z.  The walks share their prefixes: 2 + 6 + 18 independent face steps
// in three dependent rounds.
__device__ __forceinline__ void stencil27(const ffv_dmesh &m, int32_t c, int32_t e[27]) {
  int32_t x[3], y[9];
  x[1] = c;
  face_steps(m, c, 0, 2, x[0], x[2]);
#pragma unroll
  for (int ix = 0; ix < 3; ix++) {
    y[ix + 3] = x[ix];
    face_steps(m, x[ix], 3, 1, y[ix], y[ix + 6]);
  }
#pragma unroll
  for (int j = 0; j < 9; j++) {
    e[j + 9] = y[j];
    face_steps(m, y[j], 4, 5, e[j], e[j + 18]);
  }
}

// the 135 normalised features of a cell as BF16, eight per 16-byte chunk (chunk 16 holds
// features 128-134 and a zero, chunk 17 zeros), handed to put(chunk, uint4)
template <typename Put>
__device__ __forceinline__ void cell_features(const ffv_dmesh &m, const float *__restrict__ F,
                                              const float mean[5], const float istd[5], int32_t c,
                                              Put put) {
  int32_t e[27];
  stencil27(m, c, e);
  uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int o = 0; o < 27; o++)
#pragma unroll
    for (int q = 0; q < 5; q++) {
      const int k = 5 * o + q;
      const bf16 v = __float2bfloat16_rn((F[(int64_t)q * m.n + e[o]] - mean[q]) * istd[q]);
      const uint32_t u = __bfloat16_as_ushort(v);
      if ((k & 1) == 0) w[(k & 7) >> 1] = u;
      else w[(k & 7) >> 1] |= u << 16;
      if ((k & 7) == 7) put(k >> 3, make_uint4(w[0], w[1], w[2], w[3]));
    }
  put(NIN >> 3, make_uint4(w[0], w[1], w[2], w[3] & 0xFFFFu));
  put(KIN / 8 - 1, make_uint4(0u, 0u, 0u, 0u));
}

// A block builds its 128 feature rows in shared memory (row stride 146 BF16 = 73 words,
// odd, so that the threads' 4-byte accesses to their own rows fall in distinct banks) and
// then writes them out as one contiguous run of 4-byte words: a thread writing its own
// 288-byte row directly would touch 32 cache lines per warp store.
constexpr int GATHER_TPB = 128, GATHER_SW = 73;  // shared words per row (KIN / 2 = 72, +1)
__global__ void __launch_bounds__(GATHER_TPB) mlp_gather(ffv_dmesh m, const float *__restrict__ F,
                                                         const float *__restrict__ norm,
                                                         bf16 *__restrict__ X) {
  __shared__ uint32_t tile[GATHER_TPB * GATHER_SW];
  const int64_t c0 = (int64_t)blockIdx.x * GATHER_TPB;
  const int64_t c = c0 + threadIdx.x;
  if (c < m.n) {
    float mean[5], istd[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      mean[q] = norm[q];
      istd[q] = 1.0f / norm[5 + q];
    }
    uint32_t *row = tile + threadIdx.x * GATHER_SW;
    cell_features(m, F, mean, istd, (int32_t)c, [&](int ch, uint4 v) {
      row[4 * ch] = v.x;
      row[4 * ch + 1] = v.y;
      row[4 * ch + 2] = v.z;
      row[4 * ch + 3] = v.w;
    });
  }
  __syncthreads();
  const int64_t rows = m.n - c0 < GATHER_TPB ? m.n - c0 : GATHER_TPB;
  const int words = (int)rows * (KIN / 2);
  uint32_t *dst = reinterpret_cast<uint32_t *>(X + c0 * KIN);
  for (int w = threadIdx.x; w < words; w += GATHER_TPB)
    dst[w] = tile[(w / (KIN / 2)) * GATHER_SW + w % (KIN / 2)];
}

// ------------------------------------------------------------------------- weights
__global__ void mlp_pack(const float *__restrict__ P, bf16 *__restrict__ W1, bf16 *__restrict__ W2,
                         bf16 *__restrict__ W2T) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NH * KIN; i += gridDim.x * blockDim.x) {
    const int r = i / KIN, k = i % KIN;
    W1[i] = __float2bfloat16_rn(k < NIN ? P[OFF_W1 + r * NIN + k] : 0.0f);
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NH * NH; i += gridDim.x * blockDim.x) {
    const int r = i / NH, k = i % NH;
    const bf16 w = __float2bfloat16_rn(P[OFF_W2 + i]);
    W2[i] = w;
    W2T[k * NH + r] = w;
  }
}

struct Smem {
  bf16 *W1, *W2, *W2T, *X, *H1, *DA;
  float *b1, *b2, *w3;
};

// stage the BF16 weights and the FP32 biases into shared memory (whole block)
__device__ void stage_weights(const Smem &s, const bf16 *W1, const bf16 *W2, const bf16 *W2T,
                              const float *P, bool with_t) {
  for (int i = threadIdx.x; i < NH * (KIN / 8); i += blockDim.x) {
    const int r = i / (KIN / 8), ch = i % (KIN / 8);
    *reinterpret_cast<uint4 *>(s.W1 + r * SX + ch * 8) =
        *reinterpret_cast<const uint4 *>(W1 + r * KIN + ch * 8);
  }
  for (int i = threadIdx.x; i < NH * (NH / 8); i += blockDim.x) {
    const int r = i / (NH / 8), ch = i % (NH / 8);
    *reinterpret_cast<uint4 *>(s.W2 + r * SH + ch * 8) =
        *reinterpret_cast<const uint4 *>(W2 + r * NH + ch * 8);
    if (with_t)
      *reinterpret_cast<uint4 *>(s.W2T + r * SH + ch * 8) =
          *reinterpret_cast<const uint4 *>(W2T + r * NH + ch * 8);
  }
  for (int i = threadIdx.x; i < NH; i += blockDim.x) {
    s.b1[i] = P[OFF_B1 + i];
    s.b2[i] = P[OFF_B2 + i];
    s.w3[i] = P[OFF_W3 + i];
  }
}

// load 16 sample rows (row index row_of(i), or zeros past `valid`) into the warp's X tile
template <typename RowOf>
__device__ __forceinline__ void load_tile(bf16 *Xs, const bf16 *__restrict__ X, int valid,
                                          RowOf row_of) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < 16 * (KIN / 8); i += 32) {
    const int r = i / (KIN / 8), ch = i % (KIN / 8);
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (r < valid) v = *reinterpret_cast<const uint4 *>(X + row_of(r) * KIN + ch * 8);
    *reinterpret_cast<uint4 *>(Xs + r * SX + ch * 8) = v;
  }
  __syncwarp();
}

// forward pass of one 16-sample tile: a1/a2 receive the pre-activations (C-fragment
// layout: [n-tile][4], rows g, g, g+8, g+8 and columns nt*8 + 2q + {0,1}), H1s the first
// hidden layer in BF16, z the logits of rows g and g+8 (every lane of the quad)
__device__ __forceinline__ void tile_forward(const Smem &s, const bf16 *Xs, bf16 *H1s,
                                             float a1[8][4], float a2[8][4], float &zg,
                                             float &zg8) {
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 8; nt++) a1[nt][0] = a1[nt][1] = a1[nt][2] = a1[nt][3] = 0.0f;
#pragma unroll
  for (int kk = 0; kk < KIN / 16; kk++) {
    const int k0 = kk * 16 + 2 * q;
    const uint32_t x0 = ld32(Xs + g * SX + k0), x1 = ld32(Xs + (g + 8) * SX + k0);
    const uint32_t x2 = ld32(Xs + g * SX + k0 + 8), x3 = ld32(Xs + (g + 8) * SX + k0 + 8);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const bf16 *w = s.W1 + (nt * 8 + g) * SX + k0;
      mma16816(a1[nt], x0, x1, x2, x3, ld32(w), ld32(w + 8));
    }
  }
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int col = nt * 8 + 2 * q;
    a1[nt][0] += s.b1[col];
    a1[nt][1] += s.b1[col + 1];
    a1[nt][2] += s.b1[col];
    a1[nt][3] += s.b1[col + 1];
    *reinterpret_cast<__nv_bfloat162 *>(H1s + g * SH + col) =
        __floats2bfloat162_rn(gelu(a1[nt][0]), gelu(a1[nt][1]));
    *reinterpret_cast<__nv_bfloat162 *>(H1s + (g + 8) * SH + col) =
        __floats2bfloat162_rn(gelu(a1[nt][2]), gelu(a1[nt][3]));
  }
  __syncwarp();
#pragma unroll
  for (int nt = 0; nt < 8; nt++) a2[nt][0] = a2[nt][1] = a2[nt][2] = a2[nt][3] = 0.0f;
#pragma unroll
  for (int kk = 0; kk < NH / 16; kk++) {
    const int k0 = kk * 16 + 2 * q;
    const uint32_t h0 = ld32(H1s + g * SH + k0), h1 = ld32(H1s + (g + 8) * SH + k0);
    const uint32_t h2 = ld32(H1s + g * SH + k0 + 8), h3 = ld32(H1s + (g + 8) * SH + k0 + 8);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const bf16 *w = s.W2 + (nt * 8 + g) * SH + k0;
      mma16816(a2[nt], h0, h1, h2, h3, ld32(w), ld32(w + 8));
    }
  }
  zg = 0.0f;
  zg8 = 0.0f;
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int col = nt * 8 + 2 * q;
    a2[nt][0] += s.b2[col];
    a2[nt][1] += s.b2[col + 1];
    a2[nt][2] += s.b2[col];
    a2[nt][3] += s.b2[col + 1];
    zg += gelu(a2[nt][0]) * s.w3[col] + gelu(a2[nt][1]) * s.w3[col + 1];
    zg8 += gelu(a2[nt][2]) * s.w3[col] + gelu(a2[nt][3]) * s.w3[col + 1];
  }
  zg += __shfl_xor_sync(0xffffffffu, zg, 1);
  zg += __shfl_xor_sync(0xffffffffu, zg, 2);
  zg8 += __shfl_xor_sync(0xffffffffu, zg8, 1);
  zg8 += __shfl_xor_sync(0xffffffffu, zg8, 2);
}

__device__ __forceinline__ Smem carve(unsigned char *base, bool train) {
  Smem s;
  bf16 *p = reinterpret_cast<bf16 *>(base);
  s.W1 = p;
  p += NH * SX;
  s.W2 = p;
  p += NH * SH;
  s.W2T = p;
  if (train) p += NH * SH;
  s.X = p;
  p += WARPS * 16 * SX;
  s.H1 = p;
  p += WARPS * 16 * SH;
  s.DA = p;
  if (train) p += WARPS * 16 * SH;
  float *f = reinterpret_cast<float *>(p);
  s.b1 = f;
  s.b2 = f + NH;
  s.w3 = f + 2 * NH;
  return s;
}
constexpr size_t smem_bytes(bool train) {
  return sizeof(bf16) * (size_t)(NH * SX + NH * SH + (train ? NH * SH : 0) + WARPS * 16 * SX +
                                 WARPS * 16 * SH + (train ? WARPS * 16 * SH : 0)) +
         sizeof(float) * 3 * NH;
}
// FP32 gradient accumulators of a training block, after the operand area
constexpr size_t ACC_FLOATS = NH * KIN + NH * NH + 3 * NH + 1 + 1;  // ... + b3 + loss

// ------------------------------------------------------------------ inference (tcgen05)
// One CTA of 128 threads per 128-cell tile (persistent over tiles), thread r owning cell
// row r.  Shared memory, canonical K-major BF16 tiles (ffv_tc.cuh): the feature tile X
// [128][144] (later the first hidden layer H [128][64] over it), W1 [64][144], W2 [64][64],
// then b1, b2, w3 in FP32.  Tensor memory: 64 FP32 columns x 128 lanes, the accumulator of
// either layer (lane r = row r).  Per tile: rows built (stencil gather or copied feature
// rows) -> 9 MMAs (K = 16) of layer 1 -> GELU + BF16 of row r into H -> 4 MMAs of layer 2 ->
// GELU, the w3 dot product and the sigmoid of row r.  The MMAs take ~1 us of a tile's time:
// the gather dominates, and three CTAs per SM overlap one another's phases.
constexpr int TC_ROWS = 128;
constexpr int TC_SBO_X = (KIN / 8) * 128, TC_SBO_H = (NH / 8) * 128;
constexpr int TC_W1 = TC_ROWS * KIN * 2;     // byte offsets in the dynamic shared memory
constexpr int TC_W2 = TC_W1 + NH * KIN * 2;
constexpr int TC_VEC = TC_W2 + NH * NH * 2;
constexpr int TC_SMEM = TC_VEC + 3 * NH * 4;
constexpr int TC_CTAS_PER_SM = 3;
constexpr int TC_TMEM_COLS = 64;
constexpr int TC_WAIT_POLLS = 1 << 22;  // an MMA group takes ~1 us; this is far beyond it
static_assert(TC_SMEM * TC_CTAS_PER_SM <= 227 * 1024, "shared memory of three CTAs per SM");
static_assert(TC_TMEM_COLS * TC_CTAS_PER_SM <= 512, "tensor memory of three CTAs per SM");

template <bool GATHER>
__global__ void __launch_bounds__(TC_ROWS, TC_CTAS_PER_SM)
    mlp_infer_tc(ffv_dmesh m, const float *__restrict__ F, const float *__restrict__ norm,
                 const bf16 *__restrict__ X, int64_t n, const bf16 *__restrict__ W1,
                 const bf16 *__restrict__ W2, const float *__restrict__ P, float *__restrict__ prob,
                 uint8_t *__restrict__ marks, float threshold, int accumulate,
                 unsigned *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t tmem_holder;
  __shared__ __align__(8) uint64_t bar;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < NH * (KIN / 8); i += TC_ROWS) {
    const int r = i / (KIN / 8), ch = i % (KIN / 8);
    *reinterpret_cast<uint4 *>(sm + TC_W1 + tc::kmajor_offset(r, 8 * ch, KIN)) =
        *reinterpret_cast<const uint4 *>(W1 + r * KIN + 8 * ch);
  }
  for (int i = tid; i < NH * (NH / 8); i += TC_ROWS) {
    const int r = i / (NH / 8), ch = i % (NH / 8);
    *reinterpret_cast<uint4 *>(sm + TC_W2 + tc::kmajor_offset(r, 8 * ch, NH)) =
        *reinterpret_cast<const uint4 *>(W2 + r * NH + 8 * ch);
  }
  float *b1s = reinterpret_cast<float *>(sm + TC_VEC), *b2s = b1s + NH, *w3s = b2s + NH;
  for (int i = tid; i < NH; i += TC_ROWS) {
    b1s[i] = P[OFF_B1 + i];
    b2s[i] = P[OFF_B2 + i];
    w3s[i] = P[OFF_W3 + i];
  }
  if (warp == 0) tc::tmem_alloc(&tmem_holder, TC_TMEM_COLS);
  if (tid == 0) tc::mbar_init(&bar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_holder;
  const uint32_t row_tmem = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 lanes
  const uint32_t xs = tc::smem_addr(sm), w1s = tc::smem_addr(sm + TC_W1),
                 w2s = tc::smem_addr(sm + TC_W2);
  constexpr uint32_t idesc = tc::idesc_bf16_f32(TC_ROWS, NH);
  const float b3 = P[OFF_B3];
  float mean[5], istd[5];
#pragma unroll
  for (int q = 0; q < 5; q++) {
    mean[q] = GATHER ? norm[q] : 0.0f;
    istd[q] = GATHER ? 1.0f / norm[5 + q] : 1.0f;
  }
  const int64_t ntiles = (n + TC_ROWS - 1) / TC_ROWS;
  int failed_parity = -1;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t c = t * TC_ROWS + tid;
    const bool valid = c < n;
    auto put = [&](int ch, uint4 v) {
      *reinterpret_cast<uint4 *>(sm + tc::kmajor_offset(tid, 8 * ch, KIN)) = v;
    };
    if (!valid) {
#pragma unroll 1
      for (int ch = 0; ch < KIN / 8; ch++) put(ch, make_uint4(0u, 0u, 0u, 0u));
    } else if (GATHER) {
      cell_features(m, F, mean, istd, (int32_t)c, put);
    } else {
#pragma unroll
      for (int ch = 0; ch < KIN / 8; ch++) put(ch, *reinterpret_cast<const uint4 *>(X + c * KIN + 8 * ch));
    }
    // layer 1: pre-activations of the 128 rows into tensor memory
    tc::fence_async_shared();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
#pragma unroll
      for (int kk = 0; kk < KIN / 16; kk++)
        tc::mma_bf16(tmem, tc::sdesc(xs + 256 * kk, 128, TC_SBO_X), tc::sdesc(w1s + 256 * kk, 128, TC_SBO_X),
                     idesc, kk > 0);
      tc::commit(&bar);
    }
    if (__syncthreads_or(!tc::mbar_wait(&bar, 0, TC_WAIT_POLLS))) {
      failed_parity = 0;
      break;
    }
    tc::fence_after_sync();
#pragma unroll
    for (int c0 = 0; c0 < NH; c0 += 16) {
      float a[16];
      tc::tmem_ld16(row_tmem + c0, a);
      uint32_t pk[8];
#pragma unroll
      for (int j = 0; j < 8; j++)
        pk[j] = pack2(__float2bfloat16_rn(gelu(a[2 * j] + b1s[c0 + 2 * j])),
                      __float2bfloat16_rn(gelu(a[2 * j + 1] + b1s[c0 + 2 * j + 1])));
      *reinterpret_cast<uint4 *>(sm + tc::kmajor_offset(tid, c0, NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      *reinterpret_cast<uint4 *>(sm + tc::kmajor_offset(tid, c0 + 8, NH)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
    // layer 2 over H (the feature tile's first 16 KB: layer 1 has finished reading it)
    tc::fence_async_shared();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
#pragma unroll
      for (int kk = 0; kk < NH / 16; kk++)
        tc::mma_bf16(tmem, tc::sdesc(xs + 256 * kk, 128, TC_SBO_H), tc::sdesc(w2s + 256 * kk, 128, TC_SBO_H),
                     idesc, kk > 0);
      tc::commit(&bar);
    }
    if (__syncthreads_or(!tc::mbar_wait(&bar, 1, TC_WAIT_POLLS))) {
      failed_parity = 1;
      break;
    }
    tc::fence_after_sync();
    float z = 0.0f;
#pragma unroll
    for (int c0 = 0; c0 < NH; c0 += 16) {
      float a[16];
      tc::tmem_ld16(row_tmem + c0, a);
#pragma unroll
      for (int j = 0; j < 16; j++) z += gelu(a[j] + b2s[c0 + j]) * w3s[c0 + j];
    }
    if (valid) {
      const float p = 1.0f / (1.0f + expf(-(z + b3)));
      if (prob) prob[c] = p;
      if (marks) {
        const uint8_t hit = p > threshold ? 1 : 0;
        marks[c] = accumulate ? (uint8_t)(marks[c] | hit) : hit;
      }
    }
    // the next tile's MMAs (after its barrier) overwrite the accumulator these loads read
    tc::fence_before_sync();
  }
  if (failed_parity >= 0) {
    // a wait ran out: report it, give the MMAs in flight one more bounded wait, free the
    // tensor memory and leave (the tiles not finished keep their outputs)
    if (tid == 0) atomicOr(err, 1u);
    tc::mbar_wait(&bar, (uint32_t)failed_parity, TC_WAIT_POLLS);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
}

// row index of sample i of a training step: identity (seed 0) or a hashed draw
__device__ __forceinline__ int64_t sample_row(uint64_t seed, int64_t step, int64_t i, int64_t N) {
  if (seed == 0) return i;
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(step * 1315423911ll + i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (int64_t)(z % (uint64_t)N);
}

// reduce a per-lane column partial over the eight row groups (lanes with the same q)
__device__ __forceinline__ float rows_sum(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 8);
  v += __shfl_xor_sync(0xffffffffu, v, 16);
  return v;
}

// weight gradient dW[m][j] += sum_s A[s][m] B[s][j] over the tile's 16 samples, A = DA
// (16 x 64, stride SH), B = a 16 x (8 ntiles) BF16 tile of stride `sb`; columns j >= jmax
// are dropped
template <int NT>
__device__ __forceinline__ void grad_outer(const bf16 *DA, const bf16 *B, int sb, float *acc,
                                           int acc_stride, int jmax) {
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll 1
  for (int mt = 0; mt < NH / 16; mt++) {
    const int m0 = mt * 16 + g;
    const uint32_t a0 = pack2(DA[(2 * q) * SH + m0], DA[(2 * q + 1) * SH + m0]);
    const uint32_t a1 = pack2(DA[(2 * q) * SH + m0 + 8], DA[(2 * q + 1) * SH + m0 + 8]);
    const uint32_t a2 = pack2(DA[(2 * q + 8) * SH + m0], DA[(2 * q + 9) * SH + m0]);
    const uint32_t a3 = pack2(DA[(2 * q + 8) * SH + m0 + 8], DA[(2 * q + 9) * SH + m0 + 8]);
#pragma unroll 2
    for (int nt = 0; nt < NT; nt++) {
      const int j = nt * 8 + g;
      const uint32_t b0 = pack2(B[(2 * q) * sb + j], B[(2 * q + 1) * sb + j]);
      const uint32_t b1 = pack2(B[(2 * q + 8) * sb + j], B[(2 * q + 9) * sb + j]);
      float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      mma16816(c, a0, a1, a2, a3, b0, b1);
      const int col = nt * 8 + 2 * q;
      if (col < jmax) {
        atomicAdd(acc + m0 * acc_stride + col, c[0]);
        atomicAdd(acc + (m0 + 8) * acc_stride + col, c[2]);
      }
      if (col + 1 < jmax) {
        atomicAdd(acc + m0 * acc_stride + col + 1, c[1]);
        atomicAdd(acc + (m0 + 8) * acc_stride + col + 1, c[3]);
      }
    }
  }
}

// gradient of the mean binary cross-entropy over B samples (rows drawn by sample_row),
// added to G (FP32, NPARAM, zeroed by the caller); loss sum added to *loss
__global__ void __launch_bounds__(TPB) mlp_train_kernel(const bf16 *__restrict__ X,
                                                        const float *__restrict__ y, int64_t N,
                                                        int64_t B, uint64_t seed, int64_t step,
                                                        const bf16 *__restrict__ W1,
                                                        const bf16 *__restrict__ W2,
                                                        const bf16 *__restrict__ W2T,
                                                        const float *__restrict__ P,
                                                        float *__restrict__ G,
                                                        float *__restrict__ loss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Smem s = carve(smem, true);
  float *acc = reinterpret_cast<float *>(smem + smem_bytes(true));
  float *gW1 = acc, *gW2 = acc + NH * KIN, *gb1 = gW2 + NH * NH, *gb2 = gb1 + NH, *gw3 = gb2 + NH;
  float *gb3 = gw3 + NH, *gl = gb3 + 1;
  for (int i = threadIdx.x; i < (int)ACC_FLOATS; i += blockDim.x) acc[i] = 0.0f;
  stage_weights(s, W1, W2, W2T, P, true);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  bf16 *Xs = s.X + warp * 16 * SX, *H1s = s.H1 + warp * 16 * SH, *DAs = s.DA + warp * 16 * SH;
  const float b3 = P[OFF_B3], invB = 1.0f / (float)B;
  const int64_t ntiles = (B + 15) / 16;
  for (int64_t t = (int64_t)blockIdx.x * WARPS + warp; t < ntiles; t += (int64_t)gridDim.x * WARPS) {
    const int64_t i0 = t * 16;
    const int valid = (int)((B - i0) < 16 ? (B - i0) : 16);
    load_tile(Xs, X, valid, [&](int r) { return sample_row(seed, step, i0 + r, N); });
    float a1[8][4], a2[8][4], zg, zg8;
    tile_forward(s, Xs, H1s, a1, a2, zg, zg8);
    // output layer: d loss / d z = (p - y) / B
    float dzg = 0.0f, dzg8 = 0.0f;
    if (g < valid) {
      const float p = 1.0f / (1.0f + expf(-(zg + b3))), yy = y[sample_row(seed, step, i0 + g, N)];
      dzg = (p - yy) * invB;
      if (q == 0) atomicAdd(gl, -(yy * logf(fmaxf(p, 1e-12f)) + (1.0f - yy) * logf(fmaxf(1.0f - p, 1e-12f))));
    }
    if (g + 8 < valid) {
      const float p = 1.0f / (1.0f + expf(-(zg8 + b3))),
                  yy = y[sample_row(seed, step, i0 + g + 8, N)];
      dzg8 = (p - yy) * invB;
      if (q == 0)
        atomicAdd(gl, -(yy * logf(fmaxf(p, 1e-12f)) + (1.0f - yy) * logf(fmaxf(1.0f - p, 1e-12f))));
    }
    {
      float d3 = (q == 0) ? dzg + dzg8 : 0.0f;
      d3 = rows_sum(d3);
      if (lane == 0) atomicAdd(gb3, d3);
    }
    // second hidden layer
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int col = nt * 8 + 2 * q;
      float w3v[2] = {s.w3[col], s.w3[col + 1]};
      float dw[2], db[2];
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const float h_g = gelu(a2[nt][e]), h_g8 = gelu(a2[nt][2 + e]);
        dw[e] = rows_sum(dzg * h_g + dzg8 * h_g8);
        const float d_g = dzg * w3v[e] * gelu_grad(a2[nt][e]);
        const float d_g8 = dzg8 * w3v[e] * gelu_grad(a2[nt][2 + e]);
        a2[nt][e] = d_g;
        a2[nt][2 + e] = d_g8;
        db[e] = rows_sum(d_g + d_g8);
      }
      if (g == 0) {
        atomicAdd(gw3 + col, dw[0]);
        atomicAdd(gw3 + col + 1, dw[1]);
        atomicAdd(gb2 + col, db[0]);
        atomicAdd(gb2 + col + 1, db[1]);
      }
      *reinterpret_cast<__nv_bfloat162 *>(DAs + g * SH + col) = __floats2bfloat162_rn(a2[nt][0], a2[nt][1]);
      *reinterpret_cast<__nv_bfloat162 *>(DAs + (g + 8) * SH + col) =
          __floats2bfloat162_rn(a2[nt][2], a2[nt][3]);
    }
    __syncwarp();
    // dW2 = da2^T h1
    grad_outer<8>(DAs, H1s, SH, gW2, NH, NH);
    // dh1 = da2 W2, then da1 = dh1 * gelu'(a1)
    float dh[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) dh[nt][0] = dh[nt][1] = dh[nt][2] = dh[nt][3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < NH / 16; kk++) {
      const int k0 = kk * 16 + 2 * q;
      const uint32_t d0 = ld32(DAs + g * SH + k0), d1 = ld32(DAs + (g + 8) * SH + k0);
      const uint32_t d2 = ld32(DAs + g * SH + k0 + 8), d3 = ld32(DAs + (g + 8) * SH + k0 + 8);
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const bf16 *w = s.W2T + (nt * 8 + g) * SH + k0;
        mma16816(dh[nt], d0, d1, d2, d3, ld32(w), ld32(w + 8));
      }
    }
    __syncwarp();
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int col = nt * 8 + 2 * q;
      float db[2];
#pragma unroll
      for (int e = 0; e < 2; e++) {
        dh[nt][e] *= gelu_grad(a1[nt][e]);
        dh[nt][2 + e] *= gelu_grad(a1[nt][2 + e]);
        db[e] = rows_sum(dh[nt][e] + dh[nt][2 + e]);
      }
      if (g == 0) {
        atomicAdd(gb1 + col, db[0]);
        atomicAdd(gb1 + col + 1, db[1]);
      }
      *reinterpret_cast<__nv_bfloat162 *>(DAs + g * SH + col) = __floats2bfloat162_rn(dh[nt][0], dh[nt][1]);
      *reinterpret_cast<__nv_bfloat162 *>(DAs + (g + 8) * SH + col) =
          __floats2bfloat162_rn(dh[nt][2], dh[nt][3]);
    }
    __syncwarp();
    // dW1 = da1^T x
    grad_outer<KIN / 8>(DAs, Xs, SX, gW1, KIN, NIN);
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NH * NIN; i += blockDim.x) {
    const int r = i / NIN, k = i % NIN;
    const float v = gW1[r * KIN + k];
    if (v != 0.0f) atomicAdd(G + OFF_W1 + i, v);
  }
  for (int i = threadIdx.x; i < NH * NH; i += blockDim.x)
    if (gW2[i] != 0.0f) atomicAdd(G + OFF_W2 + i, gW2[i]);
  for (int i = threadIdx.x; i < NH; i += blockDim.x) {
    atomicAdd(G + OFF_B1 + i, gb1[i]);
    atomicAdd(G + OFF_B2 + i, gb2[i]);
    atomicAdd(G + OFF_W3 + i, gw3[i]);
  }
  if (threadIdx.x == 0) {
    atomicAdd(G + OFF_B3, *gb3);
    atomicAdd(loss, *gl);
  }
}

// AdamW (decoupled weight decay on W1, W2, w3; none on the biases)
__global__ void mlp_adamw(float *__restrict__ P, const float *__restrict__ G, float *__restrict__ M,
                          float *__restrict__ V, float lr, float wd, float b1, float b2, float eps,
                          float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x) {
    const float gr = G[i];
    const float m = b1 * M[i] + (1.0f - b1) * gr;
    const float v = b2 * V[i] + (1.0f - b2) * gr * gr;
    M[i] = m;
    V[i] = v;
    const bool decay = (i < OFF_B1) || (i >= OFF_W2 && i < OFF_B2) || (i >= OFF_W3 && i < OFF_B3);
    float p = P[i];
    if (decay) p -= lr * wd * p;
    p -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    P[i] = p;
  }
}

}  // namespace

struct ffv_mlp {
  int device, nsm;
  cudaStream_t stream;
  float *d_P, *d_G, *d_M, *d_V, *d_norm, *d_loss;
  bf16 *d_W1, *d_W2, *d_W2T;
  int64_t t;  // AdamW step count
  // predict buffers
  int64_t cap;
  float *d_F, *d_prob;
  // inference wait timeouts: mapped pinned word, set by the device, read by the host
  unsigned *h_err, *d_err;
};

namespace {
int mlp_cuda(cudaError_t e) { return e == cudaSuccess ? FFV_OK : FFV_ERR_CUDA; }
#define MCK(x)                                  \
  do {                                          \
    int _r = mlp_cuda(x);                       \
    if (_r != FFV_OK) return _r;                \
  } while (0)

int repack(ffv_mlp *m) {
  mlp_pack<<<64, 256, 0, m->stream>>>(m->d_P, m->d_W1, m->d_W2, m->d_W2T);
  return mlp_cuda(cudaGetLastError());
}

int ensure_cap(ffv_mlp *m, int64_t n) {
  if (m->cap >= n) return FFV_OK;
  cudaFree(m->d_F);
  cudaFree(m->d_prob);
  m->d_F = m->d_prob = nullptr;
  m->cap = 0;
  if (cudaMalloc(&m->d_F, sizeof(float) * 5 * n) != cudaSuccess ||
      cudaMalloc(&m->d_prob, sizeof(float) * n) != cudaSuccess)
    return FFV_ERR_NOMEM;
  m->cap = n;
  return FFV_OK;
}

// the fused inference kernel over n rows: feature rows X (dm unused), or the stencil gather
// of the fields F on mesh dm (X unused); probabilities and/or marks out
int infer(ffv_mlp *m, bool gather, const ffv_dmesh &dm, const float *F, const bf16 *X, int64_t n,
          float *prob, uint8_t *marks, float threshold, int accumulate, cudaStream_t st) {
  if (n <= 0) return FFV_OK;
  const int64_t tiles = (n + TC_ROWS - 1) / TC_ROWS;
  int64_t blocks = (int64_t)m->nsm * TC_CTAS_PER_SM;
  if (blocks > tiles) blocks = tiles;
  if (gather) {
    MCK(cudaFuncSetAttribute(mlp_infer_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    mlp_infer_tc<true><<<(unsigned)blocks, TC_ROWS, TC_SMEM, st>>>(
        dm, F, m->d_norm, nullptr, n, m->d_W1, m->d_W2, m->d_P, prob, marks, threshold, accumulate, m->d_err);
  } else {
    MCK(cudaFuncSetAttribute(mlp_infer_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    mlp_infer_tc<false><<<(unsigned)blocks, TC_ROWS, TC_SMEM, st>>>(
        dm, nullptr, nullptr, X, n, m->d_W1, m->d_W2, m->d_P, prob, marks, threshold, accumulate, m->d_err);
  }
  return mlp_cuda(cudaGetLastError());
}

// a timeout recorded by an inference kernel that has finished (the word is cleared)
int take_timeout(ffv_mlp *m) {
  const unsigned e = *(volatile unsigned *)m->h_err;
  if (!e) return FFV_OK;
  *(volatile unsigned *)m->h_err = 0u;
  return FFV_ERR_TIMEOUT;
}

int grad(ffv_mlp *m, const bf16 *X, const float *y, int64_t N, int64_t B, uint64_t seed,
         int64_t step) {
  MCK(cudaMemsetAsync(m->d_G, 0, sizeof(float) * NPARAM, m->stream));
  MCK(cudaMemsetAsync(m->d_loss, 0, sizeof(float), m->stream));
  const size_t sb = smem_bytes(true) + sizeof(float) * ACC_FLOATS;
  MCK(cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb));
  const int64_t tiles = (B + 15) / 16;
  int64_t blocks = (tiles + WARPS - 1) / WARPS;
  if (blocks > 152) blocks = 152;
  mlp_train_kernel<<<(unsigned)blocks, TPB, sb, m->stream>>>(X, y, N, B, seed, step, m->d_W1,
                                                             m->d_W2, m->d_W2T, m->d_P, m->d_G,
                                                             m->d_loss);
  return mlp_cuda(cudaGetLastError());
}

// seeded host initialisation: weights uniform in +-1/sqrt(fan_in), biases zero
void init_params(float *P, uint64_t seed) {
  uint64_t s = seed ? seed : 1;
  auto next = [&]() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  memset(P, 0, sizeof(float) * NPARAM);
  for (int i = 0; i < NH * NIN; i++) P[OFF_W1 + i] = (float)((2.0 * next() - 1.0) / sqrt((double)NIN));
  for (int i = 0; i < NH * NH; i++) P[OFF_W2 + i] = (float)((2.0 * next() - 1.0) / sqrt((double)NH));
  for (int i = 0; i < NH; i++) P[OFF_W3 + i] = (float)((2.0 * next() - 1.0) / sqrt((double)NH));
}
}  // namespace

// defined in ffv_api.cu
int ffv_ctx_view(ffv_ctx *ctx, int *device, cudaStream_t *st, ffv_dmesh *dm, const double **S,
                 const M5Consts **k, int *model, double *gamma0, double *pinf0);

namespace {
struct CtxView {
  int device, model;
  cudaStream_t st;
  ffv_dmesh dm;
  const double *S;
  const M5Consts *k;
  double gamma0, pinf0;
};
int view(ffv_ctx *ctx, CtxView &v) {
  return ffv_ctx_view(ctx, &v.device, &v.st, &v.dm, &v.S, &v.k, &v.model, &v.gamma0, &v.pinf0);
}
void launch_fields(const CtxView &v, float *F) {
  if (v.model == 5) ffv_m5f_indicator_fields(v.dm.n, *v.k, v.S, F, v.st);
  else ffv_m0_indicator_fields(v.dm.n, v.gamma0, v.pinf0, v.S, F, v.st);
}
}  // namespace

extern "C" {

int ffv_mlp_create(ffv_mlp **out, int device, uint64_t seed) {
  if (!out) return FFV_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return FFV_ERR_CUDA;
  MCK(cudaSetDevice(device));
  ffv_mlp *m = (ffv_mlp *)calloc(1, sizeof(ffv_mlp));
  if (!m) return FFV_ERR_NOMEM;
  m->device = device;
  if (cudaDeviceGetAttribute(&m->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      m->nsm < 1)
    m->nsm = 1;
  float *h = (float *)malloc(sizeof(float) * NPARAM);
  const float norm[10] = {0, 0, 0, 0, 0, 1, 1, 1, 1, 1};
  int rc = FFV_OK;
  if (!h || cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&m->d_P, sizeof(float) * NPARAM) != cudaSuccess ||
      cudaMalloc(&m->d_G, sizeof(float) * NPARAM) != cudaSuccess ||
      cudaMalloc(&m->d_M, sizeof(float) * NPARAM) != cudaSuccess ||
      cudaMalloc(&m->d_V, sizeof(float) * NPARAM) != cudaSuccess ||
      cudaMalloc(&m->d_norm, sizeof(float) * 10) != cudaSuccess ||
      cudaMalloc(&m->d_loss, sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->d_W1, sizeof(bf16) * NH * KIN) != cudaSuccess ||
      cudaMalloc(&m->d_W2, sizeof(bf16) * NH * NH) != cudaSuccess ||
      cudaMalloc(&m->d_W2T, sizeof(bf16) * NH * NH) != cudaSuccess ||
      cudaHostAlloc(&m->h_err, sizeof(unsigned), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer(&m->d_err, m->h_err, 0) != cudaSuccess) {
    rc = FFV_ERR_NOMEM;
  }
  if (rc == FFV_OK) *m->h_err = 0u;
  if (rc == FFV_OK) {
    init_params(h, seed);
    if (cudaMemcpy(m->d_P, h, sizeof(float) * NPARAM, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(m->d_norm, norm, sizeof(norm), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m->d_M, 0, sizeof(float) * NPARAM) != cudaSuccess ||
        cudaMemset(m->d_V, 0, sizeof(float) * NPARAM) != cudaSuccess)
      rc = FFV_ERR_CUDA;
  }
  if (rc == FFV_OK) rc = repack(m);
  if (rc == FFV_OK && cudaStreamSynchronize(m->stream) != cudaSuccess) rc = FFV_ERR_CUDA;
  free(h);
  if (rc != FFV_OK) {
    ffv_mlp_destroy(m);
    return rc;
  }
  *out = m;
  return FFV_OK;
}

int ffv_mlp_destroy(ffv_mlp *m) {
  if (!m) return FFV_OK;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  cudaFree(m->d_P);
  cudaFree(m->d_G);
  cudaFree(m->d_M);
  cudaFree(m->d_V);
  cudaFree(m->d_norm);
  cudaFree(m->d_loss);
  cudaFree(m->d_W1);
  cudaFree(m->d_W2);
  cudaFree(m->d_W2T);
  cudaFree(m->d_F);
  cudaFree(m->d_prob);
  cudaFreeHost(m->h_err);
  if (m->stream) cudaStreamDestroy(m->stream);
  free(m);
  return FFV_OK;
}

int ffv_mlp_get_params(ffv_mlp *m, float *params) {
  if (!m || !params) return FFV_ERR_ARG;
  MCK(cudaSetDevice(m->device));
  MCK(cudaMemcpyAsync(params, m->d_P, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  return FFV_OK;
}

int ffv_mlp_set_params(ffv_mlp *m, const float *params) {
  if (!m || !params) return FFV_ERR_ARG;
  MCK(cudaSetDevice(m->device));
  MCK(cudaMemcpyAsync(m->d_P, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemsetAsync(m->d_M, 0, sizeof(float) * NPARAM, m->stream));
  MCK(cudaMemsetAsync(m->d_V, 0, sizeof(float) * NPARAM, m->stream));
  m->t = 0;
  int rc = repack(m);
  if (rc != FFV_OK) return rc;
  MCK(cudaStreamSynchronize(m->stream));
  return FFV_OK;
}

int ffv_mlp_set_norm(ffv_mlp *m, const float *mean, const float *stdev) {
  if (!m || !mean || !stdev) return FFV_ERR_ARG;
  float h[10];
  for (int q = 0; q < 5; q++) {
    if (!(stdev[q] > 0.0f)) return FFV_ERR_ARG;
    h[q] = mean[q];
    h[5 + q] = stdev[q];
  }
  MCK(cudaSetDevice(m->device));
  MCK(cudaMemcpyAsync(m->d_norm, h, sizeof(h), cudaMemcpyHostToDevice, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  return FFV_OK;
}

int ffv_mlp_fields(ffv_ctx *ctx, float *F_dev) {
  CtxView v;
  int rc = view(ctx, v);
  if (rc != FFV_OK) return rc;
  if (!F_dev) return FFV_ERR_ARG;
  MCK(cudaSetDevice(v.device));
  launch_fields(v, F_dev);
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(v.st));
  return FFV_OK;
}

int ffv_mlp_features(ffv_ctx *ctx, ffv_mlp *m, void *X_dev) {
  if (!m || !X_dev) return FFV_ERR_ARG;
  CtxView v;
  int rc = view(ctx, v);
  if (rc != FFV_OK) return rc;
  if (v.device != m->device) return FFV_ERR_ARG;
  MCK(cudaSetDevice(v.device));
  rc = ensure_cap(m, v.dm.n);
  if (rc != FFV_OK) return rc;
  launch_fields(v, m->d_F);
  mlp_gather<<<(unsigned)((v.dm.n + 127) / 128), 128, 0, v.st>>>(v.dm, m->d_F, m->d_norm,
                                                                  (bf16 *)X_dev);
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(v.st));
  return FFV_OK;
}

int ffv_mlp_forward(ffv_mlp *m, const void *X_dev, int64_t n, float *prob_dev) {
  if (!m || !X_dev || !prob_dev || n < 0) return FFV_ERR_ARG;
  MCK(cudaSetDevice(m->device));
  if (n == 0) return FFV_OK;
  int rc = infer(m, false, ffv_dmesh{}, nullptr, (const bf16 *)X_dev, n, prob_dev, nullptr, 0.0f, 0,
                 m->stream);
  if (rc != FFV_OK) return rc;
  MCK(cudaStreamSynchronize(m->stream));
  return take_timeout(m);
}

int ffv_mlp_predict(ffv_ctx *ctx, ffv_mlp *m, float *prob_host) {
  if (!m || !prob_host) return FFV_ERR_ARG;
  CtxView v;
  int rc = view(ctx, v);
  if (rc != FFV_OK) return rc;
  if (v.device != m->device) return FFV_ERR_ARG;
  MCK(cudaSetDevice(v.device));
  rc = ensure_cap(m, v.dm.n);
  if (rc != FFV_OK) return rc;
  launch_fields(v, m->d_F);
  rc = infer(m, true, v.dm, m->d_F, nullptr, v.dm.n, m->d_prob, nullptr, 0.0f, 0, v.st);
  if (rc != FFV_OK) return rc;
  MCK(cudaMemcpyAsync(prob_host, m->d_prob, sizeof(float) * v.dm.n, cudaMemcpyDeviceToHost, v.st));
  MCK(cudaStreamSynchronize(v.st));
  return take_timeout(m);
}

int ffv_mlp_mark(ffv_ctx *ctx, ffv_mlp *m, float threshold, uint8_t *marks_dev,
                 int32_t accumulate) {
  if (!m || !marks_dev) return FFV_ERR_ARG;
  CtxView v;
  int rc = view(ctx, v);
  if (rc != FFV_OK) return rc;
  if (v.device != m->device) return FFV_ERR_ARG;
  MCK(cudaSetDevice(v.device));
  rc = ensure_cap(m, v.dm.n);
  if (rc != FFV_OK) return rc;
  // a timeout of an earlier call (this call is not waited for)
  rc = take_timeout(m);
  if (rc != FFV_OK) return rc;
  launch_fields(v, m->d_F);
  return infer(m, true, v.dm, m->d_F, nullptr, v.dm.n, nullptr, marks_dev, threshold, accumulate, v.st);
}

int ffv_mlp_grad(ffv_mlp *m, const void *X_dev, const float *y_dev, int64_t B, float *grad_host,
                 float *loss_host) {
  if (!m || !X_dev || !y_dev || !grad_host || B < 1) return FFV_ERR_ARG;
  MCK(cudaSetDevice(m->device));
  int rc = grad(m, (const bf16 *)X_dev, y_dev, B, B, 0, 0);
  if (rc != FFV_OK) return rc;
  MCK(cudaMemcpyAsync(grad_host, m->d_G, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, m->stream));
  float l = 0.0f;
  MCK(cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  if (loss_host) *loss_host = l / (float)B;
  return FFV_OK;
}

int ffv_mlp_train(ffv_mlp *m, const void *X_dev, const float *y_dev, int64_t N, int32_t batch,
                  int32_t steps, float lr, float wd, uint64_t seed, float *loss_host) {
  if (!m || !X_dev || !y_dev || N < 1 || batch < 1 || steps < 0 || seed == 0) return FFV_ERR_ARG;
  MCK(cudaSetDevice(m->device));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int32_t i = 0; i < steps; i++) {
    int rc = grad(m, (const bf16 *)X_dev, y_dev, N, batch, seed, m->t);
    if (rc != FFV_OK) return rc;
    m->t++;
    const float c1 = 1.0f - powf(b1, (float)m->t), c2 = 1.0f - powf(b2, (float)m->t);
    mlp_adamw<<<(NPARAM + 255) / 256, 256, 0, m->stream>>>(m->d_P, m->d_G, m->d_M, m->d_V, lr, wd,
                                                           b1, b2, eps, c1, c2);
    rc = repack(m);
    if (rc != FFV_OK) return rc;
    if (loss_host) {
      float l = 0.0f;
      MCK(cudaMemcpyAsync(&l, m->d_loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
      MCK(cudaStreamSynchronize(m->stream));
      loss_host[i] = l / (float)batch;
    }
  }
  MCK(cudaStreamSynchronize(m->stream));
  return FFV_OK;
}

}  // extern "C"
