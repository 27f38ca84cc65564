// Face-frame helpers and state layout of model 5, shared by the FP64 and FP32-flux kernels
// (templated on the scalar type; the FP64 instantiation is the reference-exact one).
#pragma once
#include "ffv_device.cuh"

namespace {

template <int N>
struct K5 {
  static constexpr int NEQ = 3 * N + 12, NC = N + 4;
  static constexpr int i0 = 0, i1 = N, i2 = N + 3, i3 = N + 4, i4 = 2 * N + 3, i5 = 3 * N + 3;
};

template <int S, typename T>
__device__ __forceinline__ T sgn(T x) {
  return S > 0 ? x : -x;
}
// frame of face F: local axis q (0 = n, 1 = t1, 2 = t2) -> global axis and sign
template <int F, int Q> struct Fr {
  static constexpr int ax = Q == 0 ? fr_n_axis(F) : (Q == 1 ? fr_t1_axis(F) : fr_t2_axis(F));
  static constexpr int sg = Q == 0 ? fr_n_sign(F) : (Q == 1 ? fr_t1_sign(F) : fr_t2_sign(F));
};
template <int F, int Q, typename T>
__device__ __forceinline__ T loc(const T v[3]) {
  return sgn<Fr<F, Q>::sg>(v[Fr<F, Q>::ax]);
}
// global component A of a*n + b*t1 + c*t2
template <int F, int A, typename T>
__device__ __forceinline__ T glob(T a, T b, T c) {
  return Fr<F, 0>::ax == A ? sgn<Fr<F, 0>::sg>(a)
                           : (Fr<F, 1>::ax == A ? sgn<Fr<F, 1>::sg>(b) : sgn<Fr<F, 2>::sg>(c));
}
// R T R^T for the frame of F (rotate_vectors.c:73-106, rows n, t1, t2): a signed permutation
template <int F, typename R>
__device__ __forceinline__ void tens_to_local(const R T[3][3], R out[3][3]) {
#define TL(I, J) out[I][J] = sgn<Fr<F, I>::sg * Fr<F, J>::sg>(T[Fr<F, I>::ax][Fr<F, J>::ax])
  TL(0, 0); TL(0, 1); TL(0, 2); TL(1, 0); TL(1, 1); TL(1, 2); TL(2, 0); TL(2, 1); TL(2, 2);
#undef TL
}
template <int F, typename R>
__device__ __forceinline__ void tens_to_global(const R T[3][3], R out[3][3]) {
#define TG(I, J) out[Fr<F, I>::ax][Fr<F, J>::ax] = sgn<Fr<F, I>::sg * Fr<F, J>::sg>(T[I][J])
  TG(0, 0); TG(0, 1); TG(0, 2); TG(1, 0); TG(1, 1); TG(1, 2); TG(2, 0); TG(2, 1); TG(2, 2);
#undef TG
}

}  // namespace
