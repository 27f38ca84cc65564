// J2 radial-return plasticity of a cell's deformation tensor, in FP64 (no counterpart in the
// reference: its plastic step is only prototyped, strdata.h:809, and the call commented out,
// m5_relaxation_solid.c:14).
//
// With G = A A^T = Q diag(lam) Q^T (cyclic Jacobi, Golub & Van Loan, Matrix Computations,
// sec. 8.5), the Hencky strain h_i = ln(lam_i) / 2 splits into its mean m (the volume, kept)
// and the deviator d_i.  The hyperelastic solid's von Mises stress (state_equation.c:143-204,
// the mu term) in the principal frame is that of s_i = -mu |G|^(-1/6) (t_i - mean t),
// t_i = g_i^2 - |G|^(1/3) g_i, g_i = exp(2 (m + beta d_i)).  Where it exceeds the yield
// stress at beta = 1, the deviator is scaled by the largest beta in [0, 1] (60 bisection
// steps) whose stress lies on or inside the yield surface, and A <- Q diag(exp((beta - 1) d_i))
// Q^T A.  The total energy and the materials' alpha rho e are kept: the elastic energy
// released goes into the materials' internal energy (the pressure recovery subtracts e_el
// from alpha rho e).  The same steps, in the same order, as the oracle's restatement.
#pragma once
#include <math.h>

#include "ffv_cvt.cuh"
#include "ffv_m5.cuh"

__device__ inline void plastic_jacobi3(const double G[9], double lam[3], double Q[9]) {
  double a[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      a[i][j] = G[3 * i + j];
      Q[3 * i + j] = (i == j) ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 32; sweep++) {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    const double dg = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (!(off > 1e-32 * dg)) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (a[p][q] == 0.0) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < 3; r++) {
          const double arp = a[r][p], arq = a[r][q];
          a[r][p] = c * arp - s * arq;
          a[r][q] = s * arp + c * arq;
        }
        for (int r = 0; r < 3; r++) {
          const double apr = a[p][r], aqr = a[q][r];
          a[p][r] = c * apr - s * aqr;
          a[q][r] = s * apr + c * aqr;
        }
        for (int r = 0; r < 3; r++) {
          const double qp = Q[3 * r + p], qq = Q[3 * r + q];
          Q[3 * r + p] = c * qp - s * qq;
          Q[3 * r + q] = s * qp + c * qq;
        }
      }
  }
  for (int i = 0; i < 3; i++) lam[i] = a[i][i];
}

__device__ inline double plastic_vm(double mu, double m, const double d[3], double beta) {
  const double g13 = exp(2.0 * m), g16 = exp(m);
  double t[3];
  for (int i = 0; i < 3; i++) {
    const double g = exp(2.0 * (m + beta * d[i]));
    t[i] = g * g - g13 * g;
  }
  const double tm = (t[0] + t[1] + t[2]) / 3.0;
  double j = 0.0;
  for (int i = 0; i < 3; i++) {
    const double s = -mu / g16 * (t[i] - tm);
    j += s * s;
  }
  return sqrt(1.5 * j);
}

// von Mises stress of the hyperelastic deviator of A for shear modulus mu, in FP32: the
// screen that lets cells far inside the yield surface skip the FP64 return (its error, ~1e-7
// of |G| mu, is far below the 1 % margin the caller leaves)
__device__ inline float plastic_vm_screen(const double *A, float mu) {
  float a[9], G[9];
  for (int q = 0; q < 9; q++) a[q] = f32_of_f64(A[q]);
  // a fluid cell carries A = 0 (G = 0, no elastic stress): nothing to screen
  if (a[0] == 0.0f && a[4] == 0.0f && a[8] == 0.0f && a[1] == 0.0f && a[2] == 0.0f &&
      a[3] == 0.0f && a[5] == 0.0f && a[6] == 0.0f && a[7] == 0.0f)
    return 0.0f;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      G[3 * i + j] = a[3 * i] * a[3 * j] + a[3 * i + 1] * a[3 * j + 1] + a[3 * i + 2] * a[3 * j + 2];
  const float det = G[0] * (G[4] * G[8] - G[5] * G[7]) - G[1] * (G[3] * G[8] - G[5] * G[6]) +
                    G[2] * (G[3] * G[7] - G[4] * G[6]);
  if (!(det > 0.0f)) return 0.0f;  // fluid cells (A = 0): no elastic stress
  const float g13 = cbrtf(det), g16 = sqrtf(g13);
  float t[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      t[3 * i + j] = G[3 * i] * G[j] + G[3 * i + 1] * G[3 + j] + G[3 * i + 2] * G[6 + j] -
                     g13 * G[3 * i + j];
  const float tm = (t[0] + t[4] + t[8]) * (1.0f / 3.0f);
  float j2 = 0.0f;
  for (int q = 0; q < 9; q++) {
    const float s = (mu / g16) * (t[q] - ((q == 0 || q == 4 || q == 8) ? tm : 0.0f));
    j2 += s * s;
  }
  return sqrtf(1.5f * j2);
}

// the return mapping on the cell state V (deformation tensor at V + i5); returns true when
// A changed
template <int N>
__device__ inline bool plastic_return(const M5Consts &k, double *V) {
  using C = K5<N>;
  double *A = V + C::i5;
  bool near = false;
  for (int v = 0; v < N; v++)
    if (k.mu[v] != 0.0 && k.yield[v] > 0.0 &&
        plastic_vm_screen(A, (float)k.mu[v]) >= 0.99f * (float)k.yield[v])
      near = true;
  if (!near) return false;
  double G[9], lam[3], Q[9];
  G[0] = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
  G[1] = A[0] * A[3] + A[1] * A[4] + A[2] * A[5];
  G[2] = A[0] * A[6] + A[1] * A[7] + A[2] * A[8];
  G[3] = A[3] * A[0] + A[4] * A[1] + A[5] * A[2];
  G[4] = A[3] * A[3] + A[4] * A[4] + A[5] * A[5];
  G[5] = A[3] * A[6] + A[4] * A[7] + A[5] * A[8];
  G[6] = A[6] * A[0] + A[7] * A[1] + A[8] * A[2];
  G[7] = A[6] * A[3] + A[7] * A[4] + A[8] * A[5];
  G[8] = A[6] * A[6] + A[7] * A[7] + A[8] * A[8];
  plastic_jacobi3(G, lam, Q);
  if (!(lam[0] > 0.0 && lam[1] > 0.0 && lam[2] > 0.0)) return false;
  double h[3], d[3];
  for (int i = 0; i < 3; i++) h[i] = 0.5 * log(lam[i]);
  const double m = (h[0] + h[1] + h[2]) / 3.0;
  for (int i = 0; i < 3; i++) d[i] = h[i] - m;
  double beta = 1.0;
  for (int v = 0; v < N; v++) {
    if (k.mu[v] == 0.0 || !(k.yield[v] > 0.0)) continue;
    if (plastic_vm(k.mu[v], m, d, beta) <= k.yield[v]) continue;
    double lo = 0.0, hi = beta;
    for (int it = 0; it < 60; it++) {
      const double mid = 0.5 * (lo + hi);
      if (plastic_vm(k.mu[v], m, d, mid) <= k.yield[v]) lo = mid;
      else hi = mid;
    }
    beta = lo;
  }
  if (beta == 1.0) return false;
  double M[9], An[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double x = 0.0;
      for (int q = 0; q < 3; q++) x += Q[3 * i + q] * exp((beta - 1.0) * d[q]) * Q[3 * j + q];
      M[3 * i + j] = x;
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      An[3 * i + j] = M[3 * i + 0] * A[0 + j] + M[3 * i + 1] * A[3 + j] + M[3 * i + 2] * A[6 + j];
  for (int q = 0; q < 9; q++) A[q] = An[q];
  return true;
}
