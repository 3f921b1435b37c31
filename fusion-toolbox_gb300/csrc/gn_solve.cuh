// FP64 Gauss-Newton step on the device: 6x6 Cholesky solve, SE(3)
// exponential, left pose update, and the float32 pose view for the next
// association.  Replaces the host code of the reference loop
// (slamtb/registration/icp.py:236-256: torch.cholesky + cholesky_solve on
// the CPU, tenviz SE3.exp, transform = update @ transform).
#pragma once

#include "stb_common.cuh"

namespace stb {

// Lower Cholesky A = L L^T with LAPACK potrf's failure rule: a pivot that is
// not > 0 (or NaN) fails.  Then solves A x = b.  Returns false on failure.
__device__ inline bool cholesky_solve6(const double A[36], const double b[6],
                                       double x[6]) {
  double L[36];
  double inv_diag[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double d = A[j * 6 + j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= L[j * 6 + k] * L[j * 6 + k];
    if (!(d > 0.0)) return false;
    const double ljj = sqrt(d);
    L[j * 6 + j] = ljj;
    inv_diag[j] = 1.0 / ljj;
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double s = A[i * 6 + j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= L[i * 6 + k] * L[j * 6 + k];
      L[i * 6 + j] = s * inv_diag[j];
    }
  }
  double y[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double s = b[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s -= L[i * 6 + k] * y[k];
    y[i] = s * inv_diag[i];
  }
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    double s = y[i];
#pragma unroll
    for (int k = i + 1; k < 6; ++k) s -= L[k * 6 + i] * x[k];
    x[i] = s * inv_diag[i];
  }
  return true;
}

// SE(3) exponential of a twist [v; w] (translation first, the order fixed by
// the Jacobian J = [n; p x n]): R = I + A W + B W^2, t = (I + B W + C W^2) v,
// A = sin t / t, B = (1 - cos t) / t^2, C = (t - sin t) / t^3, with their
// Taylor series below t = 1e-2.  Writes a row-major 4x4.
__device__ inline void se3_exp(const double xi[6], double E[16]) {
  const double wx = xi[3], wy = xi[4], wz = xi[5];
  const double t2 = wx * wx + wy * wy + wz * wz;
  double A, B, C;
  if (t2 < 1e-4) {
    const double t4 = t2 * t2, t6 = t4 * t2;
    A = 1.0 - t2 / 6.0 + t4 / 120.0 - t6 / 5040.0;
    B = 0.5 - t2 / 24.0 + t4 / 720.0 - t6 / 40320.0;
    C = 1.0 / 6.0 - t2 / 120.0 + t4 / 5040.0 - t6 / 362880.0;
  } else {
    const double t = sqrt(t2);
    double s, c;
    sincos(t, &s, &c);
    A = s / t;
    B = (1.0 - c) / t2;
    C = (t - s) / (t2 * t);
  }
  // W = hat(w), W2 = W W
  const double W[9] = {0.0, -wz, wy, wz, 0.0, -wx, -wy, wx, 0.0};
  double W2[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      W2[i * 3 + j] = W[i * 3 + 0] * W[0 * 3 + j] + W[i * 3 + 1] * W[1 * 3 + j] +
                      W[i * 3 + 2] * W[2 * 3 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double id = (i == j) ? 1.0 : 0.0;
      E[i * 4 + j] = id + A * W[i * 3 + j] + B * W2[i * 3 + j];
      t += (id + B * W[i * 3 + j] + C * W2[i * 3 + j]) * xi[j];
    }
    E[i * 4 + 3] = t;
  }
  E[12] = 0.0;
  E[13] = 0.0;
  E[14] = 0.0;
  E[15] = 1.0;
}

// Out = E * T for row-major 4x4 rigid transforms (last row 0 0 0 1).
__device__ inline void compose(const double E[16], const double T[16], double Out[16]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double s = E[i * 4 + 0] * T[0 * 4 + j] + E[i * 4 + 1] * T[1 * 4 + j] +
                 E[i * 4 + 2] * T[2 * 4 + j];
      if (j == 3) s += E[i * 4 + 3];
      Out[i * 4 + j] = s;
    }
  }
  Out[12] = 0.0;
  Out[13] = 0.0;
  Out[14] = 0.0;
  Out[15] = 1.0;
}

// float32 view of an FP64 pose: the cast transform.to(float32) of
// icp.py:53,61 and the normal matrix of RigidTransform's constructor.
__device__ inline void refresh_pose32(Pose32 &P, const double T[16]) {
#pragma unroll
  for (int k = 0; k < 12; ++k) P.rt[k] = __double2float_rn(T[k]);
  inverse_transpose(P.rt, P.nm);
}

// Upper-triangle index of (a, b), a <= b, in the 21-entry packed J^T J.
__host__ __device__ constexpr int upper_index(int a, int b) {
  return a * 6 - a * (a - 1) / 2 + (b - a);
}

}  // namespace stb
