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

// Coefficients of the SE(3) exponential, A = sin t / t, B = (1 - cos t) / t^2,
// C = (t - sin t) / t^3, of t2 = t^2.  Below t = 0.5 (every Gauss-Newton
// update of a registration that converges) they are their Maclaurin series in
// t^2 through t^14, evaluated by Horner's rule: 7 dependent FMAs instead of
// sincos and three divisions; the first omitted term is below
// 0.5^16 / 17! < 5e-20 of the sum.  Above, the closed forms.
__device__ __forceinline__ void se3_coeffs(double t2, double &A, double &B, double &C) {
  if (t2 < 0.25) {
    // A_k = (-1)^k / (2k+1)!, B_k = (-1)^k / (2k+2)!, C_k = (-1)^k / (2k+3)!
    double a = -1.0 / 1307674368000.0, b = -1.0 / 20922789888000.0,
           c = -1.0 / 355687428096000.0;
    a = fma(a, t2, 1.0 / 6227020800.0);
    b = fma(b, t2, 1.0 / 87178291200.0);
    c = fma(c, t2, 1.0 / 1307674368000.0);
    a = fma(a, t2, -1.0 / 39916800.0);
    b = fma(b, t2, -1.0 / 479001600.0);
    c = fma(c, t2, -1.0 / 6227020800.0);
    a = fma(a, t2, 1.0 / 362880.0);
    b = fma(b, t2, 1.0 / 3628800.0);
    c = fma(c, t2, 1.0 / 39916800.0);
    a = fma(a, t2, -1.0 / 5040.0);
    b = fma(b, t2, -1.0 / 40320.0);
    c = fma(c, t2, -1.0 / 362880.0);
    a = fma(a, t2, 1.0 / 120.0);
    b = fma(b, t2, 1.0 / 720.0);
    c = fma(c, t2, 1.0 / 5040.0);
    a = fma(a, t2, -1.0 / 6.0);
    b = fma(b, t2, -1.0 / 24.0);
    c = fma(c, t2, -1.0 / 120.0);
    A = fma(a, t2, 1.0);
    B = fma(b, t2, 0.5);
    C = fma(c, t2, 1.0 / 6.0);
    return;
  }
  const double t = sqrt(t2);
  double s, c;
  sincos(t, &s, &c);
  A = s / t;
  B = (1.0 - c) / t2;
  C = (t - s) / (t2 * t);
}

// SE(3) exponential of a twist [v; w] (translation first, the order fixed by
// the Jacobian J = [n; p x n]): R = I + A W + B W^2, t = (I + B W + C W^2) v
// with the coefficients of se3_coeffs.  Writes a row-major 4x4.
__device__ inline void se3_exp(const double xi[6], double E[16]) {
  const double wx = xi[3], wy = xi[4], wz = xi[5];
  const double t2 = wx * wx + wy * wy + wz * wz;
  double A, B, C;
  se3_coeffs(t2, A, B, C);
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

// ---------------------------------------------------------------------------
// Warp-parallel FP64 Gauss-Newton step.  FP64 latency is ~66 cycles per
// dependent operation on this part, so the step is laid out to keep the
// dependent chain short: lanes 0..5 hold the rows of the 6x6 system
// (right-looking Cholesky, pivot reciprocals by Newton-Raphson on the
// float32 rsqrt), divisions by constants are multiplications by
// reciprocals, and matrix products run one entry per lane.
// ---------------------------------------------------------------------------
namespace stb {

// 1/sqrt(d) for d > 0: float32 seed (relative error < 2^-22), one
// Newton-Raphson step in FP64 (y <- y + y/2 (1 - d y^2)), which squares the
// error to below 2^-43 (~1e-13): the pivots of the 6x6 factorisation carry
// 13 significant digits, the Gauss-Newton update needs fewer than 8.  Seeds
// outside the float32 range fall back to the library call.
__device__ __forceinline__ double rsqrt_fp64(double d) {
  const float f = (float)d;
  if (!(f > 1e-37f && f < 1e37f)) return 1.0 / sqrt(d);
  const double y = (double)rsqrtf(f);
  const double e = fma(-d, y * y, 1.0);
  return fma(0.5 * y, e, y);
}

// SE(3) exponential like se3_exp, entries spread over the warp: lanes 0..8
// hold R, lanes 16..24 hold V = I + B W + C W^2, lanes 0..2 then form
// t = V v.  All lanes call it with the same xi; E (16 doubles, shared
// memory) receives the row-major 4x4.
__device__ inline void warp_se3_exp(const double *xi, double *E, int lane) {
  const unsigned full = 0xffffffffu;
  const double wx = xi[3], wy = xi[4], wz = xi[5];
  const double t2 = fma(wx, wx, fma(wy, wy, wz * wz));
  double A, B, C;
  se3_coeffs(t2, A, B, C);
  // entry (i, j) of the 3x3 blocks: lanes 0..8 -> R, lanes 16..24 -> V
  const int e = lane & 15;
  const int i = e / 3, j = e % 3;
  const double w[3] = {wx, wy, wz};
  double val = 0.0;
  if (e < 9) {
    // W = hat(w): W[i][j] = -w[(i+2)%3] if j == (i+1)%3, w[(i+1)%3] if j == (i+2)%3
    const double Wij = (i == j) ? 0.0 : ((j == (i + 1) % 3) ? -w[(i + 2) % 3] : w[(i + 1) % 3]);
    const double W2ij = fma(w[i], w[j], (i == j) ? -t2 : 0.0);  // W^2 = w w^T - |w|^2 I
    const double c1 = (lane < 16) ? A : B, c2 = (lane < 16) ? B : C;
    val = fma(c1, Wij, fma(c2, W2ij, (i == j) ? 1.0 : 0.0));
  }
  if (lane < 9) E[i * 4 + j] = val;
  // t_i = sum_k V[i][k] v_k, V[i][k] on lane 16 + 3 i + k
  const double v0 = __shfl_sync(full, val, 16 + 3 * (lane % 3) + 0);
  const double v1 = __shfl_sync(full, val, 16 + 3 * (lane % 3) + 1);
  const double v2 = __shfl_sync(full, val, 16 + 3 * (lane % 3) + 2);
  if (lane < 3) E[lane * 4 + 3] = fma(v0, xi[0], fma(v1, xi[1], v2 * xi[2]));
  if (lane >= 12 && lane < 16) E[lane] = (lane == 15) ? 1.0 : 0.0;
  __syncwarp();
}

// 6x6 Cholesky solve A x = b by one warp.  A: 36 doubles (row-major, full
// symmetric), b: 6 doubles, x: 6 doubles out; all in shared memory.  Lane i
// holds row i; the forward substitution L y = b runs inside the
// factorisation loop.  Returns the LAPACK potrf verdict (false when a pivot
// is not > 0 or NaN), uniform across the warp.
__device__ inline bool warp_cholesky_solve6(const double *A, const double *b, double *x,
                                            double *L /* 36 doubles scratch */, int lane) {
  const unsigned full = 0xffffffffu;
  const int i = lane < 6 ? lane : 5;
  double row[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) row[k] = A[i * 6 + k];
  double yi = (lane < 6) ? b[lane] : 0.0;
  double my_inv = 0.0;
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double d = __shfl_sync(full, row[j], j);
    ok = ok && (d > 0.0);
    if (!ok) break;
    const double inv = rsqrt_fp64(d);
    if (lane == j) my_inv = inv;
    // column j of L and y_j
    if (i >= j) row[j] *= inv;
    const double yj = __shfl_sync(full, yi * inv, j);
    if (lane == j) yi = yj;
    if (lane > j && lane < 6) yi = fma(-row[j], yj, yi);
    // trailing update A'[i][k] -= L[i][j] L[k][j] for k > j
#pragma unroll
    for (int k = j + 1; k < 6; ++k) {
      const double lkj = __shfl_sync(full, row[j], k);
      if (i >= k) row[k] = fma(-row[j], lkj, row[k]);
    }
  }
  if (!ok) return false;
  if (lane < 6) {
#pragma unroll
    for (int k = 0; k < 6; ++k) L[lane * 6 + k] = (k <= lane) ? row[k] : 0.0;
  }
  __syncwarp();
  // backward: L^T x = y
  double xi = yi;
#pragma unroll
  for (int j = 5; j >= 0; --j) {
    const double xj = __shfl_sync(full, xi * my_inv, j);
    if (lane == j) xi = xj;
    if (lane < j) xi = fma(-L[j * 6 + lane], xj, xi);
  }
  if (lane < 6) x[lane] = xi;
  __syncwarp();
  return true;
}

// Out = E * T (rigid 4x4, row-major) by one warp: lane = entry of the 3x4.
__device__ inline void warp_compose(const double *E, const double *T, double *Out, int lane) {
  if (lane < 12) {
    const int i = lane >> 2, j = lane & 3;
    double s = fma(E[i * 4 + 0], T[0 * 4 + j],
                   fma(E[i * 4 + 1], T[1 * 4 + j], E[i * 4 + 2] * T[2 * 4 + j]));
    if (j == 3) s += E[i * 4 + 3];
    Out[lane] = s;
  } else if (lane < 16) {
    Out[lane] = (lane == 15) ? 1.0 : 0.0;
  }
  __syncwarp();
}

}  // namespace stb
