// The feature term of one matched pixel, shared by the plain and batched
// reductions: FeatureJacobianKernel (icp_jacobian_feature.cu:58-109) with
// the sampling of feature_map.hpp:15-85.
//   * gate: sum_c r_c^2 > thresh^2 rejects the pixel (decided on the
//     reference's float32 values, channels in order);
//   * per channel c (the last one only in the reference's mode, all in
//     "sum" mode): bilinear value, central differences at u +- 0.05 and
//     v +- 0.05 (lower side clamped at 0), J = [g; Tp x g] with
//     g = (du fx / z, dv fy / z, -(du fx x + dv fy y) / z^2).
// The arithmetic per channel is the same in both feature layouts, so the
// results are the same bits.
#pragma once

#include "stb_common.cuh"

namespace stb {

// J^T J (upper triangle, 21 slots, by w2) and J^T r (6 slots from 21, by
// w1) of one Jacobian row, into per-thread float32 partials (a register
// array, or StridedAcc accumulators in shared memory).
template <typename Acc>
__device__ __forceinline__ void acc_se3_terms(Acc acc, const float *Jv, float r, float w1,
                                              float w2) {
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = a; b < 6; ++b) acc[a * 6 - a * (a - 1) / 2 + (b - a)] += w2 * (Jv[a] * Jv[b]);
#pragma unroll
  for (int a = 0; a < 6; ++a) acc[21 + a] += w1 * (Jv[a] * r);
}

__device__ __forceinline__ void feature_jacobian(const float3 &Tp, float du, float dv, float j00,
                                                 float j02, float j11, float j12, float *Jv) {
  const float gx = fmul(du, j00), gy = fmul(dv, j11), gz = fadd(fmul(du, j02), fmul(dv, j12));
  Jv[0] = gx;
  Jv[1] = gy;
  Jv[2] = gz;
  Jv[3] = fsub(fmul(Tp.y, gz), fmul(Tp.z, gy));
  Jv[4] = fsub(fmul(Tp.z, gx), fmul(Tp.x, gz));
  Jv[5] = fsub(fmul(Tp.x, gy), fmul(Tp.y, gx));
}

// Returns true when the pixel passes the gate (its J terms are then in
// acc, J^T r with -wf1 as icp.py:222); sq receives sum_c r_c^2.
template <typename FT, bool kHWC, typename Acc>
__device__ __forceinline__ bool feature_term(const FeatView<FT, kHWC> &tf,
                                             const FeatView<FT, kHWC> &sf, long long i,
                                             const Pose32 &P, const float3 &Tp, int H, int W,
                                             float feat_thr2, int mode, float wf1, float wf2,
                                             Acc acc, float &sq) {
  const int C = tf.C;
  float u, v;
  project(P, Tp, u, v);
  sq = 0.f;
  for (int c = 0; c < C; ++c) {
    const float r = fsub(bilin_c(tf, c, H, W, u, v), sf.at(c, i));
    sq = fadd(sq, fmul(r, r));
  }
  if (sq > feat_thr2) return false;
  const float h = 0.05f;
  const float div = fdiv(1.f, fmul(2.f, h));
  const float uu0 = fadd(u, h), uu1 = fmaxf(fsub(u, h), 0.f);
  const float vv0 = fadd(v, h), vv1 = fmaxf(fsub(v, h), 0.f);
  const float zz = fmul(Tp.z, Tp.z);
  const float j00 = fdiv(P.fx, Tp.z), j02 = fdiv(fmul(-Tp.x, P.fx), zz);
  const float j11 = fdiv(P.fy, Tp.z), j12 = fdiv(fmul(-Tp.y, P.fy), zz);
  const int c0 = (mode == 0) ? C - 1 : 0;
  for (int c = c0; c < C; ++c) {
    const float r = fsub(bilin_c(tf, c, H, W, u, v), sf.at(c, i));
    const float du = fmul(fsub(bilin_c(tf, c, H, W, uu0, v), bilin_c(tf, c, H, W, uu1, v)), div);
    const float dv = fmul(fsub(bilin_c(tf, c, H, W, u, vv0), bilin_c(tf, c, H, W, u, vv1)), div);
    float Jv[6];
    feature_jacobian(Tp, du, dv, j00, j02, j11, j12, Jv);
    acc_se3_terms(acc, Jv, r, -wf1, wf2);
  }
  return true;
}

}  // namespace stb
