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

// ---------------------------------------------------------------------------
// Texel-major maps whose channels fill whole 16-byte vectors (a multiple of
// 8 BF16 or 4 float32 channels, 16-byte aligned maps): a tap's channels are
// read as 16-byte vectors, one load per 8 (4) channels instead of one per
// channel.  The values and the arithmetic are those of bilin_c and
// FeatView::at, so the results are the same bits.
// ---------------------------------------------------------------------------
template <typename T>
struct Vec16 {
  static constexpr int V = 16 / sizeof(T);
};

__device__ __forceinline__ void unpack16(const uint4 &w, const float *, float *out) {
  out[0] = __uint_as_float(w.x);
  out[1] = __uint_as_float(w.y);
  out[2] = __uint_as_float(w.z);
  out[3] = __uint_as_float(w.w);
}

// BF16 -> float32 is exact: the BF16 bits are the high half of the float's
// (the low address holds the lower channel).
__device__ __forceinline__ void unpack16(const uint4 &w, const __nv_bfloat16 *, float *out) {
  const unsigned q[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    out[2 * k] = __uint_as_float(q[k] << 16);
    out[2 * k + 1] = __uint_as_float(q[k] & 0xffff0000u);
  }
}

// Channels [g V, g V + V) of texel idx.
template <typename T>
__device__ __forceinline__ void load_group(const T *map, int C, long long idx, int g, float *out) {
  const uint4 w = __ldg(reinterpret_cast<const uint4 *>(map + idx * C) + g);
  unpack16(w, map, out);
}

template <typename T>
__device__ __forceinline__ bool vec_maps(const FeatView<T, true> &tf, const FeatView<T, true> &sf) {
  constexpr int V = Vec16<T>::V;
  return tf.C % V == 0 && ((reinterpret_cast<uintptr_t>(tf.p) | reinterpret_cast<uintptr_t>(sf.p)) &
                           15) == 0;
}

// bilin_c for the V channels of group g.
template <typename T>
__device__ __forceinline__ void bilin_group(const T *map, int C, int g, int H, int W, float u,
                                            float v, float *out) {
  constexpr int V = Vec16<T>::V;
  const int ui = (int)u, vi = (int)v;
  const float ur = __fsub_rn(u, (float)ui), vr = __fsub_rn(v, (float)vi);
  const long long b = (long long)vi * W + ui;
  const bool r_in = ui + 1 < W, d_in = vi + 1 < H;
  float f00[V], f10[V], f01[V], f11[V];
  load_group(map, C, b, g, f00);
#pragma unroll
  for (int j = 0; j < V; ++j) f10[j] = f01[j] = f11[j] = 0.f;
  if (r_in) load_group(map, C, b + 1, g, f10);
  if (d_in) load_group(map, C, b + W, g, f01);
  if (r_in && d_in) load_group(map, C, b + W + 1, g, f11);
  const float ur1 = __fsub_rn(1.f, ur), vr1 = __fsub_rn(1.f, vr);
#pragma unroll
  for (int j = 0; j < V; ++j) {
    const float a0 = __fadd_rn(__fmul_rn(f00[j], ur1), __fmul_rn(f10[j], ur));
    const float a1 = __fadd_rn(__fmul_rn(f01[j], ur1), __fmul_rn(f11[j], ur));
    out[j] = __fadd_rn(__fmul_rn(a0, vr1), __fmul_rn(a1, vr));
  }
}

// The gate's sum of squared channel residuals at (u, v) on 16-byte channel
// vectors (channels in order, as the scalar loop); r_last receives the last
// channel's residual.
template <typename FT>
__device__ __forceinline__ float gate_vec(const FeatView<FT, true> &tf,
                                          const FeatView<FT, true> &sf, long long i, int H,
                                          int W, float u, float v, float &r_last) {
  constexpr int V = Vec16<FT>::V;
  const int C = tf.C;
  float sq = 0.f;
  for (int g = 0; g < C / V; ++g) {
    float tv[V], sv[V];
    bilin_group(tf.p, C, g, H, W, u, v, tv);
    load_group(sf.p, C, i, g, sv);
#pragma unroll
    for (int j = 0; j < V; ++j) {
      const float r = fsub(tv[j], sv[j]);
      sq = fadd(sq, fmul(r, r));
      r_last = r;
    }
  }
  return sq;
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
  // the last channel's residual, when the vector gate formed it
  float r_last = 0.f;
  bool have_last = false;
  if constexpr (kHWC) {
    if (vec_maps(tf, sf)) {
      sq = gate_vec(tf, sf, i, H, W, u, v, r_last);
      have_last = true;
    }
  }
  if (!have_last) {
    for (int c = 0; c < C; ++c) {
      const float r = fsub(bilin_c(tf, c, H, W, u, v), sf.at(c, i));
      sq = fadd(sq, fmul(r, r));
    }
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
    const float r = (have_last && c == C - 1) ? r_last
                                              : fsub(bilin_c(tf, c, H, W, u, v), sf.at(c, i));
    const float du = fmul(fsub(bilin_c(tf, c, H, W, uu0, v), bilin_c(tf, c, H, W, uu1, v)), div);
    const float dv = fmul(fsub(bilin_c(tf, c, H, W, u, vv0), bilin_c(tf, c, H, W, u, vv1)), div);
    float Jv[6];
    feature_jacobian(Tp, du, dv, j00, j02, j11, j12, Jv);
    acc_se3_terms(acc, Jv, r, -wf1, wf2);
  }
  return true;
}

}  // namespace stb
