// Shared device code of the GB300 ICP path.
//
// Floating-point policy: every float32 operation that decides a
// correspondence (pose cast, transform, projection, distance and angle
// gates) or that feeds the bit-exact per-point partials is written with the
// round-to-nearest intrinsics (__fmul_rn, __fadd_rn, __fsub_rn, __fdiv_rn,
// __fsqrt_rn), which the compiler never contracts into FMA.  This makes the
// device results equal, bit for bit, to the reference's float32 operation
// order evaluated without contraction (the host build of the reference, and
// the numpy oracle).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace stb {

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// a0*b0 + (a1*b1 + a2*b2): the order in which the reference's Eigen sums
// the dot product and squared norm of 3-vectors (its unrolled reduction,
// Eigen/src/Core/Redux.h redux_novec_unroller, splits three terms at one).
__device__ __forceinline__ float dot3(float a0, float a1, float a2, float b0,
                                      float b1, float b2) {
  return fadd(fmul(a0, b0), fadd(fmul(a1, b1), fmul(a2, b2)));
}

// float32 view of the pose and intrinsics the kernels need:
// RigidTransform (include/slamtb/camera.hpp:118-166) and KCamera (:18-86).
struct Pose32 {
  float rt[12];  // 3x4 row-major, float32 cast of the FP64 pose
  float nm[9];   // normal matrix: inverse transpose of rt's 3x3 block
  float fx, fy, cx, cy;
};

// InverseTranspose (camera.hpp:99-116), float32, same operation order.
__device__ __forceinline__ void inverse_transpose(const float *A, float *r) {
#define E(i, j) A[(i)*4 + (j)]
  const float det =
      fadd(fsub(fmul(E(0, 0), fsub(fmul(E(1, 1), E(2, 2)), fmul(E(2, 1), E(1, 2)))),
                fmul(E(0, 1), fsub(fmul(E(1, 0), E(2, 2)), fmul(E(1, 2), E(2, 0))))),
           fmul(E(0, 2), fsub(fmul(E(1, 0), E(2, 1)), fmul(E(1, 1), E(2, 0)))));
  const float inv = fdiv(1.0f, det);
  r[0 * 3 + 0] = fmul(fsub(fmul(E(1, 1), E(2, 2)), fmul(E(2, 1), E(1, 2))), inv);
  r[1 * 3 + 0] = fmul(-fsub(fmul(E(0, 1), E(2, 2)), fmul(E(0, 2), E(2, 1))), inv);
  r[2 * 3 + 0] = fmul(fsub(fmul(E(0, 1), E(1, 2)), fmul(E(0, 2), E(1, 1))), inv);
  r[0 * 3 + 1] = fmul(-fsub(fmul(E(1, 0), E(2, 2)), fmul(E(1, 2), E(2, 0))), inv);
  r[1 * 3 + 1] = fmul(fsub(fmul(E(0, 0), E(2, 2)), fmul(E(0, 2), E(2, 0))), inv);
  r[2 * 3 + 1] = fmul(-fsub(fmul(E(0, 0), E(1, 2)), fmul(E(1, 0), E(0, 2))), inv);
  r[0 * 3 + 2] = fmul(fsub(fmul(E(1, 0), E(2, 1)), fmul(E(2, 0), E(1, 1))), inv);
  r[1 * 3 + 2] = fmul(-fsub(fmul(E(0, 0), E(2, 1)), fmul(E(2, 0), E(0, 1))), inv);
  r[2 * 3 + 2] = fmul(fsub(fmul(E(0, 0), E(1, 1)), fmul(E(1, 0), E(0, 1))), inv);
#undef E
}

// Entry e < 9 of inverse_transpose's result, computed by one lane: the
// same operations in the same order as the serial function (entry (i, j) is
// the (i, j) cofactor, from the rows and columns other than i and j in
// increasing order, times 1 / det), so the nine lanes of a warp produce
// its result bit for bit in parallel.
__device__ __forceinline__ float inverse_transpose_entry(const float *A, int e) {
#define E(i, j) A[(i)*4 + (j)]
  const float det =
      fadd(fsub(fmul(E(0, 0), fsub(fmul(E(1, 1), E(2, 2)), fmul(E(2, 1), E(1, 2)))),
                fmul(E(0, 1), fsub(fmul(E(1, 0), E(2, 2)), fmul(E(1, 2), E(2, 0))))),
           fmul(E(0, 2), fsub(fmul(E(1, 0), E(2, 1)), fmul(E(1, 1), E(2, 0)))));
  const float inv = fdiv(1.0f, det);
  const int i = e / 3, j = e % 3;
  const int a = i == 0 ? 1 : 0, b = i == 2 ? 1 : 2;
  const int c = j == 0 ? 1 : 0, d = j == 2 ? 1 : 2;
  const float m = fsub(fmul(E(a, c), E(b, d)), fmul(E(a, d), E(b, c)));
#undef E
  return fmul(((i + j) & 1) ? -m : m, inv);
}

// RigidTransform::Transform (camera.hpp:134-145).
__device__ __forceinline__ float3 transform_point(const float *rt, float x,
                                                  float y, float z) {
  float3 o;
  o.x = fadd(fadd(fadd(fmul(rt[0], x), fmul(rt[1], y)), fmul(rt[2], z)), rt[3]);
  o.y = fadd(fadd(fadd(fmul(rt[4], x), fmul(rt[5], y)), fmul(rt[6], z)), rt[7]);
  o.z = fadd(fadd(fadd(fmul(rt[8], x), fmul(rt[9], y)), fmul(rt[10], z)), rt[11]);
  return o;
}

// RigidTransform::TransformNormal (camera.hpp:150-165).
__device__ __forceinline__ float3 transform_normal(const float *nm, float x,
                                                   float y, float z) {
  float3 o;
  o.x = fadd(fadd(fmul(nm[0], x), fmul(nm[1], y)), fmul(nm[2], z));
  o.y = fadd(fadd(fmul(nm[3], x), fmul(nm[4], y)), fmul(nm[5], z));
  o.z = fadd(fadd(fmul(nm[6], x), fmul(nm[7], y)), fmul(nm[8], z));
  return o;
}

// The normal-angle gate of the association (correspondence.hpp:69-89):
// with c = (Tn . m) / (sqrt(Tn . Tn) sqrt(m . m)) in the reference's
// float32 operations, the pair is rejected when -1 <= c <= cos_max.  Only
// the outcome matters, so c is first estimated as (Tn . m) rsqrt((Tn . Tn)
// (m . m)): the dot products are the same bits, rsqrtf is within 2 ulp and
// the two products add one rounding each, so the estimate is within
// 2^-22 + 2^-23 of c relative, and c's own four roundings within 2^-22:
// |estimate - c| < 6e-7 for |c| <= 1.  Where the estimate is at least 2e-6
// from cos_max and 4e-6 above -1 (and the norms are normal, finite
// floats), it decides as c would; otherwise c is formed exactly.
__device__ __forceinline__ bool normal_angle_rejects(const float3 &Tn, float mx, float my,
                                                     float mz, float cos_max) {
  const float d = dot3(Tn.x, Tn.y, Tn.z, mx, my, mz);
  const float nn = dot3(Tn.x, Tn.y, Tn.z, Tn.x, Tn.y, Tn.z);
  const float mm = dot3(mx, my, mz, mx, my, mz);
  const float pm = nn * mm;
  if (pm > 1e-30f && pm < 1e30f) {
    const float ce = d * rsqrtf(pm);
    if (fabsf(ce - cos_max) > 2e-6f && ce > -1.0f + 4e-6f && ce < 2.0f) return ce <= cos_max;
  }
  const float c = fdiv(d, fmul(__fsqrt_rn(nn), __fsqrt_rn(mm)));
  return c >= -1.0f && c <= cos_max;
}

// KCamera::Project (camera.hpp:53-60): fx * x / z + cx.
__device__ __forceinline__ void project(const Pose32 &P, float3 p, float &u,
                                        float &v) {
  u = fadd(fdiv(fmul(P.fx, p.x), p.z), P.cx);
  v = fadd(fdiv(fmul(P.fy, p.y), p.z), P.cy);
}

// int(round(u)) with the bounds test of every kernel of the path
// (correspondence.hpp:179-182): true when round(u) lies in [0, size).
// round() is half away from zero; NaN fails the test.
__device__ __forceinline__ bool round_in(float u, int size, int &ui) {
  const float r = roundf(u);
  if (!(r >= 0.0f && r < (float)size)) return false;
  ui = (int)r;
  return true;
}

// Loads a pose block (rt: float32 3x4 or 4x4 row-major; kcam: 3x3) and
// derives the normal matrix, as RigidTransform's constructor does on the
// host (camera.hpp:123-129).
__device__ __forceinline__ void load_pose32(Pose32 &P, const float *rt_cam,
                                            const float *kcam) {
#pragma unroll
  for (int k = 0; k < 12; ++k) P.rt[k] = rt_cam[k];
  inverse_transpose(P.rt, P.nm);
  P.fx = kcam[0];
  P.cx = kcam[2];
  P.fy = kcam[4];
  P.cy = kcam[5];
}

template <typename T>
__device__ __forceinline__ float load_feat(const T *p);
template <>
__device__ __forceinline__ float load_feat<float>(const float *p) {
  return __ldg(p);
}
template <>
__device__ __forceinline__ float load_feat<__nv_bfloat16>(const __nv_bfloat16 *p) {
  return __bfloat162float(*p);
}

// Feature maps of n pixels and C channels in the reference's planar layout
// ([C][n], kHWC = false) or texel-major ([n][C], kHWC = true: the channels
// of a pixel share cache lines, so sampling all channels at a pixel touches
// a few lines instead of one per channel).
template <typename T, bool kHWC>
struct FeatView {
  const T *p;
  long long n;
  int C;
  __device__ __forceinline__ float at(int c, long long idx) const {
    return load_feat(p + (kHWC ? idx * C + c : (long long)c * n + idx));
  }
};

// Bilinear sample of channel c (BilinearInterp, feature_map.hpp:15-41):
// truncated cell, taps past the right / bottom edge read 0.
template <typename T, bool kHWC>
__device__ __forceinline__ float bilin_c(const FeatView<T, kHWC> &f, int c, int H, int W,
                                         float u, float v) {
  const int ui = (int)u, vi = (int)v;
  const float ur = __fsub_rn(u, (float)ui), vr = __fsub_rn(v, (float)vi);
  const long long b = (long long)vi * W + ui;
  const float v00 = f.at(c, b);
  const float v10 = (ui + 1 < W) ? f.at(c, b + 1) : 0.f;
  const float v01 = (vi + 1 < H) ? f.at(c, b + W) : 0.f;
  const float v11 = (ui + 1 < W && vi + 1 < H) ? f.at(c, b + W + 1) : 0.f;
  const float a0 = __fadd_rn(__fmul_rn(v00, __fsub_rn(1.f, ur)), __fmul_rn(v10, ur));
  const float a1 = __fadd_rn(__fmul_rn(v01, __fsub_rn(1.f, ur)), __fmul_rn(v11, ur));
  return __fadd_rn(__fmul_rn(a0, __fsub_rn(1.f, vr)), __fmul_rn(a1, vr));
}

// ---------------------------------------------------------------------------
// Compensated float32 sums: a value is carried as (s, c) with the exact sum
// s + c; TwoSum (Knuth) keeps the rounding error of every addition.
// ---------------------------------------------------------------------------
// Per-thread accumulators in shared memory, transposed ([slot][thread]):
// the lanes of a warp touching one slot fall in distinct banks.
template <int kStride>
struct StridedAcc {
  float *p;
  __device__ __forceinline__ float &operator[](int k) const { return p[k * kStride]; }
};

struct CSum {
  float s, c;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void csum_add(CSum &acc, float x) {
  float s, e;
  two_sum(acc.s, x, s, e);
  acc.s = s;
  acc.c = __fadd_rn(acc.c, e);
}

__device__ __forceinline__ void csum_merge(CSum &acc, float s2, float c2) {
  float s, e;
  two_sum(acc.s, s2, s, e);
  acc.s = s;
  acc.c = __fadd_rn(__fadd_rn(acc.c, c2), e);
}

__device__ __forceinline__ void csum_warp_reduce(CSum &acc) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float s2 = __shfl_down_sync(0xffffffffu, acc.s, off);
    const float c2 = __shfl_down_sync(0xffffffffu, acc.c, off);
    csum_merge(acc, s2, c2);
  }
}

}  // namespace stb
