// _cslamtb-compatible entry points: the reference-layout correspondence map
// and the per-point partial outputs of ICPJacobian, bit for bit.
//
// These keep the reference's data contract (per-point JtJ/Jr/r^2 partials,
// int64 map with index in the high word); the fused path in icp_fused.cu
// is what ICPOdometry uses.
#include <math.h>

#include "stb_common.cuh"
#include "stb_host.hpp"

namespace stb {
namespace {

constexpr int kThreads = 256;

// --------------------------------------------------------------------------
// correspondence map, reference layout
// (src/correspondence_map.cu:39-61, src/correspondence.hpp:173-193,
//  src/merge_map.hpp:63-81)
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
    k_corr_map_ref(const float *__restrict__ sp, const float *__restrict__ sn,
                   const uint8_t *__restrict__ sm, int64_t n, int64_t mask_len,
                   const float *__restrict__ rt_cam,
                   const float *__restrict__ tp, const float *__restrict__ tn,
                   const uint8_t *__restrict__ tm, int H, int W,
                   const float *__restrict__ kcam, unsigned long long *map,
                   float thr2, float cos_max) {
  __shared__ Pose32 P;
  if (threadIdx.x == 0) load_pose32(P, rt_cam, kcam);
  __syncthreads();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (mask_len == n && !sm[i]) return;
  const float3 Tp = transform_point(P.rt, sp[3 * i], sp[3 * i + 1], sp[3 * i + 2]);
  float u, v;
  project(P, Tp, u, v);
  int ui, vi;
  if (!round_in(u, W, ui) || !round_in(v, H, vi)) return;
  const int64_t pix = (int64_t)vi * W + ui;
  if (!tm[pix]) return;
  const float dx = fsub(tp[3 * pix], Tp.x), dy = fsub(tp[3 * pix + 1], Tp.y),
              dz = fsub(tp[3 * pix + 2], Tp.z);
  const float sq = dot3(dx, dy, dz, dx, dy, dz);
  if (sq > thr2) return;
  const float3 Tn = transform_normal(P.nm, sn[3 * i], sn[3 * i + 1], sn[3 * i + 2]);
  const float nx = tn[3 * pix], ny = tn[3 * pix + 1], nz = tn[3 * pix + 2];
  const float c = fdiv(dot3(Tn.x, Tn.y, Tn.z, nx, ny, nz),
                       fmul(__fsqrt_rn(dot3(Tn.x, Tn.y, Tn.z, Tn.x, Tn.y, Tn.z)),
                            __fsqrt_rn(dot3(nx, ny, nz, nx, ny, nz))));
  if (c >= -1.0f && c <= cos_max) return;
  const float dist = __fsqrt_rn(sq);

  // z-buffer with the deterministic rule: the lexicographically smallest
  // (distance, index) pair wins.  Lock-free: each failed CAS means another
  // thread stored a smaller pair, so the retries are bounded by the number
  // of competitors for this pixel.
  unsigned long long *addr = map + pix;
  const unsigned long long mine =
      ((unsigned long long)(uint32_t)i << 32) | __float_as_uint(dist);
  unsigned long long old = *(volatile unsigned long long *)addr;
  for (;;) {
    const float cur_d = __uint_as_float((uint32_t)(old & 0xffffffffu));
    const int32_t cur_i = (int32_t)(old >> 32);
    const bool better = dist < cur_d || (dist == cur_d && (int32_t)i < cur_i);
    if (!better) break;
    const unsigned long long prev = atomicCAS(addr, old, mine);
    if (prev == old) break;
    old = prev;
  }
}

// Matched source test shared by the partial kernels
// (icp_jacobian_geometric.cu:58-73): mask, projection, bounds, and the map
// entry naming this source point.
__device__ __forceinline__ bool matched_source(const Pose32 &P,
                                               const float *__restrict__ sp,
                                               const uint8_t *__restrict__ sm,
                                               const long long *__restrict__ map,
                                               int64_t i, int H, int W, float3 &Tp,
                                               float &u, float &v, int64_t &pix) {
  if (!sm[i]) return false;
  Tp = transform_point(P.rt, sp[3 * i], sp[3 * i + 1], sp[3 * i + 2]);
  project(P, Tp, u, v);
  int ui, vi;
  if (!round_in(u, W, ui) || !round_in(v, H, vi)) return false;
  pix = (int64_t)vi * W + ui;
  const int32_t owner = (int32_t)(map[pix] >> 32);
  return owner == (int32_t)i;
}

__device__ __forceinline__ void write_se3_partials(float *__restrict__ JtJ,
                                                   float *__restrict__ Jr, int64_t i,
                                                   const float *J, float r) {
  // JtJ[a][b] = J[b] * J[a], Jr[k] = J[k] * r (icp_jacobian_common.hpp:50-60)
  float *o = JtJ + 36 * i;
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = 0; b < 6; ++b) o[a * 6 + b] = fmul(J[b], J[a]);
#pragma unroll
  for (int k = 0; k < 6; ++k) Jr[6 * i + k] = fmul(J[k], r);
}

__device__ __forceinline__ void zero_partials(float *__restrict__ JtJ,
                                              float *__restrict__ Jr, int64_t i) {
  float *o = JtJ + 36 * i;
#pragma unroll
  for (int k = 0; k < 36; ++k) o[k] = 0.f;
#pragma unroll
  for (int k = 0; k < 6; ++k) Jr[6 * i + k] = 0.f;
}

// --------------------------------------------------------------------------
// GeometricJacobianKernel (icp_jacobian_geometric.cu:54-85)
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
    k_geom_partials(const float *__restrict__ sp, const uint8_t *__restrict__ sm,
                    int64_t n, const float *__restrict__ rt_cam,
                    const float *__restrict__ tp, const float *__restrict__ tn,
                    int H, int W, const float *__restrict__ kcam,
                    const long long *__restrict__ map, float *__restrict__ JtJ,
                    float *__restrict__ Jr, float *__restrict__ r2,
                    int32_t *count) {
  __shared__ Pose32 P;
  if (threadIdx.x == 0) load_pose32(P, rt_cam, kcam);
  __syncthreads();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool matched = false;
  if (i < n) {
    float3 Tp;
    float u, v;
    int64_t pix;
    if (matched_source(P, sp, sm, map, i, H, W, Tp, u, v, pix)) {
      matched = true;
      const float qx = tp[3 * pix], qy = tp[3 * pix + 1], qz = tp[3 * pix + 2];
      const float nx = tn[3 * pix], ny = tn[3 * pix + 1], nz = tn[3 * pix + 2];
      const float r = dot3(fsub(qx, Tp.x), fsub(qy, Tp.y), fsub(qz, Tp.z), nx, ny, nz);
      const float J[6] = {nx, ny, nz, fsub(fmul(Tp.y, nz), fmul(Tp.z, ny)),
                          fsub(fmul(Tp.z, nx), fmul(Tp.x, nz)),
                          fsub(fmul(Tp.x, ny), fmul(Tp.y, nx))};
      write_se3_partials(JtJ, Jr, i, J, r);
      r2[i] = fmul(r, r);
    } else {
      zero_partials(JtJ, Jr, i);
      r2[i] = 0.f;
    }
  }
  const int nmatch = __syncthreads_count(matched);
  if (threadIdx.x == 0 && nmatch) atomicAdd(count, nmatch);
}

// --------------------------------------------------------------------------
// FeatureJacobianKernel (icp_jacobian_feature.cu:58-109) with FeatureMap /
// BilinearInterp / BilinearInterpGrad (src/feature_map.hpp:8-85)
// --------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ float bilinear(const T *__restrict__ f, int H, int W,
                                          float u, float v) {
  const int ui = (int)u, vi = (int)v;  // truncation, as int(u) in the reference
  const float ur = fsub(u, (float)ui), vr = fsub(v, (float)vi);
  const float v00 = load_feat(f + (int64_t)vi * W + ui);
  const float v10 = (ui + 1 < W) ? load_feat(f + (int64_t)vi * W + ui + 1) : 0.f;
  const float v01 = (vi + 1 < H) ? load_feat(f + (int64_t)(vi + 1) * W + ui) : 0.f;
  const float v11 =
      (ui + 1 < W && vi + 1 < H) ? load_feat(f + (int64_t)(vi + 1) * W + ui + 1) : 0.f;
  const float a0 = fadd(fmul(v00, fsub(1.f, ur)), fmul(v10, ur));
  const float a1 = fadd(fmul(v01, fsub(1.f, ur)), fmul(v11, ur));
  return fadd(fmul(a0, fsub(1.f, vr)), fmul(a1, vr));
}

template <typename T, bool kSO3>
__global__ void __launch_bounds__(kThreads)
    k_feat_partials(const float *__restrict__ sp, const T *__restrict__ sf,
                    const uint8_t *__restrict__ sm, int64_t n,
                    const float *__restrict__ rt_cam, const T *__restrict__ tf,
                    int C, int H, int W, const float *__restrict__ kcam,
                    const long long *__restrict__ map, float thresh,
                    float *__restrict__ JtJ, float *__restrict__ Jr,
                    float *__restrict__ r2, int32_t *count) {
  __shared__ Pose32 P;
  if (threadIdx.x == 0) load_pose32(P, rt_cam, kcam);
  __syncthreads();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool counted = false;
  if (i < n) {
    zero_partials(JtJ, Jr, i);
    r2[i] = 0.f;
    float3 Tp;
    float u, v;
    int64_t pix;
    if (matched_source(P, sp, sm, map, i, H, W, Tp, u, v, pix)) {
      const float h = 0.05f;
      const float div = fdiv(1.f, fmul(2.f, h));
      const float uu0 = fadd(u, h), uu1 = fmaxf(fsub(u, h), 0.f);
      const float vv0 = fadd(v, h), vv1 = fmaxf(fsub(v, h), 0.f);
      // Dx_Project (camera.hpp:65-78)
      const float zz = fmul(Tp.z, Tp.z);
      const float j00 = fdiv(P.fx, Tp.z), j02 = fdiv(fmul(-Tp.x, P.fx), zz);
      const float j11 = fdiv(P.fy, Tp.z), j12 = fdiv(fmul(-Tp.y, P.fy), zz);
      const int64_t plane = (int64_t)H * W;
      float sq = 0.f, J[6], r = 0.f;
      for (int c = 0; c < C; ++c) {
        const T *fc = tf + c * plane;
        const float val = bilinear(fc, H, W, u, v);
        r = fsub(val, load_feat(sf + (int64_t)c * n + i));
        const float du = fmul(fsub(bilinear(fc, H, W, uu0, v), bilinear(fc, H, W, uu1, v)), div);
        const float dv = fmul(fsub(bilinear(fc, H, W, u, vv0), bilinear(fc, H, W, u, vv1)), div);
        const float gx = fmul(du, j00), gy = fmul(dv, j11),
                    gz = fadd(fmul(du, j02), fmul(dv, j12));
        const float cx = fsub(fmul(Tp.y, gz), fmul(Tp.z, gy));
        const float cy = fsub(fmul(Tp.z, gx), fmul(Tp.x, gz));
        const float cz = fsub(fmul(Tp.x, gy), fmul(Tp.y, gx));
        if (kSO3) {
          J[0] = cx; J[1] = cy; J[2] = cz;
        } else {
          J[0] = gx; J[1] = gy; J[2] = gz; J[3] = cx; J[4] = cy; J[5] = cz;
        }
        sq = fadd(sq, fmul(r, r));
      }
      if (!(sq > fmul(thresh, thresh))) {
        counted = true;
        if (kSO3) {
          // SO3ICPJacobian::Compute (icp_jacobian_common.hpp:91-112): 3x3
          // block, the rest of the 6x6 / 6 buffers left at zero
#pragma unroll
          for (int a = 0; a < 3; ++a) {
#pragma unroll
            for (int b = 0; b < 3; ++b) JtJ[36 * i + a * 6 + b] = fmul(J[b], J[a]);
            Jr[6 * i + a] = fmul(J[a], r);
          }
        } else {
          write_se3_partials(JtJ, Jr, i, J, r);
        }
        r2[i] = sq;
      }
    }
  }
  const int nmatch = __syncthreads_count(counted);
  if (threadIdx.x == 0 && nmatch) atomicAdd(count, nmatch);
}

// --------------------------------------------------------------------------
// InformationMatrixKernel (icp_jacobian_geometric.cu:118-158)
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
    k_info_partials(const float *__restrict__ sp, const uint8_t *__restrict__ sm,
                    int64_t n, const float *__restrict__ rt_cam,
                    const float *__restrict__ tp, int H, int W,
                    const float *__restrict__ kcam, const long long *__restrict__ map,
                    float *__restrict__ GtG) {
  __shared__ Pose32 P;
  if (threadIdx.x == 0) load_pose32(P, rt_cam, kcam);
  __syncthreads();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float *o = GtG + 36 * i;
  float3 Tp;
  float u, v;
  int64_t pix;
  if (!matched_source(P, sp, sm, map, i, H, W, Tp, u, v, pix)) {
#pragma unroll
    for (int k = 0; k < 36; ++k) o[k] = 0.f;
    return;
  }
  const float qx = tp[3 * pix], qy = tp[3 * pix + 1], qz = tp[3 * pix + 2];
  const float G0[6] = {0.f, qz, -qy, 1.f, 0.f, 0.f};
  const float G1[6] = {-qz, 0.f, qx, 0.f, 1.f, 0.f};
  const float G2[6] = {qy, -qx, 0.f, 0.f, 0.f, 1.f};
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = 0; b < 6; ++b)
      o[a * 6 + b] = fadd(fadd(fmul(G0[a], G0[b]), fmul(G1[a], G1[b])), fmul(G2[a], G2[b]));
}

}  // namespace

// Host helpers shared with icp_fused.cu.
float distance_thresh_sq(double d) { return (float)(d * d); }

float angle_cos_max(double angle) {
  const float th = (float)angle;
  if (isnan(th) || (double)th >= M_PI) return -INFINITY;
  const double c = (th <= 0.0f) ? 1.0 : cos((double)th);
  float f = (float)c;
  if ((double)f > c) f = nextafterf(f, -INFINITY);
  return f;
}

}  // namespace stb

using namespace stb;

static int check_common(int64_t n, int32_t H, int32_t W) {
  if (n < 0 || n > INT32_MAX)
    return fail(STB_EINVAL, "Check failed: num_source must be in [0, 2^31), got %lld",
                (long long)n);
  if (H <= 0 || W <= 0)
    return fail(STB_EINVAL, "Check failed: target size must be positive, got %dx%d", H, W);
  return STB_OK;
}

extern "C" int stb_correspondence_map(
    const float *source_points, const float *source_normals, const uint8_t *source_mask,
    int64_t num_source, int64_t source_mask_len, const float *rt_cam,
    const float *target_points, const float *target_normals, const uint8_t *target_mask,
    int32_t height, int32_t width, const float *kcam, int64_t *merge_map,
    double distance_thresh, double normal_angle_thresh, void *stream) {
  clear_error();
  STB_TRY(check_common(num_source, height, width));
  STB_TRY(check_device_ptr(source_points, "source_points"));
  STB_TRY(check_device_ptr(source_normals, "source_normals"));
  STB_TRY(check_device_ptr(source_mask, "source_mask"));
  STB_TRY(check_device_ptr(rt_cam, "rt_cam"));
  STB_TRY(check_device_ptr(target_points, "target_points"));
  STB_TRY(check_device_ptr(target_normals, "target_normals"));
  STB_TRY(check_device_ptr(target_mask, "target_mask"));
  STB_TRY(check_device_ptr(kcam, "kcam"));
  STB_TRY(check_device_ptr(merge_map, "merge_map"));
  if (num_source == 0) return STB_OK;
  k_corr_map_ref<<<blocks_for(num_source, kThreads), kThreads, 0, as_stream(stream)>>>(
      source_points, source_normals, source_mask, num_source, source_mask_len, rt_cam,
      target_points, target_normals, target_mask, height, width, kcam,
      reinterpret_cast<unsigned long long *>(merge_map), distance_thresh_sq(distance_thresh),
      angle_cos_max(normal_angle_thresh));
  return check_launch("stb_correspondence_map");
}

extern "C" int stb_icp_jacobian_geometric(
    const float *src_points, const uint8_t *src_mask, int64_t num_source,
    const float *rt_cam, const float *tgt_points, const float *tgt_normals,
    int32_t height, int32_t width, const float *kcam, const int64_t *merge_map,
    float *JtJ_partial, float *Jr_partial, float *squared_residual,
    int32_t *match_count, void *stream) {
  clear_error();
  STB_TRY(check_common(num_source, height, width));
  STB_TRY(check_device_ptr(src_points, "src_points"));
  STB_TRY(check_device_ptr(src_mask, "src_mask"));
  STB_TRY(check_device_ptr(rt_cam, "rt_cam"));
  STB_TRY(check_device_ptr(tgt_points, "tgt_points"));
  STB_TRY(check_device_ptr(tgt_normals, "tgt_normals"));
  STB_TRY(check_device_ptr(kcam, "kcam"));
  STB_TRY(check_device_ptr(merge_map, "merge_map"));
  STB_TRY(check_device_ptr(JtJ_partial, "JtJ_partial"));
  STB_TRY(check_device_ptr(Jr_partial, "Jr_partial"));
  STB_TRY(check_device_ptr(squared_residual, "squared_residual"));
  STB_TRY(check_device_ptr(match_count, "match_count"));
  if (num_source == 0) return STB_OK;
  k_geom_partials<<<blocks_for(num_source, kThreads), kThreads, 0, as_stream(stream)>>>(
      src_points, src_mask, num_source, rt_cam, tgt_points, tgt_normals, height, width,
      kcam, reinterpret_cast<const long long *>(merge_map), JtJ_partial, Jr_partial,
      squared_residual, match_count);
  return check_launch("stb_icp_jacobian_geometric");
}

template <bool kSO3>
static int feature_entry(const float *src_points, const void *src_feats,
                         const uint8_t *src_mask, int64_t num_source,
                         const float *rt_cam, const void *tgt_feats, int32_t channels,
                         int32_t height, int32_t width, int32_t feat_dtype,
                         const float *kcam, const int64_t *merge_map,
                         float residual_thresh, float *JtJ_partial, float *Jr_partial,
                         float *squared_residuals, int32_t *match_count, void *stream,
                         const char *name) {
  clear_error();
  STB_TRY(check_common(num_source, height, width));
  if (channels <= 0)
    return fail(STB_EINVAL, "Check failed: channels must be positive, got %d", channels);
  if (feat_dtype != STB_F32 && feat_dtype != STB_BF16)
    return fail(STB_EDTYPE, "Check failed: feature maps must be float32 or bfloat16");
  STB_TRY(check_device_ptr(src_points, "src_points"));
  STB_TRY(check_device_ptr(src_feats, "src_feats"));
  STB_TRY(check_device_ptr(src_mask, "src_mask"));
  STB_TRY(check_device_ptr(rt_cam, "rt_cam"));
  STB_TRY(check_device_ptr(tgt_feats, "tgt_feats"));
  STB_TRY(check_device_ptr(kcam, "kcam"));
  STB_TRY(check_device_ptr(merge_map, "merge_map"));
  STB_TRY(check_device_ptr(JtJ_partial, "JtJ_partial"));
  STB_TRY(check_device_ptr(Jr_partial, "Jr_partial"));
  STB_TRY(check_device_ptr(squared_residuals, "squared_residuals"));
  STB_TRY(check_device_ptr(match_count, "match_count"));
  if (num_source == 0) return STB_OK;
  const unsigned grid = blocks_for(num_source, kThreads);
  const long long *map = reinterpret_cast<const long long *>(merge_map);
  if (feat_dtype == STB_F32)
    k_feat_partials<float, kSO3><<<grid, kThreads, 0, as_stream(stream)>>>(
        src_points, static_cast<const float *>(src_feats), src_mask, num_source, rt_cam,
        static_cast<const float *>(tgt_feats), channels, height, width, kcam, map,
        residual_thresh, JtJ_partial, Jr_partial, squared_residuals, match_count);
  else
    k_feat_partials<__nv_bfloat16, kSO3><<<grid, kThreads, 0, as_stream(stream)>>>(
        src_points, static_cast<const __nv_bfloat16 *>(src_feats), src_mask, num_source,
        rt_cam, static_cast<const __nv_bfloat16 *>(tgt_feats), channels, height, width,
        kcam, map, residual_thresh, JtJ_partial, Jr_partial, squared_residuals,
        match_count);
  return check_launch(name);
}

extern "C" int stb_icp_jacobian_feature(
    const float *src_points, const void *src_feats, const uint8_t *src_mask,
    int64_t num_source, const float *rt_cam, const void *tgt_feats, int32_t channels,
    int32_t height, int32_t width, int32_t feat_dtype, const float *kcam,
    const int64_t *merge_map, float residual_thresh, float *JtJ_partial,
    float *Jr_partial, float *squared_residuals, int32_t *match_count, void *stream) {
  return feature_entry<false>(src_points, src_feats, src_mask, num_source, rt_cam,
                              tgt_feats, channels, height, width, feat_dtype, kcam,
                              merge_map, residual_thresh, JtJ_partial, Jr_partial,
                              squared_residuals, match_count, stream,
                              "stb_icp_jacobian_feature");
}

extern "C" int stb_icp_jacobian_feature_so3(
    const float *src_points, const void *src_feats, const uint8_t *src_mask,
    int64_t num_source, const float *rt_cam, const void *tgt_feats, int32_t channels,
    int32_t height, int32_t width, int32_t feat_dtype, const float *kcam,
    const int64_t *merge_map, float residual_thresh, float *JtJ_partial,
    float *Jr_partial, float *squared_residuals, int32_t *match_count, void *stream) {
  return feature_entry<true>(src_points, src_feats, src_mask, num_source, rt_cam,
                             tgt_feats, channels, height, width, feat_dtype, kcam,
                             merge_map, residual_thresh, JtJ_partial, Jr_partial,
                             squared_residuals, match_count, stream,
                             "stb_icp_jacobian_feature_so3");
}

extern "C" int stb_icp_information_partials(
    const float *src_points, const uint8_t *src_mask, int64_t num_source,
    const float *rt_cam, const float *tgt_points, int32_t height, int32_t width,
    const float *kcam, const int64_t *merge_map, float *GtG_partial, void *stream) {
  clear_error();
  STB_TRY(check_common(num_source, height, width));
  STB_TRY(check_device_ptr(src_points, "src_points"));
  STB_TRY(check_device_ptr(src_mask, "src_mask"));
  STB_TRY(check_device_ptr(rt_cam, "rt_cam"));
  STB_TRY(check_device_ptr(tgt_points, "tgt_points"));
  STB_TRY(check_device_ptr(kcam, "kcam"));
  STB_TRY(check_device_ptr(merge_map, "merge_map"));
  STB_TRY(check_device_ptr(GtG_partial, "GtG_partial"));
  if (num_source == 0) return STB_OK;
  k_info_partials<<<blocks_for(num_source, kThreads), kThreads, 0, as_stream(stream)>>>(
      src_points, src_mask, num_source, rt_cam, tgt_points, height, width, kcam,
      reinterpret_cast<const long long *>(merge_map), GtG_partial);
  return check_launch("stb_icp_information_partials");
}
