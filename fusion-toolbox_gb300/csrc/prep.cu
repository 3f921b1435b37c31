// Frame preparation feeding the ICP path: depth back-projection, mask
// erosion, central-difference normals, and the XYZ / mask / feature
// pyramids.  Each kernel restates one reference kernel in its float32
// operation order (no contraction), so results are bit-exact with the
// reference's host build; the 3x3 Gaussian blur restates kornia's
// GaussianBlur2d (reflect border) and is compared within a tolerance.
#include <math.h>

#include "stb_common.cuh"
#include "stb_host.hpp"

namespace stb {
namespace {

constexpr int kBX = 32, kBY = 8;

inline dim3 grid2(int w, int h) { return dim3((w + kBX - 1) / kBX, (h + kBY - 1) / kBY); }

// _utils.py:11-37 (depth * scale + bias, u/v grid) and camera.py:127-149
// (x = (u - cx) * z / fx); raw mask = depth > 0 (frame.py:290).
__global__ void k_depth_to_points(const float *__restrict__ depth, float scale, float bias,
                                  const float *__restrict__ kcam, float *__restrict__ pts,
                                  uint8_t *__restrict__ raw_mask, int H, int W) {
  const int c = blockIdx.x * kBX + threadIdx.x, r = blockIdx.y * kBY + threadIdx.y;
  if (c >= W || r >= H) return;
  const int64_t i = (int64_t)r * W + c;
  const float d = depth[i];
  const float z = fadd(fmul(d, scale), bias);
  const float fx = kcam[0], cx = kcam[2], fy = kcam[4], cy = kcam[5];
  pts[3 * i] = fdiv(fmul(fsub((float)c, cx), z), fx);
  pts[3 * i + 1] = fdiv(fmul(fsub((float)r, cy), z), fy);
  pts[3 * i + 2] = z;
  raw_mask[i] = d > 0.0f;
}

// ErodeMaskKernel (src/erode_mask.cu:18-39).  Its neighbourhood table lists
// {0, 1} twice, so the pixels above, right and left are tested and the
// pixel below never is; kept as is.
__global__ void k_erode(const uint8_t *__restrict__ in, uint8_t *__restrict__ out, int H,
                        int W) {
  const int c = blockIdx.x * kBX + threadIdx.x, r = blockIdx.y * kBY + threadIdx.y;
  if (c >= W || r >= H) return;
  const int64_t i = (int64_t)r * W + c;
  bool ok = in[i];
  if (ok && r > 0) ok = in[i - W];
  if (ok && c + 1 < W) ok = in[i + 1];
  if (ok && c > 0) ok = in[i - 1];
  out[i] = ok;
}

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
  return f3(fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z));
}
__device__ __forceinline__ float sq3(float3 a) { return dot3(a.x, a.y, a.z, a.x, a.y, a.z); }

// CentralDifferencesKernel (src/normals.cu:27-100).
__global__ void k_normals(const float *__restrict__ xyz, const uint8_t *__restrict__ mask,
                          float *__restrict__ out, int H, int W) {
  const int c = blockIdx.x * kBX + threadIdx.x, r = blockIdx.y * kBY + threadIdx.y;
  if (c >= W || r >= H) return;
  const int64_t i = (int64_t)r * W + c;
  if (!mask[i]) {
    out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = 0.f;
    return;
  }
  auto at = [&](int64_t j) { return f3(xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2]); };
  const float3 zero = f3(0.f, 0.f, 0.f);
  const float3 center = at(i);
  const float3 left = (c > 0 && mask[i - 1]) ? at(i - 1) : zero;
  const float3 right = (c < W - 1 && mask[i + 1]) ? at(i + 1) : zero;
  const float3 top = (r > 0 && mask[i - W]) ? at(i - W) : zero;
  const float3 bottom = (r < H - 1 && mask[i + W]) ? at(i + W) : zero;
  const float thr2 = 4.0f, inv_thr2 = 0.25f;

  const float lds = sq3(sub3(left, center)), rds = sq3(sub3(right, center));
  const float lr = fdiv(lds, rds);
  float3 l2r;
  if (lr < thr2 && lr > inv_thr2)
    l2r = sub3(right, left);
  else if (lds < rds)
    l2r = sub3(center, left);
  else
    l2r = sub3(right, center);

  const float bds = sq3(sub3(bottom, center)), tds = sq3(sub3(top, center));
  const float bt = fdiv(bds, tds);
  float3 b2t;
  if (bt < thr2 && bt > inv_thr2)
    b2t = sub3(top, bottom);
  else if (bds < tds)
    b2t = sub3(center, bottom);
  else
    b2t = sub3(top, center);

  float3 n = f3(fsub(fmul(l2r.y, b2t.z), fmul(l2r.z, b2t.y)),
                fsub(fmul(l2r.z, b2t.x), fmul(l2r.x, b2t.z)),
                fsub(fmul(l2r.x, b2t.y), fmul(l2r.y, b2t.x)));
  const float len = __fsqrt_rn(sq3(n));
  if (!(len > 1e-6f)) {
    n = f3(0.f, 0.f, -1.f);
  } else {
    n = f3(fdiv(n.x, len), fdiv(n.y, len), fdiv(n.z, len));
  }
  out[3 * i] = n.x;
  out[3 * i + 1] = n.y;
  out[3 * i + 2] = n.z;
}

// DownsampleXYZNearestKernel (src/downsample.cu:25-72): the valid point of
// the 2x2 block nearest to the block's mean.  Source rows past the image
// (odd heights) are skipped; the reference reads past the end there.
__global__ void k_downsample_xyz(const float *__restrict__ xyz, const uint8_t *__restrict__ mask,
                                 int H, int W, float inv_scale, float *__restrict__ dst,
                                 int DH, int DW) {
  const int dc = blockIdx.x * kBX + threadIdx.x, dr = blockIdx.y * kBY + threadIdx.y;
  if (dc >= DW || dr >= DH) return;
  const int r0 = (int)fmul((float)dr, inv_scale), c0 = (int)fmul((float)dc, inv_scale);
  const int off[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
  float3 mean = f3(0.f, 0.f, 0.f);
  int count = 0;
  float3 p[4];
  bool ok[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int r = r0 + off[k][0], c = c0 + off[k][1];
    ok[k] = c < W && r < H && mask[(int64_t)r * W + c];
    if (ok[k]) {
      const int64_t j = (int64_t)r * W + c;
      p[k] = f3(xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2]);
      mean = f3(fadd(mean.x, p[k].x), fadd(mean.y, p[k].y), fadd(mean.z, p[k].z));
      ++count;
    }
  }
  const float fc = (float)count;
  mean = f3(fdiv(mean.x, fc), fdiv(mean.y, fc), fdiv(mean.z, fc));
  float best = INFINITY;
  float3 near = f3(0.f, 0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (!ok[k]) continue;
    const float d = sq3(sub3(p[k], mean));
    if (d < best) {
      best = d;
      near = p[k];
    }
  }
  const int64_t o = (int64_t)dr * DW + dc;
  dst[3 * o] = near.x;
  dst[3 * o + 1] = near.y;
  dst[3 * o + 2] = near.z;
}

// DownsampleMaskKernel (src/downsample.cu:112-116).
__global__ void k_downsample_mask(const uint8_t *__restrict__ mask, int H, int W,
                                  float inv_scale, uint8_t *__restrict__ dst, int DH, int DW) {
  const int dc = blockIdx.x * kBX + threadIdx.x, dr = blockIdx.y * kBY + threadIdx.y;
  if (dc >= DW || dr >= DH) return;
  const int r = (int)fmul((float)dr, inv_scale), c = (int)fmul((float)dc, inv_scale);
  dst[(int64_t)dr * DW + dc] = (r < H && c < W) ? mask[(int64_t)r * W + c] : 0;
}

template <typename T>
__device__ __forceinline__ T to_t(float v);
template <>
__device__ __forceinline__ float to_t<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 to_t<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}

// DownsampleFeatureKernel (src/downsample.cu:145-168): 2x2 mean per channel.
template <typename T>
__global__ void k_downsample_feat(const T *__restrict__ f, int C, int H, int W,
                                  float inv_scale, T *__restrict__ dst, int DH, int DW) {
  const int dc = blockIdx.x * kBX + threadIdx.x, dr = blockIdx.y * kBY + threadIdx.y;
  if (dc >= DW || dr >= DH) return;
  const int r0 = (int)fmul((float)dr, inv_scale), c0 = (int)fmul((float)dc, inv_scale);
  const int off[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
  for (int ch = 0; ch < C; ++ch) {
    const T *fc = f + (int64_t)ch * H * W;
    float s = 0.f;
    int count = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int r = r0 + off[k][0], c = c0 + off[k][1];
      if (c >= W || r >= H) continue;
      s = fadd(s, load_feat(fc + (int64_t)r * W + c));
      ++count;
    }
    dst[(int64_t)ch * DH * DW + (int64_t)dr * DW + dc] = to_t<T>(fdiv(s, (float)count));
  }
}

__device__ __forceinline__ int reflect(int i, int n) {
  if (i < 0) return -i;
  if (i >= n) return 2 * n - 2 - i;
  return i;
}

struct Kernel3 {
  float w[9];
};

// 3x3 Gaussian with reflect border (kornia GaussianBlur2d, used by
// slamtb/processing.py:148); taps summed row by row.
template <typename T>
__global__ void k_blur3(const T *__restrict__ f, int C, int H, int W, Kernel3 k,
                        T *__restrict__ dst) {
  const int c = blockIdx.x * kBX + threadIdx.x, r = blockIdx.y * kBY + threadIdx.y;
  if (c >= W || r >= H) return;
  for (int ch = 0; ch < C; ++ch) {
    const T *fc = f + (int64_t)ch * H * W;
    float s = 0.f;
#pragma unroll
    for (int dy = 0; dy < 3; ++dy) {
      const int rr = reflect(r + dy - 1, H);
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        const int cc = reflect(c + dx - 1, W);
        s = fadd(s, fmul(k.w[dy * 3 + dx], load_feat(fc + (int64_t)rr * W + cc)));
      }
    }
    dst[(int64_t)ch * H * W + (int64_t)r * W + c] = to_t<T>(s);
  }
}

int check_hw(int H, int W) {
  if (H <= 0 || W <= 0)
    return fail(STB_EINVAL, "Check failed: image size must be positive, got %dx%d", H, W);
  return STB_OK;
}

int check_down(int H, int W, float scale, int DH, int DW) {
  STB_TRY(check_hw(H, W));
  if (!(scale > 0.f && scale <= 1.f))
    return fail(STB_EINVAL, "Check failed: scale must be in (0, 1], got %g", scale);
  if (DH != (int)(H * scale) || DW != (int)(W * scale) || DH <= 0 || DW <= 0)
    return fail(STB_EINVAL, "Check failed: destination must be int(size * scale), got %dx%d",
                DH, DW);
  return STB_OK;
}

// [C][n] -> [n][C] through a shared-memory tile of kTX pixels x up to kTC
// channels: loads coalesced along pixels, stores coalesced along channels.
constexpr int kTX = 32, kTC = 32;
template <typename T>
__global__ void k_interleave(const T *__restrict__ src, T *__restrict__ dst, int C, int64_t n) {
  __shared__ T tile[kTC][kTX + 1];
  const int64_t x0 = (int64_t)blockIdx.x * kTX;
  for (int c0 = 0; c0 < C; c0 += kTC) {
    // load: thread (tx, ty) reads channel c0 + ty, pixel x0 + tx
    for (int ty = threadIdx.y; ty < kTC; ty += blockDim.y) {
      const int c = c0 + ty;
      const int64_t x = x0 + threadIdx.x;
      if (c < C && x < n) tile[ty][threadIdx.x] = src[(int64_t)c * n + x];
    }
    __syncthreads();
    // store: consecutive threads write consecutive channels of a pixel
    const int cw = min(kTC, C - c0);
    for (int k = threadIdx.y * kTX + threadIdx.x; k < kTX * cw; k += blockDim.x * blockDim.y) {
      const int px = k / cw, c = k % cw;
      const int64_t x = x0 + px;
      if (x < n) dst[x * C + c0 + c] = tile[c][px];
    }
    __syncthreads();
  }
}

// BilateralDepthFilterKernel (src/bilateral_depth_filter.cu:15-72).  A block
// computes a kBX x kBLR tile of outputs from a shared-memory copy of the
// scaled depth and the mask over the tile plus the filter's halo (read once
// from HBM, coalesced); every output then walks its (2 hw + 1)^2 taps in
// shared memory, rows outer and columns inner as the reference, with its
// float32 operations uncontracted.  Taps outside the image read as masked.
constexpr int kBLR = 16;           // output rows per block (2 per thread)
constexpr int kMaxHalfWidth = 15;  // filter_width <= 31
constexpr int kBLW = kBX + 2 * kMaxHalfWidth, kBLH = kBLR + 2 * kMaxHalfWidth;

template <typename T>
__device__ __forceinline__ float scaled_depth(T v, float scale) {
  return fmul((float)v, scale);
}
template <>
__device__ __forceinline__ float scaled_depth<double>(double v, float scale) {
  return __double2float_rn(__dmul_rn(v, (double)scale));
}
template <typename T>
__device__ __forceinline__ T from_float(float x) {
  return (T)x;  // integers truncate toward zero, as the reference's scalar_t(...)
}

template <typename T>
__global__ void __launch_bounds__(kBX * kBY) k_bilateral(const T *__restrict__ depth,
                                                         const uint8_t *__restrict__ mask,
                                                         T *__restrict__ out, int H, int W,
                                                         int hw, float inv_sc, float inv_ss,
                                                         float scale, float inv_scale) {
  __shared__ float zs[kBLH][kBLW];
  __shared__ uint8_t ms[kBLH][kBLW];
  const int c0 = blockIdx.x * kBX - hw, r0 = blockIdx.y * kBLR - hw;
  const int tw = kBX + 2 * hw, th = kBLR + 2 * hw;
  for (int k = threadIdx.y * kBX + threadIdx.x; k < tw * th; k += kBX * kBY) {
    const int ty = k / tw, tx = k % tw;
    const int r = r0 + ty, c = c0 + tx;
    const bool in = r >= 0 && r < H && c >= 0 && c < W;
    const int64_t i = in ? (int64_t)r * W + c : 0;
    ms[ty][tx] = in && mask[i];
    zs[ty][tx] = in ? scaled_depth(depth[i], scale) : 0.f;
  }
  __syncthreads();
#pragma unroll
  for (int half = 0; half < kBLR / kBY; ++half) {
    const int ly = threadIdx.y + half * kBY, lx = threadIdx.x;
    const int row = blockIdx.y * kBLR + ly, col = blockIdx.x * kBX + lx;
    if (row >= H || col >= W) continue;
    const int64_t o = (int64_t)row * W + col;
    if (!ms[ly + hw][lx + hw]) {
      out[o] = from_float<T>(0.f);
      continue;
    }
    const float z = zs[ly + hw][lx + hw];
    float color_sum = 0.f, weight_sum = 0.f;
    for (int y = -hw; y <= hw; ++y) {
      for (int x = -hw; x <= hw; ++x) {
        if (!ms[ly + hw + y][lx + hw + x]) continue;
        const float cz = zs[ly + hw + y][lx + hw + x];
        const float dx = (float)(-x), dy = (float)(-y);
        const float space_sqr = fadd(fmul(dx, dx), fmul(dy, dy));
        const float dcolor = fsub(z, cz);
        const float color_sqr = fmul(dcolor, dcolor);
        const float weight =
            expf(fmul(-0.5f, fadd(fmul(space_sqr, inv_ss), fmul(color_sqr, inv_sc))));
        color_sum = fadd(color_sum, fmul(cz, weight));
        weight_sum = fadd(weight_sum, weight);
      }
    }
    out[o] = from_float<T>(weight_sum > 0.f ? fmul(fdiv(color_sum, weight_sum), inv_scale)
                                            : 0.f);
  }
}

}  // namespace
}  // namespace stb

using namespace stb;

extern "C" int stb_depth_to_points(const float *depth, float depth_scale, float depth_bias,
                                   const float *kcam, float *points, uint8_t *raw_mask,
                                   int32_t height, int32_t width, void *stream) {
  clear_error();
  STB_TRY(check_hw(height, width));
  STB_TRY(check_device_ptr(depth, "depth"));
  STB_TRY(check_device_ptr(kcam, "kcam"));
  STB_TRY(check_device_ptr(points, "points"));
  STB_TRY(check_device_ptr(raw_mask, "mask"));
  k_depth_to_points<<<grid2(width, height), dim3(kBX, kBY), 0, as_stream(stream)>>>(
      depth, depth_scale, depth_bias, kcam, points, raw_mask, height, width);
  return check_launch("stb_depth_to_points");
}

extern "C" int stb_erode_mask(const uint8_t *in_mask, uint8_t *out_mask, int32_t height,
                              int32_t width, void *stream) {
  clear_error();
  STB_TRY(check_hw(height, width));
  STB_TRY(check_device_ptr(in_mask, "in_mask"));
  STB_TRY(check_device_ptr(out_mask, "out_mask"));
  if (in_mask == out_mask) return fail(STB_EINVAL, "Check failed: erosion cannot run in place");
  k_erode<<<grid2(width, height), dim3(kBX, kBY), 0, as_stream(stream)>>>(in_mask, out_mask,
                                                                          height, width);
  return check_launch("stb_erode_mask");
}

extern "C" int stb_estimate_normals(const float *xyz, const uint8_t *mask, float *normals,
                                    int32_t height, int32_t width, void *stream) {
  clear_error();
  STB_TRY(check_hw(height, width));
  STB_TRY(check_device_ptr(xyz, "xyz_image"));
  STB_TRY(check_device_ptr(mask, "mask_image"));
  STB_TRY(check_device_ptr(normals, "out_normals"));
  k_normals<<<grid2(width, height), dim3(kBX, kBY), 0, as_stream(stream)>>>(xyz, mask, normals,
                                                                           height, width);
  return check_launch("stb_estimate_normals");
}

extern "C" int stb_downsample_xyz(const float *xyz, const uint8_t *mask, int32_t height,
                                  int32_t width, float scale, float *dst, int32_t dst_height,
                                  int32_t dst_width, void *stream) {
  clear_error();
  STB_TRY(check_down(height, width, scale, dst_height, dst_width));
  STB_TRY(check_device_ptr(xyz, "xyz_image"));
  STB_TRY(check_device_ptr(mask, "mask"));
  STB_TRY(check_device_ptr(dst, "dst"));
  k_downsample_xyz<<<grid2(dst_width, dst_height), dim3(kBX, kBY), 0, as_stream(stream)>>>(
      xyz, mask, height, width, 1.0f / scale, dst, dst_height, dst_width);
  return check_launch("stb_downsample_xyz");
}

extern "C" int stb_downsample_mask(const uint8_t *mask, int32_t height, int32_t width,
                                   float scale, uint8_t *dst, int32_t dst_height,
                                   int32_t dst_width, void *stream) {
  clear_error();
  STB_TRY(check_down(height, width, scale, dst_height, dst_width));
  STB_TRY(check_device_ptr(mask, "mask"));
  STB_TRY(check_device_ptr(dst, "dst"));
  k_downsample_mask<<<grid2(dst_width, dst_height), dim3(kBX, kBY), 0, as_stream(stream)>>>(
      mask, height, width, 1.0f / scale, dst, dst_height, dst_width);
  return check_launch("stb_downsample_mask");
}

extern "C" int stb_downsample_features(const void *feats, int32_t channels, int32_t height,
                                       int32_t width, int32_t feat_dtype, float scale,
                                       void *dst, int32_t dst_height, int32_t dst_width,
                                       void *stream) {
  clear_error();
  STB_TRY(check_down(height, width, scale, dst_height, dst_width));
  if (channels <= 0) return fail(STB_EINVAL, "Check failed: channels must be positive");
  STB_TRY(check_device_ptr(feats, "feature_image"));
  STB_TRY(check_device_ptr(dst, "dst"));
  const dim3 g = grid2(dst_width, dst_height), b(kBX, kBY);
  if (feat_dtype == STB_F32)
    k_downsample_feat<float><<<g, b, 0, as_stream(stream)>>>(
        static_cast<const float *>(feats), channels, height, width, 1.0f / scale,
        static_cast<float *>(dst), dst_height, dst_width);
  else if (feat_dtype == STB_BF16)
    k_downsample_feat<__nv_bfloat16><<<g, b, 0, as_stream(stream)>>>(
        static_cast<const __nv_bfloat16 *>(feats), channels, height, width, 1.0f / scale,
        static_cast<__nv_bfloat16 *>(dst), dst_height, dst_width);
  else
    return fail(STB_EDTYPE, "Check failed: feature maps must be float32 or bfloat16");
  return check_launch("stb_downsample_features");
}

extern "C" int stb_gaussian_blur3(const void *feats, int32_t channels, int32_t height,
                                  int32_t width, int32_t feat_dtype, double sigma, void *dst,
                                  void *stream) {
  clear_error();
  STB_TRY(check_hw(height, width));
  if (height < 2 || width < 2)
    return fail(STB_EINVAL, "Check failed: reflect padding needs at least 2x2 pixels");
  if (channels <= 0) return fail(STB_EINVAL, "Check failed: channels must be positive");
  if (!(sigma > 0.0)) return fail(STB_EINVAL, "Check failed: sigma must be positive");
  STB_TRY(check_device_ptr(feats, "feature_image"));
  STB_TRY(check_device_ptr(dst, "dst"));
  if (feats == dst) return fail(STB_EINVAL, "Check failed: blur cannot run in place");
  double g[3], sum = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double x = k - 1;
    g[k] = exp(-(x * x) / (2.0 * sigma * sigma));
    sum += g[k];
  }
  Kernel3 k3;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) k3.w[a * 3 + b] = (float)((g[a] / sum) * (g[b] / sum));
  const dim3 gr = grid2(width, height), bl(kBX, kBY);
  if (feat_dtype == STB_F32)
    k_blur3<float><<<gr, bl, 0, as_stream(stream)>>>(static_cast<const float *>(feats), channels,
                                                     height, width, k3,
                                                     static_cast<float *>(dst));
  else if (feat_dtype == STB_BF16)
    k_blur3<__nv_bfloat16><<<gr, bl, 0, as_stream(stream)>>>(
        static_cast<const __nv_bfloat16 *>(feats), channels, height, width, k3,
        static_cast<__nv_bfloat16 *>(dst));
  else
    return fail(STB_EDTYPE, "Check failed: feature maps must be float32 or bfloat16");
  return check_launch("stb_gaussian_blur3");
}

extern "C" int stb_feature_interleave(const void *src, void *dst, int32_t channels,
                                      int64_t count, int32_t feat_dtype, void *stream) {
  clear_error();
  if (channels <= 0) return fail(STB_EINVAL, "Check failed: channels must be positive");
  if (count <= 0) return fail(STB_EINVAL, "Check failed: count must be positive");
  STB_TRY(check_device_ptr(src, "src"));
  STB_TRY(check_device_ptr(dst, "dst"));
  if (src == dst) return fail(STB_EINVAL, "Check failed: interleave cannot run in place");
  const dim3 grid((unsigned)((count + kTX - 1) / kTX)), block(kTX, 8);
  if (feat_dtype == STB_F32)
    k_interleave<float><<<grid, block, 0, as_stream(stream)>>>(
        static_cast<const float *>(src), static_cast<float *>(dst), channels, count);
  else if (feat_dtype == STB_BF16)
    k_interleave<__nv_bfloat16><<<grid, block, 0, as_stream(stream)>>>(
        static_cast<const __nv_bfloat16 *>(src), static_cast<__nv_bfloat16 *>(dst), channels,
        count);
  else
    return fail(STB_EDTYPE, "Check failed: feature maps must be float32 or bfloat16");
  return check_launch("stb_feature_interleave");
}

extern "C" int stb_bilateral_depth_filter(const void *depth, const uint8_t *mask, void *out,
                                          int32_t height, int32_t width, int32_t dtype,
                                          int32_t filter_width, float sigma_color,
                                          float sigma_space, float depth_scale, void *stream) {
  clear_error();
  STB_TRY(check_hw(height, width));
  if (filter_width < 0 || filter_width / 2 > kMaxHalfWidth)
    return fail(STB_EINVAL, "Check failed: filter_width must be in [0, %d], got %d",
                2 * kMaxHalfWidth + 1, filter_width);
  STB_TRY(check_device_ptr(depth, "depth"));
  STB_TRY(check_device_ptr(mask, "mask"));
  STB_TRY(check_device_ptr(out, "out"));
  if (depth == out) return fail(STB_EINVAL, "Check failed: the filter cannot run in place");
  const int hw = filter_width / 2;
  // as the reference: 1.0 / (sigma * sigma) with the product in float and
  // the quotient in double, both kept as float; 1.0 / depth_scale likewise
  const float inv_sc = (float)(1.0 / (double)(sigma_color * sigma_color));
  const float inv_ss = (float)(1.0 / (double)(sigma_space * sigma_space));
  const float inv_scale = (float)(1.0 / (double)depth_scale);
  const dim3 grid((width + kBX - 1) / kBX, (height + kBLR - 1) / kBLR), block(kBX, kBY);
  const cudaStream_t st = as_stream(stream);
#define STB_BILATERAL(T)                                                                  \
  k_bilateral<T><<<grid, block, 0, st>>>(static_cast<const T *>(depth), mask,           \
                                         static_cast<T *>(out), height, width, hw, inv_sc, \
                                         inv_ss, depth_scale, inv_scale)
  switch (dtype) {
    case STB_F32: STB_BILATERAL(float); break;
    case STB_F64: STB_BILATERAL(double); break;
    case STB_U8: STB_BILATERAL(uint8_t); break;
    case STB_I16: STB_BILATERAL(int16_t); break;
    case STB_U16: STB_BILATERAL(uint16_t); break;
    case STB_I32: STB_BILATERAL(int32_t); break;
    case STB_I64: STB_BILATERAL(int64_t); break;
    default: return fail(STB_EDTYPE, "Check failed: unsupported depth dtype %d", dtype);
  }
#undef STB_BILATERAL
  return check_launch("stb_bilateral_depth_filter");
}
