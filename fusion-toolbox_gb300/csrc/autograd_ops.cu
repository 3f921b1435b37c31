// Differentiable registration layer of the reference's AutogradICP
// (slamtb/registration/autogradicp.py:145-239):
//   * ExpRtToMatrixOp (src/exp_rt_to_matrix.cu:12-121, src/exp_rt.hpp:9-142):
//     a twist [t; w] (w = rotation axis x angle) to the 3x4 matrix [R(w) | t]
//     and its backward by the derivative of Gallego and Yezzi;
//   * MatrixToExpRtOp (src/matrix_to_exp_rt.cu:12-50): the inverse map;
//   * FPCLMatcherOp (src/fpcl_matcher.cu:13-229, src/feature_map.hpp): the
//     projective match of transformed source points against a target frame
//     (points, normals and bilinearly sampled features), and the gradient of
//     a loss on the sampled features with respect to the source points.
// One thread per element.  The float32 instantiations use round-to-nearest
// intrinsics (no FMA contraction) so that the matcher's samples and
// gradients follow the reference's float32 operation order exactly.
#include <math.h>

#include "stb_common.cuh"
#include "stb_host.hpp"

namespace stb {
namespace {

constexpr int kOpThreads = 256;

template <typename T>
struct Arith;
template <>
struct Arith<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
  static __device__ __forceinline__ void sincos_(float a, float *s, float *c) { sincosf(a, s, c); }
  static __device__ __forceinline__ float atan2_(float y, float x) { return atan2f(y, x); }
};
template <>
struct Arith<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
  static __device__ __forceinline__ void sincos_(double a, double *s, double *c) { sincos(a, s, c); }
  static __device__ __forceinline__ double atan2_(double y, double x) { return atan2(y, x); }
};

// ---------------------------------------------------------------------------
// ExpRt: twist [t; w] <-> [R(w) | t]
// ---------------------------------------------------------------------------

// R(w) by Rodrigues' formula, R = cos(a) I + sin(a) [k]x + (1 - cos(a)) k k^T
// with a = |w| and k = w / a (k = w when a = 0, as a normalised zero
// vector stays zero), the construction AngleAxis(|w|, w / |w|) of
// exp_rt.hpp:27-32 followed by its rotation matrix.
template <typename T>
__device__ __forceinline__ void rodrigues(T wx, T wy, T wz, T R[9]) {
  using A = Arith<T>;
  const T n2 = A::add(A::add(A::mul(wx, wx), A::mul(wy, wy)), A::mul(wz, wz));
  const T ang = A::sqrt_(n2);
  T kx = wx, ky = wy, kz = wz;
  if (n2 > T(0)) {
    kx = A::div(wx, ang);
    ky = A::div(wy, ang);
    kz = A::div(wz, ang);
  }
  T s, c;
  A::sincos_(ang, &s, &c);
  const T c1 = A::sub(T(1), c);
  const T sx = A::mul(s, kx), sy = A::mul(s, ky), sz = A::mul(s, kz);
  const T cx = A::mul(c1, kx), cy = A::mul(c1, ky), cz = A::mul(c1, kz);
  R[0] = A::add(A::mul(cx, kx), c);
  R[4] = A::add(A::mul(cy, ky), c);
  R[8] = A::add(A::mul(cz, kz), c);
  const T xy = A::mul(cx, ky), xz = A::mul(cx, kz), yz = A::mul(cy, kz);
  R[1] = A::sub(xy, sz);
  R[3] = A::add(xy, sz);
  R[2] = A::add(xz, sy);
  R[6] = A::sub(xz, sy);
  R[5] = A::sub(yz, sx);
  R[7] = A::add(yz, sx);
}

template <typename T>
__global__ void __launch_bounds__(kOpThreads) k_exp_rt_to_matrix(const T *__restrict__ x,
                                                                 T *__restrict__ m,
                                                                 long long count) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= count) return;
  const T *xi = x + 6 * i;
  T R[9];
  rodrigues<T>(xi[3], xi[4], xi[5], R);
  T *mi = m + 12 * i;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c) mi[4 * r + c] = R[3 * r + c];
    mi[4 * r + 3] = xi[r];
  }
}

// d loss / d [t; w] from d loss / d M (3x4) and the forward's M
// (exp_rt_to_matrix.cu:56-98, exp_rt.hpp:90-138).  dM / dt_r is the unit at
// (r, 3).  dR / dw_k = [u_k]x R with u_k = (w w_k + w x ((I - R) e_k)) /
// |w|^2 (Gallego and Yezzi, "A compact formula for the derivative of a 3-D
// rotation in exponential coordinates", JMIV 51(3), 2015), and u_k = e_k
// when |w|^2 <= 1e-12.
template <typename T>
__global__ void __launch_bounds__(kOpThreads) k_exp_rt_to_matrix_backward(
    const T *__restrict__ dm, const T *__restrict__ x, const T *__restrict__ m,
    T *__restrict__ dx, long long count) {
  using A = Arith<T>;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= count) return;
  const T *xi = x + 6 * i, *mi = m + 12 * i, *g = dm + 12 * i;
  const T v[3] = {xi[3], xi[4], xi[5]};
  const T vn = A::add(A::add(A::mul(v[0], v[0]), A::mul(v[1], v[1])), A::mul(v[2], v[2]));
  T R[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) R[3 * r + c] = mi[4 * r + c];
  T *o = dx + 6 * i;
  o[0] = g[3];
  o[1] = g[7];
  o[2] = g[11];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T u[3];
    if (vn > T(1e-12)) {
      // e = column k of I - R
      const T e[3] = {A::sub(k == 0 ? T(1) : T(0), R[k]), A::sub(k == 1 ? T(1) : T(0), R[3 + k]),
                      A::sub(k == 2 ? T(1) : T(0), R[6 + k])};
      const T vxe[3] = {A::sub(A::mul(v[1], e[2]), A::mul(v[2], e[1])),
                        A::sub(A::mul(v[2], e[0]), A::mul(v[0], e[2])),
                        A::sub(A::mul(v[0], e[1]), A::mul(v[1], e[0]))};
#pragma unroll
      for (int r = 0; r < 3; ++r) u[r] = A::div(A::add(A::mul(v[r], v[k]), vxe[r]), vn);
    } else {
      u[0] = k == 0 ? T(1) : T(0);
      u[1] = k == 1 ? T(1) : T(0);
      u[2] = k == 2 ? T(1) : T(0);
    }
    // [u]x = [[0, -u2, u1], [u2, 0, -u0], [-u1, u0, 0]]; dR = [u]x R
    const T S[9] = {T(0), -u[2], u[1], u[2], T(0), -u[0], -u[1], u[0], T(0)};
    T acc = T(0);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const T d = A::add(A::add(A::mul(S[3 * r], R[c]), A::mul(S[3 * r + 1], R[3 + c])),
                           A::mul(S[3 * r + 2], R[6 + c]));
        acc = A::add(acc, A::mul(d, g[4 * r + c]));
      }
    o[3 + k] = acc;
  }
}

// [R | t] -> [t; w], w = axis x angle of R (matrix_to_exp_rt.cu:20-32: the
// AngleAxis of R).  R to a unit quaternion by Shepperd's method (the trace
// branch when the trace is positive, else the branch of the largest
// diagonal entry; Shepperd, J. Guidance and Control 1(3), 1978), then
// angle = 2 atan2(|q_v|, |q_w|) and axis = sign(q_w) q_v / |q_v|, w = 0 when
// |q_v| = 0.
template <typename T>
__global__ void __launch_bounds__(kOpThreads) k_matrix_to_exp_rt(const T *__restrict__ m,
                                                                 T *__restrict__ x,
                                                                 long long count) {
  using A = Arith<T>;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= count) return;
  const T *mi = m + 12 * i;
#define M(r, c) mi[4 * (r) + (c)]
  T q[3], w;
  const T tr = A::add(A::add(M(0, 0), M(1, 1)), M(2, 2));
  if (tr > T(0)) {
    T t = A::sqrt_(A::add(tr, T(1)));
    w = A::mul(T(0.5), t);
    t = A::div(T(0.5), t);
    q[0] = A::mul(A::sub(M(2, 1), M(1, 2)), t);
    q[1] = A::mul(A::sub(M(0, 2), M(2, 0)), t);
    q[2] = A::mul(A::sub(M(1, 0), M(0, 1)), t);
  } else {
    int a = 0;
    if (M(1, 1) > M(0, 0)) a = 1;
    if (M(2, 2) > M(a, a)) a = 2;
    const int b = (a + 1) % 3, c = (b + 1) % 3;
    T t = A::sqrt_(A::add(A::sub(A::sub(M(a, a), M(b, b)), M(c, c)), T(1)));
    q[a] = A::mul(T(0.5), t);
    t = A::div(T(0.5), t);
    w = A::mul(A::sub(M(c, b), M(b, c)), t);
    q[b] = A::mul(A::add(M(b, a), M(a, b)), t);
    q[c] = A::mul(A::add(M(c, a), M(a, c)), t);
  }
  T *xi = x + 6 * i;
  xi[0] = M(0, 3);
  xi[1] = M(1, 3);
  xi[2] = M(2, 3);
#undef M
  const T n = A::sqrt_(A::add(A::add(A::mul(q[0], q[0]), A::mul(q[1], q[1])), A::mul(q[2], q[2])));
  if (n == T(0)) {
    xi[3] = xi[4] = xi[5] = T(0);
    return;
  }
  const T ang = A::mul(T(2), A::atan2_(n, fabs(w)));
  const T f = A::div(w < T(0) ? -ang : ang, n);
  xi[3] = A::mul(q[0], f);
  xi[4] = A::mul(q[1], f);
  xi[5] = A::mul(q[2], f);
}

// ---------------------------------------------------------------------------
// FPCLMatcherOp
// ---------------------------------------------------------------------------

// Bilinear sample of channel c at (u, v) (feature_map.hpp:8-43): the cell
// of (int(u), int(v)) (truncation), its right / lower neighbours read as 0
// past the last column / row, weights u - int(u) and v - int(v).
template <typename T>
__device__ __forceinline__ T bilinear_fm(const T *__restrict__ f, int H, int W, T u, T v) {
  using A = Arith<T>;
  const int ui = (int)u, vi = (int)v;
  const T ur = A::sub(u, (T)ui), vr = A::sub(v, (T)vi);
  const bool r = ui + 1 < W, d = vi + 1 < H;
  const long long o = (long long)vi * W + ui;
  const T v00 = f[o];
  const T v10 = r ? f[o + 1] : T(0);
  const T v01 = d ? f[o + W] : T(0);
  const T v11 = (r && d) ? f[o + W + 1] : T(0);
  const T u0 = A::add(A::mul(v00, A::sub(T(1), ur)), A::mul(v10, ur));
  const T u1 = A::add(A::mul(v01, A::sub(T(1), ur)), A::mul(v11, ur));
  return A::add(A::mul(u0, A::sub(T(1), vr)), A::mul(u1, vr));
}

// KCamera::Project (camera.hpp:52-59): (fx x) / z + cx.
template <typename T>
__device__ __forceinline__ void project_k(const T *k, T x, T y, T z, T &u, T &v) {
  using A = Arith<T>;
  u = A::add(A::div(A::mul(k[0], x), z), k[2]);
  v = A::add(A::div(A::mul(k[4], y), z), k[5]);
}

template <typename T>
__device__ __forceinline__ bool round_in_t(T u, int size, int &ui) {
  const T r = round(u);
  if (!(r >= T(0) && r < (T)size)) return false;
  ui = (int)r;
  return true;
}

// Forward (fpcl_matcher.cu:46-80): source point i matches when it projects
// into the target image and the correspondence map's winner at that pixel
// is i.  A match takes the target point and normal at the pixel and the
// bilinear feature sample at the unrounded projection.  Points that do not
// match get mask 0 and zero outputs (the reference leaves them unwritten).
template <typename T>
__global__ void __launch_bounds__(kOpThreads) k_fpcl_forward(
    const T *__restrict__ tp, const T *__restrict__ tn, const T *__restrict__ tf, int C, int H,
    int W, const T *__restrict__ sp, long long n, const T *__restrict__ kcam,
    const long long *__restrict__ merge_map, T *__restrict__ op, T *__restrict__ on,
    T *__restrict__ of, uint8_t *__restrict__ mask) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  T u, v;
  project_k<T>(kcam, sp[3 * i], sp[3 * i + 1], sp[3 * i + 2], u, v);
  int ui = 0, vi = 0;
  bool ok = round_in_t<T>(u, W, ui) && round_in_t<T>(v, H, vi);
  const long long pix = (long long)vi * W + ui;
  ok = ok && (long long)(int)(merge_map[pix] >> 32) == i;
  mask[i] = ok;
  if (!ok) {
#pragma unroll
    for (int d = 0; d < 3; ++d) op[3 * i + d] = on[3 * i + d] = T(0);
    for (int c = 0; c < C; ++c) of[c * n + i] = T(0);
    return;
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    op[3 * i + d] = tp[3 * pix + d];
    on[3 * i + d] = tn[3 * pix + d];
  }
  const long long plane = (long long)H * W;
  for (int c = 0; c < C; ++c) of[c * n + i] = bilinear_fm<T>(tf + c * plane, H, W, u, v);
}

// Backward (fpcl_matcher.cu:126-190): the feature gradient by central
// differences of the bilinear sample with step h (the lower sample clamped
// at 0, feature_map.hpp:45-63), contracted with d loss / d feature over the
// channels, then through the projection's Jacobian (camera.hpp:64-77).
// 0 < h < 0.5 keeps every sample inside the map.
template <typename T>
__global__ void __launch_bounds__(kOpThreads) k_fpcl_backward(
    const T *__restrict__ tf, int C, int H, int W, const T *__restrict__ sp, long long n,
    const uint8_t *__restrict__ mask, const T *__restrict__ dl, const T *__restrict__ kcam,
    T h, T *__restrict__ dx) {
  using A = Arith<T>;
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T x = sp[3 * i], y = sp[3 * i + 1], z = sp[3 * i + 2];
  T u, v;
  project_k<T>(kcam, x, y, z, u, v);
  // a match projects inside the map (re-tested, so that no mask can lead a
  // sample out of it): with h < 0.5 every sample then stays inside
  int ui, vi;
  if (!mask[i] || !round_in_t<T>(u, W, ui) || !round_in_t<T>(v, H, vi)) {
    dx[3 * i] = dx[3 * i + 1] = dx[3 * i + 2] = T(0);
    return;
  }
  const T div = A::div(T(1), A::mul(T(2), h));
  const T up = A::add(u, h), um = fmax(A::sub(u, h), T(0));
  const T vp = A::add(v, h), vm = fmax(A::sub(v, h), T(0));
  const long long plane = (long long)H * W;
  T gu = T(0), gv = T(0);
  for (int c = 0; c < C; ++c) {
    const T *f = tf + c * plane;
    const T du = A::mul(A::sub(bilinear_fm<T>(f, H, W, up, v), bilinear_fm<T>(f, H, W, um, v)), div);
    const T dv = A::mul(A::sub(bilinear_fm<T>(f, H, W, u, vp), bilinear_fm<T>(f, H, W, u, vm)), div);
    const T g = dl[c * n + i];
    gu = A::add(gu, A::mul(du, g));
    gv = A::add(gv, A::mul(dv, g));
  }
  const T fx = kcam[0], fy = kcam[4];
  const T z2 = A::mul(z, z);
  const T j00 = A::div(fx, z), j02 = A::div(A::mul(-x, fx), z2);
  const T j11 = A::div(fy, z), j12 = A::div(A::mul(-y, fy), z2);
  dx[3 * i] = A::mul(j00, gu);
  dx[3 * i + 1] = A::mul(j11, gv);
  dx[3 * i + 2] = A::add(A::mul(j02, gu), A::mul(j12, gv));
}

unsigned grid1(long long n) { return (unsigned)((n + kOpThreads - 1) / kOpThreads); }

int check_float_dtype(int32_t dtype) {
  if (dtype != STB_F32 && dtype != STB_F64)
    return fail(STB_EDTYPE, "Check failed: expected float32 or float64 (dtype %d)", dtype);
  return STB_OK;
}

int check_hw(int H, int W) {
  if (H <= 0 || W <= 0)
    return fail(STB_EINVAL, "Check failed: image size must be positive, got %dx%d", H, W);
  return STB_OK;
}

int check_count(long long count) {
  if (count < 0 || count >= (1ll << 31) * kOpThreads)
    return fail(STB_EINVAL, "Check failed: count %lld out of range", count);
  return STB_OK;
}

}  // namespace
}  // namespace stb

using namespace stb;

extern "C" int stb_exp_rt_to_matrix(const void *exp_rt, void *matrix, int64_t count,
                                    int32_t dtype, void *stream) {
  clear_error();
  STB_TRY(check_float_dtype(dtype));
  STB_TRY(check_count(count));
  if (count == 0) return STB_OK;
  STB_TRY(check_device_ptr(exp_rt, "exp_rt"));
  STB_TRY(check_device_ptr(matrix, "matrix"));
  const cudaStream_t st = as_stream(stream);
  if (dtype == STB_F32)
    k_exp_rt_to_matrix<float><<<grid1(count), kOpThreads, 0, st>>>(
        static_cast<const float *>(exp_rt), static_cast<float *>(matrix), count);
  else
    k_exp_rt_to_matrix<double><<<grid1(count), kOpThreads, 0, st>>>(
        static_cast<const double *>(exp_rt), static_cast<double *>(matrix), count);
  return check_launch("stb_exp_rt_to_matrix");
}

extern "C" int stb_exp_rt_to_matrix_backward(const void *d_matrix, const void *exp_rt,
                                             const void *matrix, void *d_exp_rt, int64_t count,
                                             int32_t dtype, void *stream) {
  clear_error();
  STB_TRY(check_float_dtype(dtype));
  STB_TRY(check_count(count));
  if (count == 0) return STB_OK;
  STB_TRY(check_device_ptr(d_matrix, "d_matrix"));
  STB_TRY(check_device_ptr(exp_rt, "exp_rt"));
  STB_TRY(check_device_ptr(matrix, "matrix"));
  STB_TRY(check_device_ptr(d_exp_rt, "d_exp_rt"));
  const cudaStream_t st = as_stream(stream);
  if (dtype == STB_F32)
    k_exp_rt_to_matrix_backward<float><<<grid1(count), kOpThreads, 0, st>>>(
        static_cast<const float *>(d_matrix), static_cast<const float *>(exp_rt),
        static_cast<const float *>(matrix), static_cast<float *>(d_exp_rt), count);
  else
    k_exp_rt_to_matrix_backward<double><<<grid1(count), kOpThreads, 0, st>>>(
        static_cast<const double *>(d_matrix), static_cast<const double *>(exp_rt),
        static_cast<const double *>(matrix), static_cast<double *>(d_exp_rt), count);
  return check_launch("stb_exp_rt_to_matrix_backward");
}

extern "C" int stb_matrix_to_exp_rt(const void *matrix, void *exp_rt, int64_t count,
                                    int32_t dtype, void *stream) {
  clear_error();
  STB_TRY(check_float_dtype(dtype));
  STB_TRY(check_count(count));
  if (count == 0) return STB_OK;
  STB_TRY(check_device_ptr(matrix, "matrix"));
  STB_TRY(check_device_ptr(exp_rt, "exp_rt"));
  const cudaStream_t st = as_stream(stream);
  if (dtype == STB_F32)
    k_matrix_to_exp_rt<float><<<grid1(count), kOpThreads, 0, st>>>(
        static_cast<const float *>(matrix), static_cast<float *>(exp_rt), count);
  else
    k_matrix_to_exp_rt<double><<<grid1(count), kOpThreads, 0, st>>>(
        static_cast<const double *>(matrix), static_cast<double *>(exp_rt), count);
  return check_launch("stb_matrix_to_exp_rt");
}

extern "C" int stb_fpcl_match_forward(const void *tgt_points, const void *tgt_normals,
                                      const void *tgt_feats, int32_t channels, int32_t height,
                                      int32_t width, const void *src_points, int64_t num_source,
                                      const void *kcam, const int64_t *merge_map,
                                      void *out_points, void *out_normals, void *out_feats,
                                      uint8_t *match_mask, int32_t dtype, void *stream) {
  clear_error();
  STB_TRY(check_float_dtype(dtype));
  STB_TRY(check_hw(height, width));
  STB_TRY(check_count(num_source));
  if (channels < 0) return fail(STB_EINVAL, "Check failed: channels must be >= 0");
  if (num_source == 0) return STB_OK;
  STB_TRY(check_device_ptr(tgt_points, "target_points"));
  STB_TRY(check_device_ptr(tgt_normals, "target_normals"));
  if (channels > 0) {
    STB_TRY(check_device_ptr(tgt_feats, "target_features"));
    STB_TRY(check_device_ptr(out_feats, "out_features"));
  }
  STB_TRY(check_device_ptr(src_points, "source_points"));
  STB_TRY(check_device_ptr(kcam, "kcam"));
  STB_TRY(check_device_ptr(merge_map, "merge_map"));
  STB_TRY(check_device_ptr(out_points, "out_points"));
  STB_TRY(check_device_ptr(out_normals, "out_normals"));
  STB_TRY(check_device_ptr(match_mask, "match_mask"));
  const cudaStream_t st = as_stream(stream);
#define STB_FPCL_FWD(T)                                                                      \
  k_fpcl_forward<T><<<grid1(num_source), kOpThreads, 0, st>>>(                               \
      static_cast<const T *>(tgt_points), static_cast<const T *>(tgt_normals),                \
      static_cast<const T *>(tgt_feats), channels, height, width,                            \
      static_cast<const T *>(src_points), num_source, static_cast<const T *>(kcam),          \
      reinterpret_cast<const long long *>(merge_map), static_cast<T *>(out_points),           \
      static_cast<T *>(out_normals), static_cast<T *>(out_feats), match_mask)
  if (dtype == STB_F32)
    STB_FPCL_FWD(float);
  else
    STB_FPCL_FWD(double);
#undef STB_FPCL_FWD
  return check_launch("stb_fpcl_match_forward");
}

extern "C" int stb_fpcl_match_backward(const void *tgt_feats, int32_t channels, int32_t height,
                                       int32_t width, const void *src_points, int64_t num_source,
                                       const uint8_t *match_mask, const void *dl_feats,
                                       const void *kcam, double grad_precision, void *dx_points,
                                       int32_t dtype, void *stream) {
  clear_error();
  STB_TRY(check_float_dtype(dtype));
  STB_TRY(check_hw(height, width));
  STB_TRY(check_count(num_source));
  if (channels < 0) return fail(STB_EINVAL, "Check failed: channels must be >= 0");
  if (!(grad_precision > 0.0 && grad_precision < 0.5))
    return fail(STB_EINVAL, "Check failed: grad_precision must be in (0, 0.5), got %g",
                grad_precision);
  if (num_source == 0) return STB_OK;
  if (channels > 0) {
    STB_TRY(check_device_ptr(tgt_feats, "target_features"));
    STB_TRY(check_device_ptr(dl_feats, "dl_features"));
  }
  STB_TRY(check_device_ptr(src_points, "source_points"));
  STB_TRY(check_device_ptr(match_mask, "match_mask"));
  STB_TRY(check_device_ptr(kcam, "kcam"));
  STB_TRY(check_device_ptr(dx_points, "dx_points"));
  const cudaStream_t st = as_stream(stream);
  if (dtype == STB_F32)
    k_fpcl_backward<float><<<grid1(num_source), kOpThreads, 0, st>>>(
        static_cast<const float *>(tgt_feats), channels, height, width,
        static_cast<const float *>(src_points), num_source, match_mask,
        static_cast<const float *>(dl_feats), static_cast<const float *>(kcam),
        (float)grad_precision, static_cast<float *>(dx_points));
  else
    k_fpcl_backward<double><<<grid1(num_source), kOpThreads, 0, st>>>(
        static_cast<const double *>(tgt_feats), channels, height, width,
        static_cast<const double *>(src_points), num_source, match_mask,
        static_cast<const double *>(dl_feats), static_cast<const double *>(kcam),
        grad_precision, static_cast<double *>(dx_points));
  return check_launch("stb_fpcl_match_backward");
}
