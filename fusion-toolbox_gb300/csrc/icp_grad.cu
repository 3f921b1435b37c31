// Differentiable point-to-plane loss for batches of frame pairs, with a
// hand-written adjoint.
//
// Forward (per pair p, pose T_p): the ICPOdometry association at the float32
// cast of T_p (64-bit atomicMin z-buffer, the reference's gates) and
// L_p = sum over the correspondences of r^2, r = (q - T_p s).n
// (icp_jacobian_geometric.cu:82), summed in compensated float32.
// Adjoint (correspondences frozen): dL/dxi = -2 sum r J with J = [n; Tp x n]
// for T <- exp(xi) T_p (the sign convention of icp_jacobian_common.hpp:41-48,
// J = -dr/dxi), and dL/dz_i = -2 r_i (R^T n) . d_i for the source depth z_i,
// s_i = z_i d_i, d_i = ((u_i - cx)/fx, (v_i - cy)/fy, 1) (the back-projection
// of slamtb/camera.py:127-149).
//
// Grid: x = work items of a pair, y = pair.  Per-pair totals use per-block
// partials and a last-block ticket (deterministic order).
#include <math.h>

#include "gn_solve.cuh"
#include "stb_common.cuh"
#include "stb_host.hpp"

namespace stb {

float distance_thresh_sq(double d);
float angle_cos_max(double angle);

namespace {

constexpr int kT = 256;
constexpr int kItem = kT * 4;        // pixels per block
constexpr int kMaxBlocksX = 1024;    // blocks per pair (grid-stride beyond)
constexpr unsigned kTag = 254u;

struct GradLayout {
  size_t err, tickets, part, keys, total;
};

inline int blocks_x(int64_t max_px) {
  int64_t b = (max_px + kItem - 1) / kItem;
  return (int)(b < 1 ? 1 : (b > kMaxBlocksX ? kMaxBlocksX : b));
}

inline size_t al(size_t x) { return (x + 255) & ~size_t(255); }

inline GradLayout grad_layout(int B, int64_t max_px) {
  GradLayout g;
  size_t o = 0;
  g.err = o;
  o += 256;
  g.tickets = o;
  o += al(sizeof(unsigned) * (size_t)B);
  g.part = o;
  o += al(sizeof(float) * 16 * (size_t)B * blocks_x(max_px));
  g.keys = o;
  o += al(sizeof(unsigned long long) * (size_t)B * max_px);
  g.total = o;
  return g;
}

// Level descriptor and float32 pose of pair blockIdx.y, into shared memory.
__device__ __forceinline__ void pair_setup(const stb_level *levels, const double *poses,
                                           stb_level &lv, Pose32 &P) {
  if (threadIdx.x == 0) {
    lv = levels[blockIdx.y];
    double T[16];
    for (int k = 0; k < 16; ++k) T[k] = poses[blockIdx.y * 16 + k];
    P.fx = lv.fx;
    P.fy = lv.fy;
    P.cx = lv.cx;
    P.cy = lv.cy;
    refresh_pose32(P, T);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kT) k_g_assoc(const stb_level *levels, const double *poses,
                                                int64_t max_px, unsigned long long *keys_all,
                                                float thr2, float cos_max, unsigned *err) {
  __shared__ stb_level lv;
  __shared__ Pose32 P;
  pair_setup(levels, poses, lv, P);
  const int H = lv.height, W = lv.width;
  if ((int64_t)H * W > max_px) {
    if (threadIdx.x == 0) atomicOr(err, 2u);
    return;
  }
  unsigned long long *keys = keys_all + (size_t)blockIdx.y * max_px;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < lv.num_source;
       i += (int64_t)gridDim.x * kT) {
    if (!lv.src_mask[i]) continue;
    const float3 Tp = transform_point(P.rt, lv.src_points[3 * i], lv.src_points[3 * i + 1],
                                      lv.src_points[3 * i + 2]);
    float u, v;
    project(P, Tp, u, v);
    int ui, vi;
    if (!round_in(u, W, ui) || !round_in(v, H, vi)) continue;
    const int64_t pix = (int64_t)vi * W + ui;
    if (!lv.tgt_mask[pix]) continue;
    const float *tp = lv.tgt_points, *tn = lv.tgt_normals, *sn = lv.src_normals;
    const float dx = fsub(tp[3 * pix], Tp.x), dy = fsub(tp[3 * pix + 1], Tp.y),
                dz = fsub(tp[3 * pix + 2], Tp.z);
    const float sq = dot3(dx, dy, dz, dx, dy, dz);
    if (sq > thr2) continue;
    const float3 Tn = transform_normal(P.nm, sn[3 * i], sn[3 * i + 1], sn[3 * i + 2]);
    const float nx = tn[3 * pix], ny = tn[3 * pix + 1], nz = tn[3 * pix + 2];
    const float c = fdiv(dot3(Tn.x, Tn.y, Tn.z, nx, ny, nz),
                         fmul(__fsqrt_rn(dot3(Tn.x, Tn.y, Tn.z, Tn.x, Tn.y, Tn.z)),
                              __fsqrt_rn(dot3(nx, ny, nz, nx, ny, nz))));
    if (c >= -1.0f && c <= cos_max) continue;
    atomicMin(keys + pix, ((unsigned long long)kTag << 56) |
                              ((unsigned long long)__float_as_uint(__fsqrt_rn(sq)) << 24) |
                              (unsigned long long)i);
  }
}

// kN compensated sums of the block -> slot; last block of the pair folds the
// pair's slots into tot (FP64, smem); returns true in that block.
template <int kN>
__device__ bool pair_fold(CSum *acc, float *part_all, unsigned *tickets, double *tot) {
  __shared__ float ws[kT / 32][kN][2];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < kN; ++a) {
    csum_warp_reduce(acc[a]);
    if (lane == 0) {
      ws[warp][a][0] = acc[a].s;
      ws[warp][a][1] = acc[a].c;
    }
  }
  __syncthreads();
  float *slot = part_all + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 16;
  if (threadIdx.x < kN) {
    CSum t = {0.f, 0.f};
    for (int w = 0; w < kT / 32; ++w) csum_merge(t, ws[w][threadIdx.x][0], ws[w][threadIdx.x][1]);
    slot[threadIdx.x] = t.s;
    slot[8 + threadIdx.x] = t.c;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    s_last = atomicAdd(tickets + blockIdx.y, 1u) == gridDim.x - 1;
    if (s_last) tickets[blockIdx.y] = 0;
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  if (warp < kN) {
    CSum t = {0.f, 0.f};
    const float *base = part_all + (size_t)blockIdx.y * gridDim.x * 16;
    for (int b = lane; b < (int)gridDim.x; b += 32)
      csum_merge(t, __ldcg(base + (size_t)b * 16 + warp), __ldcg(base + (size_t)b * 16 + 8 + warp));
    csum_warp_reduce(t);
    if (lane == 0) tot[warp] = (double)t.s + (double)t.c;
  }
  __syncthreads();
  return true;
}

__global__ void __launch_bounds__(kT) k_g_loss(const stb_level *levels, const double *poses,
                                               int64_t max_px, const unsigned long long *keys_all,
                                               float *part, unsigned *tickets, double *loss) {
  __shared__ stb_level lv;
  __shared__ Pose32 P;
  __shared__ double tot[8];
  pair_setup(levels, poses, lv, P);
  const int64_t npix = (int64_t)lv.height * lv.width;
  const unsigned long long *keys = keys_all + (size_t)blockIdx.y * max_px;
  CSum acc[1] = {{0.f, 0.f}};
  if (npix <= max_px) {
    for (int64_t pix = blockIdx.x * (int64_t)kT + threadIdx.x; pix < npix;
         pix += (int64_t)gridDim.x * kT) {
      const unsigned long long key = __ldcg(keys + pix);
      if ((unsigned)(key >> 56) != kTag) continue;
      const int64_t i = (int64_t)(key & 0xffffffull);
      const float3 Tp = transform_point(P.rt, lv.src_points[3 * i], lv.src_points[3 * i + 1],
                                        lv.src_points[3 * i + 2]);
      const float *tp = lv.tgt_points + 3 * pix, *tn = lv.tgt_normals + 3 * pix;
      const float r = dot3(fsub(tp[0], Tp.x), fsub(tp[1], Tp.y), fsub(tp[2], Tp.z), tn[0], tn[1],
                           tn[2]);
      csum_add(acc[0], r * r);
    }
  }
  if (pair_fold<1>(acc, part, tickets, tot) && threadIdx.x == 0) loss[blockIdx.y] = tot[0];
}

__global__ void __launch_bounds__(kT) k_g_adjoint(const stb_level *levels, const double *poses,
                                                  int64_t max_px,
                                                  const unsigned long long *keys_all,
                                                  const double *grad_loss, float *part,
                                                  unsigned *tickets, double *grad_twist,
                                                  float *const *grad_depth) {
  __shared__ stb_level lv;
  __shared__ Pose32 P;
  __shared__ double tot[8];
  pair_setup(levels, poses, lv, P);
  const int H = lv.height, W = lv.width;
  const int64_t npix = (int64_t)H * W;
  const unsigned long long *keys = keys_all + (size_t)blockIdx.y * max_px;
  const float g = (float)grad_loss[blockIdx.y];
  float *gz = grad_depth ? grad_depth[blockIdx.y] : nullptr;
  CSum acc[6];
#pragma unroll
  for (int a = 0; a < 6; ++a) acc[a] = {0.f, 0.f};
  if (npix <= max_px) {
    for (int64_t pix = blockIdx.x * (int64_t)kT + threadIdx.x; pix < npix;
         pix += (int64_t)gridDim.x * kT) {
      const unsigned long long key = __ldcg(keys + pix);
      if ((unsigned)(key >> 56) != kTag) continue;
      const int64_t i = (int64_t)(key & 0xffffffull);
      const float3 Tp = transform_point(P.rt, lv.src_points[3 * i], lv.src_points[3 * i + 1],
                                        lv.src_points[3 * i + 2]);
      const float *tp = lv.tgt_points + 3 * pix, *tn = lv.tgt_normals + 3 * pix;
      const float nx = tn[0], ny = tn[1], nz = tn[2];
      const float r = dot3(fsub(tp[0], Tp.x), fsub(tp[1], Tp.y), fsub(tp[2], Tp.z), nx, ny, nz);
      const float Jv[6] = {nx, ny, nz, Tp.y * nz - Tp.z * ny, Tp.z * nx - Tp.x * nz,
                           Tp.x * ny - Tp.y * nx};
      const float s = -2.f * g * r;
#pragma unroll
      for (int a = 0; a < 6; ++a) csum_add(acc[a], s * Jv[a]);
      if (gz) {
        // R^T n, with R the float32 rotation of the pose
        const float *R = P.rt;
        const float rn0 = R[0] * nx + R[4] * ny + R[8] * nz;
        const float rn1 = R[1] * nx + R[5] * ny + R[9] * nz;
        const float rn2 = R[2] * nx + R[6] * ny + R[10] * nz;
        const float u = (float)(i % W), v = (float)(i / W);
        const float d0 = (u - P.cx) / P.fx, d1 = (v - P.cy) / P.fy;
        gz[i] = s * (rn0 * d0 + rn1 * d1 + rn2);
      }
    }
  }
  if (pair_fold<6>(acc, part, tickets, tot) && grad_twist && threadIdx.x < 6)
    grad_twist[blockIdx.y * 6 + threadIdx.x] = tot[threadIdx.x];
}

__global__ void k_zero_depth_grads(const stb_level *levels, float *const *grad_depth) {
  float *gz = grad_depth[blockIdx.y];
  const int64_t n = levels[blockIdx.y].num_source;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    gz[i] = 0.f;
}

__global__ void k_se3_exp_compose(const double *twist, const double *base, double *out, int B) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= B) return;
  double xi[6], E[16], T[16], O[16];
  for (int k = 0; k < 6; ++k) xi[k] = twist[p * 6 + k];
  for (int k = 0; k < 16; ++k) T[k] = base[p * 16 + k];
  se3_exp(xi, E);
  compose(E, T, O);
  for (int k = 0; k < 16; ++k) out[p * 16 + k] = O[k];
}

// g_out = J_l(xi)^T g_in per pair, with J_l the left Jacobian of SE(3) for
// xi = [rho; phi]: exp(xi + d) = exp(J_l(xi) d) exp(xi) + O(|d|^2).  J_l is
// summed from its series J_l = sum_n ad(xi)^n / (n + 1)!, with
// ad(xi) = [[phi^, rho^], [0, phi^]] (Barfoot, State Estimation for
// Robotics, sec. 7.1.5), in FP64 until the term falls below 1e-20 of the
// sum (at most 96 terms).
__global__ void k_se3_twist_grad(const double *twist, const double *g_in, double *g_out, int B) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= B) return;
  double ad[36] = {0};
  const double r0 = twist[p * 6], r1 = twist[p * 6 + 1], r2 = twist[p * 6 + 2];
  const double w0 = twist[p * 6 + 3], w1 = twist[p * 6 + 4], w2 = twist[p * 6 + 5];
  auto put_hat = [&](int r, int c, double x, double y, double z) {
    ad[(r + 0) * 6 + c + 1] = -z;
    ad[(r + 0) * 6 + c + 2] = y;
    ad[(r + 1) * 6 + c + 0] = z;
    ad[(r + 1) * 6 + c + 2] = -x;
    ad[(r + 2) * 6 + c + 0] = -y;
    ad[(r + 2) * 6 + c + 1] = x;
  };
  put_hat(0, 0, w0, w1, w2);
  put_hat(0, 3, r0, r1, r2);
  put_hat(3, 3, w0, w1, w2);
  double S[36], term[36], next[36];
  for (int k = 0; k < 36; ++k) S[k] = term[k] = (k % 7 == 0) ? 1.0 : 0.0;
  for (int n = 1; n <= 96; ++n) {
    double tmax = 0.0, smax = 0.0;
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        double a = 0.0;
        for (int k = 0; k < 6; ++k) a += term[i * 6 + k] * ad[k * 6 + j];
        next[i * 6 + j] = a / (double)(n + 1);
      }
    for (int k = 0; k < 36; ++k) {
      term[k] = next[k];
      S[k] += term[k];
      tmax = fmax(tmax, fabs(term[k]));
      smax = fmax(smax, fabs(S[k]));
    }
    if (tmax <= 1e-20 * smax) break;
  }
  double g[6];
  for (int k = 0; k < 6; ++k) g[k] = g_in[p * 6 + k];
  for (int j = 0; j < 6; ++j) {
    double a = 0.0;
    for (int i = 0; i < 6; ++i) a += S[i * 6 + j] * g[i];
    g_out[p * 6 + j] = a;
  }
}

int check_loss_args(const stb_level *levels, int B, const double *poses, int64_t max_px,
                    void *workspace, size_t ws_bytes) {
  if (B <= 0) return fail(STB_EINVAL, "Check failed: num_pairs must be positive");
  if (max_px <= 0) return fail(STB_EINVAL, "Check failed: max_target_pixels must be positive");
  const GradLayout g = grad_layout(B, max_px);
  if (ws_bytes < g.total)
    return fail(STB_EINVAL, "Check failed: workspace of %zu bytes, %zu needed", ws_bytes, g.total);
  if (((uintptr_t)workspace & 255) != 0)
    return fail(STB_EINVAL, "Check failed: workspace must be 256-byte aligned");
  STB_TRY(check_device_ptr(levels, "levels"));
  STB_TRY(check_device_ptr(poses, "poses"));
  STB_TRY(check_device_ptr(workspace, "workspace"));
  return STB_OK;
}

}  // namespace
}  // namespace stb

using namespace stb;

extern "C" int stb_se3_exp_compose(const double *twist, const double *base, double *out,
                                   int32_t num_pairs, void *stream) {
  clear_error();
  if (num_pairs <= 0) return fail(STB_EINVAL, "Check failed: num_pairs must be positive");
  STB_TRY(check_device_ptr(twist, "twist"));
  STB_TRY(check_device_ptr(base, "base"));
  STB_TRY(check_device_ptr(out, "out"));
  k_se3_exp_compose<<<(num_pairs + 63) / 64, 64, 0, as_stream(stream)>>>(twist, base, out,
                                                                        num_pairs);
  return check_launch("stb_se3_exp_compose");
}

extern "C" int stb_se3_twist_grad(const double *twist, const double *grad_tangent,
                                  double *grad_twist, int32_t num_pairs, void *stream) {
  clear_error();
  if (num_pairs <= 0) return fail(STB_EINVAL, "Check failed: num_pairs must be positive");
  STB_TRY(check_device_ptr(twist, "twist"));
  STB_TRY(check_device_ptr(grad_tangent, "grad_tangent"));
  STB_TRY(check_device_ptr(grad_twist, "grad_twist"));
  k_se3_twist_grad<<<(num_pairs + 63) / 64, 64, 0, as_stream(stream)>>>(twist, grad_tangent,
                                                                      grad_twist, num_pairs);
  return check_launch("stb_se3_twist_grad");
}

extern "C" size_t stb_icp_loss_workspace_bytes(int32_t num_pairs, int64_t max_target_pixels) {
  if (num_pairs <= 0 || max_target_pixels <= 0) return 0;
  return grad_layout(num_pairs, max_target_pixels).total;
}

extern "C" int stb_icp_loss_forward(const stb_level *levels, int32_t num_pairs,
                                    const double *poses, double distance_thresh,
                                    double normal_angle_thresh, int64_t max_target_pixels,
                                    void *workspace, size_t workspace_bytes, double *loss,
                                    void *stream) {
  clear_error();
  STB_TRY(check_loss_args(levels, num_pairs, poses, max_target_pixels, workspace,
                          workspace_bytes));
  STB_TRY(check_device_ptr(loss, "loss"));
  const GradLayout g = grad_layout(num_pairs, max_target_pixels);
  char *ws = static_cast<char *>(workspace);
  const cudaStream_t st = as_stream(stream);
  unsigned *err = reinterpret_cast<unsigned *>(ws + g.err);
  unsigned *tickets = reinterpret_cast<unsigned *>(ws + g.tickets);
  unsigned long long *keys = reinterpret_cast<unsigned long long *>(ws + g.keys);
  cudaMemsetAsync(ws, 0, g.part, st);  // error word and tickets
  cudaMemsetAsync(keys, 0xff, sizeof(unsigned long long) * (size_t)num_pairs * max_target_pixels,
                  st);
  const dim3 grid(blocks_x(max_target_pixels), num_pairs);
  k_g_assoc<<<grid, kT, 0, st>>>(levels, poses, max_target_pixels, keys,
                                 distance_thresh_sq(distance_thresh),
                                 angle_cos_max(normal_angle_thresh), err);
  k_g_loss<<<grid, kT, 0, st>>>(levels, poses, max_target_pixels, keys,
                                reinterpret_cast<float *>(ws + g.part), tickets, loss);
  return check_launch("stb_icp_loss_forward");
}

extern "C" int stb_icp_loss_backward(const stb_level *levels, int32_t num_pairs,
                                     const double *poses, const double *grad_loss,
                                     int64_t max_target_pixels, void *workspace,
                                     size_t workspace_bytes, double *grad_twist,
                                     float *const *grad_depth, void *stream) {
  clear_error();
  STB_TRY(check_loss_args(levels, num_pairs, poses, max_target_pixels, workspace,
                          workspace_bytes));
  STB_TRY(check_device_ptr(grad_loss, "grad_loss"));
  STB_TRY(check_device_ptr(grad_twist, "grad_twist", true));
  STB_TRY(check_device_ptr(grad_depth, "grad_depth", true));
  const GradLayout g = grad_layout(num_pairs, max_target_pixels);
  char *ws = static_cast<char *>(workspace);
  const cudaStream_t st = as_stream(stream);
  const dim3 grid(blocks_x(max_target_pixels), num_pairs);
  if (grad_depth) k_zero_depth_grads<<<grid, kT, 0, st>>>(levels, grad_depth);
  k_g_adjoint<<<grid, kT, 0, st>>>(levels, poses, max_target_pixels,
                                   reinterpret_cast<const unsigned long long *>(ws + g.keys),
                                   grad_loss, reinterpret_cast<float *>(ws + g.part),
                                   reinterpret_cast<unsigned *>(ws + g.tickets), grad_twist,
                                   grad_depth);
  return check_launch("stb_icp_loss_backward");
}
