// Differentiable point-to-plane loss for batches of frame pairs, with a
// hand-written adjoint.
//
// Layout: every field is one dense device array over the batch, pair p at
// offset p * H * W pixels: source depth (float32, metres), source normals
// (float32 xyz), source mask (uint8), target points / normals (float32
// xyz), target mask (uint8); all pairs share the size and the intrinsics.
// Source points are back-projected in the kernels exactly as
// stb_depth_to_points does (x = ((u - cx) z) / fx, slamtb/camera.py:127-149),
// so the loss reads 4 bytes of depth per source pixel instead of 12 of
// points and the depth gradient needs no chain through a points tensor.
//
// Forward (per pair p, pose T_p): the ICPOdometry association at the float32
// cast of T_p (64-bit atomicMin z-buffer, the reference's gates) and
// L_p = sum over the correspondences of r^2, r = (q - T_p s).n
// (icp_jacobian_geometric.cu:82), summed in compensated float32.
// Adjoint (correspondences frozen): dL/dxi = -2 sum r J with J = [n; Tp x n]
// for T <- exp(xi) T_p (the sign convention of icp_jacobian_common.hpp:41-48,
// J = -dr/dxi), and dL/dz_i = -2 r_i (R^T n) . d_i for the source depth z_i,
// s_i = z_i d_i, d_i = ((u_i - cx)/fx, (v_i - cy)/fy, 1).
//
// Grid: x = work items of a pair, y = pair.  Per-pair totals use per-block
// partials and a last-block ticket (deterministic order).
#include <math.h>

#include "gn_solve.cuh"
#include "keymap.cuh"
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

struct LossArgs {
  const float *depth, *sn;
  const uint8_t *sm;
  const float *tp, *tn;
  const uint8_t *tm;
  int B, H, W;
  float fx, fy, cx, cy;
  const double *poses;
};

struct GradLayout {
  size_t tickets, part, keys, total;
};

inline int blocks_x(int64_t px) {
  int64_t b = (px + kItem - 1) / kItem;
  return (int)(b < 1 ? 1 : (b > kMaxBlocksX ? kMaxBlocksX : b));
}

inline size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// Blocks per pair of the per-pixel loss passes: about two waves of 4
// blocks per SM over the whole batch, at most blocks_x(npix); the grid-
// stride loops cover the rest, and the slots of the workspace fit any grid
// up to blocks_x.  A block of k_g_loss / k_g_adjoint ends with a per-pair
// fold and ticket, and every block sets up its pair's float32 pose first,
// so with few pixels a block those set the time (32 pairs of 640x480,
// graph-captured step: 300 blocks a pair 94 k pairs/s; the folding passes
// on 38 a pair 106 k; the association too 110 k).  The loss and both forms
// of the adjoint use the same grid, so their sums agree bit for bit; the
// association's key map does not depend on the grid.
int fold_blocks(int B, int64_t npix) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms <= 0) {
    cudaGetLastError();
    sms = 152;
  }
  const int want = (8 * sms + B - 1) / B;
  const int cap = blocks_x(npix);
  return want < 1 ? 1 : (want > cap ? cap : want);
}

inline GradLayout grad_layout(int B, int64_t px) {
  GradLayout g;
  size_t o = 0;
  g.tickets = o;
  o += al(sizeof(unsigned) * (size_t)B);
  g.part = o;
  o += al(sizeof(float) * 16 * (size_t)B * blocks_x(px));
  g.keys = o;
  o += al(sizeof(unsigned long long) * (size_t)B * px);
  g.total = o;
  return g;
}

// float32 pose of pair blockIdx.y, into shared memory (refresh_pose32's
// values), in two halves so that a kernel can issue its first pixel loads
// in between: pose_load starts lanes 0..11 loading one FP64 entry each;
// pose_finish converts them, forms the normal matrix on thread 0 and ends
// with the block barrier.
__device__ __forceinline__ double pose_load(const LossArgs &a) {
  return threadIdx.x < 12 ? a.poses[blockIdx.y * 16 + threadIdx.x] : 0.0;
}

__device__ __forceinline__ void pose_finish(const LossArgs &a, Pose32 &P, double t) {
  if (threadIdx.x < 32) {
    if (threadIdx.x < 12) P.rt[threadIdx.x] = __double2float_rn(t);
    __syncwarp();
    if (threadIdx.x == 0) {
      P.fx = a.fx;
      P.fy = a.fy;
      P.cx = a.cx;
      P.cy = a.cy;
      inverse_transpose(P.rt, P.nm);
    }
  }
  __syncthreads();
}

// Source point i of a pair from its depth (stb_depth_to_points' arithmetic).
__device__ __forceinline__ float3 source_point(const LossArgs &a, float z, int i) {
  const float u = (float)(i % a.W), v = (float)(i / a.W);
  return make_float3(fdiv(fmul(fsub(u, a.cx), z), a.fx), fdiv(fmul(fsub(v, a.cy), z), a.fy), z);
}

// Pixels per thread per round of the loss kernels: every load of a round
// is issued before the first dependent use, so a thread waits for one
// gather round trip per round instead of one per pixel.  The pixels of a
// thread keep the grid-stride order, so sums are the same bits.  Two
// pixels keep 4-5 blocks of 256 resident per SM (the register caps of the
// launch bounds: k_g_assoc 64, k_g_adjoint 64, k_g_loss 48);
// four pixels need about 115 registers and halve the occupancy, which
// costs more than the extra loads in flight win.
constexpr int kP = 2;

// The source half of a round of k_g_assoc (pose-independent): mask and
// depth of pixels i0 + k * stride.
struct SourceRound {
  bool ok[kP];
  float z[kP];
};

__device__ __forceinline__ void load_sources(const LossArgs &a, size_t po, int npix, int i0,
                                             int stride, SourceRound &S) {
#pragma unroll
  for (int k = 0; k < kP; ++k) {
    const int i = i0 + k * stride;
    const int ic = i < npix ? i : 0;
    S.ok[k] = i < npix && a.sm[po + ic];
    S.z[k] = a.depth[po + ic];
  }
}

__global__ void __launch_bounds__(kT, 4) k_g_assoc(const LossArgs a, unsigned long long *keys_all,
                                                float thr2, float cos_max) {
  __shared__ Pose32 P;
  const double pose_entry = pose_load(a);
  const int H = a.H, W = a.W;
  const int npix = H * W;  // < 2^24, checked on the host
  const size_t po = (size_t)blockIdx.y * npix;
  unsigned long long *keys = keys_all + po;
  const float *tp = a.tp + 3 * po, *tn = a.tn + 3 * po, *sn = a.sn + 3 * po;
  const uint8_t *tm = a.tm + po;
  const int stride = gridDim.x * kT;
  int i0 = blockIdx.x * kT + threadIdx.x;
  SourceRound S;
  load_sources(a, po, npix, i0, stride, S);  // in flight across the barrier
  pose_finish(a, P, pose_entry);
  while (true) {
    // the projections of the source pixels, and the gathers of the
    // projected target pixels
    bool ok[kP];
    int pix[kP];
    float3 Tp[kP];
#pragma unroll
    for (int k = 0; k < kP; ++k) {
      const int i = i0 + k * stride;
      const float3 s = source_point(a, S.z[k], i < npix ? i : 0);
      Tp[k] = transform_point(P.rt, s.x, s.y, s.z);
      float u, v;
      project(P, Tp[k], u, v);
      int ui = 0, vi = 0;
      ok[k] = S.ok[k] && round_in(u, W, ui) && round_in(v, H, vi);
      pix[k] = ok[k] ? vi * W + ui : 0;
    }
    // (the source normals go out with the gathers: one round trip)
    float q[kP][3], m[kP][3], ns[kP][3];
    bool tv[kP];
#pragma unroll
    for (int k = 0; k < kP; ++k) {
      const int i = i0 + k * stride;
      const int ic = i < npix ? i : 0;
      tv[k] = tm[pix[k]];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        q[k][d] = tp[3 * pix[k] + d];
        m[k][d] = tn[3 * pix[k] + d];
        ns[k][d] = sn[3 * ic + d];
      }
    }
    // the gates and the z-buffer
#pragma unroll
    for (int k = 0; k < kP; ++k) {
      if (!ok[k] || !tv[k]) continue;
      const int i = i0 + k * stride;
      const float dx = fsub(q[k][0], Tp[k].x), dy = fsub(q[k][1], Tp[k].y),
                  dz = fsub(q[k][2], Tp[k].z);
      const float sq = dot3(dx, dy, dz, dx, dy, dz);
      if (sq > thr2) continue;
      const float3 Tn = transform_normal(P.nm, ns[k][0], ns[k][1], ns[k][2]);
      if (normal_angle_rejects(Tn, m[k][0], m[k][1], m[k][2], cos_max)) continue;
      atomicMin(keys + pix[k], ((unsigned long long)kTag << 56) |
                                   ((unsigned long long)__float_as_uint(__fsqrt_rn(sq)) << 24) |
                                   (unsigned long long)i);
    }
    i0 += stride * kP;
    if (i0 >= npix) break;
    load_sources(a, po, npix, i0, stride, S);
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

// The inputs of a round's residuals: keys, then (matched pixels) the
// winners' depths (the gather) and the target points and normals.
struct Round {
  bool m[kP];
  int i[kP];
  float z[kP], q[kP][3], n[kP][3];
};

__device__ __forceinline__ void load_round(const LossArgs &a, size_t po, int npix,
                                           const unsigned long long *keys, int p0, int stride,
                                           Round &R) {
  unsigned long long key[kP];
#pragma unroll
  for (int k = 0; k < kP; ++k) {
    const int pix = p0 + k * stride;
    key[k] = pix < npix ? __ldcg(keys + pix) : 0ull;
  }
#pragma unroll
  for (int k = 0; k < kP; ++k) {
    const int pix = p0 + k * stride;
    R.m[k] = (unsigned)(key[k] >> 56) == kTag;
    R.i[k] = R.m[k] ? (int)(key[k] & 0xffffffull) : 0;
    const int pc = R.m[k] ? pix : 0;
    R.z[k] = a.depth[po + R.i[k]];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      R.q[k][d] = a.tp[3 * (po + pc) + d];
      R.n[k][d] = a.tn[3 * (po + pc) + d];
    }
  }
}

// r = (q - Tp) . n of pixel k of a round (icp_jacobian_geometric.cu:82), with Tp the
// transformed back-projection of the winner and q, n the target point and normal.
__device__ __forceinline__ float round_residual(const LossArgs &a, const Pose32 &P,
                                                const Round &R, int k, float3 &Tp,
                                                float3 &n) {
  const float3 s = source_point(a, R.z[k], R.i[k]);
  Tp = transform_point(P.rt, s.x, s.y, s.z);
  n = make_float3(R.n[k][0], R.n[k][1], R.n[k][2]);
  return dot3(fsub(R.q[k][0], Tp.x), fsub(R.q[k][1], Tp.y), fsub(R.q[k][2], Tp.z), n.x, n.y,
              n.z);
}

// The loss of every pair, and with kAdj its adjoint at a unit output
// gradient in the same pass (the tangent sums -2 sum r J and the depth
// adjoint -2 r (R^T n).d at each matched source pixel), so that a backward
// pass only scales them by dL/dL_p (k_g_scale) instead of reading the
// correspondences, the gathers and the target frame again.  The adjoint
// terms use k_g_adjoint's expressions with its factor -2 g at g = 1, so at
// a unit output gradient the two give the same bits.
template <bool kAdj>
__global__ void __launch_bounds__(kT, kAdj ? 4 : 5)
    k_g_loss(const LossArgs a, const unsigned long long *keys_all, float *part,
             unsigned *tickets, double *loss, double *tangent, float *depth_adj) {
  __shared__ Pose32 P;
  __shared__ double tot[8];
  constexpr int kN = kAdj ? 7 : 1;
  const double pose_entry = pose_load(a);
  const int npix = a.H * a.W;
  const size_t po = (size_t)blockIdx.y * npix;
  const unsigned long long *keys = keys_all + po;
  float *gz = (kAdj && depth_adj) ? depth_adj + po : nullptr;
  const int stride = gridDim.x * kT;
  CSum acc[kN];
#pragma unroll
  for (int k = 0; k < kN; ++k) acc[k] = {0.f, 0.f};
  int p0 = blockIdx.x * kT + threadIdx.x;
  Round R;
  load_round(a, po, npix, keys, p0, stride, R);  // in flight across the barrier
  pose_finish(a, P, pose_entry);
  while (true) {
#pragma unroll
    for (int k = 0; k < kP; ++k) {
      if (!R.m[k]) continue;
      float3 Tp, n;
      const float r = round_residual(a, P, R, k, Tp, n);
      csum_add(acc[0], r * r);
      if (kAdj) {
        const int i = R.i[k];
        const float Jv[6] = {n.x, n.y, n.z, Tp.y * n.z - Tp.z * n.y, Tp.z * n.x - Tp.x * n.z,
                             Tp.x * n.y - Tp.y * n.x};
        const float s = -2.f * r;
#pragma unroll
        for (int c = 0; c < 6; ++c) csum_add(acc[1 + c], s * Jv[c]);
        if (gz) {
          const float *Rt = P.rt;
          const float rn0 = Rt[0] * n.x + Rt[4] * n.y + Rt[8] * n.z;
          const float rn1 = Rt[1] * n.x + Rt[5] * n.y + Rt[9] * n.z;
          const float rn2 = Rt[2] * n.x + Rt[6] * n.y + Rt[10] * n.z;
          const float d0 = ((float)(i % a.W) - P.cx) / P.fx,
                      d1 = ((float)(i / a.W) - P.cy) / P.fy;
          gz[i] = s * (rn0 * d0 + rn1 * d1 + rn2);
        }
      }
    }
    p0 += stride * kP;
    if (p0 >= npix) break;
    load_round(a, po, npix, keys, p0, stride, R);
  }
  if (pair_fold<kN>(acc, part, tickets, tot)) {
    if (threadIdx.x == 0) loss[blockIdx.y] = tot[0];
    if (kAdj && threadIdx.x < 6) tangent[blockIdx.y * 6 + threadIdx.x] = tot[1 + threadIdx.x];
  }
}

// Backward of the fused forward: grad_tangent[p] = g_p tangent[p] (FP64) and
// grad_depth[p][i] = (float)g_p depth_adj[p][i], g_p = grad_loss[p]; 16-byte
// vectors where a pair's pixels start on a 16-byte boundary.
__global__ void k_g_scale(const double *grad_loss, const double *tangent,
                          const float *depth_adj, int npix, double *grad_tangent,
                          float *grad_depth) {
  const int p = blockIdx.y;
  const double g = grad_loss[p];
  if (grad_tangent && blockIdx.x == 0 && threadIdx.x < 6)
    grad_tangent[p * 6 + threadIdx.x] = g * tangent[p * 6 + threadIdx.x];
  if (!grad_depth) return;
  const float gf = (float)g;
  const size_t po = (size_t)p * npix;
  const float *src = depth_adj + po;
  float *dst = grad_depth + po;
  const int stride = gridDim.x * blockDim.x;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if ((((uintptr_t)src | (uintptr_t)dst) & 15) == 0) {
    const int n4 = npix >> 2;
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    float4 *d4 = reinterpret_cast<float4 *>(dst);
    for (int k = t; k < n4; k += stride) {
      const float4 v = __ldcs(s4 + k);
      __stcs(d4 + k, make_float4(gf * v.x, gf * v.y, gf * v.z, gf * v.w));
    }
    for (int k = 4 * n4 + t; k < npix; k += stride) dst[k] = gf * src[k];
  } else {
    for (int k = t; k < npix; k += stride) dst[k] = gf * src[k];
  }
}

__global__ void __launch_bounds__(kT, 4) k_g_adjoint(const LossArgs a,
                                                  const unsigned long long *keys_all,
                                                  const double *grad_loss, float *part,
                                                  unsigned *tickets, double *grad_tangent,
                                                  float *grad_depth) {
  __shared__ Pose32 P;
  __shared__ double tot[8];
  const double pose_entry = pose_load(a);
  const int npix = a.H * a.W;
  const size_t po = (size_t)blockIdx.y * npix;
  const unsigned long long *keys = keys_all + po;
  const float g = (float)grad_loss[blockIdx.y];
  float *gz = grad_depth ? grad_depth + po : nullptr;
  const int stride = gridDim.x * kT;
  CSum acc[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) acc[k] = {0.f, 0.f};
  int p0 = blockIdx.x * kT + threadIdx.x;
  Round R;
  load_round(a, po, npix, keys, p0, stride, R);  // in flight across the barrier
  pose_finish(a, P, pose_entry);
  while (true) {
#pragma unroll
    for (int k = 0; k < kP; ++k) {
      if (!R.m[k]) continue;
      const int i = R.i[k];
      float3 Tp, n;
      const float r = round_residual(a, P, R, k, Tp, n);
      const float Jv[6] = {n.x, n.y, n.z, Tp.y * n.z - Tp.z * n.y, Tp.z * n.x - Tp.x * n.z,
                           Tp.x * n.y - Tp.y * n.x};
      const float s = -2.f * g * r;
#pragma unroll
      for (int c = 0; c < 6; ++c) csum_add(acc[c], s * Jv[c]);
      if (gz) {
        // R^T n, with R the float32 rotation of the pose
        const float *Rt = P.rt;
        const float rn0 = Rt[0] * n.x + Rt[4] * n.y + Rt[8] * n.z;
        const float rn1 = Rt[1] * n.x + Rt[5] * n.y + Rt[9] * n.z;
        const float rn2 = Rt[2] * n.x + Rt[6] * n.y + Rt[10] * n.z;
        const float d0 = ((float)(i % a.W) - P.cx) / P.fx, d1 = ((float)(i / a.W) - P.cy) / P.fy;
        gz[i] = s * (rn0 * d0 + rn1 * d1 + rn2);
      }
    }
    p0 += stride * kP;
    if (p0 >= npix) break;
    load_round(a, po, npix, keys, p0, stride, R);
  }
  if (pair_fold<6>(acc, part, tickets, tot) && grad_tangent && threadIdx.x < 6)
    grad_tangent[blockIdx.y * 6 + threadIdx.x] = tot[threadIdx.x];
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
//
// Every term ad^n / (n + 1)! has the form [[A, B], [0, A]] (3x3 blocks), so
// one warp per pair carries its 18 distinct entries, one per lane (lanes
// 0..8 A row-major, 9..17 B), through the recurrence
// A' = A phi^ / (n + 1), B' = (A rho^ + B phi^) / (n + 1), the terms in
// shared memory.  A thread per pair would issue all 36 entries' FP64
// products and divisions one after the other.
constexpr int kTwistWarps = 4;  // pairs per block

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Column j of the hat matrix of (x, y, z): [[0, -z, y], [z, 0, -x], [-y, x, 0]].
__device__ __forceinline__ void hat_column(double x, double y, double z, int j, double c[3]) {
  c[0] = j == 0 ? 0.0 : (j == 1 ? -z : y);
  c[1] = j == 0 ? z : (j == 1 ? 0.0 : -x);
  c[2] = j == 0 ? -y : (j == 1 ? x : 0.0);
}

__global__ void __launch_bounds__(32 * kTwistWarps)
    k_se3_twist_grad(const double *twist, const double *g_in, double *g_out, int B) {
  __shared__ double s_term[kTwistWarps][18], s_sum[kTwistWarps][18];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int p = blockIdx.x * kTwistWarps + w;
  if (p >= B) return;  // the whole warp
  const double r0 = twist[p * 6], r1 = twist[p * 6 + 1], r2 = twist[p * 6 + 2];
  const double w0 = twist[p * 6 + 3], w1 = twist[p * 6 + 4], w2 = twist[p * 6 + 5];
  const bool mine = lane < 18, in_a = lane < 9;
  const int e = in_a ? lane : (mine ? lane - 9 : 0);
  const int i = e / 3, j = e % 3;
  double wc[3], rc[3];
  hat_column(w0, w1, w2, j, wc);
  hat_column(r0, r1, r2, j, rc);
  // the n = 0 term and the sum: the identity
  double sum = (lane == 0 || lane == 4 || lane == 8) ? 1.0 : 0.0;
  if (mine) s_term[w][lane] = sum;
  __syncwarp();
  for (int n = 1; n <= 96; ++n) {
    double a = 0.0;
    if (mine) {
      const double *A = s_term[w], *Bm = s_term[w] + 9;
#pragma unroll
      for (int k = 0; k < 3; ++k) a += A[i * 3 + k] * (in_a ? wc[k] : rc[k]);
      if (!in_a) {
#pragma unroll
        for (int k = 0; k < 3; ++k) a += Bm[i * 3 + k] * wc[k];
      }
    }
    const double next = a / (double)(n + 1);
    __syncwarp();
    double tabs = 0.0, sabs = 0.0;
    if (mine) {
      s_term[w][lane] = next;
      sum += next;
      tabs = fabs(next);
      sabs = fabs(sum);
    }
    __syncwarp();
    const double tmax = warp_max(tabs), smax = warp_max(sabs);
    if (tmax <= 1e-20 * smax) break;
  }
  if (mine) s_sum[w][lane] = sum;
  __syncwarp();
  if (lane < 6) {
    // column `lane` of J_l = [[SA, SB], [0, SA]] against g
    const double *SA = s_sum[w], *SB = s_sum[w] + 9;
    const int c = lane;
    double acc = 0.0;
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      const double s = r < 3 ? (c < 3 ? SA[r * 3 + c] : SB[r * 3 + c - 3])
                             : (c < 3 ? 0.0 : SA[(r - 3) * 3 + c - 3]);
      acc += s * g_in[p * 6 + r];
    }
    g_out[p * 6 + c] = acc;
  }
}

int check_loss_args(const LossArgs &a, void *workspace, size_t ws_bytes) {
  if (a.B <= 0) return fail(STB_EINVAL, "Check failed: num_pairs must be positive");
  if (a.H <= 0 || a.W <= 0)
    return fail(STB_EINVAL, "Check failed: frame size must be positive, got %dx%d", a.H, a.W);
  if ((int64_t)a.H * a.W >= (1ll << 24))
    return fail(STB_EINVAL, "Check failed: frames must have fewer than 2^24 pixels");
  const GradLayout g = grad_layout(a.B, (int64_t)a.H * a.W);
  if (ws_bytes < g.total)
    return fail(STB_EINVAL, "Check failed: workspace of %zu bytes, %zu needed", ws_bytes, g.total);
  if (((uintptr_t)workspace & 255) != 0)
    return fail(STB_EINVAL, "Check failed: workspace must be 256-byte aligned");
  STB_TRY(check_device_ptr(a.depth, "source_depth"));
  STB_TRY(check_device_ptr(a.sn, "source_normals"));
  STB_TRY(check_device_ptr(a.sm, "source_mask"));
  STB_TRY(check_device_ptr(a.tp, "target_points"));
  STB_TRY(check_device_ptr(a.tn, "target_normals"));
  STB_TRY(check_device_ptr(a.tm, "target_mask"));
  STB_TRY(check_device_ptr(a.poses, "poses"));
  STB_TRY(check_device_ptr(workspace, "workspace"));
  return STB_OK;
}

LossArgs loss_args(const float *src_depth, const float *src_normals, const uint8_t *src_mask,
                   const float *tgt_points, const float *tgt_normals, const uint8_t *tgt_mask,
                   int32_t num_pairs, int32_t height, int32_t width, float fx, float fy,
                   float cx, float cy, const double *poses) {
  LossArgs a;
  a.depth = src_depth;
  a.sn = src_normals;
  a.sm = src_mask;
  a.tp = tgt_points;
  a.tn = tgt_normals;
  a.tm = tgt_mask;
  a.B = num_pairs;
  a.H = height;
  a.W = width;
  a.fx = fx;
  a.fy = fy;
  a.cx = cx;
  a.cy = cy;
  a.poses = poses;
  return a;
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
  k_se3_twist_grad<<<(num_pairs + kTwistWarps - 1) / kTwistWarps, 32 * kTwistWarps, 0,
                     as_stream(stream)>>>(twist, grad_tangent, grad_twist, num_pairs);
  return check_launch("stb_se3_twist_grad");
}

extern "C" size_t stb_icp_loss_workspace_bytes(int32_t num_pairs, int32_t height,
                                               int32_t width) {
  if (num_pairs <= 0 || height <= 0 || width <= 0) return 0;
  return grad_layout(num_pairs, (int64_t)height * width).total;
}

extern "C" int stb_icp_loss_forward(const float *src_depth, const float *src_normals,
                                    const uint8_t *src_mask, const float *tgt_points,
                                    const float *tgt_normals, const uint8_t *tgt_mask,
                                    int32_t num_pairs, int32_t height, int32_t width, float fx,
                                    float fy, float cx, float cy, const double *poses,
                                    double distance_thresh, double normal_angle_thresh,
                                    void *workspace, size_t workspace_bytes, double *loss,
                                    void *stream) {
  clear_error();
  const LossArgs a = loss_args(src_depth, src_normals, src_mask, tgt_points, tgt_normals,
                               tgt_mask, num_pairs, height, width, fx, fy, cx, cy, poses);
  STB_TRY(check_loss_args(a, workspace, workspace_bytes));
  STB_TRY(check_device_ptr(loss, "loss"));
  const int64_t npix = (int64_t)height * width;
  const GradLayout g = grad_layout(num_pairs, npix);
  char *ws = static_cast<char *>(workspace);
  const cudaStream_t st = as_stream(stream);
  unsigned long long *keys = reinterpret_cast<unsigned long long *>(ws + g.keys);
  cudaMemsetAsync(ws + g.tickets, 0, sizeof(unsigned) * (size_t)num_pairs, st);
  cudaMemsetAsync(keys, 0xff, sizeof(unsigned long long) * (size_t)num_pairs * npix, st);
  const dim3 grid(fold_blocks(num_pairs, npix), num_pairs);
  k_g_assoc<<<grid, kT, 0, st>>>(a, keys, distance_thresh_sq(distance_thresh),
                                 angle_cos_max(normal_angle_thresh));
  k_g_loss<false><<<grid, kT, 0, st>>>(a, keys, reinterpret_cast<float *>(ws + g.part),
                                       reinterpret_cast<unsigned *>(ws + g.tickets), loss,
                                       nullptr, nullptr);
  return check_launch("stb_icp_loss_forward");
}

extern "C" int stb_icp_loss_forward_adjoint(
    const float *src_depth, const float *src_normals, const uint8_t *src_mask,
    const float *tgt_points, const float *tgt_normals, const uint8_t *tgt_mask,
    int32_t num_pairs, int32_t height, int32_t width, float fx, float fy, float cx, float cy,
    const double *poses, double distance_thresh, double normal_angle_thresh, void *workspace,
    size_t workspace_bytes, double *loss, double *tangent, float *depth_adjoint,
    void *stream) {
  clear_error();
  const LossArgs a = loss_args(src_depth, src_normals, src_mask, tgt_points, tgt_normals,
                               tgt_mask, num_pairs, height, width, fx, fy, cx, cy, poses);
  STB_TRY(check_loss_args(a, workspace, workspace_bytes));
  STB_TRY(check_device_ptr(loss, "loss"));
  STB_TRY(check_device_ptr(tangent, "tangent"));
  STB_TRY(check_device_ptr(depth_adjoint, "depth_adjoint", true));
  const int64_t npix = (int64_t)height * width;
  const GradLayout g = grad_layout(num_pairs, npix);
  char *ws = static_cast<char *>(workspace);
  const cudaStream_t st = as_stream(stream);
  unsigned long long *keys = reinterpret_cast<unsigned long long *>(ws + g.keys);
  cudaMemsetAsync(ws + g.tickets, 0, sizeof(unsigned) * (size_t)num_pairs, st);
  cudaMemsetAsync(keys, 0xff, sizeof(unsigned long long) * (size_t)num_pairs * npix, st);
  if (depth_adjoint)
    cudaMemsetAsync(depth_adjoint, 0, sizeof(float) * (size_t)num_pairs * npix, st);
  const dim3 grid(fold_blocks(num_pairs, npix), num_pairs);
  k_g_assoc<<<grid, kT, 0, st>>>(a, keys, distance_thresh_sq(distance_thresh),
                                 angle_cos_max(normal_angle_thresh));
  k_g_loss<true><<<grid, kT, 0, st>>>(a, keys, reinterpret_cast<float *>(ws + g.part),
                                      reinterpret_cast<unsigned *>(ws + g.tickets), loss,
                                      tangent, depth_adjoint);
  return check_launch("stb_icp_loss_forward_adjoint");
}

extern "C" int stb_icp_loss_scale_adjoint(const double *grad_loss, const double *tangent,
                                          const float *depth_adjoint, int32_t num_pairs,
                                          int32_t height, int32_t width, double *grad_tangent,
                                          float *grad_depth, void *stream) {
  clear_error();
  if (num_pairs <= 0 || height <= 0 || width <= 0)
    return fail(STB_EINVAL, "Check failed: sizes must be positive, got %d pairs of %dx%d",
                num_pairs, height, width);
  if ((int64_t)height * width >= (1ll << 24))
    return fail(STB_EINVAL, "Check failed: frames must have fewer than 2^24 pixels");
  STB_TRY(check_device_ptr(grad_loss, "grad_loss"));
  STB_TRY(check_device_ptr(grad_tangent, "grad_tangent", true));
  STB_TRY(check_device_ptr(grad_depth, "grad_depth", true));
  if (grad_tangent) STB_TRY(check_device_ptr(tangent, "tangent"));
  if (grad_depth) STB_TRY(check_device_ptr(depth_adjoint, "depth_adjoint"));
  const int npix = height * width;
  int bx = (npix / 4 + 255) / 256;
  bx = bx < 1 ? 1 : (bx > 256 ? 256 : bx);
  k_g_scale<<<dim3(bx, num_pairs), 256, 0, as_stream(stream)>>>(
      grad_loss, tangent, depth_adjoint, npix, grad_tangent, grad_depth);
  return check_launch("stb_icp_loss_scale_adjoint");
}

extern "C" int stb_icp_loss_backward(const float *src_depth, const float *src_normals,
                                     const uint8_t *src_mask, const float *tgt_points,
                                     const float *tgt_normals, const uint8_t *tgt_mask,
                                     int32_t num_pairs, int32_t height, int32_t width, float fx,
                                     float fy, float cx, float cy, const double *poses,
                                     const double *grad_loss, void *workspace,
                                     size_t workspace_bytes, double *grad_tangent,
                                     float *grad_depth, void *stream) {
  clear_error();
  const LossArgs a = loss_args(src_depth, src_normals, src_mask, tgt_points, tgt_normals,
                               tgt_mask, num_pairs, height, width, fx, fy, cx, cy, poses);
  STB_TRY(check_loss_args(a, workspace, workspace_bytes));
  STB_TRY(check_device_ptr(grad_loss, "grad_loss"));
  STB_TRY(check_device_ptr(grad_tangent, "grad_tangent", true));
  STB_TRY(check_device_ptr(grad_depth, "grad_depth", true));
  const int64_t npix = (int64_t)height * width;
  const GradLayout g = grad_layout(num_pairs, npix);
  char *ws = static_cast<char *>(workspace);
  const cudaStream_t st = as_stream(stream);
  if (grad_depth) cudaMemsetAsync(grad_depth, 0, sizeof(float) * (size_t)num_pairs * npix, st);
  const dim3 fgrid(fold_blocks(num_pairs, npix), num_pairs);
  k_g_adjoint<<<fgrid, kT, 0, st>>>(a, reinterpret_cast<const unsigned long long *>(ws + g.keys),
                                   grad_loss, reinterpret_cast<float *>(ws + g.part),
                                   reinterpret_cast<unsigned *>(ws + g.tickets), grad_tangent,
                                   grad_depth);
  return check_launch("stb_icp_loss_backward");
}

extern "C" int stb_icp_loss_correspondences(const void *workspace, int32_t num_pairs,
                                            int32_t height, int32_t width, int64_t *merge_map,
                                            void *stream) {
  clear_error();
  if (num_pairs <= 0 || height <= 0 || width <= 0)
    return fail(STB_EINVAL, "Check failed: sizes must be positive, got %d pairs of %dx%d",
                num_pairs, height, width);
  if (((uintptr_t)workspace & 255) != 0)
    return fail(STB_EINVAL, "Check failed: workspace must be 256-byte aligned");
  STB_TRY(check_device_ptr(workspace, "workspace"));
  STB_TRY(check_device_ptr(merge_map, "merge_map"));
  const int64_t n = (int64_t)num_pairs * height * width;
  const GradLayout g = grad_layout(num_pairs, (int64_t)height * width);
  const auto *keys = reinterpret_cast<const unsigned long long *>(
      static_cast<const char *>(workspace) + g.keys);
  k_keys_to_merge_map<<<keys_grid(n), 256, 0, as_stream(stream)>>>(
      keys, nullptr, n, kTag, reinterpret_cast<long long *>(merge_map));
  return check_launch("stb_icp_loss_correspondences");
}
