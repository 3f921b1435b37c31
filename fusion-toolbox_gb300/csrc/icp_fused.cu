// Fused Gauss-Newton ICP for one frame pair (ICPOdometry.estimate,
// slamtb/registration/icp.py:152-262) without host synchronisation.
//
// Per iteration, two kernels:
//   k_assoc  -- one thread per source point: transform, project, gate
//               (bounds, target mask, distance, normal angle) and a 64-bit
//               atomicMin of (epoch tag, distance bits, source index) into a
//               per-pixel key map.  The epoch tag makes entries of earlier
//               iterations read as empty, so the map is cleared once per
//               call instead of once per iteration (the reference refills a
//               fresh int64 map per term and iteration,
//               slamtb/registration/correspondence_map.py:66-70).
//   k_reduce -- one thread per TARGET pixel: the pixel's winner (if any)
//               gives the source index; point-to-plane and feature residuals
//               and Jacobians are formed and the 30 unique normal-equation
//               terms are summed with compensated float32 (TwoSum) through
//               warp shuffles, a per-block partial and a last-block-done
//               ticket.  The last block finishes the sum in FP64, solves the
//               6x6 system, applies the SE(3) update and writes the float32
//               pose view for the next iteration.  This replaces the
//               per-point partials + three torch.sum(0) + host solve of the
//               reference (icp.py:39-82, 216-256).
// After the loop one more association at the final pose feeds k_info, the
// information matrix sum of G^T G (icp_jacobian_geometric.cu:118-158).
#include <math.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "feature_term.cuh"
#include "fused_common.cuh"
#include "gn_solve.cuh"
#include "keymap.cuh"
#include "stb_common.cuh"
#include "stb_host.hpp"

namespace stb {

float distance_thresh_sq(double d);
float angle_cos_max(double angle);

using namespace fused;

namespace {

// ---------------------------------------------------------------------------
__global__ void k_begin(Job job, Job *dst) {
  if (threadIdx.x != 0) return;
  *dst = job;
  State *S = job.state;
  double T[16];
  for (int k = 0; k < 16; ++k)
    T[k] = job.init ? job.init[k]
                    : (job.has_init_v ? job.init_v[k] : ((k % 5) == 0 ? 1.0 : 0.0));
  S->pose.fx = job.kcam ? job.kcam[0] : job.kcam_v[0];
  S->pose.cx = job.kcam ? job.kcam[2] : job.kcam_v[1];
  S->pose.fy = job.kcam ? job.kcam[4] : job.kcam_v[2];
  S->pose.cy = job.kcam ? job.kcam[5] : job.kcam_v[3];
  refresh_pose32(S->pose, T);
  for (int k = 0; k < 16; ++k) {
    S->Td[k] = T[k];
    S->Tw[k] = dw_of_double(T[k]);
  }
  S->ticket = 0;
  S->stopped = 0;
  S->status = 0;
  S->iters_done = 0;
  for (int k = 0; k < STB_RES_SIZE; ++k) job.result[k] = 0.0;
  job.result[STB_RES_RESIDUAL] = INFINITY;
}

// ---------------------------------------------------------------------------
// Programmatic dependent launch: a kernel launched with the attribute may
// start while its predecessor in the stream still runs; it does work that
// does not depend on the predecessor, then waits here for its completion
// (and the visibility of its writes).  Without the attribute the wait
// returns at once.
__device__ __forceinline__ void grid_dependency_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
// Lets the next kernel of the stream be scheduled (it still waits for this
// one to complete before reading what this one writes).
__device__ __forceinline__ void grid_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__global__ void __launch_bounds__(kAssocThreads) k_assoc(const Job *__restrict__ J,
                                                         int epoch, int force) {
  __shared__ Pose32 P;
  __shared__ int skip;
  // pose-independent prologue: this thread's source point and normal (the
  // inputs and the Job are not written by the preceding kernel)
  const long long n = J->n;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool in = i < n && J->sm[i];
  const float *__restrict__ sp = J->sp;
  const float *__restrict__ sn = J->sn;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, n0 = 0.f, n1 = 0.f, n2 = 0.f;
  if (in) {
    s0 = sp[3 * i], s1 = sp[3 * i + 1], s2 = sp[3 * i + 2];
    n0 = sn[3 * i], n1 = sn[3 * i + 1], n2 = sn[3 * i + 2];
  }
  grid_dependency_wait();  // the previous reduction has written the pose
  grid_launch_dependents();
  const State *S = J->state;
  if (threadIdx.x == 0) skip = !force && S->stopped;
  load_shared_pose(P, S);
  __syncthreads();
  if (skip || !in) return;
  const int H = J->H, W = J->W;
  const float3 Tp = transform_point(P.rt, s0, s1, s2);
  float u, v;
  project(P, Tp, u, v);
  int ui, vi;
  if (!round_in(u, W, ui) || !round_in(v, H, vi)) return;
  const int64_t pix = (int64_t)vi * W + ui;
  // the target pixel's mask, point and normal in one round trip (the point
  // and normal of a masked-out pixel are read and discarded)
  const float *__restrict__ tp = J->tp;
  const float *__restrict__ tn = J->tn;
  const bool valid = J->tm[pix];
  const float qx = tp[3 * pix], qy = tp[3 * pix + 1], qz = tp[3 * pix + 2];
  const float nx = tn[3 * pix], ny = tn[3 * pix + 1], nz = tn[3 * pix + 2];
  if (!valid) return;
  const float dx = fsub(qx, Tp.x), dy = fsub(qy, Tp.y), dz = fsub(qz, Tp.z);
  const float sq = dot3(dx, dy, dz, dx, dy, dz);
  if (sq > J->thr2) return;
  const float3 Tn = transform_normal(P.nm, n0, n1, n2);
  const float c = fdiv(dot3(Tn.x, Tn.y, Tn.z, nx, ny, nz),
                       fmul(__fsqrt_rn(dot3(Tn.x, Tn.y, Tn.z, Tn.x, Tn.y, Tn.z)),
                            __fsqrt_rn(dot3(nx, ny, nz, nx, ny, nz))));
  if (c >= -1.0f && c <= J->cos_max) return;
  const float dist = __fsqrt_rn(sq);
  const unsigned long long key = ((unsigned long long)tag_of(epoch) << 56) |
                                 ((unsigned long long)__float_as_uint(dist) << 24) |
                                 (unsigned long long)i;
  atomicMin(J->keys + pix, key);
}

// One Gauss-Newton step from the FP64 totals in shared memory, by warp 0 of
// the last block: the FP64 solve and exponential (warp_gn_update of
// gn_solve.cuh), then what the next kernel reads (the FP64 pose and its
// float32 view with the normal matrix, the status, the stop flag, the
// iteration count) and the totals of a successful step for the result.
// When a history is recorded, warp 1 writes this iteration's record
// meanwhile and, after the solve status is known (named barrier 1), its
// pose.
__device__ void gn_step(const Job *J, const StateView &V, const double *tot, int iter) {
  __shared__ float rt32[12];
  __shared__ double s_tn[16];
  __shared__ int s_ok;
  const int lane = threadIdx.x & 31;
  State *S = J->state;
  double *H = J->history ? J->history + (size_t)iter * STB_HIST_SIZE : nullptr;
  if (threadIdx.x < 32) {
    double xs[6];
    double tn;
    const bool ok = warp_gn_update(tot, tot + kJr, V.Td, xs, tn, lane);
    const double cg = tot[kCountGeom], cf = tot[kCountFeat];
    const bool no_match = (J->use_geom ? fmax(cg, cf) : cf) == 0.0;
    if (ok) {
      if (lane < 16) {
        s_tn[lane] = tn;
        S->Td[lane] = tn;
      }
      if (lane < 12) {
        const float f = __double2float_rn(tn);  // transform.to(float32)
        rt32[lane] = f;
        S->pose.rt[lane] = f;
      }
      if (lane < kAccs) S->last_totd[lane] = tot[lane];
      __syncwarp();
    }
    if (lane == 0) {
      bool finite = true;
      for (int k = 0; k < 6; ++k) finite &= isfinite(xs[k]);
      if (ok) {
        float nm[9];
        inverse_transpose(rt32, nm);
        for (int k = 0; k < 9; ++k) S->pose.nm[k] = nm[k];
        S->iters_done = V.iters_done + 1;
      }
      S->status = step_status(V.status, ok, finite, no_match, S);
      s_ok = ok;
    }
    if (H) asm volatile("bar.sync 1, 64;" ::: "memory");
    return;
  }
  if (!H) return;
  // warp 1: the history record
  for (int k = lane; k < 36; k += 32) {
    const int r = k / 6, c = k % 6;
    H[STB_HIST_JTJ + k] = tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
  }
  if (lane < 6) H[STB_HIST_JR + lane] = tot[kJr + lane];
  if (lane == 0) {
    H[STB_HIST_R2] = tot[kR2];
    H[STB_HIST_GEOM_COUNT] = tot[kCountGeom];
    H[STB_HIST_FEAT_COUNT] = tot[kCountFeat];
  }
  asm volatile("bar.sync 1, 64;" ::: "memory");
  const bool ok = s_ok;
  if (lane == 0) H[STB_HIST_OK] = ok ? 1.0 : 0.0;
  if (ok && lane < 16) H[STB_HIST_TRANSFORM + lane] = s_tn[lane];
}

// The same step in double-words (the opt-in STB_OPT_DW_SOLVE): the solve
// on the double-words (warp_gn_update_dw of gn_solve.cuh), the pose kept as
// double-words.  No FP64 instruction is on this path: the FP64 result block
// is written once per registration by the information pass, the history
// record by warp 1.
__device__ void gn_step_dw(const Job *J, const StateView &V, const float2 *totw, int iter) {
  __shared__ float rt32[12];
  __shared__ float2 s_tn[16];
  __shared__ int s_ok;
  __shared__ double s_tot[kAccs];
  const int lane = threadIdx.x & 31;
  State *S = J->state;
  double *H = J->history ? J->history + (size_t)iter * STB_HIST_SIZE : nullptr;
  if (threadIdx.x < 32) {
    float xs[6];
    float2 tn;
    const bool ok = warp_gn_update_dw(totw, totw + kJr, V.Tw, xs, tn, lane);
    // count == 0 on the high words (counts are non-negative)
    const float cg = totw[kCountGeom].x, cf = totw[kCountFeat].x;
    const bool no_match = (J->use_geom ? fmaxf(cg, cf) : cf) == 0.f;
    if (ok) {
      if (lane < 16) {
        s_tn[lane] = tn;
        S->Tw[lane] = tn;
      }
      if (lane < 12) {
        rt32[lane] = tn.x;  // the float32 rounding of the pose entry
        S->pose.rt[lane] = tn.x;
      }
      if (lane < kAccs) S->last_tot[lane] = totw[lane];
      __syncwarp();
    }
    if (lane == 0) {
      bool finite = true;
      for (int k = 0; k < 6; ++k) finite &= isfinite(xs[k]);
      if (ok) {
        float nm[9];
        inverse_transpose(rt32, nm);
        for (int k = 0; k < 9; ++k) S->pose.nm[k] = nm[k];
        S->iters_done = V.iters_done + 1;
      }
      S->status = step_status(V.status, ok, finite, no_match, S);
      s_ok = ok;
    }
    if (H) asm volatile("bar.sync 1, 64;" ::: "memory");
    return;
  }
  if (!H) return;
  // warp 1: the FP64 history record (exact conversions: a normalised
  // double-word has at most 49 significant bits)
  if (lane < kAccs) s_tot[lane] = (double)totw[lane].x + (double)totw[lane].y;
  __syncwarp();
  for (int k = lane; k < 36; k += 32) {
    const int r = k / 6, c = k % 6;
    H[STB_HIST_JTJ + k] = s_tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
  }
  if (lane < 6) H[STB_HIST_JR + lane] = s_tot[kJr + lane];
  if (lane == 0) {
    H[STB_HIST_R2] = s_tot[kR2];
    H[STB_HIST_GEOM_COUNT] = s_tot[kCountGeom];
    H[STB_HIST_FEAT_COUNT] = s_tot[kCountFeat];
  }
  asm volatile("bar.sync 1, 64;" ::: "memory");
  const bool ok = s_ok;
  if (lane == 0) H[STB_HIST_OK] = ok ? 1.0 : 0.0;
  if (ok && lane < 16) H[STB_HIST_TRANSFORM + lane] = (double)s_tn[lane].x + (double)s_tn[lane].y;
}

// Pixels of one thread per round of the reduction loop; all their loads
// that do not depend on the correspondence are issued together.
constexpr int kRP = kPixelsPerThread;

// The transposed block sum of k_reduce lives in dynamic shared memory
// (kAccs x kT floats: 60 KB at 512 threads).
extern __shared__ __align__(16) float s_red[];

template <typename FT, bool kGeom, bool kFeat, bool kHWC, int kT>
__global__ void __launch_bounds__(kT) k_reduce(const Job *__restrict__ J, int epoch) {
  __shared__ Pose32 P;
  __shared__ StateView V;
  __shared__ int skip;
  float(*red)[kT] = reinterpret_cast<float(*)[kT]>(s_red);
  __shared__ float2 bsum[kAccs];
  __shared__ int is_last;
  __shared__ float2 totw[kAccs];
  __shared__ double tot[kAccs];
  State *S = J->state;
  grid_dependency_wait();  // the association has written the key map
  grid_launch_dependents();
  const bool solve_dw = J->solve_dw;
  if (threadIdx.x == 0) skip = S->stopped;
  load_shared_pose(P, S);
  load_state_view(V, S, solve_dw);
  __syncthreads();
  if (skip) return;

  // per-thread partials are plain float32: a thread adds kRP pixels per
  // round and few rounds, so its rounding stays below ~1e-6 of the sum of
  // magnitudes; compensation (TwoSum) starts at the block level
  float acc[kAccs];
#pragma unroll
  for (int a = 0; a < kAccs; ++a) acc[a] = 0.f;

  const int H = J->H, W = J->W;
  const int64_t npix = (int64_t)H * W;
  const unsigned tag = tag_of(epoch);
  const unsigned long long *__restrict__ keys = J->keys;
  const float *__restrict__ sp = J->sp;
  const float *__restrict__ tp = J->tp;
  const float *__restrict__ tn = J->tn;
  const float wg1 = J->wg1, wg2 = J->wg2, wf1 = J->wf1, wf2 = J->wf2;
  const int64_t per_block = (int64_t)kT * kRP;
  for (int64_t base = blockIdx.x * per_block; base < npix;
       base += (int64_t)gridDim.x * per_block) {
    unsigned long long key[kRP];
    float tq[kRP][3], tnm[kRP][3];
#pragma unroll
    for (int k = 0; k < kRP; ++k) {
      const int64_t pix = base + k * kT + threadIdx.x;
      const int64_t pc = pix < npix ? pix : 0;
      key[k] = pix < npix ? keys[pix] : 0ull;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        tq[k][d] = kGeom ? tp[3 * pc + d] : 0.f;
        tnm[k][d] = kGeom ? tn[3 * pc + d] : 0.f;
      }
    }
    float spt[kRP][3];
#pragma unroll
    for (int k = 0; k < kRP; ++k) {
      const int64_t i = ((unsigned)(key[k] >> 56) == tag) ? (int64_t)(key[k] & 0xffffffull) : 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) spt[k][d] = sp[3 * i + d];
    }
#pragma unroll
    for (int k = 0; k < kRP; ++k) {
      if ((unsigned)(key[k] >> 56) != tag) continue;
      const int64_t i = (int64_t)(key[k] & 0xffffffull);
      const float3 Tp = transform_point(P.rt, spt[k][0], spt[k][1], spt[k][2]);
      if (kGeom) {
        // r = (q - Tp).n, J = [n; Tp x n] (icp_jacobian_geometric.cu:82,
        // icp_jacobian_common.hpp:41-48)
        const float nx = tnm[k][0], ny = tnm[k][1], nz = tnm[k][2];
        const float r = dot3(fsub(tq[k][0], Tp.x), fsub(tq[k][1], Tp.y),
                             fsub(tq[k][2], Tp.z), nx, ny, nz);
        const float Jv[6] = {nx, ny, nz, fsub(fmul(Tp.y, nz), fmul(Tp.z, ny)),
                             fsub(fmul(Tp.z, nx), fmul(Tp.x, nz)),
                             fsub(fmul(Tp.x, ny), fmul(Tp.y, nx))};
        accumulate_se3(acc, Jv, r, wg1, wg2);
        acc[kR2] += wg1 * (r * r);
        acc[kCountGeom] += 1.f;
      }
      if (kFeat) {
        // FeatureJacobianKernel (icp_jacobian_feature.cu:65-108)
        const FeatView<FT, kHWC> tf{static_cast<const FT *>(J->tf), npix, J->C};
        const FeatView<FT, kHWC> sf{static_cast<const FT *>(J->sf), J->n, J->C};
        float sq;
        if (feature_term(tf, sf, i, P, Tp, H, W, J->feat_thr2, J->channel_mode, wf1, wf2, acc,
                         sq)) {
          acc[kR2] += wf1 * sq;
          acc[kCountFeat] += 1.f;
        }
      }
    }
  }

  block_reduce<kAccs, kT>(acc, red, bsum);
  if (!publish_slot<kAccs>(bsum, J->part, &S->ticket, &is_last)) return;
  if (solve_dw) {
    grid_totals<kAccs, kT>(J->part, gridDim.x, nullptr, totw);
    if (threadIdx.x < 64) {
      if (threadIdx.x == 0) S->ticket = 0;
      gn_step_dw(J, V, totw, epoch);
    }
  } else {
    grid_totals<kAccs, kT>(J->part, gridDim.x, tot, nullptr);
    if (threadIdx.x < 64) {
      if (threadIdx.x == 0) S->ticket = 0;
      gn_step(J, V, tot, epoch);
    }
  }
}

// Information matrix: sum over winners of G^T G with G from the target point
// (icp_jacobian_geometric.cu:141-151), summed as icp.py:108.
__global__ void __launch_bounds__(kReduceThreads) k_info(const Job *__restrict__ J,
                                                         int epoch) {
  __shared__ float red[kInfoAccs][kReduceThreads];
  __shared__ float2 bsum[kInfoAccs];
  __shared__ int is_last;
  __shared__ double tot[kInfoAccs];
  State *S = J->state;
  grid_dependency_wait();
  float acc[kInfoAccs];
#pragma unroll
  for (int a = 0; a < kInfoAccs; ++a) acc[a] = 0.f;
  const int64_t npix = (int64_t)J->H * J->W;
  const unsigned tag = tag_of(epoch);
  const unsigned long long *__restrict__ keys = J->keys;
  const float *__restrict__ tp = J->tp;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t pix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pix < npix;
       pix += stride) {
    if ((unsigned)(keys[pix] >> 56) != tag) continue;
    const float qx = tp[3 * pix], qy = tp[3 * pix + 1], qz = tp[3 * pix + 2];
    const float G0[6] = {0.f, qz, -qy, 1.f, 0.f, 0.f};
    const float G1[6] = {-qz, 0.f, qx, 0.f, 1.f, 0.f};
    const float G2[6] = {qy, -qx, 0.f, 0.f, 0.f, 1.f};
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
      for (int b = a; b < 6; ++b)
        acc[upper_index(a, b)] += G0[a] * G0[b] + G1[a] * G1[b] + G2[a] * G2[b];
  }
  block_reduce<kInfoAccs, kReduceThreads>(acc, red, bsum);
  if (!publish_slot<kInfoAccs>(bsum, J->part, &S->ticket, &is_last)) return;
  grid_totals<kInfoAccs, kReduceThreads>(J->part, gridDim.x, tot);
  double *R = J->result;
  for (int k = threadIdx.x; k < 36; k += blockDim.x) {
    const int r = k / 6, c = k % 6;
    R[STB_RES_INFO + k] = tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
  }
  // the result of the last successful step (its pose, J^T J, match count,
  // residual r2 / count, icp.py:249-253), once per registration
  const int done = S->iters_done;
  const bool dw = J->solve_dw;
  // a total of the last successful step, from the solve's representation
  auto last = [&](int a) -> double {
    if (!dw) return S->last_totd[a];
    const float2 v = S->last_tot[a];
    return (double)v.x + (double)v.y;
  };
  if (done > 0) {
    for (int k = threadIdx.x; k < 36; k += blockDim.x) {
      const int r = k / 6, c = k % 6;
      R[STB_RES_JTJ + k] = last(r <= c ? upper_index(r, c) : upper_index(c, r));
    }
    if (threadIdx.x < 16)
      R[STB_RES_TRANSFORM + threadIdx.x] =
          dw ? (double)S->Tw[threadIdx.x].x + (double)S->Tw[threadIdx.x].y
             : S->Td[threadIdx.x];
  }
  if (threadIdx.x == 0) {
    S->ticket = 0;
    if (done > 0) {
      const double cg = last(kCountGeom), cf = last(kCountFeat);
      const double count = J->use_geom ? fmax(cg, cf) : cf;
      R[STB_RES_MATCHES] = count;
      R[STB_RES_ITERS] = (double)done;
      R[STB_RES_RESIDUAL] = last(kR2) / count;
    }
    R[STB_RES_STATUS] = (double)S->status;
  }
}

// ---------------------------------------------------------------------------
// Per-kernel CUDA-event timing (stb_profile_*): when enabled, every launch of
// the sequence is bracketed by two events recorded on the launching stream
// (captured as event nodes when the sequence is a graph).
// ---------------------------------------------------------------------------
enum ProfKind {
  kProfAssoc = 0,
  kProfReduce = 1,
  kProfInfo = 2,
  kProfSetup = 3,
  kProfPersist = 4,
  kProfKinds = 5
};
constexpr int kProfKindsRequired = 4;  // callers written for the first four kinds

struct ProfSet {
  std::vector<cudaEvent_t> start, stop;
  std::vector<int> kind;
  int used = 0;
  void reset() { used = 0; }
  void before(int k, cudaStream_t st) {
    if ((int)start.size() <= used) {
      cudaEvent_t a, b;
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      start.push_back(a);
      stop.push_back(b);
      kind.push_back(k);
    }
    kind[used] = k;
    record(start[used], st);
  }
  void after(cudaStream_t st) { record(stop[used++], st); }
  // Inside stream capture an External record becomes an event-record node
  // that records at every replay (a plain record only orders the capture);
  // outside capture a plain record.
  static void record(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    if (cs == cudaStreamCaptureStatusActive)
      cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
    else
      cudaEventRecord(ev, st);
  }
};

std::mutex g_prof_mutex;
bool g_prof_on = false;
ProfSet g_prof_direct;
ProfSet *g_prof_last = nullptr;

struct Timed {
  ProfSet *ps;
  cudaStream_t st;
  Timed(ProfSet *p, int k, cudaStream_t s) : ps(p), st(s) {
    if (ps) ps->before(k, st);
  }
  ~Timed() {
    if (ps) ps->after(st);
  }
};

// ---------------------------------------------------------------------------
// Launch sequence and CUDA-graph cache
// ---------------------------------------------------------------------------

using ReduceFn = void (*)(const Job *, int);

// The reduction kernel of a configuration with its block size and dynamic
// shared memory: the geometric-only kernel runs 512 threads per block (one
// block per SM at 640x480: half the block partials of 256, so the last
// block's fold is one round of loads); the feature kernels, whose sampling
// needs more registers, 256.
struct ReduceLaunch {
  ReduceFn fn;
  int threads;
  int smem;
};

template <typename FT, bool kGeom, bool kFeat, bool kHWC, int kT>
ReduceLaunch reduce_launch() {
  return ReduceLaunch{k_reduce<FT, kGeom, kFeat, kHWC, kT>, kT, (int)(sizeof(float) * kAccs * kT)};
}

// The 512-thread kernel needs more than the default 48 KB of dynamic shared
// memory; allowed once per device, outside any stream capture.
int prepare_reduce_kernels() {
  static std::mutex m;
  static unsigned long long done = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("cudaGetDevice");
  std::lock_guard<std::mutex> lock(m);
  if (dev < 64 && (done >> dev) & 1ull) return STB_OK;
  const ReduceLaunch r = reduce_launch<float, true, false, false, 512>();
  if (cudaFuncSetAttribute(r.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, r.smem) !=
      cudaSuccess)
    return check_launch("cudaFuncSetAttribute");
  if (dev < 64) done |= 1ull << dev;
  return STB_OK;
}

template <typename FT, bool kHWC>
ReduceLaunch feat_reduce(bool use_geom) {
  return use_geom ? reduce_launch<FT, true, true, kHWC, 256>()
                  : reduce_launch<FT, false, true, kHWC, 256>();
}

ReduceLaunch pick_reduce(const Plan &p) {
  if (!p.use_feat) return reduce_launch<float, true, false, false, 512>();
  switch (p.dtype) {
    case STB_F32: return feat_reduce<float, false>(p.use_geom);
    case STB_BF16: return feat_reduce<__nv_bfloat16, false>(p.use_geom);
    case STB_F32_HWC: return feat_reduce<float, true>(p.use_geom);
    default: return feat_reduce<__nv_bfloat16, true>(p.use_geom);
  }
}

// Launch with programmatic stream serialisation (the kernel may start while
// its predecessor finishes; it waits in grid_dependency_wait).
template <typename... Args>
void launch_pdl(void (*kern)(Args...), unsigned grid, unsigned block, size_t smem,
                cudaStream_t st, bool pdl, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = pdl ? attr : nullptr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kern, args...);
}

// Everything after k_begin; k_begin itself is launched by the caller so that
// a captured graph can take new Job parameters per call.  The first
// association follows k_begin (which writes the Job) without overlap; every
// later kernel overlaps its predecessor's tail, except when profiling (event
// records sit between the kernels).
int launch_body(const Plan &p, cudaStream_t st, ProfSet *ps) {
  const unsigned agrid = blocks_for(p.n, kAssocThreads);
  const ReduceLaunch red = pick_reduce(p);
  const unsigned rgrid = reduce_blocks((int64_t)p.H * p.W, red.threads);
  const bool pdl = ps == nullptr;
  const Job *job = p.job_dev;
  for (int it = 0; it < p.iters; ++it) {
    if (p.n > 0) {
      Timed t(ps, kProfAssoc, st);
      launch_pdl(k_assoc, agrid, kAssocThreads, 0, st, pdl && it > 0, job, it, 0);
    }
    Timed t(ps, kProfReduce, st);
    launch_pdl(red.fn, rgrid, red.threads, red.smem, st, pdl && (p.n > 0 || it > 0), job, it);
  }
  if (p.n > 0) {
    Timed t(ps, kProfAssoc, st);
    launch_pdl(k_assoc, agrid, kAssocThreads, 0, st, pdl && p.iters > 0, job, p.iters, 1);
  }
  {
    Timed t(ps, kProfInfo, st);
    launch_pdl(k_info, p.nblocks, kReduceThreads, 0, st, pdl, job, p.iters);
  }
  return check_launch("stb_icp_estimate");
}

// Key-map clear and k_begin (the Job for this call).
void launch_setup(const Plan &p, Job &job, cudaStream_t st, ProfSet *ps) {
  Timed t(ps, kProfSetup, st);
  cudaMemsetAsync(p.keys, 0xff, sizeof(unsigned long long) * (size_t)p.H * p.W, st);
  k_begin<<<1, 32, 0, st>>>(job, p.job_dev);
}

struct GraphEntry {
  cudaGraph_t graph = nullptr;  // kept alive: its node handle updates the exec
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t begin_node = nullptr;
  cudaKernelNodeParams begin_params{};
  ProfSet *prof = nullptr;  // event pairs captured in the graph (profiling)
  unsigned long long last_use = 0;
};

// Graphs kept at most; past it the least recently replayed one is
// destroyed (an executable graph destroyed while a replay is in flight is
// freed when that replay completes).
constexpr size_t kMaxGraphs = 64;

using GraphKey =
    std::tuple<void *, int64_t, int, int, int, int, int, int, int, int, int, bool, bool>;
std::mutex g_graph_mutex;
std::map<GraphKey, GraphEntry> g_graphs;
unsigned long long g_graph_tick = 0;

void evict_oldest_graph() {
  auto oldest = g_graphs.begin();
  for (auto it = g_graphs.begin(); it != g_graphs.end(); ++it)
    if (it->second.last_use < oldest->second.last_use) oldest = it;
  GraphEntry &e = oldest->second;
  {
    std::lock_guard<std::mutex> plock(g_prof_mutex);
    if (g_prof_last == e.prof) g_prof_last = nullptr;
  }
  cudaGraphExecDestroy(e.exec);
  cudaGraphDestroy(e.graph);
  delete e.prof;
  g_graphs.erase(oldest);
}

int run_graph(const Plan &p, const Job &job, bool with_history, cudaStream_t st) {
  std::lock_guard<std::mutex> lock(g_graph_mutex);
  const bool prof = g_prof_on;
  const GraphKey key{(void *)p.job_dev, p.n, p.H, p.W, p.C, p.dtype, p.iters,
                     p.use_geom, p.use_feat, p.channel_mode, p.solve_dw, with_history,
                     prof};
  auto it = g_graphs.find(key);
  Job job_copy = job;
  Job *dst = p.job_dev;
  void *args[] = {&job_copy, &dst};
  if (it == g_graphs.end()) {
    if (g_graphs.size() >= kMaxGraphs) evict_oldest_graph();
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess)
      return check_launch("cudaStreamCreate");
    cudaGraph_t graph;
    ProfSet *ps = prof ? new ProfSet() : nullptr;
    cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    launch_setup(p, job_copy, cap, ps);
    launch_body(p, cap, ps);
    const cudaError_t cerr = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (cerr != cudaSuccess)
      return fail(STB_ECUDA, "Cuda call error stb_icp_estimate (graph capture): %s",
                  cudaGetErrorString(cerr));
    GraphEntry e;
    e.prof = ps;
    // locate k_begin's node to update its parameters on later calls
    size_t count = 0;
    cudaGraphGetNodes(graph, nullptr, &count);
    cudaGraphNode_t *nodes = new cudaGraphNode_t[count];
    cudaGraphGetNodes(graph, nodes, &count);
    for (size_t k = 0; k < count; ++k) {
      cudaGraphNodeType type;
      cudaGraphNodeGetType(nodes[k], &type);
      if (type != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp;
      cudaGraphKernelNodeGetParams(nodes[k], &kp);
      if (kp.func == (void *)k_begin) {
        e.begin_node = nodes[k];
        e.begin_params = kp;
      }
    }
    delete[] nodes;
    const cudaError_t ierr = cudaGraphInstantiate(&e.exec, graph, 0);
    if (ierr != cudaSuccess || !e.begin_node) {
      cudaGraphDestroy(graph);
      return fail(STB_ECUDA, "Cuda call error stb_icp_estimate (graph instantiate): %s",
                  cudaGetErrorString(ierr));
    }
    e.graph = graph;
    it = g_graphs.emplace(key, e).first;
  }
  GraphEntry &e = it->second;
  e.last_use = ++g_graph_tick;
  if (e.prof) {
    std::lock_guard<std::mutex> plock(g_prof_mutex);
    g_prof_last = e.prof;
  }
  cudaKernelNodeParams kp = e.begin_params;
  kp.kernelParams = args;
  kp.extra = nullptr;
  if (cudaGraphExecKernelNodeSetParams(e.exec, e.begin_node, &kp) != cudaSuccess)
    return check_launch("cudaGraphExecKernelNodeSetParams");
  if (cudaGraphLaunch(e.exec, st) != cudaSuccess) return check_launch("cudaGraphLaunch");
  return STB_OK;
}

}  // namespace
}  // namespace stb

using namespace stb;

extern "C" size_t stb_icp_workspace_bytes(int64_t num_source, int32_t height,
                                          int32_t width) {
  (void)num_source;
  return workspace_bytes((int64_t)height * width);
}

namespace stb {
namespace {

// The arguments of a registration call, as the entry points take them.
struct EstimateArgs {
  const float *kcam, *src_points, *src_normals;
  const uint8_t *src_mask;
  int64_t num_source;
  const void *src_feats;
  const float *tgt_points, *tgt_normals;
  const uint8_t *tgt_mask;
  int32_t height, width;
  const void *tgt_feats;
  int32_t channels, feat_dtype;
  const double *init_transform;
  int32_t num_iters;
  double geom_weight, feat_weight, distance_thresh, normal_angle_thresh,
      feat_residual_thresh;
  int32_t channel_mode;  // channel mode (low byte) | STB_OPT_* bits
  double *result, *history;
};

// Checks the arguments shared by both registration entry points (sizes,
// options, device pointers); tells whether kcam and init_transform are host
// memory.
int check_args(const EstimateArgs &a, bool *kcam_host, bool *init_host) {
  if (a.num_source < 0 || (unsigned long long)a.num_source >= kMaxSources)
    return fail(STB_EINVAL, "Check failed: num_source must be in [0, 2^24), got %lld",
                (long long)a.num_source);
  if (a.height <= 0 || a.width <= 0)
    return fail(STB_EINVAL, "Check failed: target size must be positive, got %dx%d",
                a.height, a.width);
  if (a.num_iters < 0 || a.num_iters > 254)
    return fail(STB_EINVAL, "Check failed: num_iters must be in [0, 254], got %d",
                a.num_iters);
  constexpr unsigned kOpts = STB_OPT_DW_SOLVE | STB_OPT_MULTI_LAUNCH;
  if (((unsigned)a.channel_mode & ~(0xffu | kOpts)) != 0)
    return fail(STB_EINVAL, "Check failed: unknown option bits 0x%x in channel_mode",
                (unsigned)a.channel_mode & ~(0xffu | kOpts));
  const int cmode = a.channel_mode & 0xff;
  const bool use_feat = a.feat_weight > 0.0 && a.src_feats && a.tgt_feats;
  if (use_feat) {
    if (a.channels <= 0)
      return fail(STB_EINVAL, "Check failed: channels must be positive, got %d", a.channels);
    if (a.feat_dtype < STB_F32 || a.feat_dtype > STB_BF16_HWC)
      return fail(STB_EDTYPE, "Check failed: feature maps must be float32 or bfloat16");
    if (cmode != 0 && cmode != 1)
      return fail(STB_EINVAL, "Check failed: channel_mode must be 0 or 1");
  }
  STB_TRY(check_small_input(a.kcam, "kcam", false, kcam_host));
  STB_TRY(check_device_ptr(a.src_points, "src_points"));
  STB_TRY(check_device_ptr(a.src_normals, "src_normals"));
  STB_TRY(check_device_ptr(a.src_mask, "src_mask"));
  STB_TRY(check_device_ptr(a.tgt_points, "tgt_points"));
  STB_TRY(check_device_ptr(a.tgt_normals, "tgt_normals"));
  STB_TRY(check_device_ptr(a.tgt_mask, "tgt_mask"));
  if (use_feat) {
    STB_TRY(check_device_ptr(a.src_feats, "src_feats"));
    STB_TRY(check_device_ptr(a.tgt_feats, "tgt_feats"));
  }
  STB_TRY(check_small_input(a.init_transform, "transform", true, init_host));
  STB_TRY(check_device_ptr(a.result, "result"));
  STB_TRY(check_device_ptr(a.history, "history", true));
  return STB_OK;
}

// The plan and the Job of a checked call on the workspace at ws.
void make_plan(const EstimateArgs &a, bool kcam_host, bool init_host, char *ws, Plan &p,
               Job &job) {
  const bool use_feat = a.feat_weight > 0.0 && a.src_feats && a.tgt_feats;
  const bool use_geom = a.geom_weight > 0.0;
  const int64_t npix = (int64_t)a.height * a.width;
  p.n = a.num_source;
  p.H = a.height;
  p.W = a.width;
  p.C = use_feat ? a.channels : 0;
  p.dtype = use_feat ? a.feat_dtype : 0;
  p.iters = a.num_iters;
  p.use_geom = use_geom;
  p.use_feat = use_feat;
  p.channel_mode = use_feat ? (a.channel_mode & 0xff) : 0;
  p.solve_dw = (a.channel_mode & STB_OPT_DW_SOLVE) != 0;
  p.multi_launch = (a.channel_mode & STB_OPT_MULTI_LAUNCH) != 0;
  p.nblocks = reduce_blocks(npix);
  p.job_dev = reinterpret_cast<Job *>(ws);

  job.sp = a.src_points;
  job.sn = a.src_normals;
  job.sm = a.src_mask;
  job.n = a.num_source;
  job.sf = a.src_feats;
  job.tp = a.tgt_points;
  job.tn = a.tgt_normals;
  job.tm = a.tgt_mask;
  job.H = a.height;
  job.W = a.width;
  job.tf = a.tgt_feats;
  job.C = p.C;
  job.dtype = p.dtype;
  set_small_inputs(job, a.kcam, kcam_host, a.init_transform, init_host);
  job.iters = a.num_iters;
  job.channel_mode = p.channel_mode;
  job.use_geom = use_geom;
  job.use_feat = use_feat;
  job.solve_dw = p.solve_dw;
  job.wg1 = (float)a.geom_weight;
  job.wg2 = (float)(a.geom_weight * a.geom_weight);
  job.wf1 = (float)a.feat_weight;
  job.wf2 = (float)(a.feat_weight * a.feat_weight);
  job.thr2 = distance_thresh_sq(a.distance_thresh);
  job.cos_max = angle_cos_max(a.normal_angle_thresh);
  {
    const float t = (float)a.feat_residual_thresh;  // a float in the reference
    job.feat_thr2 = t * t;
  }
  job.result = a.result;
  job.history = a.history;
  job.state = reinterpret_cast<State *>(ws + kSlot);
  job.part = reinterpret_cast<float2 *>(ws + 2 * kSlot);
  job.keys = reinterpret_cast<unsigned long long *>(ws + keys_offset(npix));
  job.nblocks = p.nblocks;
  p.keys = job.keys;
  static_assert(sizeof(Job) <= kSlot && sizeof(State) <= kSlot, "workspace slots");
}

}  // namespace
}  // namespace stb

extern "C" int stb_icp_correspondences(const void *workspace, int32_t height, int32_t width,
                                       int32_t num_iters, int64_t *merge_map, void *stream) {
  clear_error();
  if (height <= 0 || width <= 0)
    return fail(STB_EINVAL, "Check failed: target size must be positive, got %dx%d",
                height, width);
  if (num_iters < 0 || num_iters > 254)
    return fail(STB_EINVAL, "Check failed: num_iters must be in [0, 254], got %d", num_iters);
  if (((uintptr_t)workspace & 255) != 0)
    return fail(STB_EINVAL, "Check failed: workspace must be 256-byte aligned");
  STB_TRY(check_device_ptr(workspace, "workspace"));
  STB_TRY(check_device_ptr(merge_map, "merge_map"));
  const int64_t npix = (int64_t)height * width;
  const auto *keys = reinterpret_cast<const unsigned long long *>(
      static_cast<const char *>(workspace) + keys_offset(npix));
  k_keys_to_merge_map<<<keys_grid(npix), 256, 0, as_stream(stream)>>>(
      keys, nullptr, npix, tag_of_host(num_iters), reinterpret_cast<long long *>(merge_map));
  return check_launch("stb_icp_correspondences");
}

extern "C" int stb_icp_estimate(
    const float *kcam, const float *src_points, const float *src_normals,
    const uint8_t *src_mask, int64_t num_source, const void *src_feats,
    const float *tgt_points, const float *tgt_normals, const uint8_t *tgt_mask,
    int32_t height, int32_t width, const void *tgt_feats, int32_t channels,
    int32_t feat_dtype, const double *init_transform, int32_t num_iters,
    double geom_weight, double feat_weight, double distance_thresh,
    double normal_angle_thresh, double feat_residual_thresh, int32_t channel_mode,
    void *workspace, size_t workspace_bytes_, double *result, double *history,
    int32_t use_graph, void *stream) {
  clear_error();
  const EstimateArgs a{kcam, src_points, src_normals, src_mask, num_source, src_feats,
                       tgt_points, tgt_normals, tgt_mask, height, width, tgt_feats, channels,
                       feat_dtype, init_transform, num_iters, geom_weight, feat_weight,
                       distance_thresh, normal_angle_thresh, feat_residual_thresh,
                       channel_mode, result, history};
  bool kcam_host, init_host;
  STB_TRY(check_args(a, &kcam_host, &init_host));
  const int64_t npix = (int64_t)height * width;
  if (workspace_bytes_ < workspace_bytes(npix))
    return fail(STB_EINVAL, "Check failed: workspace of %zu bytes, %zu needed",
                workspace_bytes_, workspace_bytes(npix));
  if (((uintptr_t)workspace & 255) != 0)
    return fail(STB_EINVAL, "Check failed: workspace must be 256-byte aligned");
  STB_TRY(check_device_ptr(workspace, "workspace"));
  STB_TRY(prepare_reduce_kernels());
  Plan p;
  Job job;
  make_plan(a, kcam_host, init_host, static_cast<char *>(workspace), p, job);

  const cudaStream_t st = as_stream(stream);
  ProfSet *ps = nullptr;
  if (g_prof_on) {
    std::lock_guard<std::mutex> plock(g_prof_mutex);
    g_prof_direct.reset();
    ps = g_prof_last = &g_prof_direct;
  }
  if (!p.multi_launch) {
    STB_TRY(reset_persistent(job, st));
    Timed t(ps, kProfPersist, st);
    return launch_persistent(p, job, st);
  }
  if (use_graph) return run_graph(p, job, history != nullptr, st);
  launch_setup(p, job, st, ps);
  return launch_body(p, st, ps);
}

extern "C" int stb_profile_enable(int32_t on) {
  clear_error();
  std::lock_guard<std::mutex> plock(g_prof_mutex);
  g_prof_on = on != 0;
  g_prof_last = nullptr;
  return STB_OK;
}

extern "C" int stb_profile_read(double *ms_by_kind, int64_t *launches_by_kind,
                                int32_t num_kinds) {
  clear_error();
  if (num_kinds < kProfKindsRequired)
    return fail(STB_EINVAL, "Check failed: num_kinds must be at least %d", kProfKindsRequired);
  for (int k = 0; k < num_kinds; ++k) {
    ms_by_kind[k] = 0.0;
    launches_by_kind[k] = 0;
  }
  std::lock_guard<std::mutex> plock(g_prof_mutex);
  if (!g_prof_last) return STB_OK;
  for (int i = 0; i < g_prof_last->used; ++i) {
    float ms = 0.f;
    const cudaError_t err =
        cudaEventElapsedTime(&ms, g_prof_last->start[i], g_prof_last->stop[i]);
    if (err != cudaSuccess)
      return fail(STB_ECUDA, "Cuda call error stb_profile_read: %s", cudaGetErrorString(err));
    const int kind = g_prof_last->kind[i];
    if (kind >= num_kinds) continue;
    ms_by_kind[kind] += ms;
    launches_by_kind[kind] += 1;
  }
  return STB_OK;
}

// ---------------------------------------------------------------------------
// Registration without any allocation: the same launch sequence as
// stb_icp_estimate, with its scratch in a fixed device array.
//
// Who needs it: callers that cannot call cudaMalloc while they track --
// hosts that bind the C ABI from a runtime without a CUDA allocator of its
// own (a plain C or FFI host, no torch caching allocator to borrow from),
// and applications that fix their device-memory budget at start-up and
// forbid later allocations (cudaMalloc and cudaFree synchronise the device,
// which stalls a real-time tracking loop sharing the GPU).
//
// The scratch is kStaticMaxPixels target pixels' worth (about 8.9 MB) in
// g_static_workspace, which every GPU that loads this library holds until
// the process exits.  The first call on a device looks up the array's device
// address with cudaGetSymbolAddress (host code cannot use the symbol itself:
// it names a host-side stand-in); make that first call before any stream
// capture.  The address is cached for the life of the process, so a device
// reset (cudaDeviceReset) ends this entry point's use on that device.  All calls share the one array: two calls whose work overlaps on
// the GPU race and corrupt each other.  What must start cleared is cleared by
// every call (the key map and the per-call state), the rest is written
// before it is read.
// ---------------------------------------------------------------------------
namespace stb {
namespace {

constexpr int64_t kStaticMaxPixels = 1 << 20;  // e.g. 1280x720 and 1024x1024 fit
// The layout of stb_icp_estimate's workspace at the largest frame: every
// frame up to kStaticMaxPixels fits (workspace_bytes grows with the pixels).
constexpr size_t kStaticWorkspaceBytes = workspace_bytes(kStaticMaxPixels);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_workspace[kStaticWorkspaceBytes];

std::mutex g_static_mutex;
void *g_static_ptr[kMaxDevices] = {};

// Device address of g_static_workspace on the current device (looked up
// once per device).
int static_workspace(void **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(STB_ECUDA, "Cuda call error stb_icp_estimate_static: no usable device");
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&p, g_static_workspace);
    if (err != cudaSuccess || !p)
      return fail(STB_ECUDA, "Cuda call error stb_icp_estimate_static "
                  "(cudaGetSymbolAddress): %s", cudaGetErrorString(err));
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return STB_OK;
}

}  // namespace
}  // namespace stb

extern "C" int stb_icp_estimate_static(
    const float *kcam, const float *src_points, const float *src_normals,
    const uint8_t *src_mask, int64_t num_source, const void *src_feats,
    const float *tgt_points, const float *tgt_normals, const uint8_t *tgt_mask,
    int32_t height, int32_t width, const void *tgt_feats, int32_t channels,
    int32_t feat_dtype, const double *init_transform, int32_t num_iters,
    double geom_weight, double feat_weight, double distance_thresh,
    double normal_angle_thresh, double feat_residual_thresh, int32_t channel_mode,
    double *result, double *history, void *stream) {
  clear_error();
  if (height <= 0 || width <= 0)
    return fail(STB_EINVAL, "Check failed: target size must be positive, got %dx%d",
                height, width);
  const int64_t npix = (int64_t)height * width;
  if (npix > kStaticMaxPixels)
    return fail(STB_EINVAL,
                "Check failed: stb_icp_estimate_static handles at most %lld target pixels "
                "(its fixed scratch), got %dx%d = %lld; use stb_icp_estimate with a "
                "caller-provided workspace", (long long)kStaticMaxPixels, height, width,
                (long long)npix);
  const EstimateArgs a{kcam, src_points, src_normals, src_mask, num_source, src_feats,
                       tgt_points, tgt_normals, tgt_mask, height, width, tgt_feats, channels,
                       feat_dtype, init_transform, num_iters, geom_weight, feat_weight,
                       distance_thresh, normal_angle_thresh, feat_residual_thresh,
                       channel_mode, result, history};
  bool kcam_host, init_host;
  STB_TRY(check_args(a, &kcam_host, &init_host));
  STB_TRY(prepare_reduce_kernels());
  void *workspace = nullptr;
  STB_TRY(static_workspace(&workspace));
  if (workspace_bytes(npix) > kStaticWorkspaceBytes)
    return fail(STB_EINVAL, "Check failed: stb_icp_estimate_static scratch too small");
  Plan p;
  Job job;
  make_plan(a, kcam_host, init_host, static_cast<char *>(workspace), p, job);

  // Direct launches only: no graph, no stream and no event is created here.
  const cudaStream_t st = as_stream(stream);
  if (!p.multi_launch) {
    STB_TRY(reset_persistent(job, st));
    return launch_persistent(p, job, st);
  }
  launch_setup(p, job, st, nullptr);
  return launch_body(p, st, nullptr);
}

extern "C" int stb_set_wait_test_limits(uint32_t spin_limit, int32_t phantom_arrivals) {
  clear_error();
  if (phantom_arrivals < 0)
    return fail(STB_EINVAL, "Check failed: phantom_arrivals must be >= 0, got %d",
                phantom_arrivals);
  set_persist_test_limits(spin_limit, phantom_arrivals);
  return STB_OK;
}
