// Shared pieces of the fused single-pair registration (the multi-launch
// path of icp_fused.cu and the persistent kernel of icp_persist.cu): the
// workspace layout, the loop state, the per-call parameters (Job) and the
// block- and grid-level compensated reductions.
#pragma once

#include <stdint.h>

#include "gn_solve.cuh"
#include "stb_common.cuh"
#include "slamtb_gb300.h"

namespace stb {
namespace fused {

constexpr int kAccs = 30;      // 21 JtJ (upper) + 6 Jr + r2 + count_geom + count_feat
constexpr int kInfoAccs = 21;  // GtG upper triangle
constexpr int kAssocThreads = 256;
constexpr int kReduceThreads = 256;
constexpr int kPixelsPerThread = 4;
constexpr int kMaxReduceBlocks = 152 * 8;
constexpr unsigned long long kMaxSources = 1ull << 24;

// Accumulator slots.
constexpr int kJr = 21, kR2 = 27, kCountGeom = 28, kCountFeat = 29;

// The loop state.  The pose and the totals of the last successful step are
// FP64 (Td, last_totd) under the default FP64 solve, double-words (Tw,
// last_tot) under the opt-in double-word solve (Job::solve_dw).
struct State {
  double Td[16];
  double last_totd[32];
  float2 Tw[16];  // pose as double-words (within ~1e-14 of FP64)
  Pose32 pose;    // float32 view of the pose + intrinsics
  float2 last_tot[32];
  unsigned ticket;
  unsigned stopped;
  unsigned status;
  int iters_done;
  // grid barrier of the persistent kernel: arrivals (only grow during a
  // call) and error
  unsigned bar_count, bar_err;
};
static_assert(sizeof(State) <= 1024, "the workspace's State slot is 1024 bytes");

struct Job {
  const float *kcam;
  const float *sp, *sn;
  const uint8_t *sm;
  long long n;
  const void *sf;
  const float *tp, *tn;
  const uint8_t *tm;
  int H, W;
  const void *tf;
  int C, dtype;
  const double *init;
  int iters, channel_mode;
  int use_geom, use_feat;
  int solve_dw;  // 1: double-word solve (STB_OPT_DW_SOLVE), 0: FP64
  float wg1, wg2, wf1, wf2;
  float thr2, cos_max, feat_thr2;
  double *result, *history;
  unsigned long long *keys;
  float2 *part;  // per block: kSlotAccs (sum, compensation) pairs; two
                 // such buffers (the persistent kernel alternates them)
  int nblocks;
  State *state;
  // intrinsics (fx, cx, fy, cy) and initial pose given as host values
  // (kcam / init null): carried in the launch parameters, no copy
  float kcam_v[4];
  double init_v[16];
  int has_init_v;
  // the persistent kernel's grid barriers: polls before a wait gives up,
  // and arrivals expected beyond the grid's blocks (0; a test sets more so
  // that the waits run out)
  unsigned spin_limit;
  int bar_phantom;
  // rounds of source points the persistent kernel keeps in shared memory
  int src_cache_rounds;
};
static_assert(sizeof(Job) <= 1024, "the workspace's Job slot is 1024 bytes");

// Host-side: intrinsics and initial pose into the Job, by pointer (device
// memory) or by value (host memory, read here).
inline void set_small_inputs(Job &job, const float *kcam, bool kcam_host, const double *init,
                             bool init_host) {
  job.kcam = kcam_host ? nullptr : kcam;
  if (kcam_host) {
    job.kcam_v[0] = kcam[0];
    job.kcam_v[1] = kcam[2];
    job.kcam_v[2] = kcam[4];
    job.kcam_v[3] = kcam[5];
  }
  job.init = init_host ? nullptr : init;
  job.has_init_v = init != nullptr && init_host;
  for (int k = 0; k < 16; ++k) job.init_v[k] = job.has_init_v ? init[k] : 0.0;
}

constexpr size_t kSlot = 1024;

__host__ __device__ constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Blocks of the reduction for `threads` threads of kPixelsPerThread pixels;
// the workspace holds slots for the 256-thread count (the largest grid).
constexpr int reduce_blocks(int64_t pixels, int threads = kReduceThreads) {
  const int64_t per_block = (int64_t)threads * kPixelsPerThread;
  int64_t b = (pixels + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > kMaxReduceBlocks) b = kMaxReduceBlocks;
  return (int)b;
}

constexpr int kSlotAccs = 32;  // accumulator pairs per block slot (>= kAccs)

// Workspace: [Job slot][State slot][block slots: 2 x nblocks x kSlotAccs
// float2][keys H*W]
constexpr size_t keys_offset(int64_t pixels) {
  return 2 * kSlot + align256(2 * sizeof(float2) * kSlotAccs * reduce_blocks(pixels));
}
constexpr size_t workspace_bytes(int64_t pixels) {
  return keys_offset(pixels) + align256(sizeof(unsigned long long) * pixels);
}

__device__ __forceinline__ unsigned tag_of(int epoch) { return 254u - (unsigned)epoch; }
inline unsigned tag_of_host(int epoch) { return 254u - (unsigned)epoch; }

__device__ __forceinline__ void load_shared_pose(Pose32 &P, const State *S) {
  const float *src = reinterpret_cast<const float *>(&S->pose);
  float *dst = reinterpret_cast<float *>(&P);
  for (int k = threadIdx.x; k < (int)(sizeof(Pose32) / sizeof(float)); k += blockDim.x)
    dst[k] = src[k];
}


__device__ __forceinline__ void accumulate_se3(float *acc, const float *Jv, float r, float w1,
                                               float w2) {
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = a; b < 6; ++b) acc[upper_index(a, b)] += w2 * (Jv[a] * Jv[b]);
#pragma unroll
  for (int a = 0; a < 6; ++a) acc[kJr + a] += w1 * (Jv[a] * r);
}

// Block-level compensated reduction of kN per-thread float32 partials,
// transposed through shared memory: thread t stores its partial a at
// red[a][t]; warp w then sums accumulators w, w + 8, ... (each lane eight
// of the block's threads with TwoSum, then the warp's lanes by shuffles),
// its accumulators interleaved so that their dependent chains overlap.
// Threads 0..kN-1 of the block end with the totals in out (shared).
template <int kN, int kT>
__device__ __forceinline__ void block_reduce(const float *acc, float (*red)[kT], float2 *out) {
  constexpr int kW = kT / 32;
  constexpr int kPer = (kN + kW - 1) / kW;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < kN; ++a) red[a][threadIdx.x] = acc[a];
  __syncthreads();
  CSum t[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int a = warp + q * kW;
    float v[kW];
#pragma unroll
    for (int j = 0; j < kW; ++j) v[j] = (a < kN) ? red[a < kN ? a : 0][lane + 32 * j] : 0.f;
    t[q] = {v[0], 0.f};
#pragma unroll
    for (int j = 1; j < kW; ++j) csum_add(t[q], v[j]);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      const float s2 = __shfl_down_sync(0xffffffffu, t[q].s, off);
      const float c2 = __shfl_down_sync(0xffffffffu, t[q].c, off);
      csum_merge(t[q], s2, c2);
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      const int a = warp + q * kW;
      if (a < kN) out[a] = make_float2(t[q].s, t[q].c);
    }
  }
  __syncthreads();
}

// Writes the block's totals to its slot and takes a ticket; true in the
// last block to finish (which then sees every slot).
template <int kN>
__device__ __forceinline__ bool publish_slot(const float2 *bsum, float2 *part, unsigned *ticket,
                                             int *is_last) {
  if (threadIdx.x < kN) part[(size_t)blockIdx.x * kSlotAccs + threadIdx.x] = bsum[threadIdx.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!*is_last) return false;
  __threadfence();
  return true;
}

// Last block: totals of kN accumulators from all block slots, in FP64 (when
// tot is given) and as double-words (when totw is given).  Warp w
// folds slots w, w + 8, ... with lane = accumulator; every load of a round
// (kFoldLoads slots) is issued before its additions, so 300 slots cost two
// L2 round trips.  The eight warp results are merged through shared memory.
constexpr int kFoldLoads = 24;
template <int kN, int kT>
__device__ __forceinline__ void grid_totals(const float2 *part, int nblocks, double *tot,
                                            float2 *totw = nullptr) {
  __shared__ float2 wsum[kT / 32][32];
  constexpr int kW = kT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  CSum t = {0.f, 0.f};
  for (int b0 = warp; b0 < nblocks; b0 += kW * kFoldLoads) {
    float2 v[kFoldLoads];
#pragma unroll
    for (int k = 0; k < kFoldLoads; ++k) {
      const int b = b0 + k * kW;
      v[k] = (b < nblocks && lane < kN) ? __ldcg(part + (size_t)b * kSlotAccs + lane)
                                        : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < kFoldLoads; ++k) csum_merge(t, v[k].x, v[k].y);
  }
  wsum[warp][lane] = make_float2(t.s, t.c);
  __syncthreads();
  if (threadIdx.x < kN) {
    CSum u = {0.f, 0.f};
#pragma unroll
    for (int w = 0; w < kW; ++w) csum_merge(u, wsum[w][threadIdx.x].x, wsum[w][threadIdx.x].y);
    if (tot) tot[threadIdx.x] = (double)u.s + (double)u.c;
    if (totw) totw[threadIdx.x] = dw_of_csum(u.s, u.c);
  }
  __syncthreads();
}

// Per-block copy of the loop state, loaded at kernel start (the last block
// then finds it in shared memory instead of paying an L2 round trip in the
// serial tail).
struct StateView {
  double Td[16];
  float2 Tw[16];
  unsigned status;
  int iters_done;
};

__device__ __forceinline__ void load_state_view(StateView &V, const State *S, bool dw) {
  if (threadIdx.x < 16) {
    if (dw)
      V.Tw[threadIdx.x] = S->Tw[threadIdx.x];
    else
      V.Td[threadIdx.x] = S->Td[threadIdx.x];
  }
  if (threadIdx.x == 16) V.status = S->status;
  if (threadIdx.x == 17) V.iters_done = S->iters_done;
}

// Status bits of a step (lane 0): what warp_gn_update's verdict, the
// update's finiteness and the match counts say, and the stop flag.
__device__ __forceinline__ unsigned step_status(unsigned st, bool ok, bool finite,
                                                bool no_match, State *S) {
  if (!ok) {
    st |= STB_ST_NOT_PD;
    S->stopped = 1;
  } else if (!finite) {
    st |= STB_ST_NAN;
  }
  if (no_match) st |= STB_ST_NO_MATCHES;
  return st;
}


// Sizes and options of one call, and where its Job and key map live.
struct Plan {
  int64_t n;
  int H, W, C, dtype, iters, use_geom, use_feat, channel_mode, solve_dw, multi_launch, nblocks;
  Job *job_dev;
  unsigned long long *keys;
};

// The persistent single-launch registration (icp_persist.cu): launches the
// whole registration of Job (whose Job slot, State and key map live in the
// workspace of the Plan) on stream st, after reset_persistent has cleared
// its barrier words on the same stream.
int reset_persistent(const Job &job, cudaStream_t st);
int launch_persistent(const Plan &p, Job job, cudaStream_t st);

// Test hook of the persistent kernels' bounded waits: a wait gives up after
// spin_limit polls (0: the default), and every grid barrier expects phantom
// more arrivals than the grid has blocks (0: none).
void set_persist_test_limits(unsigned spin_limit, int phantom);

}  // namespace fused
}  // namespace stb
