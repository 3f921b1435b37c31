// Batched multiscale ICP with the grid split into groups: each group of
// blocks registers whole frame pairs, one after the other, with the phases
// of the single-pair kernel (persist_phases.cuh) and barriers of its own.
//
// The lock-step batch kernel (icp_batch.cu) advances every pair through the
// same phase at once, so each phase streams all pairs' frames from memory
// and waits at grid barriers for the slowest.  Here a group keeps one pair
// (a few to ~60 MB for 640x480 to 1280x720 frames) resident in L2 for all
// of its iterations, the groups' serial parts (barriers, the FP64 step)
// overlap each other, and no pair waits for another: for many small and
// mid-size pairs this is the faster schedule; the batch entry point runs
// whichever the caller (or BatchRegistration.autotune) picks.
//
// Per pair (MultiscaleRegistration.estimate_frame,
// slamtb/registration/multiscale.py:30-67): the group clears the pair's key
// map; per level, coarsest first, the pose carries over (identity when the
// previous level's first iteration failed), and each Gauss-Newton
// iteration is association (correspondence_map.cu:39-61), group barrier,
// reduction into the group's slots, the polled fold and the step
// (icp.py:152-262), as ICPOdometry.estimate; after the finest level, the
// association at the final pose and the information sum
// (icp_jacobian_geometric.cu:118-158).  Pairs are handed out from a queue
// ordered by decreasing size, so large pairs start first.
//
// Every wait is bounded; a wait that gives up sets the error word (shared
// with the lock-step kernel), every block leaves, and the status pass
// flags STB_ST_TIMEOUT in every pair's result.
#include <math.h>
#include <stddef.h>

#include "group_launch.hpp"
#include "persist_phases.cuh"
#include "stb_host.hpp"

namespace stb {
namespace fused {

// One level of one pair as a group runs it (kept in shared memory; the
// phase templates read the fields they need).
struct GLevel {
  const float *sp, *sn;
  const uint8_t *sm;
  long long n;
  const void *sf;
  const float *tp, *tn;
  const uint8_t *tm;
  int H, W;
  const void *tf;
  int C, channel_mode;
  int use_geom, use_feat;
  float wg1, wg2, wf1, wf2, thr2, cos_max, feat_thr2;
  unsigned long long *keys;
  float2 *part;
  unsigned *bar, *err;
  unsigned spin_limit;
  int bar_phantom;
  int rank, size;
};

__device__ __forceinline__ int rank_of(const GLevel &x) { return x.rank; }
__device__ __forceinline__ int size_of(const GLevel &x) { return x.size; }
__device__ __forceinline__ unsigned *bar_word(const GLevel &x) { return x.bar; }
__device__ __forceinline__ unsigned *err_word(const GLevel &x) { return x.err; }

// The whole grid as one barrier group (set-up phase).
struct GridSync {
  unsigned *bar, *err;
  unsigned spin_limit;
  int bar_phantom;
};
__device__ __forceinline__ int rank_of(const GridSync &) { return blockIdx.x; }
__device__ __forceinline__ int size_of(const GridSync &) { return gridDim.x; }
__device__ __forceinline__ unsigned *bar_word(const GridSync &x) { return x.bar; }
__device__ __forceinline__ unsigned *err_word(const GridSync &x) { return x.err; }

namespace {

// Barrier words in the sync region: [0] grid arrivals, [2] error word (bit
// 0 timeout, bit 1 capacity), [3] the pair queue; group g's arrival counter
// at kGroupWords + 32 g and its published ticket one word later.
constexpr int kGroupWords = 64;

// A pair's state while its group runs it (every block of the group holds
// the same copy).
struct PairLoop {
  LoopShared L;
  int p;            // pair
  int stopped;      // the level's solve failed: its remaining iterations skip
  int level_iters;  // successful iterations of the current level
  double last_r2, last_count;  // of the level's last successful step
};

// The step of one iteration (warp 0 of every block of the group): the
// solve, the pose, and the record (rank 0: the result block and the
// history row), as the lock-step kernel's pair step.
__device__ void group_step(const GroupLaunch &a, const GLevel &X, PairLoop &S, int s, int lane) {
  LoopShared &L = S.L;
  const bool dw = a.solve_dw;
  const double cg = L.tot[kCountGeom], cf = L.tot[kCountFeat];
  const double count = X.use_geom ? fmax(cg, cf) : cf;
  double xs[6];
  double tn;
  bool ok;
  if (dw) {
    if (lane < 16) L.Tw[lane] = dw_of_double(L.Td[lane]);
    __syncwarp();
    float2 tnw;
    float xf[6];
    ok = warp_gn_update_dw(L.totw, L.totw + kJr, L.Tw, xf, tnw, lane);
    tn = (double)tnw.x + (double)tnw.y;
    for (int k = 0; k < 6; ++k) xs[k] = xf[k];
  } else {
    ok = warp_gn_update(L.tot, L.tot + kJr, L.Td, xs, tn, lane);
  }
  const bool rec = X.rank == 0;
  double *R = a.results + (size_t)S.p * STB_RES_SIZE;
  double *H = (rec && a.history)
                  ? a.history + ((size_t)S.p * a.total_iters + s) * STB_HIST_SIZE
                  : nullptr;
  for (int k = lane; k < 36; k += 32) {
    const int r = k / 6, c = k % 6;
    const double v = L.tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
    if (H) H[STB_HIST_JTJ + k] = v;
    if (rec && ok) R[STB_RES_JTJ + k] = v;
  }
  if (H && lane < 6) H[STB_HIST_JR + lane] = L.tot[kJr + lane];
  if (H && lane == 0) {
    H[STB_HIST_R2] = L.tot[kR2];
    H[STB_HIST_GEOM_COUNT] = cg;
    H[STB_HIST_FEAT_COUNT] = cf;
  }
  __syncwarp();
  if (!ok) {
    if (lane == 0) {
      unsigned st = L.status | STB_ST_NOT_PD;
      if (count == 0.0) st |= STB_ST_NO_MATCHES;
      L.status = st;
      S.stopped = 1;
      if (rec) R[STB_RES_STATUS] = (double)st;
      if (H) H[STB_HIST_OK] = 0.0;
    }
    __syncwarp();
    return;
  }
  if (lane < 16) {
    L.Td[lane] = tn;
    if (rec) R[STB_RES_TRANSFORM + lane] = tn;
    if (H) H[STB_HIST_TRANSFORM + lane] = tn;
  }
  __syncwarp();
  refresh_view(L, false, lane);
  if (lane == 0) {
    unsigned st = L.status;
    bool finite = true;
    for (int k = 0; k < 6; ++k) finite &= isfinite(xs[k]);
    if (!finite) st |= STB_ST_NAN;
    if (count == 0.0) st |= STB_ST_NO_MATCHES;
    L.status = st;
    S.level_iters += 1;
    S.last_r2 = L.tot[kR2];
    S.last_count = count;
    if (rec) {
      R[STB_RES_MATCHES] = count;
      R[STB_RES_ITERS] = (double)S.level_iters;
      R[STB_RES_STATUS] = (double)st;
    }
    if (H) H[STB_HIST_OK] = 1.0;
  }
  __syncwarp();
}

// Level l of pair p into the shared GLevel (thread 0).
__device__ void set_level(const GroupLaunch &a, GLevel &X, int p, int l) {
  const stb_level lv = a.levels[(size_t)p * a.L + l];
  const GroupLevelParams &q = a.lp[l];
  X.sp = lv.src_points;
  X.sn = lv.src_normals;
  X.sm = lv.src_mask;
  X.n = lv.num_source;
  X.sf = lv.src_feats;
  X.tp = lv.tgt_points;
  X.tn = lv.tgt_normals;
  X.tm = lv.tgt_mask;
  X.H = lv.height;
  X.W = lv.width;
  X.tf = lv.tgt_feats;
  X.use_geom = q.use_geom;
  X.use_feat = q.use_feat;
  X.wg1 = q.wg1;
  X.wg2 = q.wg2;
  X.wf1 = q.wf1;
  X.wf2 = q.wf2;
  X.thr2 = q.thr2;
  X.cos_max = q.cos_max;
  X.feat_thr2 = q.feat_thr2;
  X.keys = a.keys + a.key_off[p];
}

extern __shared__ __align__(16) float s_group_dyn[];

template <typename FT, bool kFeat, bool kHWC>
__global__ void __launch_bounds__(kPT, 1) k_group(const __grid_constant__ GroupLaunch a, int gs,
                                                  int cache_rounds) {
  __shared__ GLevel X;
  __shared__ PairLoop S;
  __shared__ int s_t;
  const int lane = threadIdx.x & 31;
  const int groups = gridDim.x / gs;
  const int g = blockIdx.x / gs;
  unsigned *err = a.sync + 2;
  const GridSync grid{a.sync, err, a.spin_limit, a.bar_phantom};

  // set-up (block 0): the pairs' key-map offsets (each pair's largest
  // level) and the queue order (decreasing size; equal sizes by index)
  if (blockIdx.x == 0) {
    for (int p = threadIdx.x; p < a.B; p += blockDim.x) {
      long long big = 0;
      for (int l = 0; l < a.L; ++l) {
        const stb_level &lv = a.levels[(size_t)p * a.L + l];
        big = max(big, (long long)lv.height * lv.width);
      }
      // (rounded up to an even count, as the lock-step kernel's maps)
      a.key_off[p + 1] = (big + 1) & ~1ll;  // sizes, summed below
    }
    __syncthreads();
    for (int p = threadIdx.x; p < a.B; p += blockDim.x) {
      const long long mine = a.key_off[p + 1];
      int rank = 0;
      for (int q = 0; q < a.B; ++q) {
        const long long other = a.key_off[q + 1];
        rank += other > mine || (other == mine && q < p);
      }
      a.order[rank] = p;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      long long acc = 0;
      a.key_off[0] = 0;
      for (int p = 0; p < a.B; ++p) {
        acc += a.key_off[p + 1];
        a.key_off[p + 1] = acc;
      }
      if (acc > a.keys_cap) atomicOr(err, 2u);
    }
  }
  // every pair's result block starts empty (a pair whose group never runs,
  // as after a timeout, still has a defined block for the status pass)
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
       k < (long long)a.B * STB_RES_SIZE; k += (long long)gridDim.x * blockDim.x)
    a.results[k] = (k % STB_RES_SIZE == STB_RES_RESIDUAL) ? INFINITY : 0.0;
  if (!group_barrier(grid, 0, true) || ld_relaxed(err)) return;
  if (g >= groups) return;  // blocks past the last whole group stay idle

  if (threadIdx.x == 0) {
    X.C = a.C;
    X.channel_mode = a.mode;
    X.part = a.part + (size_t)(g * gs) * 2 * kSlotAccs;
    X.bar = a.sync + kGroupWords + 32 * g;
    X.err = err;
    X.spin_limit = a.spin_limit;
    X.bar_phantom = a.bar_phantom;
    X.rank = blockIdx.x - g * gs;
    X.size = gs;
  }
  __syncthreads();
  SrcCache C;
  C.cap = cache_rounds * kPR * kPT;
  C.f = s_group_dyn;
  C.m = reinterpret_cast<uint8_t *>(C.f + 6 * C.cap);
  unsigned nbar = 0;
  bool alive = true;

  for (;;) {
    // the next pair of the queue, taken by the group's rank 0 and
    // published by the barrier
    if (X.rank == 0 && threadIdx.x == 0)
      st_relaxed_u32(X.bar + 1, atomicAdd(a.sync + 3, 1u));
    if (!(alive = group_barrier(X, nbar++, true))) break;
    if (threadIdx.x == 0) s_t = (int)ld_relaxed(X.bar + 1);
    __syncthreads();
    const int t = s_t;
    if (t >= a.B) break;
    const int p = a.order[t];

    // the pair's state, key map cleared, own slots poisoned
    if (threadIdx.x < 32) {
      if (lane < 16) {
        S.L.Td[lane] = a.init ? a.init[(size_t)p * 16 + lane] : ((lane % 5) == 0 ? 1.0 : 0.0);
      }
      if (lane == 0) {
        S.p = p;
        S.stopped = 0;
        S.level_iters = 0;
        S.last_r2 = 0.0;
        S.last_count = 0.0;
        S.L.status = 0;
      }
    }
    {
      unsigned long long *keys = a.keys + a.key_off[p];
      const long long nk = a.key_off[p + 1] - a.key_off[p];
      for (long long k = (long long)X.rank * kPT + threadIdx.x; k < nk;
           k += (long long)gs * kPT)
        keys[k] = ~0ull;
    }
    poison_slot(X, 0);
    poison_slot(X, 1);
    if (!(alive = group_barrier(X, nbar++, true))) break;

    int s = 0;     // iterations of the pair so far (history row, epoch)
    int used = 0;  // iterations that ran (slot buffer parity)
    for (int l = 0; l < a.L && alive; ++l) {
      // level start: the pose carries over, identity when the previous
      // level's first iteration failed (multiscale.py:52-60)
      if (threadIdx.x == 0) set_level(a, X, p, l);
      __syncthreads();
      if (threadIdx.x < 32) {
        const stb_level &lv = a.levels[(size_t)p * a.L + l];
        if (lane < 16 && l > 0 && S.level_iters == 0)
          S.L.Td[lane] = (lane % 5) == 0 ? 1.0 : 0.0;
        __syncwarp();
        if (lane == 0) {
          S.stopped = 0;
          S.level_iters = 0;
          S.last_r2 = 0.0;
          S.last_count = 0.0;
          S.L.P.fx = lv.fx;
          S.L.P.fy = lv.fy;
          S.L.P.cx = lv.cx;
          S.L.P.cy = lv.cy;
          if (X.rank == 0) {
            double *R = a.results + (size_t)p * STB_RES_SIZE;
            R[STB_RES_ITERS] = 0.0;
            R[STB_RES_RESIDUAL] = INFINITY;
          }
        }
        __syncwarp();
        refresh_view(S.L, false, lane);
      }
      const Share src = share_of(X.n, X.rank, gs);
      const Share tgt = share_of((long long)X.H * X.W, X.rank, gs);
      C.rounds = min(cache_rounds, src.rounds);
      for (int r = 0; r < C.rounds; ++r) {
#pragma unroll
        for (int k = 0; k < kPR; ++k) {
          const long long i = unit_of(r, k, X.rank, gs);
          const int c = cache_index(r, k);
          const bool in = i < X.n;
          C.m[c] = in ? __ldg(X.sm + i) : (uint8_t)0;
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            C.f[d * C.cap + c] = in ? __ldg(X.sp + 3 * i + d) : 0.f;
            C.f[(3 + d) * C.cap + c] = in ? __ldg(X.sn + 3 * i + d) : 0.f;
          }
        }
      }
      __syncthreads();
      const int iters = a.lp[l].iters;
      for (int it = 0; it < iters; ++it, ++s) {
        if (S.stopped) continue;  // the same in every block of the group
        associate(X, S.L.P, src, C, s);
        if (!(alive = group_barrier(X, nbar++, true))) break;
        float acc[kAccs];
#pragma unroll
        for (int k = 0; k < kAccs; ++k) acc[k] = 0.f;
        if (X.use_geom)
          reduce_pixels<FT, true, kFeat, kHWC>(X, S.L.P, tgt, s, acc);
        else
          reduce_pixels<FT, false, kFeat, kHWC>(X, S.L.P, tgt, s, acc);
        if (used > 0) poison_slot(X, (used + 1) & 1);
        write_slot<kAccs>(X, acc, used & 1);
        if (!(alive = fold_slots<kAccs>(X, S.L, used & 1, true))) break;
        ++used;
        if (threadIdx.x < 32) group_step(a, X, S, s, lane);
        __syncthreads();
      }
    }
    if (!alive) break;

    // the information matrix at the final pose (finest level, whose
    // GLevel is still set)
    const Share src = share_of(X.n, X.rank, gs);
    const Share tgt = share_of((long long)X.H * X.W, X.rank, gs);
    associate(X, S.L.P, src, C, s);
    if (!(alive = group_barrier(X, nbar++, true))) break;
    float acc[kInfoAccs];
#pragma unroll
    for (int k = 0; k < kInfoAccs; ++k) acc[k] = 0.f;
    info_pixels(X, tgt, s, acc);
    // (buffer `used & 1`: its last reader folded it before the barrier
    // above, and the next pair poisons both buffers after its first one)
    write_slot<kInfoAccs>(X, acc, used & 1);
    // (every block waits: an arrival that does not wait would let a block
    // reach the next barrier before the others reached this one, and the
    // arrival counter cannot tell the two barriers' arrivals apart)
    if (!(alive = group_barrier(X, nbar++, true))) break;
    if (X.rank == 0) {
      fold_slots<kInfoAccs>(X, S.L, used & 1, false);
      double *R = a.results + (size_t)p * STB_RES_SIZE;
      for (int k = threadIdx.x; k < 36; k += blockDim.x) {
        const int r = k / 6, c = k % 6;
        R[STB_RES_INFO + k] = S.L.tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
      }
      if (threadIdx.x == 0)
        R[STB_RES_RESIDUAL] = S.last_count > 0.0 ? S.last_r2 / S.last_count : INFINITY;
    }
    __syncthreads();
  }
}

// Flags every pair's status when the kernel stopped early (error word bit
// 0: a bounded wait gave up; bit 1: the workspace holds fewer key-map
// entries than the pairs need).
__global__ void k_group_status(const unsigned *sync, double *results, int B) {
  const unsigned err = *(volatile const unsigned *)(sync + 2);
  if (!err) return;
  const unsigned bits = ((err & 1u) ? STB_ST_TIMEOUT : 0u) | ((err & 2u) ? STB_ST_CAPACITY : 0u);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < B; p += gridDim.x * blockDim.x)
    results[(size_t)p * STB_RES_SIZE + STB_RES_STATUS] =
        (double)((unsigned)results[(size_t)p * STB_RES_SIZE + STB_RES_STATUS] | bits);
}

constexpr size_t group_cache_smem(int rounds) {
  return ((size_t)rounds * kPR * kPT * kCachePointBytes + 15) & ~size_t(15);
}

template <typename FT, bool kFeat, bool kHWC>
int launch_group_kernel(const GroupLaunch &g, cudaStream_t st) {
  auto kern = k_group<FT, kFeat, kHWC>;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return check_launch("stb_icp_estimate_batch (grouped kernel set-up)");
  const size_t max_smem = group_cache_smem(kMaxCacheRounds);
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPT, max_smem) !=
          cudaSuccess)
    return check_launch("stb_icp_estimate_batch (grouped kernel set-up)");
  if (per_sm < 1)
    return fail(STB_ECUDA, "Cuda call error stb_icp_estimate_batch: the grouped kernel does "
                "not fit an SM");
  int grid = sms < kGroupMaxBlocks ? sms : kGroupMaxBlocks;
  const int groups = g.groups < grid ? g.groups : grid;
  const int gs = grid / groups;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kPT);
  cfg.dynamicSmemBytes = max_smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t err = cudaLaunchKernelEx(&cfg, kern, g, gs, (int)kMaxCacheRounds);
  if (err != cudaSuccess)
    return fail(STB_ECUDA, "Cuda call error stb_icp_estimate_batch (grouped kernel): %s",
                cudaGetErrorString(err));
  k_group_status<<<(g.B + 255) / 256, 256, 0, st>>>(g.sync, g.results, g.B);
  return check_launch("stb_icp_estimate_batch");
}

}  // namespace

int launch_grouped(const GroupLaunch &g, cudaStream_t st) {
  if (g.groups < 1 || g.groups > kMaxGroups)
    return fail(STB_EINVAL, "Check failed: groups must be in [1, %d], got %d", kMaxGroups,
                g.groups);
  if (g.C == 0) return launch_group_kernel<float, false, false>(g, st);
  switch (g.dtype) {
    case STB_F32: return launch_group_kernel<float, true, false>(g, st);
    case STB_BF16: return launch_group_kernel<__nv_bfloat16, true, false>(g, st);
    case STB_F32_HWC: return launch_group_kernel<float, true, true>(g, st);
    default: return launch_group_kernel<__nv_bfloat16, true, true>(g, st);
  }
}

}  // namespace fused
}  // namespace stb
