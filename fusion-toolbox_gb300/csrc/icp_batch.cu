// Batched multiscale ICP in one persistent cooperative kernel.
//
// All frame pairs run the same schedule (levels coarsest first, each level's
// Gauss-Newton iterations), so the whole batch advances in lock step through
// phases separated by grid barriers:
//
//   A  association   -- work list of source tiles over all pairs; one
//                       thread per source point, float32 gates in the
//                       reference's operation order, 64-bit atomicMin of
//                       (epoch tag, distance, index) into the pair's key map
//   B  reduction     -- work list of target tiles over all pairs; one thread
//                       per target pixel, residuals and Jacobians summed in
//                       compensated float32 into a per-tile partial; the last
//                       tile of a group of 32 folds the group, the last group
//                       of a pair folds the pair and its warp 0 runs the FP64
//                       Cholesky solve, SE(3) exponential and pose update
//
// After the last level, one more association at the final pose feeds the
// information-matrix reduction.  Barriers spin with a bound; a barrier that
// waits too long flags STB_ST_TIMEOUT and every block returns.
//
// Reference: MultiscaleRegistration.estimate_frame
// (slamtb/registration/multiscale.py:30-67) over ICPOdometry.estimate
// (slamtb/registration/icp.py:152-262) for each pair.
#include <math.h>

#include "feature_term.cuh"
#include "gn_solve.cuh"
#include "group_launch.hpp"
#include "keymap.cuh"
#include "stb_common.cuh"
#include "stb_host.hpp"

namespace stb {

float distance_thresh_sq(double d);
float angle_cos_max(double angle);

namespace {

constexpr int kThreads = 256;
constexpr int kMaxLevels = 4;
constexpr int kGroup = 32;            // tiles per first-level reduction group
constexpr int kAccsB = 30;            // 21 JtJ + 6 Jr + r2 + count_geom + count_feat
constexpr int kSlotFloats = 64;       // (s[32], c[32]) per partial slot
constexpr int kMinTile = kThreads * 2;
constexpr unsigned kSpinLimit = 1u << 26;  // x >= 32 ns sleeps: a few seconds
constexpr int kJrB = 21, kR2B = 27, kCountGeomB = 28, kCountFeatB = 29;
// barrier words: [0] root arrivals, [1] generation, [2] error, [4] and [5]
// the tile counters of alternating phases, [8 + g] the arrivals of group g
// (room for 4088 groups of 8 blocks)
constexpr size_t kSyncBytes = 16384;

struct LevelP {
  int iters, use_geom, use_feat;
  float wg1, wg2, wf1, wf2, thr2, cos_max, feat_thr2;
};

struct PairState {
  double T[16];
  Pose32 pose;
  double last_r2, last_count;  // of the level's last successful step
  unsigned stopped, status;
  int level_iters, iters_done;
};

struct BatchArgs {
  const stb_level *levels;
  int B, L, C, dtype, mode, total_iters;
  int tile;          // largest pixels per work item (a multiple of kMinTile)
  int *level_tile;   // [kMaxLevels] pixels per work item of each level
  LevelP lp[kMaxLevels];
  const double *init;
  double *results, *history;
  int solve_dw;    // 1: double-word solve (STB_OPT_DW_SOLVE), 0: FP64
  unsigned spin_limit, bar_phantom;  // grid barriers' bounded waits
  unsigned *sync;  // [0] arrivals, [1] generation, [2] error
  PairState *ps;
  long long *key_off;   // [B + 1]
  long long *src_off;   // [L][B + 1] source tiles
  long long *tgt_off;   // [L][B + 1] target tiles
  long long *grp_off;   // [L][B + 1] groups
  unsigned *grp_ticket, *pair_ticket;
  float *tile_part, *grp_part;
  unsigned long long *keys;
  long long keys_cap, tiles_cap, groups_cap;
  int off_cap;  // offset-row entries staged in shared memory (0: read from L2)
};

__host__ __device__ inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

struct Layout {
  size_t sync, level_tile, ps, key_off, src_off, tgt_off, grp_off, grp_ticket, pair_ticket, tile_part,
      grp_part, order, gpart, keys, total;
  long long tiles_cap, groups_cap;
};

inline Layout layout(int B, long long total_pixels) {
  Layout l;
  l.tiles_cap = total_pixels / kMinTile + B;
  l.groups_cap = l.tiles_cap / kGroup + B;
  size_t o = 0;
  l.sync = o;
  o += kSyncBytes;
  l.level_tile = o;
  o += 256;
  l.ps = o;
  o += al256(sizeof(PairState) * (size_t)B);
  l.key_off = o;
  o += al256(sizeof(long long) * (B + 1));
  l.src_off = o;
  o += al256(sizeof(long long) * kMaxLevels * (B + 1));
  l.tgt_off = o;
  o += al256(sizeof(long long) * kMaxLevels * (B + 1));
  l.grp_off = o;
  o += al256(sizeof(long long) * kMaxLevels * (B + 1));
  l.grp_ticket = o;
  o += al256(sizeof(unsigned) * (size_t)l.groups_cap);
  l.pair_ticket = o;
  o += al256(sizeof(unsigned) * (size_t)B);
  l.tile_part = o;
  o += al256(sizeof(float) * kSlotFloats * (size_t)l.tiles_cap);
  l.grp_part = o;
  o += al256(sizeof(float) * kSlotFloats * (size_t)l.groups_cap);
  // the grouped kernel: its pair queue and its groups' slot buffers
  l.order = o;
  o += al256(sizeof(int) * (size_t)B);
  l.gpart = o;
  o += al256(sizeof(float2) * 2 * 32 * (size_t)fused::kGroupMaxBlocks);
  l.keys = o;
  // one key per pixel of each pair's largest level, each pair's map rounded
  // up to an even count so that it starts on a 16-byte boundary (bulk copies)
  o += al256(sizeof(unsigned long long) * (size_t)(total_pixels + B));
  l.total = o;
  return l;
}

// ---------------------------------------------------------------------------
// grid barrier with a bounded wait
// ---------------------------------------------------------------------------
// Arrivals are counted in two levels (groups of kBarGroup blocks, then the
// groups) so that no counter takes more than a few dozen atomics; the last
// arrival bumps the generation word that the others poll.
constexpr int kBarGroup = 8;

// spin_limit: polls before a wait gives up; phantom: arrivals expected
// beyond the grid's (0; a test sets more so that the waits run out).
__device__ bool grid_sync(unsigned *sync, unsigned spin_limit, unsigned phantom) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *vgen = sync + 1;
    volatile unsigned *verr = sync + 2;
    unsigned *root = sync;
    unsigned *group = sync + 8 + blockIdx.x / kBarGroup;
    const unsigned ngroups = (gridDim.x + kBarGroup - 1) / kBarGroup;
    const unsigned gsize = min((unsigned)kBarGroup, gridDim.x - (blockIdx.x / kBarGroup) * kBarGroup);
    const unsigned gen = *vgen;
    __threadfence();
    bool last = false;
    if (atomicAdd(group, 1u) == gsize - 1) {
      atomicExch(group, 0u);
      __threadfence();
      if (atomicAdd(root, 1u) == ngroups - 1 + phantom) {
        atomicExch(root, 0u);
        __threadfence();
        atomicAdd(sync + 1, 1u);
        last = true;
      }
    }
    if (!last) {
      unsigned spins = 0;
      while (*vgen == gen) {
        if (*verr) break;
        if (++spins > spin_limit) {
          atomicOr(sync + 2, 1u);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    s_ok = (*verr == 0);
  }
  __syncthreads();
  return s_ok;
}

// Dynamic tile scheduling.  A block's first tile of a phase is its block
// index; later ones are handed out by an atomic counter (sync[4 + (phase &
// 1)], offset by the grid size) rather than by a fixed stride, so a block
// whose tiles finish early takes more.  With the fixed stride, blocks spent
// about a seventh of the 256-pair run waiting at the phases' grid barriers
// for the slowest block.  Thread 0 fetches the next index while the block
// works on the current tile, so a phase with at most one tile per block (a
// single pair) pays no fetch latency.  Block 0 zeroes the other counter at
// the start of a phase: its last user ended at the previous grid barrier,
// and its next user starts after the next one.  The fetched index alternates
// between two shared words: a word is rewritten two tiles later, after a
// barrier that every thread passes only once it has read it.
template <typename F>
__device__ __forceinline__ void for_each_tile(unsigned *sync, int phase, long long ntiles, F f) {
  __shared__ unsigned s_next[2];
  unsigned *ctr = sync + 4 + (phase & 1);
  if (blockIdx.x == 0 && threadIdx.x == 0) sync[4 + ((phase + 1) & 1)] = 0u;
  long long t = blockIdx.x;
  for (int i = 0; t < ntiles; i ^= 1) {
    if (threadIdx.x == 0) s_next[i] = gridDim.x + atomicAdd(ctr, 1u);
    f(t);
    __syncthreads();
    t = s_next[i];
  }
}

// An offset row (B + 1 entries) is staged in the dynamic shared memory after
// the two stages when the launch has room for it without losing a block per
// SM (a.off_cap >= B + 1, decided on the host); otherwise it is read from L2.

// Entry k of an offset row: a shared-memory load when the row was staged,
// an L2 load (coherent with other blocks' writes) when it was not.
__device__ __forceinline__ long long off_at(const long long *off, const BatchArgs &a,
                                            long long k) {
  return (a.B + 1 <= a.off_cap) ? off[k] : __ldcg(off + k);
}

// Pair owning work item t: off[lo] <= t < off[lo + 1].
__device__ __forceinline__ int find_pair(const long long *off, const BatchArgs &a, long long t) {
  int lo = 0, hi = a.B;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off_at(off, a, mid) <= t)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Copies one level's offset row to shared memory (when it fits) and returns
// the array the phase should search.
__device__ __forceinline__ const long long *stage_offsets(const long long *row,
                                                          const BatchArgs &a, long long *smem) {
  __syncthreads();
  if (a.B + 1 > a.off_cap) return row;
  for (int k = threadIdx.x; k <= a.B; k += blockDim.x) smem[k] = __ldcg(row + k);
  __syncthreads();
  return smem;
}

__device__ __forceinline__ unsigned btag(int s) { return 254u - (unsigned)s; }

// Block-wide exclusive scans of the per-pair tile counts (block 0).
__device__ void build_offsets(const BatchArgs &a) {
  __shared__ long long carry[5];
  __shared__ long long warp_sum[kThreads / 32][5];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ long long s_lvl_px;
  __shared__ int s_tile;
  for (int l = 0; l < a.L; ++l) {
    // this level's work-item size: the largest power of two (at most a.tile,
    // at least kMinTile) that still gives every other block an item per phase
    if (threadIdx.x == 0) s_lvl_px = 0;
    __syncthreads();
    long long mine = 0;
    for (int p = threadIdx.x; p < a.B; p += kThreads) {
      const stb_level lv = a.levels[(size_t)p * a.L + l];
      mine += (long long)lv.height * lv.width;
    }
    atomicAdd((unsigned long long *)&s_lvl_px, (unsigned long long)mine);
    __syncthreads();
    if (threadIdx.x == 0) {
      int tile = a.tile;
      while (tile > kMinTile && s_lvl_px / tile < (long long)(gridDim.x / 2)) tile >>= 1;
      s_tile = tile;
      a.level_tile[l] = tile;
    }
    if (threadIdx.x < 5) carry[threadIdx.x] = 0;
    __syncthreads();
    const int tile = s_tile;
    for (int base = 0; base < a.B; base += kThreads) {
      const int p = base + threadIdx.x;
      long long v[4] = {0, 0, 0, 0};
      if (p < a.B) {
        const stb_level lv = a.levels[(size_t)p * a.L + l];
        const long long npix = (long long)lv.height * lv.width;
        const long long tt = (npix + tile - 1) / tile;
        v[0] = (lv.num_source + tile - 1) / tile;  // source tiles
        v[1] = tt;                                         // target tiles
        v[2] = (tt + kGroup - 1) / kGroup;                 // groups
        if (l == a.L - 1) {  // key map: the pair's largest level
          long long m = 0;
          for (int k = 0; k < a.L; ++k) {
            const stb_level lk = a.levels[(size_t)p * a.L + k];
            m = max(m, (long long)lk.height * lk.width);
          }
          v[3] = (m + 1) & ~1ll;  // even: 16-byte aligned maps
        }
      }
      // inclusive warp scans
      long long inc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        inc[q] = v[q];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const long long n = __shfl_up_sync(0xffffffffu, inc[q], off);
          if (lane >= off) inc[q] += n;
        }
      }
      if (lane == 31)
        for (int q = 0; q < 4; ++q) warp_sum[warp][q] = inc[q];
      __syncthreads();
      if (p < a.B) {
        long long pre[4];
        for (int q = 0; q < 4; ++q) {
          pre[q] = carry[q] + inc[q] - v[q];
          for (int w = 0; w < warp; ++w) pre[q] += warp_sum[w][q];
        }
        const size_t row = (size_t)l * (a.B + 1);
        a.src_off[row + p] = pre[0];
        a.tgt_off[row + p] = pre[1];
        a.grp_off[row + p] = pre[2];
        if (l == a.L - 1) a.key_off[p] = pre[3];
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int q = 0; q < 4; ++q) {
          long long tot = 0;
          for (int w = 0; w < kThreads / 32; ++w) tot += warp_sum[w][q];
          carry[q] += tot;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const size_t row = (size_t)l * (a.B + 1);
      a.src_off[row + a.B] = carry[0];
      a.tgt_off[row + a.B] = carry[1];
      a.grp_off[row + a.B] = carry[2];
      if (l == a.L - 1) a.key_off[a.B] = carry[3];
      if (carry[1] > a.tiles_cap || carry[2] > a.groups_cap ||
          (l == a.L - 1 && carry[3] > a.keys_cap))
        atomicOr(a.sync + 2, 2u);
    }
    __syncthreads();
  }
}


// Per-thread partial sums are plain float32: a thread adds at most
// tile / 256 <= 16 pixels, so its rounding error stays below ~1e-6 of the
// sum of magnitudes; compensation (TwoSum) starts at the warp level.
template <typename Acc>
__device__ __forceinline__ void acc_se3(Acc acc, const float *Jv, float r, float w1,
                                        float w2) {
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = a; b < 6; ++b) acc[upper_index(a, b)] += w2 * (Jv[a] * Jv[b]);
#pragma unroll
  for (int a = 0; a < 6; ++a) acc[kJrB + a] += w1 * (Jv[a] * r);
}

// Dynamic shared memory of the kernel: two staging buffers, then the staged
// offset row, then (kernels with a feature term) the per-thread
// accumulators of the reduction.  Between a tile's pipeline and the next tile's first copy the
// staging buffers are idle: the block sum and the slot folds of the tile's
// epilogue use their first bytes as scratch.
extern __shared__ __align__(128) unsigned char s_stage[];

// block reduction of kN accumulators into smem out_s/out_c (threads < kN)
template <int kN, typename Acc>
__device__ __forceinline__ void block_sum(Acc acc_in, float *out_s, float *out_c) {
  float(*ws)[kN][2] = reinterpret_cast<float(*)[kN][2]>(s_stage);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < kN; ++a) {
    CSum acc = {acc_in[a], 0.f};
    csum_warp_reduce(acc);
    if (lane == 0) {
      ws[warp][a][0] = acc.s;
      ws[warp][a][1] = acc.c;
    }
  }
  __syncthreads();
  if (threadIdx.x < kN) {
    CSum t = {0.f, 0.f};
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w)
      csum_merge(t, ws[w][threadIdx.x][0], ws[w][threadIdx.x][1]);
    out_s[threadIdx.x] = t.s;
    out_c[threadIdx.x] = t.c;
  }
  __syncthreads();
}

// Fold `count` partial slots (kN accumulators each) into out_s/out_c.  All
// loads are issued before the additions.
template <int kN>
__device__ __forceinline__ void fold_slots(const float *slots, int count, float *out_s,
                                           float *out_c) {
  float(*fs)[32][2] = reinterpret_cast<float(*)[32][2]>(s_stage + 2048);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // thread (warp w, lane a) sums slots w, w + 8, ... for accumulator a
  CSum t = {0.f, 0.f};
  if (lane < kN) {
    float vs[4], vc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int j = warp + k * (kThreads / 32);
      vs[k] = (j < count) ? __ldcg(slots + (size_t)j * kSlotFloats + lane) : 0.f;
      vc[k] = (j < count) ? __ldcg(slots + (size_t)j * kSlotFloats + 32 + lane) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) csum_merge(t, vs[k], vc[k]);
  }
  fs[warp][lane][0] = t.s;
  fs[warp][lane][1] = t.c;
  __syncthreads();
  if (threadIdx.x < kN) {
    CSum u = {0.f, 0.f};
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) csum_merge(u, fs[w][threadIdx.x][0], fs[w][threadIdx.x][1]);
    out_s[threadIdx.x] = u.s;
    out_c[threadIdx.x] = u.c;
  }
  __syncthreads();
}

__device__ __forceinline__ void load_pose(Pose32 &P, const PairState *ps) {
  const float *src = reinterpret_cast<const float *>(&ps->pose);
  float *dst = reinterpret_cast<float *>(&P);
  for (int k = threadIdx.x; k < (int)(sizeof(Pose32) / sizeof(float)); k += blockDim.x)
    dst[k] = __ldcg(src + k);
}

// Per-block cache of the pair a work item belongs to: consecutive work items
// of a block usually share the pair, so its descriptor and pose are loaded
// once per phase, not once per item.
struct TileCache {
  stb_level lv;
  Pose32 P;
  double T[16];  // the pair's FP64 pose (read by the pair's last block in its step)
  int p, skip;
};

__device__ __forceinline__ void reset_cache(TileCache &tc) {
  __syncthreads();
  if (threadIdx.x == 0) tc.p = -1;
  __syncthreads();
}

// Resolves work item t (thread 0), reloading descriptor and pose when the
// pair changes.  Returns the pair; tc.skip is uniform.
__device__ __forceinline__ int cache_pair(const BatchArgs &a, const long long *off, int level,
                                          long long t, bool check_stop, TileCache &tc) {
  __shared__ int s_new;
  // every thread is done with the previous work item before the cache and
  // the shared flags are rewritten
  __syncthreads();
  if (threadIdx.x == 0) {
    const int p = find_pair(off, a, t);
    s_new = (p != tc.p);
    if (s_new) {
      tc.p = p;
      tc.lv = a.levels[(size_t)p * a.L + level];
      tc.skip = check_stop && __ldcg(&a.ps[p].stopped);
    }
  }
  __syncthreads();
  if (s_new && !tc.skip) {
    load_pose(tc.P, a.ps + tc.p);
    if (threadIdx.x >= 32 && threadIdx.x < 48) tc.T[threadIdx.x - 32] = __ldcg(a.ps[tc.p].T + threadIdx.x - 32);
    __syncthreads();
  }
  return tc.p;
}

// ---------------------------------------------------------------------------
// phase A: association of one source tile
// ---------------------------------------------------------------------------
// Pixels per thread of a staged sub-chunk (kCh, a template parameter of
// the tile functions) and blocks per SM of the kernel, measured on GB300:
//   * geometric only: 3 blocks of 256 threads per SM (80 registers, 4-pixel
//     sub-chunks; two 32 KB stages per block fit three blocks' shared memory
//     because the epilogue scratch lives in the idle stages).  24 warps
//     instead of 16 hide more of the gathers' latency: the 256-pair run
//     took 27.9 ms, against 32.6 with 2 blocks and 29.5 with 3-pixel
//     sub-chunks (the run tracks the pixels in flight per SM).
//   * with a feature term: 2 blocks of 128 registers and 2-pixel sub-chunks.
//     Three blocks at 80 registers spill enough to lose (16 x 1080p: 264
//     pairs/s against 382); 2-pixel sub-chunks spill less than 4-pixel ones
//     (16 x 1080p: 409 pairs/s against 382).
template <bool kFeat>
struct BatchShape {
  static constexpr int kCh = kFeat ? 2 : 4;
  static constexpr int kBlocksPerSM = kFeat ? 2 : 3;
};

// ---------------------------------------------------------------------------
// Bulk-copy staging of a tile's contiguous streams.  A tile is walked in
// sub-chunks of kThreads * kCh pixels; each sub-chunk's streams (reduction: keys,
// target points, target normals; association: source points, normals,
// mask) are copied into one of two shared-memory stages by cp.async.bulk
// (issued by thread 0, completion counted on the stage's mbarrier) while the
// block computes on the other stage.  This keeps a stage per block in flight
// independently of occupancy; only the true gathers (winners' source points,
// projected target pixels, feature taps) remain per-thread loads.
// A stream whose base is not 16-byte aligned, and the bytes of a stream past
// its last 16-byte multiple, are copied by the threads with plain loads.
// ---------------------------------------------------------------------------
// a stage holds one sub-chunk of kThreads * kCh pixels at 32 bytes per pixel
// (keys 8 + xyz 12 + normal 12)
__host__ __device__ constexpr int stage_bytes(int kCh) { return kThreads * kCh * 32; }

struct StageCtl {
  unsigned long long bar[2];  // mbarriers of the two stages
  int failed;                 // a wait ran out: the block takes no further tiles
};

struct StageStream {
  void *dst;
  const void *src;
  unsigned bytes;
  unsigned elem;  // element size of the plain copy (1, 4 or 8)
};


// offset row bytes after the stages (B + 1 entries when staged), 16-aligned
__host__ __device__ inline int off_row_bytes(int off_cap) { return (8 * off_cap + 15) & ~15; }
constexpr int kAccSmemBytes = kAccsB * kThreads * 4;  // feature kernels' accumulators

template <int kCh>
__device__ __forceinline__ float *smem_acc(const BatchArgs &a) {
  return reinterpret_cast<float *>(s_stage + 2 * stage_bytes(kCh) + off_row_bytes(a.off_cap));
}

template <bool kSmem>
struct AccPick;
template <>
struct AccPick<false> {
  static __device__ __forceinline__ float *get(float *regs, float *) { return regs; }
};
template <>
struct AccPick<true> {
  static __device__ __forceinline__ StridedAcc<kThreads> get(float *, float *smem) {
    return {smem};
  }
};

template <int kCh>
__device__ __forceinline__ unsigned char *stage_buf(int st) {
  return s_stage + st * stage_bytes(kCh);
}

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void stage_init(StageCtl &ctl) {
  if (threadIdx.x == 0) {
    for (int k = 0; k < 2; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&ctl.bar[k])));
    ctl.failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// Copies the streams of one sub-chunk into stage st.  All threads call it
// (after a __syncthreads that ends every read of the stage).
// One 4-byte word global -> shared, asynchronously (waited by
// cp_async_wait_all in the same thread).
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

__device__ __forceinline__ void stage_issue(const StageStream *ss, int count, int st,
                                            StageCtl &ctl) {
  unsigned bulk[3];
  unsigned total = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    bulk[i] = 0;
    if (i < count) {
      const bool al = (((uintptr_t)ss[i].src | (uintptr_t)ss[i].dst) & 15) == 0;
      bulk[i] = al ? (ss[i].bytes & ~15u) : 0u;
      total += bulk[i];
    }
  }
  if (threadIdx.x == 0) {
    const unsigned bar = smem_addr(&ctl.bar[st]);
    // order the block's earlier generic reads of the stage, and the grid's
    // generic writes of the key map, before the async-proxy copies
    asm volatile("fence.proxy.async;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(total)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 3; ++i)
      if (i < count && bulk[i])
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
            "[%3];" ::"r"(smem_addr(ss[i].dst)),
            "l"(ss[i].src), "r"(bulk[i]), "r"(bar)
            : "memory");
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (i >= count) continue;
    const unsigned e = ss[i].elem;
    for (unsigned off = bulk[i] + threadIdx.x * e; off < ss[i].bytes; off += kThreads * e) {
      const char *src = static_cast<const char *>(ss[i].src) + off;
      char *dst = static_cast<char *>(ss[i].dst) + off;
      if (e == 8)
        *reinterpret_cast<unsigned long long *>(dst) =
            __ldcg(reinterpret_cast<const unsigned long long *>(src));
      else if (e == 4)
        *reinterpret_cast<float *>(dst) = __ldg(reinterpret_cast<const float *>(src));
      else
        *dst = *src;
    }
  }
}

// Bounded wait for stage st's copies.  ph holds this thread's expected
// parity of both stages (bit st) and flips on success; every thread waits,
// so every thread's ph stays the same.  False after the limit (error bit 4).
__device__ __forceinline__ bool stage_wait(int st, StageCtl &ctl, unsigned &ph, unsigned *err) {
  const unsigned bar = smem_addr(&ctl.bar[st]);
  const unsigned parity = (ph >> st) & 1u;
  for (unsigned spins = 0; spins <= kSpinLimit; ++spins) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) {
      ph ^= 1u << st;
      return true;
    }
    __nanosleep(32);
  }
  atomicOr(err, 4u);
  return false;
}

// Runs a tile of nsub sub-chunks: issue(c) stages sub-chunk c (all threads
// call it), compute(c, st) consumes stage st.  Sub-chunk c + 1 is in flight
// while c is computed.  After a wait that ran out, every thread (the
// decision is a block vote) waits once more, bounded, for the copies still in
// flight, marks the block failed and returns; grid barriers then see the
// error bit and end the kernel.
template <typename Issue, typename Compute>
__device__ __forceinline__ void stage_pipeline(int nsub, StageCtl &ctl, unsigned &ph,
                                               unsigned *err, Issue issue, Compute compute) {
  if (nsub <= 0 || ctl.failed) return;
  issue(0);
  if (nsub > 1) issue(1);
  bool ok = stage_wait(0, ctl, ph, err);
  for (int c = 0;; ++c) {
    if (__syncthreads_or(!ok)) {
      stage_wait(0, ctl, ph, err);
      if (nsub > 1) stage_wait(1, ctl, ph, err);
      if (threadIdx.x == 0) ctl.failed = 1;
      __syncthreads();
      return;
    }
    if (c > 0 && c + 1 < nsub) issue(c + 1);
    if (c >= nsub) return;
    const int st = c & 1;
    compute(c, st);
    ok = (c + 1 < nsub) ? stage_wait(st ^ 1, ctl, ph, err) : true;
  }
}

template <int kCh>
__device__ __forceinline__ void assoc_tile(const BatchArgs &a, const long long *off, int level,
                                           long long t, int s, bool force, TileCache &tc,
                                           StageCtl &ctl, unsigned &ph) {
  constexpr int kSub = kThreads * kCh;  // pixels of a staged sub-chunk
  const int p = cache_pair(a, off, level, t, !force, tc);
  if (tc.skip) return;
  const Pose32 &P = tc.P;
  const stb_level &lv = tc.lv;
  const long long lt = t - off_at(off, a, p);
  const LevelP &q = a.lp[level];
  const int H = lv.height, W = lv.width;
  unsigned long long *keys = a.keys + __ldcg(a.key_off + p);
  const unsigned long long tag = (unsigned long long)btag(s) << 56;
  const long long tile = __ldcg(a.level_tile + level);
  const long long start = lt * tile;
  const long long end = min((lt + 1) * tile, (long long)lv.num_source);
  const int nsub = start < end ? (int)((end - start + kSub - 1) / kSub) : 0;
  // stage layout: source xyz [kSub][3] | source normal [kSub][3] | mask [kSub]
  auto issue = [&](int c) {
    const long long b0 = start + (long long)c * kSub;
    const unsigned n = (unsigned)min((long long)kSub, end - b0);
    unsigned char *buf = stage_buf<kCh>(c & 1);
    const StageStream ss[3] = {{buf, lv.src_points + 3 * b0, 12u * n, 4},
                               {buf + kSub * 12, lv.src_normals + 3 * b0, 12u * n, 4},
                               {buf + kSub * 24, lv.src_mask + b0, n, 1}};
    stage_issue(ss, 3, c & 1, ctl);
  };
  auto compute = [&](int c, int st) {
    const long long b0 = start + (long long)c * kSub;
    const int n = (int)min((long long)kSub, end - b0);
    const float *sp = reinterpret_cast<const float *>(stage_buf<kCh>(st));
    const float *sn = sp + kSub * 3;
    const unsigned char *sm = stage_buf<kCh>(st) + kSub * 24;
    // pass 1: projection and target gathers
    float3 Tp[kCh];
    long long pix[kCh];
    bool ok[kCh];
    float qx[kCh], qy[kCh], qz[kCh], mx[kCh], my[kCh], mz[kCh];
#pragma unroll
    for (int k = 0; k < kCh; ++k) {
      const int j = k * kThreads + threadIdx.x;
      ok[k] = j < n && sm[j < n ? j : 0];
      const int jj = ok[k] ? j : 0;
      Tp[k] = transform_point(P.rt, sp[3 * jj], sp[3 * jj + 1], sp[3 * jj + 2]);
      float u, v;
      project(P, Tp[k], u, v);
      int ui = 0, vi = 0;
      ok[k] = ok[k] && round_in(u, W, ui) && round_in(v, H, vi);
      pix[k] = ok[k] ? (long long)vi * W + ui : 0;
      ok[k] = ok[k] && __ldg(lv.tgt_mask + pix[k]);
      qx[k] = __ldg(lv.tgt_points + 3 * pix[k]);
      qy[k] = __ldg(lv.tgt_points + 3 * pix[k] + 1);
      qz[k] = __ldg(lv.tgt_points + 3 * pix[k] + 2);
      mx[k] = __ldg(lv.tgt_normals + 3 * pix[k]);
      my[k] = __ldg(lv.tgt_normals + 3 * pix[k] + 1);
      mz[k] = __ldg(lv.tgt_normals + 3 * pix[k] + 2);
    }
    // pass 2: gates and the z-buffer
#pragma unroll
    for (int k = 0; k < kCh; ++k) {
      if (!ok[k]) continue;
      const int j = k * kThreads + threadIdx.x;
      const float dx = fsub(qx[k], Tp[k].x), dy = fsub(qy[k], Tp[k].y),
                  dz = fsub(qz[k], Tp[k].z);
      const float sq = dot3(dx, dy, dz, dx, dy, dz);
      if (sq > q.thr2) continue;
      const float3 Tn = transform_normal(P.nm, sn[3 * j], sn[3 * j + 1], sn[3 * j + 2]);
      if (normal_angle_rejects(Tn, mx[k], my[k], mz[k], q.cos_max)) continue;
      const float dist = __fsqrt_rn(sq);
      atomicMin(keys + pix[k], tag | ((unsigned long long)__float_as_uint(dist) << 24) |
                                   (unsigned long long)(b0 + j));
    }
  };
  stage_pipeline(nsub, ctl, ph, a.sync + 2, issue, compute);
}

// ---------------------------------------------------------------------------
// per-pair Gauss-Newton step by warp 0 (totals in smem)
// ---------------------------------------------------------------------------
__device__ void pair_step(const BatchArgs &a, int p, int level, int s, const double *tot,
                          const float2 *totw, const double *T) {
  const int lane = threadIdx.x & 31;
  PairState *ps = a.ps + p;
  const LevelP &q = a.lp[level];
  const double cg = tot[kCountGeomB], cf = tot[kCountFeatB];
  const double count = q.use_geom ? fmax(cg, cf) : cf;
  double *H = a.history ? a.history + ((size_t)p * a.total_iters + s) * STB_HIST_SIZE : nullptr;
  // the solve: FP64 (default) or double-words (STB_OPT_DW_SOLVE)
  double xs[6];
  double tn;
  bool ok;
  if (a.solve_dw) {
    __shared__ float2 s_tw[16];
    if (lane < 16) s_tw[lane] = dw_of_double(T[lane]);
    __syncwarp();
    float2 tnw;
    float xf[6];
    ok = warp_gn_update_dw(totw, totw + kJrB, s_tw, xf, tnw, lane);
    tn = (double)tnw.x + (double)tnw.y;
    for (int k = 0; k < 6; ++k) xs[k] = xf[k];
  } else {
    ok = warp_gn_update(tot, tot + kJrB, T, xs, tn, lane);
  }
  double *R = a.results + (size_t)p * STB_RES_SIZE;
  for (int k = lane; k < 36; k += 32) {
    const int r = k / 6, c = k % 6;
    const double v = tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
    if (H) H[STB_HIST_JTJ + k] = v;
    if (ok) R[STB_RES_JTJ + k] = v;
  }
  if (H && lane < 6) H[STB_HIST_JR + lane] = tot[kJrB + lane];
  if (H && lane == 0) {
    H[STB_HIST_R2] = tot[kR2B];
    H[STB_HIST_GEOM_COUNT] = cg;
    H[STB_HIST_FEAT_COUNT] = cf;
  }
  if (!ok) {
    if (lane == 0) {
      unsigned st = __ldcg(&ps->status) | STB_ST_NOT_PD;
      if (count == 0.0) st |= STB_ST_NO_MATCHES;
      ps->status = st;
      ps->stopped = 1;
      R[STB_RES_STATUS] = (double)st;
      if (H) H[STB_HIST_OK] = 0.0;
    }
    return;
  }
  __shared__ float rt32[12];
  if (lane < 12) {
    rt32[lane] = __double2float_rn(tn);
    ps->pose.rt[lane] = rt32[lane];
  }
  if (lane < 16) {
    ps->T[lane] = tn;
    R[STB_RES_TRANSFORM + lane] = tn;
    if (H) H[STB_HIST_TRANSFORM + lane] = tn;
  }
  __syncwarp();
  if (lane == 0) {
    unsigned st = __ldcg(&ps->status);
    bool finite = true;
    for (int k = 0; k < 6; ++k) finite &= isfinite(xs[k]);
    if (!finite) st |= STB_ST_NAN;
    if (count == 0.0) st |= STB_ST_NO_MATCHES;
    ps->status = st;
    float nm[9];
    inverse_transpose(rt32, nm);
    for (int k = 0; k < 9; ++k) ps->pose.nm[k] = nm[k];
    const int li = __ldcg(&ps->level_iters) + 1;
    ps->level_iters = li;
    ps->iters_done = __ldcg(&ps->iters_done) + 1;
    ps->last_r2 = tot[kR2B];
    ps->last_count = count;
    R[STB_RES_MATCHES] = count;
    R[STB_RES_ITERS] = (double)li;
    R[STB_RES_STATUS] = (double)st;
    if (H) H[STB_HIST_OK] = 1.0;
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// phase B: reduction of one target tile (+ group / pair folds and the step)
// ---------------------------------------------------------------------------
// match_list: the block's per-warp lists of matched pixels (kThreads / 32
// lists of kCh x 32 entries, shared memory)
template <typename FT, bool kFeat, bool kInfo, bool kHWC, int kCh>
__device__ __forceinline__ void reduce_tile(unsigned *match_list, const BatchArgs &a,
                                            const long long *off, int level,
                                            long long t, int s, TileCache &tc, StageCtl &ctl,
                                            unsigned &ph) {
  constexpr int kN = kInfo ? 21 : kAccsB;
  constexpr int kSub = kThreads * kCh;  // pixels of a staged sub-chunk
  __shared__ int s_last;
  __shared__ float bs[32], bc[32];
  __shared__ double tot[32];
  __shared__ float2 totw[32];
  static_assert(kCh <= 4, "the match list packs the slot in two bits");
  const int p = cache_pair(a, off, level, t, !kInfo, tc);
  if (tc.skip) return;
  const Pose32 &P = tc.P;
  const stb_level &lv = tc.lv;
  const size_t row = (size_t)level * (a.B + 1);
  const long long t0 = off_at(off, a, p);
  const long long ntiles = off_at(off, a, p + 1) - t0;
  const long long lt = t - t0;
  const LevelP &q = a.lp[level];
  const int H = lv.height, W = lv.width;
  const long long npix = (long long)H * W;
  const unsigned long long *keys = a.keys + __ldcg(a.key_off + p);
  const unsigned tag = btag(s);

  // With a feature term the 30 accumulators live in shared memory (their
  // registers would spill at this kernel's 128); otherwise in registers.
  constexpr bool kSmemAcc = kFeat && !kInfo;
  float acc_r[kSmemAcc ? 1 : kN];
  const auto acc = AccPick<kSmemAcc>::get(acc_r, smem_acc<kCh>(a) + threadIdx.x);
#pragma unroll
  for (int k = 0; k < kN; ++k) acc[k] = 0.f;

  const long long tile = __ldcg(a.level_tile + level);
  const long long start = lt * tile;
  const long long end = min((lt + 1) * tile, npix);
  const int nsub = start < end ? (int)((end - start + kSub - 1) / kSub) : 0;
  const bool need_n = !kInfo && q.use_geom;
  // stage layout: keys [kSub] | target xyz [kSub][3] | target normal [kSub][3].
  // Only the keys are staged for every pixel; the target point and normal
  // of the (about one in ten) matched pixels are gathered into their slots
  // by the lanes that process them (cp.async, 4 bytes a word), so the
  // reduction reads 8 B per pixel plus ~2.4 B of targets instead of 32 B.
  auto issue = [&](int c) {
    const long long b0 = start + (long long)c * kSub;
    const unsigned n = (unsigned)min((long long)kSub, end - b0);
    unsigned char *buf = stage_buf<kCh>(c & 1);
    const StageStream ss[1] = {{buf, keys + b0, 8u * n, 8}};
    stage_issue(ss, 1, c & 1, ctl);
  };
  auto compute = [&](int c, int st) {
    const long long b0 = start + (long long)c * kSub;
    const int nn = (int)min((long long)kSub, end - b0);
    const unsigned long long *skeys = reinterpret_cast<const unsigned long long *>(stage_buf<kCh>(st));
    float *stq = reinterpret_cast<float *>(stage_buf<kCh>(st) + kSub * 8);
    float *stn = reinterpret_cast<float *>(stage_buf<kCh>(st) + kSub * 20);
    // pass 1: the warp's matched pixels of the sub-chunk packed into its
    // list in ballot order ((source index << 7) | (slot << 5) | lane), so
    // that the arithmetic below runs with full lanes (about one pixel in
    // ten matches); then each lane's entries' target points and normals
    // (into their stage slots) and source points, all issued before the
    // first use
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned *list = match_list + warp * (kCh * 32);
    int count = 0;
#pragma unroll
    for (int k = 0; k < kCh; ++k) {
      const int j = k * kThreads + threadIdx.x;
      const unsigned long long key = j < nn ? skeys[j] : 0ull;
      const bool m = (unsigned)(key >> 56) == tag;
      const unsigned bal = __ballot_sync(0xffffffffu, m);
      if (m)
        list[count + __popc(bal & ((1u << lane) - 1u))] =
            ((unsigned)(key & 0xffffffull) << 7) | ((unsigned)k << 5) | (unsigned)lane;
      count += __popc(bal);
    }
    __syncwarp();
    const int rounds = (count + 31) >> 5;  // warp-uniform, at most kCh
    int jj[kCh];
    long long ii[kCh];
    float spt[kCh][3];
#pragma unroll
    for (int k = 0; k < kCh; ++k) {
      if (k >= rounds) break;
      const int d = lane + 32 * k;
      const unsigned ent = d < count ? list[d] : 0u;
      jj[k] = d < count ? (int)((ent >> 5) & 3u) * kThreads + warp * 32 + (int)(ent & 31u) : -1;
      ii[k] = (long long)(ent >> 7);
      if (jj[k] >= 0) {
        const long long g = b0 + jj[k];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          cp_async4(stq + 3 * jj[k] + c, lv.tgt_points + 3 * g + c);
          if (need_n) cp_async4(stn + 3 * jj[k] + c, lv.tgt_normals + 3 * g + c);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c)
        spt[k][c] = kInfo ? 0.f : __ldg(lv.src_points + 3 * ii[k] + c);
    }
    cp_async_wait_all();  // this lane's gathers (each lane reads only its own)
    // pass 2: residuals, Jacobians and the per-thread sums
#pragma unroll
    for (int k = 0; k < kCh; ++k) {
      if (k >= rounds) break;
      if (jj[k] < 0) continue;
      const int j = jj[k];
      const float qx = stq[3 * j], qy = stq[3 * j + 1], qz = stq[3 * j + 2];
      if (kInfo) {
        const float G0[6] = {0.f, qz, -qy, 1.f, 0.f, 0.f};
        const float G1[6] = {-qz, 0.f, qx, 0.f, 1.f, 0.f};
        const float G2[6] = {qy, -qx, 0.f, 0.f, 0.f, 1.f};
  #pragma unroll
        for (int i = 0; i < 6; ++i)
  #pragma unroll
          for (int j = i; j < 6; ++j)
            acc[upper_index(i, j)] += G0[i] * G0[j] + G1[i] * G1[j] + G2[i] * G2[j];
        continue;
      }
      const long long i = ii[k];
      const float3 Tp = transform_point(P.rt, spt[k][0], spt[k][1], spt[k][2]);
      if (q.use_geom) {
        const float nx = stn[3 * j], ny = stn[3 * j + 1], nz = stn[3 * j + 2];
        const float r = dot3(fsub(qx, Tp.x), fsub(qy, Tp.y), fsub(qz, Tp.z), nx, ny, nz);
        const float Jv[6] = {nx, ny, nz, fsub(fmul(Tp.y, nz), fmul(Tp.z, ny)),
                             fsub(fmul(Tp.z, nx), fmul(Tp.x, nz)),
                             fsub(fmul(Tp.x, ny), fmul(Tp.y, nx))};
        acc_se3(acc, Jv, r, q.wg1, q.wg2);
        acc[kR2B] += q.wg1 * (r * r);
        acc[kCountGeomB] += 1.f;
      }
      if (kFeat && q.use_feat) {
        const FeatView<FT, kHWC> tf{static_cast<const FT *>(lv.tgt_feats), npix, a.C};
        const FeatView<FT, kHWC> sf{static_cast<const FT *>(lv.src_feats), lv.num_source, a.C};
        float sq;
        if (feature_term(tf, sf, i, P, Tp, H, W, q.feat_thr2, a.mode, q.wf1, q.wf2, acc, sq)) {
          acc[kR2B] += q.wf1 * sq;
          acc[kCountFeatB] += 1.f;
        }
      }
    }
    __syncwarp();  // the list is rewritten by the next sub-chunk
  };
  stage_pipeline(nsub, ctl, ph, a.sync + 2, issue, compute);

  block_sum<kN>(acc, bs, bc);
  float *slot = a.tile_part + (size_t)t * kSlotFloats;
  if (threadIdx.x < kN) {
    slot[threadIdx.x] = bs[threadIdx.x];
    slot[32 + threadIdx.x] = bc[threadIdx.x];
  }
  __threadfence();
  __syncthreads();
  const long long g_local = lt / kGroup;
  const long long g = __ldcg(a.grp_off + row + p) + g_local;
  const int gsize = (int)min((long long)kGroup, ntiles - g_local * kGroup);
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(a.grp_ticket + g, 1u);
    s_last = (prev == (unsigned)gsize - 1);
    if (s_last) a.grp_ticket[g] = 0;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  fold_slots<kN>(a.tile_part + (size_t)(t0 + g_local * kGroup) * kSlotFloats, gsize, bs, bc);
  float *gslot = a.grp_part + (size_t)g * kSlotFloats;
  if (threadIdx.x < kN) {
    gslot[threadIdx.x] = bs[threadIdx.x];
    gslot[32 + threadIdx.x] = bc[threadIdx.x];
  }
  __threadfence();
  __syncthreads();
  const long long ngroups = (ntiles + kGroup - 1) / kGroup;
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(a.pair_ticket + p, 1u);
    s_last = (prev == (unsigned)ngroups - 1);
    if (s_last) a.pair_ticket[p] = 0;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const long long g0 = __ldcg(a.grp_off + row + p);
  // a pair has at most 4 * 8 * kGroup tiles per fold_slots call; fold in
  // chunks of 32 groups
  CSum run[1];
  if (threadIdx.x < kN) run[0] = {0.f, 0.f};
  for (long long c0 = 0; c0 < ngroups; c0 += 32) {
    const int cnt = (int)min(32LL, ngroups - c0);
    fold_slots<kN>(a.grp_part + (size_t)(g0 + c0) * kSlotFloats, cnt, bs, bc);
    if (threadIdx.x < kN) csum_merge(run[0], bs[threadIdx.x], bc[threadIdx.x]);
  }
  if (threadIdx.x < kN) {
    tot[threadIdx.x] = (double)run[0].s + (double)run[0].c;
    totw[threadIdx.x] = dw_of_csum(run[0].s, run[0].c);
  }
  __syncthreads();
  if (kInfo) {
    double *R = a.results + (size_t)p * STB_RES_SIZE;
    for (int k = threadIdx.x; k < 36; k += blockDim.x) {
      const int r = k / 6, c = k % 6;
      R[STB_RES_INFO + k] = tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
    }
    if (threadIdx.x == 0) {
      // residual r2 / count of the finest level's last successful step (icp.py:251)
      const double n = __ldcg(&a.ps[p].last_count);
      R[STB_RES_RESIDUAL] = n > 0.0 ? __ldcg(&a.ps[p].last_r2) / n : INFINITY;
    }
  } else if (threadIdx.x < 32) {
    pair_step(a, p, level, s, tot, totw, tc.T);
  }
  __syncthreads();
}

template <typename FT, bool kFeat, bool kHWC>
__global__ void __launch_bounds__(kThreads, BatchShape<kFeat>::kBlocksPerSM)
    k_batch(const BatchArgs args) {
  constexpr int kCh = BatchShape<kFeat>::kCh;
  long long *s_off = reinterpret_cast<long long *>(s_stage + 2 * stage_bytes(kCh));
  // the argument block is staged in shared memory so that device functions
  // can take it by reference without a per-thread local copy
  __shared__ BatchArgs a;
  __shared__ TileCache tc;
  __shared__ StageCtl ctl;
  __shared__ unsigned s_match[(kThreads / 32) * kCh * 32];
  unsigned ph = 0;  // expected parities of the two staging barriers
  for (int k = threadIdx.x; k < (int)(sizeof(BatchArgs) / sizeof(int)); k += blockDim.x)
    reinterpret_cast<int *>(&a)[k] = reinterpret_cast<const int *>(&args)[k];
  stage_init(ctl);
  // phase 0: offsets (block 0), then pair states, key map, tickets
  if (blockIdx.x == 0) build_offsets(a);
  if (!grid_sync(a.sync, a.spin_limit, a.bar_phantom)) return;
  const long long gthreads = (long long)gridDim.x * blockDim.x;
  const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long p = gtid; p < a.B; p += gthreads) {
    PairState *ps = a.ps + p;
    for (int k = 0; k < 16; ++k)
      ps->T[k] = a.init ? a.init[p * 16 + k] : ((k % 5) == 0 ? 1.0 : 0.0);
    ps->stopped = 0;
    ps->status = 0;
    ps->level_iters = 0;
    ps->iters_done = 0;
    ps->last_r2 = 0.0;
    ps->last_count = 0.0;
    a.pair_ticket[p] = 0;
    double *R = a.results + p * STB_RES_SIZE;
    for (int k = 0; k < STB_RES_SIZE; ++k) R[k] = 0.0;
    R[STB_RES_RESIDUAL] = INFINITY;
  }
  const long long nkeys = __ldcg(a.key_off + a.B);
  for (long long k = gtid; k < nkeys; k += gthreads) a.keys[k] = ~0ull;
  for (long long k = gtid; k < a.groups_cap; k += gthreads) a.grp_ticket[k] = 0;
  if (!grid_sync(a.sync, a.spin_limit, a.bar_phantom)) return;

  int s = 0;
  int phase = 0;  // tile phases so far (selects the tile counter)
  for (int level = 0; level < a.L; ++level) {
    // level start: the reference's next estimator gets the previous result's
    // transform, None (identity) when that level's first iteration failed
    for (long long p = gtid; p < a.B; p += gthreads) {
      PairState *ps = a.ps + p;
      double T[16];
      const bool reset = level > 0 && __ldcg(&ps->level_iters) == 0;
      for (int k = 0; k < 16; ++k)
        T[k] = reset ? ((k % 5) == 0 ? 1.0 : 0.0) : __ldcg(ps->T + k);
      for (int k = 0; k < 16; ++k) ps->T[k] = T[k];
      ps->stopped = 0;
      ps->level_iters = 0;
      ps->last_r2 = 0.0;
      ps->last_count = 0.0;
      const stb_level lv = a.levels[p * a.L + level];
      Pose32 P;
      P.fx = lv.fx;
      P.fy = lv.fy;
      P.cx = lv.cx;
      P.cy = lv.cy;
      refresh_pose32(P, T);
      ps->pose = P;
      double *R = a.results + p * STB_RES_SIZE;
      R[STB_RES_ITERS] = 0.0;
      R[STB_RES_RESIDUAL] = INFINITY;
    }
    if (!grid_sync(a.sync, a.spin_limit, a.bar_phantom)) return;
    const size_t row = (size_t)level * (a.B + 1);
    const long long src_tiles = __ldcg(a.src_off + row + a.B);
    const long long tgt_tiles = __ldcg(a.tgt_off + row + a.B);
    for (int it = 0; it < a.lp[level].iters; ++it, ++s) {
      const long long *off = stage_offsets(a.src_off + row, a, s_off);
      reset_cache(tc);
      for_each_tile(a.sync, phase++, src_tiles, [&](long long t) {
        assoc_tile<kCh>(a, off, level, t, s, false, tc, ctl, ph);
      });
      if (!grid_sync(a.sync, a.spin_limit, a.bar_phantom)) return;
      off = stage_offsets(a.tgt_off + row, a, s_off);
      reset_cache(tc);
      for_each_tile(a.sync, phase++, tgt_tiles, [&](long long t) {
        reduce_tile<FT, kFeat, false, kHWC, kCh>(s_match, a, off, level, t, s, tc, ctl, ph);
      });
      if (!grid_sync(a.sync, a.spin_limit, a.bar_phantom)) return;
    }
  }
  // information matrix at the final pose (finest level)
  const int level = a.L - 1;
  const size_t row = (size_t)level * (a.B + 1);
  const long long src_tiles = __ldcg(a.src_off + row + a.B);
  const long long tgt_tiles = __ldcg(a.tgt_off + row + a.B);
  const long long *off = stage_offsets(a.src_off + row, a, s_off);
  reset_cache(tc);
  for_each_tile(a.sync, phase++, src_tiles, [&](long long t) {
    assoc_tile<kCh>(a, off, level, t, s, true, tc, ctl, ph);
  });
  if (!grid_sync(a.sync, a.spin_limit, a.bar_phantom)) return;
  off = stage_offsets(a.tgt_off + row, a, s_off);
  reset_cache(tc);
  for_each_tile(a.sync, phase++, tgt_tiles, [&](long long t) {
    reduce_tile<FT, false, true, false, kCh>(s_match, a, off, level, t, s, tc, ctl, ph);
  });
}

// Flags every pair's status when the persistent kernel stopped early:
// STB_ST_TIMEOUT (a barrier gave up) or STB_ST_CAPACITY (the workspace was
// sized for fewer pixels than the levels hold).
__global__ void k_batch_status(const unsigned *sync, double *results, int B) {
  const unsigned err = *(volatile const unsigned *)(sync + 2);
  if (!err) return;
  const unsigned bits = ((err & 1u) ? STB_ST_TIMEOUT : 0u) | ((err & 2u) ? STB_ST_CAPACITY : 0u);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < B; p += gridDim.x * blockDim.x)
    results[(size_t)p * STB_RES_SIZE + STB_RES_STATUS] =
        (double)((unsigned)results[(size_t)p * STB_RES_SIZE + STB_RES_STATUS] | bits);
}

template <typename FT, bool kFeat, bool kHWC>
int launch_batch(const BatchArgs &args, cudaStream_t st) {
  auto kern = k_batch<FT, kFeat, kHWC>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  constexpr int kStageSmem = 2 * stage_bytes(BatchShape<kFeat>::kCh) +
                             (kFeat ? kAccSmemBytes : 0);
  // the offset rows go after the stages when that keeps the blocks per SM
  const int off_bytes = off_row_bytes(args.B + 1);
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kStageSmem + off_bytes) != cudaSuccess)
    return check_launch("cudaFuncSetAttribute");
  int with_off = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, kStageSmem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&with_off, kern, kThreads,
                                                kStageSmem + off_bytes);
  const bool stage_off = with_off >= per_sm;
  const int smem = kStageSmem + (stage_off ? off_bytes : 0);
  if (per_sm < 1) return fail(STB_ECUDA, "Cuda call error stb_icp_estimate_batch: kernel does not fit an SM");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(sms * per_sm);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  BatchArgs a = args;
  a.off_cap = stage_off ? args.B + 1 : 0;
  const cudaError_t err = cudaLaunchKernelEx(&cfg, kern, a);
  if (err != cudaSuccess)
    return fail(STB_ECUDA, "Cuda call error stb_icp_estimate_batch: %s", cudaGetErrorString(err));
  k_batch_status<<<(args.B + 255) / 256, 256, 0, st>>>(args.sync, args.results, args.B);
  return check_launch("stb_icp_estimate_batch");
}

}  // namespace
}  // namespace stb

using namespace stb;

extern "C" size_t stb_icp_batch_workspace_bytes(int32_t num_pairs, int64_t total_target_pixels) {
  if (num_pairs <= 0 || total_target_pixels < 0) return 0;
  return layout(num_pairs, total_target_pixels).total;
}

extern "C" int stb_icp_estimate_batch(const stb_level *levels, int32_t num_pairs,
                                      int32_t num_levels, const stb_level_params *params,
                                      int32_t channels, int32_t feat_dtype, int32_t channel_mode,
                                      const double *init_transforms, int64_t total_target_pixels,
                                      void *workspace, size_t workspace_bytes, double *results,
                                      double *history, int32_t tile_config, void *stream) {
  clear_error();
  if (num_pairs <= 0) return fail(STB_EINVAL, "Check failed: num_pairs must be positive");
  if (num_levels <= 0 || num_levels > kMaxLevels)
    return fail(STB_EINVAL, "Check failed: num_levels must be in [1, %d]", kMaxLevels);
  if (!params) return fail(STB_EINVAL, "Check failed: params: null pointer");
  int total_iters = 0;
  bool any_feat = false;
  for (int l = 0; l < num_levels; ++l) {
    if (params[l].num_iters < 0) return fail(STB_EINVAL, "Check failed: num_iters must be >= 0");
    total_iters += params[l].num_iters;
    any_feat = any_feat || params[l].feat_weight > 0.0;
  }
  if (total_iters > 253)
    return fail(STB_EINVAL, "Check failed: at most 253 iterations over all levels, got %d",
                total_iters);
  if (any_feat) {
    if (channels <= 0)
      return fail(STB_EINVAL, "Check failed: channels must be positive, got %d", channels);
    if (feat_dtype < STB_F32 || feat_dtype > STB_BF16_HWC)
      return fail(STB_EDTYPE, "Check failed: feature maps must be float32 or bfloat16");
  }
  if ((channel_mode & ~(0xff | STB_OPT_DW_SOLVE | STB_OPT_GROUPS)) != 0)
    return fail(STB_EINVAL, "Check failed: unknown option bits 0x%x in channel_mode",
                (unsigned)channel_mode & ~(0xffu | STB_OPT_DW_SOLVE | STB_OPT_GROUPS));
  const bool grouped = (channel_mode & STB_OPT_GROUPS) != 0;
  if ((channel_mode & 0xff) != 0 && (channel_mode & 0xff) != 1)
    return fail(STB_EINVAL, "Check failed: channel_mode must be 0 or 1");
  const Layout lay = layout(num_pairs, total_target_pixels);
  if (workspace_bytes < lay.total)
    return fail(STB_EINVAL, "Check failed: workspace of %zu bytes, %zu needed", workspace_bytes,
                lay.total);
  if (((uintptr_t)workspace & 255) != 0)
    return fail(STB_EINVAL, "Check failed: workspace must be 256-byte aligned");
  if (!grouped && (tile_config < 0 || tile_config > 5))
    return fail(STB_EINVAL, "Check failed: tile_config must be in [0, 5]");
  if (grouped && (tile_config < 1 || tile_config > fused::kMaxGroups))
    return fail(STB_EINVAL, "Check failed: with STB_OPT_GROUPS, tile_config (the number of "
                "groups) must be in [1, %d], got %d", fused::kMaxGroups, tile_config);
  STB_TRY(check_device_ptr(levels, "levels"));
  STB_TRY(check_device_ptr(init_transforms, "init_transforms", true));
  STB_TRY(check_device_ptr(workspace, "workspace"));
  STB_TRY(check_device_ptr(results, "results"));
  STB_TRY(check_device_ptr(history, "history", true));

  char *ws = static_cast<char *>(workspace);
  BatchArgs a;
  a.levels = levels;
  a.B = num_pairs;
  a.L = num_levels;
  a.C = any_feat ? channels : 0;
  a.dtype = feat_dtype;
  a.mode = channel_mode & 0xff;
  a.solve_dw = (channel_mode & STB_OPT_DW_SOLVE) != 0;
  {
    unsigned limit = 0;
    int phantom = 0;
    wait_test_limits(&limit, &phantom);
    a.spin_limit = limit ? limit : kSpinLimit;
    a.bar_phantom = (unsigned)phantom;
  }
  a.total_iters = total_iters;
  // largest pixels per work item: 0 -> default (8192), 1..5 -> 512 ... 8192;
  // each level uses the largest power of two below it that still gives
  // every block several work items
  a.tile = kMinTile << (tile_config == 0 ? 4 : tile_config - 1);
  for (int l = 0; l < kMaxLevels; ++l) {
    LevelP &q = a.lp[l];
    if (l >= num_levels) {
      q = LevelP{};
      continue;
    }
    const stb_level_params &pp = params[l];
    q.iters = pp.num_iters;
    q.use_geom = pp.geom_weight > 0.0;
    q.use_feat = any_feat && pp.feat_weight > 0.0;
    q.wg1 = (float)pp.geom_weight;
    q.wg2 = (float)(pp.geom_weight * pp.geom_weight);
    q.wf1 = (float)pp.feat_weight;
    q.wf2 = (float)(pp.feat_weight * pp.feat_weight);
    q.thr2 = distance_thresh_sq(pp.distance_thresh);
    q.cos_max = angle_cos_max(pp.normal_angle_thresh);
    const float ft = (float)pp.feat_residual_thresh;
    q.feat_thr2 = ft * ft;
  }
  a.init = init_transforms;
  a.results = results;
  a.history = history;
  a.sync = reinterpret_cast<unsigned *>(ws + lay.sync);
  a.level_tile = reinterpret_cast<int *>(ws + lay.level_tile);
  a.ps = reinterpret_cast<PairState *>(ws + lay.ps);
  a.key_off = reinterpret_cast<long long *>(ws + lay.key_off);
  a.src_off = reinterpret_cast<long long *>(ws + lay.src_off);
  a.tgt_off = reinterpret_cast<long long *>(ws + lay.tgt_off);
  a.grp_off = reinterpret_cast<long long *>(ws + lay.grp_off);
  a.grp_ticket = reinterpret_cast<unsigned *>(ws + lay.grp_ticket);
  a.pair_ticket = reinterpret_cast<unsigned *>(ws + lay.pair_ticket);
  a.tile_part = reinterpret_cast<float *>(ws + lay.tile_part);
  a.grp_part = reinterpret_cast<float *>(ws + lay.grp_part);
  a.keys = reinterpret_cast<unsigned long long *>(ws + lay.keys);
  a.keys_cap = total_target_pixels + num_pairs;
  a.tiles_cap = lay.tiles_cap;
  a.groups_cap = lay.groups_cap;

  const cudaStream_t st = as_stream(stream);
  // barrier counters start at zero for every launch
  if (cudaMemsetAsync(a.sync, 0, kSyncBytes, st) != cudaSuccess)
    return check_launch("cudaMemsetAsync");
  if (grouped) {
    fused::GroupLaunch g;
    g.levels = levels;
    g.B = a.B;
    g.L = a.L;
    g.C = a.C;
    g.dtype = a.dtype;
    g.mode = a.mode;
    g.total_iters = a.total_iters;
    g.solve_dw = a.solve_dw;
    for (int l = 0; l < fused::kGroupMaxLevels; ++l) {
      const LevelP &q = a.lp[l];
      g.lp[l] = fused::GroupLevelParams{q.iters, q.use_geom, q.use_feat, q.wg1, q.wg2, q.wf1,
                                        q.wf2, q.thr2, q.cos_max, q.feat_thr2};
    }
    g.init = a.init;
    g.results = a.results;
    g.history = a.history;
    g.spin_limit = a.spin_limit;
    g.bar_phantom = (int)a.bar_phantom;
    g.sync = a.sync;
    g.key_off = a.key_off;
    g.order = reinterpret_cast<int *>(ws + lay.order);
    g.part = reinterpret_cast<float2 *>(ws + lay.gpart);
    g.keys = a.keys;
    g.keys_cap = a.keys_cap;
    g.groups = tile_config;
    return fused::launch_grouped(g, st);
  }
  if (!any_feat) return launch_batch<float, false, false>(a, st);
  switch (feat_dtype) {
    case STB_F32: return launch_batch<float, true, false>(a, st);
    case STB_BF16: return launch_batch<__nv_bfloat16, true, false>(a, st);
    case STB_F32_HWC: return launch_batch<float, true, true>(a, st);
    default: return launch_batch<__nv_bfloat16, true, true>(a, st);
  }
}

extern "C" int stb_icp_batch_correspondences(const void *workspace, int32_t num_pairs,
                                             int64_t total_target_pixels, int32_t pair,
                                             int32_t height, int32_t width,
                                             int32_t total_iters, int64_t *merge_map,
                                             void *stream) {
  clear_error();
  if (num_pairs <= 0) return fail(STB_EINVAL, "Check failed: num_pairs must be positive");
  if (pair < 0 || pair >= num_pairs)
    return fail(STB_EINVAL, "Check failed: pair must be in [0, %d), got %d", num_pairs, pair);
  if (height <= 0 || width <= 0)
    return fail(STB_EINVAL, "Check failed: target size must be positive, got %dx%d",
                height, width);
  if ((int64_t)height * width > total_target_pixels)
    return fail(STB_EINVAL, "Check failed: %dx%d is more than the batch's %lld target pixels",
                height, width, (long long)total_target_pixels);
  if (total_iters < 0 || total_iters > 253)
    return fail(STB_EINVAL, "Check failed: total_iters must be in [0, 253], got %d",
                total_iters);
  if (((uintptr_t)workspace & 255) != 0)
    return fail(STB_EINVAL, "Check failed: workspace must be 256-byte aligned");
  STB_TRY(check_device_ptr(workspace, "workspace"));
  STB_TRY(check_device_ptr(merge_map, "merge_map"));
  const Layout lay = layout(num_pairs, total_target_pixels);
  const char *ws = static_cast<const char *>(workspace);
  const auto *keys = reinterpret_cast<const unsigned long long *>(ws + lay.keys);
  const auto *key_off = reinterpret_cast<const long long *>(ws + lay.key_off);
  const long long npix = (long long)height * width;
  // the information pass associates at step total_iters (tag btag of it)
  k_keys_to_merge_map<<<keys_grid(npix), 256, 0, as_stream(stream)>>>(
      keys, key_off + pair, npix, 254u - (unsigned)total_iters,
      reinterpret_cast<long long *>(merge_map));
  return check_launch("stb_icp_batch_correspondences");
}
