// One frame pair's whole registration (ICPOdometry.estimate,
// slamtb/registration/icp.py:152-262) in ONE cooperative launch.
//
// The grid holds one 512-thread block per SM (at most one block per slot of
// the workspace).  Block b owns a fixed share of the source points and of
// the target pixels for the whole registration (interleaved chunks, below).
// Per Gauss-Newton iteration:
//
//   association   each block transforms, projects and gates its source
//                 points and atomicMins (epoch tag, distance bits, index)
//                 into the per-pixel key map (correspondence_map.cu:39-61,
//                 merge_map.hpp:54-81 with the (distance, index) order);
//   grid barrier
//   reduction     each block forms the point-to-plane (and feature) terms of
//                 its target pixels' winners and writes its compensated
//                 block sums to its slot (icp_jacobian_geometric.cu:54-85,
//                 icp.py:78-80);
//   grid barrier
//   step          EVERY block folds all slots in the same fixed order and
//                 solves the 6x6 system with the same instructions, so every
//                 block holds the same new pose without a release barrier
//                 (icp.py:236-256); block 0 writes the history record.
//
// Then the association at the final pose, a barrier, the information sum of
// G^T G per block (icp_jacobian_geometric.cu:118-158), and block 0 writes
// the result block after the last barrier (the other blocks only arrive).
//
// Compared with the multi-launch sequence of icp_fused.cu (two kernels per
// iteration, the last block of the reduction folding and solving while
// the others have exited), this removes the kernel boundaries and the
// serial fold-then-solve tail's release: 2 barriers per iteration.
//
// Every barrier wait is bounded (Job::spin_limit polls); a wait that gives
// up sets the error word, every block leaves at its next barrier (waiting
// blocks notice the word within 64 polls), and block 0 writes
// STB_ST_TIMEOUT into the result status.
#include <math.h>
#include <stddef.h>

#include <mutex>

#include "feature_term.cuh"
#include "fused_common.cuh"
#include "gn_solve.cuh"
#include "stb_common.cuh"
#include "stb_host.hpp"

namespace stb {
namespace fused {
namespace {

constexpr int kPT = 512;          // threads per block
constexpr int kPW = kPT / 32;     // warps per block
constexpr int kPR = 4;            // pixels per thread per round

// Work ownership.  The source points (association) and the target pixels
// (reduction, information) are cut into chunks of kChunk consecutive units;
// block b of a grid of G blocks owns chunks b, b + G, b + 2G, ..., so every
// block's share is spread over the whole frame and content that costs more
// per unit (valid, matched pixels) is shared evenly (with contiguous ranges
// the blocks over the middle of a frame finished their association about
// 1.4 us after the others).  One round of a block covers kChunksPerRound of
// its chunks: thread t takes unit t % kChunk of chunk slot
// k (kPT / kChunk) + t / kChunk for k < kPR, so four warps read one chunk,
// coalesced.
constexpr int kChunk = 128;
constexpr int kChunksPerRound = kPT * kPR / kChunk;
static_assert(kPT % kChunk == 0, "a chunk is a whole number of warps");

struct Share {
  long long total;  // units in the frame
  int rounds;       // rounds of this block
};

__device__ __forceinline__ Share share_of(long long total) {
  const long long nch = (total + kChunk - 1) / kChunk, b = blockIdx.x, G = gridDim.x;
  const long long mine = nch > b ? (nch - 1 - b) / G + 1 : 0;
  return Share{total, (int)((mine + kChunksPerRound - 1) / kChunksPerRound)};
}

// Unit of this thread's k-th slot in round r (>= the total: no unit).
__device__ __forceinline__ long long unit_of(int r, int k) {
  const long long slot =
      (long long)r * kChunksPerRound + k * (kPT / kChunk) + threadIdx.x / kChunk;
  return (blockIdx.x + (long long)gridDim.x * slot) * kChunk + (threadIdx.x % kChunk);
}

// The block's source points of its first Job::src_cache_rounds rounds,
// copied to shared memory at the start of the registration (they are the
// same points in every association): the association then reads them
// there instead of making a memory round trip before its target gathers.
// Entry (r kPR + k) kPT + t holds the point of thread t's k-th slot in
// round r; the floats are six arrays of cap entries (x, y, z, nx, ny, nz),
// then cap mask bytes.
constexpr int kMaxCacheRounds = 2;
constexpr int kCachePointBytes = 6 * sizeof(float) + 1;

struct SrcCache {
  float *f;
  uint8_t *m;
  int cap, rounds;
};

__device__ __forceinline__ int cache_index(int r, int k) { return (r * kPR + k) * kPT + threadIdx.x; }

// Per-block shared state of the loop.
struct LoopShared {
  Pose32 P;              // float32 pose view, normal matrix, intrinsics
  double Td[16];         // pose (FP64 solve)
  float2 Tw[16];         // pose (double-word solve)
  double tot[32];        // totals of the current step, FP64
  float2 totw[32];       // the same as double-words
  double last_tot[32];   // totals of the last successful step
  float rt32[12];
  unsigned status;
  int done;              // successful iterations
  int ok;                // verdict of the last solve
};

// Loads and atomics of the grid barrier's words at GPU scope.
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_add_release(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier number `k` of this launch (counted by every block alike),
// with a bounded wait.  The arrival counter only grows: barrier k is
// complete when it reaches (k + 1) x the expected arrivals, so an arrival is
// one release-add and a wait polls one word (no generation word to read
// first, no reset).  The release orders the block's writes before the
// barrier (key-map atomics, slot stores; made block-wide by the preceding
// __syncthreads), the acquiring poll orders the reads after it.
// `wait` false: arrive and return at once (the block has no work after the
// barrier).  Returns false when a wait gave up (here or in another block).
__device__ __forceinline__ bool grid_barrier(State *S, const Job &J, unsigned k, bool wait) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned target = (k + 1) * (gridDim.x + (unsigned)J.bar_phantom);
    red_add_release(&S->bar_count, 1u);
    bool ok = true;
    if (wait) {
      unsigned spins = 0;
      while (ld_acquire(&S->bar_count) < target) {
        if (++spins > J.spin_limit) {
          atomicOr(&S->bar_err, 1u);
          ok = false;
          break;
        }
        // another block's wait gave up: checked every 64 polls
        if ((spins & 63u) == 0 && ld_relaxed(&S->bar_err)) {
          ok = false;
          break;
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok;
}

// The float32 view of the pose in Td (or Tw) and its normal matrix, by
// warp 0 (lanes 0..11 convert, lanes 0..8 form one entry each of the
// normal matrix).
__device__ __forceinline__ void refresh_view(LoopShared &L, bool dw, int lane) {
  if (lane < 12) {
    const float f = dw ? L.Tw[lane].x : __double2float_rn(L.Td[lane]);
    L.rt32[lane] = f;
    L.P.rt[lane] = f;
  }
  __syncwarp();
  if (lane < 9) L.P.nm[lane] = inverse_transpose_entry(L.rt32, lane);
  __syncwarp();
}

// Association of this block's share of the source points at epoch e.
__device__ __forceinline__ void associate(const Job &J, const Pose32 &P, Share sh,
                                          const SrcCache &C, int e) {
  const unsigned long long tag = (unsigned long long)(254u - (unsigned)e) << 56;
  const int H = J.H, W = J.W;
  const float *__restrict__ sp = J.sp;
  const float *__restrict__ sn = J.sn;
  const float *__restrict__ tp = J.tp;
  const float *__restrict__ tn = J.tn;
  const uint8_t *__restrict__ sm = J.sm;
  const uint8_t *__restrict__ tm = J.tm;
  unsigned long long *__restrict__ keys = J.keys;
  const long long n = sh.total;
  for (int r = 0; r < sh.rounds; ++r) {
    // the source mask, point and normal of every point of the round in one
    // batch of loads (none depends on another), then the projected target
    // pixels' in a second: two dependent memory round trips before the
    // atomic
    uint8_t msk[kPR];
    float sxyz[kPR][3], snrm[kPR][3];
    if (r < C.rounds) {
#pragma unroll
      for (int k = 0; k < kPR; ++k) {
        const int c = cache_index(r, k);
        msk[k] = C.m[c];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          sxyz[k][d] = C.f[d * C.cap + c];
          snrm[k][d] = C.f[(3 + d) * C.cap + c];
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kPR; ++k) {
        const long long i = unit_of(r, k);
        const long long ic = i < n ? i : 0;
        msk[k] = __ldg(sm + ic);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          sxyz[k][d] = __ldg(sp + 3 * ic + d);
          snrm[k][d] = __ldg(sn + 3 * ic + d);
        }
      }
    }
    float3 Tp[kPR];
    long long pix[kPR];
    bool ok[kPR];
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      const long long i = unit_of(r, k);
      ok[k] = i < n && msk[k];
      Tp[k] = transform_point(P.rt, sxyz[k][0], sxyz[k][1], sxyz[k][2]);
      float u, v;
      project(P, Tp[k], u, v);
      int ui = 0, vi = 0;
      ok[k] = ok[k] && round_in(u, W, ui) && round_in(v, H, vi);
      pix[k] = ok[k] ? (long long)vi * W + ui : 0;
    }
    float q[kPR][3], m[kPR][3];
    bool valid[kPR];
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      valid[k] = __ldg(tm + pix[k]);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        q[k][d] = __ldg(tp + 3 * pix[k] + d);
        m[k][d] = __ldg(tn + 3 * pix[k] + d);
      }
    }
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      if (!ok[k] || !valid[k]) continue;
      const long long i = unit_of(r, k);
      const float dx = fsub(q[k][0], Tp[k].x), dy = fsub(q[k][1], Tp[k].y),
                  dz = fsub(q[k][2], Tp[k].z);
      const float sq = dot3(dx, dy, dz, dx, dy, dz);
      if (sq > J.thr2) continue;
      const float3 Tn = transform_normal(P.nm, snrm[k][0], snrm[k][1], snrm[k][2]);
      const float c = fdiv(dot3(Tn.x, Tn.y, Tn.z, m[k][0], m[k][1], m[k][2]),
                           fmul(__fsqrt_rn(dot3(Tn.x, Tn.y, Tn.z, Tn.x, Tn.y, Tn.z)),
                                __fsqrt_rn(dot3(m[k][0], m[k][1], m[k][2], m[k][0], m[k][1],
                                                m[k][2]))));
      if (c >= -1.0f && c <= J.cos_max) continue;
      atomicMin(keys + pix[k],
                tag | ((unsigned long long)__float_as_uint(__fsqrt_rn(sq)) << 24) |
                    (unsigned long long)i);
    }
  }
}

// Per-thread partials of the normal equations over this block's share of
// the target pixels at epoch e.
template <typename FT, bool kGeom, bool kFeat, bool kHWC>
__device__ __forceinline__ void reduce_pixels(const Job &J, const Pose32 &P, Share sh, int e,
                                              float *acc) {
  const unsigned tag = 254u - (unsigned)e;
  const int H = J.H, W = J.W;
  const long long npix = (long long)H * W;
  const unsigned long long *__restrict__ keys = J.keys;
  const float *__restrict__ sp = J.sp;
  const float *__restrict__ tp = J.tp;
  const float *__restrict__ tn = J.tn;
  for (int r = 0; r < sh.rounds; ++r) {
    unsigned long long key[kPR];
    float q[kPR][3], m[kPR][3];
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      const long long pix = unit_of(r, k);
      const long long pc = pix < npix ? pix : 0;
      key[k] = pix < npix ? __ldcg(keys + pix) : 0ull;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        q[k][d] = kGeom ? __ldg(tp + 3 * pc + d) : 0.f;
        m[k][d] = kGeom ? __ldg(tn + 3 * pc + d) : 0.f;
      }
    }
    float s[kPR][3];
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      const bool match = (unsigned)(key[k] >> 56) == tag;
      const long long i = (long long)(key[k] & 0xffffffull);
#pragma unroll
      for (int d = 0; d < 3; ++d) s[k][d] = match ? __ldg(sp + 3 * i + d) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      if ((unsigned)(key[k] >> 56) != tag) continue;
      const long long i = (long long)(key[k] & 0xffffffull);
      const float3 Tp = transform_point(P.rt, s[k][0], s[k][1], s[k][2]);
      if (kGeom) {
        const float nx = m[k][0], ny = m[k][1], nz = m[k][2];
        const float r = dot3(fsub(q[k][0], Tp.x), fsub(q[k][1], Tp.y), fsub(q[k][2], Tp.z), nx,
                             ny, nz);
        const float Jv[6] = {nx, ny, nz, fsub(fmul(Tp.y, nz), fmul(Tp.z, ny)),
                             fsub(fmul(Tp.z, nx), fmul(Tp.x, nz)),
                             fsub(fmul(Tp.x, ny), fmul(Tp.y, nx))};
        accumulate_se3(acc, Jv, r, J.wg1, J.wg2);
        acc[kR2] += J.wg1 * (r * r);
        acc[kCountGeom] += 1.f;
      }
      if (kFeat) {
        const FeatView<FT, kHWC> tf{static_cast<const FT *>(J.tf), npix, J.C};
        const FeatView<FT, kHWC> sf{static_cast<const FT *>(J.sf), J.n, J.C};
        float sq;
        if (feature_term(tf, sf, i, P, Tp, H, W, J.feat_thr2, J.channel_mode, J.wf1, J.wf2, acc,
                         sq)) {
          acc[kR2] += J.wf1 * sq;
          acc[kCountFeat] += 1.f;
        }
      }
    }
  }
}

// Information partials G^T G over this block's share of the target pixels
// at epoch e.
__device__ __forceinline__ void info_pixels(const Job &J, Share sh, int e, float *acc) {
  const unsigned tag = 254u - (unsigned)e;
  const unsigned long long *__restrict__ keys = J.keys;
  const float *__restrict__ tp = J.tp;
  for (int slot = 0; slot < sh.rounds * kPR; ++slot) {
    const long long pix = unit_of(slot / kPR, slot % kPR);
    if (pix >= sh.total || (unsigned)(__ldcg(keys + pix) >> 56) != tag) continue;
    const float qx = __ldg(tp + 3 * pix), qy = __ldg(tp + 3 * pix + 1),
                qz = __ldg(tp + 3 * pix + 2);
    const float G0[6] = {0.f, qz, -qy, 1.f, 0.f, 0.f};
    const float G1[6] = {-qz, 0.f, qx, 0.f, 1.f, 0.f};
    const float G2[6] = {qy, -qx, 0.f, 0.f, 0.f, 1.f};
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
      for (int b = a; b < 6; ++b)
        acc[upper_index(a, b)] += G0[a] * G0[b] + G1[a] * G1[b] + G2[a] * G2[b];
  }
}

// isfinite on the exponent bits (integer instructions: on this part every
// FP64 instruction, comparisons included, costs the FP64 pipe's ~64 cycles
// per warp).
__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}

// The Gauss-Newton step of every block from the totals in L (FP64 or
// double-word solve); block 0 records the iteration.  Warp 0 only.
__device__ void persist_step(const Job &J, LoopShared &L, int iter, int lane) {
  const bool dw = J.solve_dw;
  bool ok;
  bool finite = true;
  if (dw) {
    float xs[6];
    float2 tn;
    ok = warp_gn_update_dw(L.totw, L.totw + kJr, L.Tw, xs, tn, lane);
    for (int k = 0; k < 6; ++k) finite &= isfinite(xs[k]);
    __syncwarp();
    if (ok && lane < 16) {
      L.Tw[lane] = tn;
      L.Td[lane] = (double)tn.x + (double)tn.y;
    }
  } else {
    // (the double-word pose Tw is not kept up to date: only the
    // double-word solve reads it)
    double xs[6];
    double tn;
    ok = warp_gn_update(L.tot, L.tot + kJr, L.Td, xs, tn, lane);
    for (int k = 0; k < 6; ++k) finite &= finite_bits(xs[k]);
    __syncwarp();
    if (ok && lane < 16) L.Td[lane] = tn;
  }
  __syncwarp();
  if (ok) {
    if (lane < kAccs) L.last_tot[lane] = L.tot[lane];
    refresh_view(L, dw, lane);
  }
  const double cg = L.tot[kCountGeom], cf = L.tot[kCountFeat];
  // the counts are sums of ones (never -0): zero exactly when all bits are
  const bool no_match = (__double_as_longlong(cf) |
                         (J.use_geom ? __double_as_longlong(cg) : 0ll)) == 0ll;
  if (lane == 0) {
    unsigned st = L.status;
    if (!ok)
      st |= STB_ST_NOT_PD;
    else if (!finite)
      st |= STB_ST_NAN;
    if (no_match) st |= STB_ST_NO_MATCHES;
    L.status = st;
    L.ok = ok;
    if (ok) L.done += 1;
  }
  __syncwarp();
  if (blockIdx.x == 0 && J.history) {
    double *Hh = J.history + (size_t)iter * STB_HIST_SIZE;
    for (int k = lane; k < 36; k += 32) {
      const int r = k / 6, c = k % 6;
      Hh[STB_HIST_JTJ + k] = L.tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
    }
    if (lane < 6) Hh[STB_HIST_JR + lane] = L.tot[kJr + lane];
    if (lane == 0) {
      Hh[STB_HIST_R2] = L.tot[kR2];
      Hh[STB_HIST_GEOM_COUNT] = cg;
      Hh[STB_HIST_FEAT_COUNT] = cf;
      Hh[STB_HIST_OK] = ok ? 1.0 : 0.0;
    }
    if (ok && lane < 16) Hh[STB_HIST_TRANSFORM + lane] = L.Td[lane];
  }
}

// Slot words at GPU scope: relaxed stores by the writing block, relaxed
// loads by the polling ones (every 32-bit word is written whole, so a load
// sees either the poison or the new value of each word).
__device__ __forceinline__ void st_relaxed_f2(float2 *p, float2 v) {
  asm volatile("st.relaxed.gpu.global.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(v.x), "f"(v.y)
               : "memory");
}
__device__ __forceinline__ float2 ld_relaxed_f2(const float2 *p) {
  float2 v;
  asm volatile("ld.relaxed.gpu.global.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p)
               : "memory");
  return v;
}

// The slots of the Gauss-Newton sums are double-buffered by iteration
// parity and carry their own completion: a slot word holds kPoison until
// its block writes the iteration's value, so the blocks fold the slots as
// they arrive instead of waiting at a grid barrier first (one L2 round trip
// less per iteration).  kPoison is a NaN payload that arithmetic never
// produces (the GPU's arithmetic returns the canonical NaN 0x7fffffff), so
// no sum can be mistaken for it.  A buffer is poisoned again by its blocks
// in the next iteration, after the association barrier: by then every
// block has folded it, and that barrier orders the poison before any
// block's reads of the buffer's next use.
constexpr unsigned kPoison = 0x7fbadbadu;

__device__ __forceinline__ float2 *slot_of(const Job &J, int buf, int block) {
  return J.part + ((size_t)buf * gridDim.x + block) * kSlotAccs;
}

__device__ __forceinline__ void poison_slot(const Job &J, int buf) {
  if (threadIdx.x < kSlotAccs)
    st_relaxed_f2(slot_of(J, buf, blockIdx.x) + threadIdx.x,
                  make_float2(__uint_as_float(kPoison), __uint_as_float(kPoison)));
}

// Totals of kN accumulators over the grid's slots of buffer buf into L.tot
// (FP64) and L.totw (double-words), in every block in the same order: warp
// w merges slots w, w + 16, ... with lane = accumulator, then the warps'
// sums are merged in warp order.  poll: the slots may still be arriving
// (reload a slot while any of its words holds kPoison, at most
// J.spin_limit times); otherwise a grid barrier has ordered them.  Returns
// false when a poll gave up (here or, seen on the error word, elsewhere).
template <int kN>
__device__ __forceinline__ bool fold_slots(const Job &J, LoopShared &L, State *S, int buf,
                                           bool poll) {
  __shared__ float2 wsum[kPW][32];
  __shared__ int s_fail[kPW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  CSum t = {0.f, 0.f};
  bool fail = false;
  // slots per warp in one round of loads: a grid of up to 192 blocks is
  // folded with every load in flight at once
  constexpr int kLoads = 12;
  for (int b0 = warp; b0 < (int)gridDim.x && !fail; b0 += kPW * kLoads) {
    float2 v[kLoads];
#pragma unroll
    for (int k = 0; k < kLoads; ++k) {
      const int b = b0 + k * kPW;
      v[k] = (b < (int)gridDim.x && lane < kN) ? ld_relaxed_f2(slot_of(J, buf, b) + lane)
                                               : make_float2(0.f, 0.f);
    }
    if (poll) {
      unsigned spins = 0;
      for (;;) {
        unsigned pending = 0;
#pragma unroll
        for (int k = 0; k < kLoads; ++k) {
          const bool bad = __float_as_uint(v[k].x) == kPoison || __float_as_uint(v[k].y) == kPoison;
          if (__any_sync(0xffffffffu, bad)) pending |= 1u << k;
        }
        if (!pending) break;
        if (++spins > J.spin_limit) {
          if (lane == 0) atomicOr(&S->bar_err, 1u);
          fail = true;
          break;
        }
        if ((spins & 63u) == 0 && ld_relaxed(&S->bar_err)) {
          fail = true;
          break;
        }
#pragma unroll
        for (int k = 0; k < kLoads; ++k)
          if ((pending & (1u << k)) && lane < kN)
            v[k] = ld_relaxed_f2(slot_of(J, buf, b0 + k * kPW) + lane);
      }
    }
#pragma unroll
    for (int k = 0; k < kLoads; ++k) csum_merge(t, v[k].x, v[k].y);
  }
  wsum[warp][lane] = make_float2(t.s, t.c);
  if (lane == 0) s_fail[warp] = fail;
  __syncthreads();
  if (threadIdx.x < kN) {
    CSum u = {0.f, 0.f};
#pragma unroll
    for (int w = 0; w < kPW; ++w) csum_merge(u, wsum[w][threadIdx.x].x, wsum[w][threadIdx.x].y);
    L.tot[threadIdx.x] = (double)u.s + (double)u.c;
    L.totw[threadIdx.x] = dw_of_csum(u.s, u.c);
  }
  bool any_fail = false;
#pragma unroll
  for (int w = 0; w < kPW; ++w) any_fail |= s_fail[w] != 0;
  __syncthreads();
  return !any_fail;
}

// This block's compensated sums of kN per-thread partials into its slot of
// buffer buf.
template <int kN>
__device__ __forceinline__ void write_slot(const Job &J, const float *acc, float (*red)[kPT],
                                           int buf) {
  __shared__ float2 bsum[32];
  block_reduce<kN, kPT>(acc, red, bsum);
  if (threadIdx.x < kN) st_relaxed_f2(slot_of(J, buf, blockIdx.x) + threadIdx.x, bsum[threadIdx.x]);
}

extern __shared__ __align__(16) float s_red_p[];

template <typename FT, bool kGeom, bool kFeat, bool kHWC>
__global__ void __launch_bounds__(kPT, 1) k_persist(const __grid_constant__ Job J) {
  __shared__ LoopShared L;
  float(*red)[kPT] = reinterpret_cast<float(*)[kPT]>(s_red_p);
  State *S = J.state;
  const int lane = threadIdx.x & 31;
  const long long n = J.n, npix = (long long)J.H * J.W;
  const long long G = gridDim.x, b = blockIdx.x;
  const long long pc = (npix + G - 1) / G;
  const long long p0 = min(npix, b * pc), p1 = min(npix, p0 + pc);
  const Share src = share_of(n), tgt = share_of(npix);
  SrcCache C;
  C.rounds = min(J.src_cache_rounds, src.rounds);
  C.cap = J.src_cache_rounds * kPR * kPT;
  C.f = s_red_p + kAccs * kPT;
  C.m = reinterpret_cast<uint8_t *>(C.f + 6 * C.cap);

  // set-up: the initial pose in every block; this block's key-map range
  // cleared (a key of an earlier registration may carry a current tag);
  // its source points copied to the cache; its slots of both buffers
  // poisoned
  for (int r = 0; r < C.rounds; ++r) {
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      const long long i = unit_of(r, k);
      const int c = cache_index(r, k);
      const bool in = i < n;
      C.m[c] = in ? __ldg(J.sm + i) : (uint8_t)0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        C.f[d * C.cap + c] = in ? __ldg(J.sp + 3 * i + d) : 0.f;
        C.f[(3 + d) * C.cap + c] = in ? __ldg(J.sn + 3 * i + d) : 0.f;
      }
    }
  }
  poison_slot(J, 0);
  poison_slot(J, 1);
  if (threadIdx.x < 32) {
    if (lane < 16) {
      const double v = J.init ? J.init[lane]
                              : (J.has_init_v ? J.init_v[lane] : ((lane % 5) == 0 ? 1.0 : 0.0));
      L.Td[lane] = v;
      L.Tw[lane] = dw_of_double(v);
    }
    if (lane == 0) {
      L.P.fx = J.kcam ? J.kcam[0] : J.kcam_v[0];
      L.P.cx = J.kcam ? J.kcam[2] : J.kcam_v[1];
      L.P.fy = J.kcam ? J.kcam[4] : J.kcam_v[2];
      L.P.cy = J.kcam ? J.kcam[5] : J.kcam_v[3];
      L.status = 0;
      L.done = 0;
      L.ok = 1;
    }
    __syncwarp();
    // the float32 cast of the initial pose (refresh_pose32's values)
    if (lane < 12) {
      L.rt32[lane] = __double2float_rn(L.Td[lane]);
      L.P.rt[lane] = L.rt32[lane];
    }
    __syncwarp();
    if (lane == 0) inverse_transpose(L.rt32, L.P.nm);
  }
  for (long long pix = p0 + threadIdx.x; pix < p1; pix += kPT) J.keys[pix] = ~0ull;
  unsigned nbar = 0;  // grid barriers passed
  bool alive = grid_barrier(S, J, nbar++, true);

  for (int iter = 0; alive && iter < J.iters; ++iter) {
    associate(J, L.P, src, C, iter);
    if (!(alive = grid_barrier(S, J, nbar++, true))) break;
    float acc[kAccs];
#pragma unroll
    for (int a = 0; a < kAccs; ++a) acc[a] = 0.f;
    reduce_pixels<FT, kGeom, kFeat, kHWC>(J, L.P, tgt, iter, acc);
    // every block has folded the previous iteration's buffer (it passed the
    // barrier above after its fold): poisoned again for the next iteration
    if (iter > 0) poison_slot(J, (iter + 1) & 1);
    write_slot<kAccs>(J, acc, red, iter & 1);
    if (!(alive = fold_slots<kAccs>(J, L, S, iter & 1, true))) break;
    if (threadIdx.x < 32) persist_step(J, L, iter, lane);
    __syncthreads();
    if (!L.ok) break;  // a failed solve ends the loop (icp.py:241-242 `except: break`)
  }

  // the association at the final pose and the information sum
  if (alive) {
    associate(J, L.P, src, C, J.iters);
    alive = grid_barrier(S, J, nbar++, true);
  }
  if (alive) {
    float acc[kInfoAccs];
#pragma unroll
    for (int a = 0; a < kInfoAccs; ++a) acc[a] = 0.f;
    info_pixels(J, tgt, J.iters, acc);
    // (buffer 0: every block has folded the last iteration's sums)
    write_slot<kInfoAccs>(J, acc, red, 0);
    alive = grid_barrier(S, J, nbar++, blockIdx.x == 0);
  }
  if (blockIdx.x != 0) return;
  double *R = J.result;
  if (alive) {
    fold_slots<kInfoAccs>(J, L, S, 0, false);
    for (int k = threadIdx.x; k < 36; k += kPT) {
      const int r = k / 6, c = k % 6;
      R[STB_RES_INFO + k] = L.tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
    }
  }
  const int done = L.done;
  for (int k = threadIdx.x; k < STB_RES_SIZE; k += kPT) {
    if (k >= STB_RES_INFO && k < STB_RES_INFO + 36 && alive) continue;
    double v = 0.0;
    if (done > 0 && k >= STB_RES_TRANSFORM && k < STB_RES_TRANSFORM + 16)
      v = L.Td[k - STB_RES_TRANSFORM];
    if (done > 0 && k >= STB_RES_JTJ && k < STB_RES_JTJ + 36) {
      const int r = (k - STB_RES_JTJ) / 6, c = (k - STB_RES_JTJ) % 6;
      v = L.last_tot[r <= c ? upper_index(r, c) : upper_index(c, r)];
    }
    if (k == STB_RES_RESIDUAL || k == STB_RES_MATCHES) {
      const double cg = L.last_tot[kCountGeom], cf = L.last_tot[kCountFeat];
      const double count = J.use_geom ? fmax(cg, cf) : cf;
      v = done > 0 ? (k == STB_RES_MATCHES ? count : L.last_tot[kR2] / count)
                   : (k == STB_RES_RESIDUAL ? INFINITY : 0.0);
    }
    if (k == STB_RES_ITERS) v = (double)done;
    if (k == STB_RES_STATUS) v = (double)(L.status | (alive ? 0u : STB_ST_TIMEOUT));
    R[k] = v;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
using PersistFn = void (*)(Job);

template <typename FT, bool kGeom, bool kFeat, bool kHWC>
PersistFn persist_fn() {
  return k_persist<FT, kGeom, kFeat, kHWC>;
}

template <typename FT, bool kHWC>
PersistFn persist_feat(bool use_geom) {
  return use_geom ? persist_fn<FT, true, true, kHWC>() : persist_fn<FT, false, true, kHWC>();
}

PersistFn pick_persist(const Plan &p) {
  if (!p.use_feat) return persist_fn<float, true, false, false>();
  switch (p.dtype) {
    case STB_F32: return persist_feat<float, false>(p.use_geom);
    case STB_BF16: return persist_feat<__nv_bfloat16, false>(p.use_geom);
    case STB_F32_HWC: return persist_feat<float, true>(p.use_geom);
    default: return persist_feat<__nv_bfloat16, true>(p.use_geom);
  }
}

// Dynamic shared memory: the block reduction's transpose (kAccs x kPT
// floats), then the source-point cache of Job::src_cache_rounds rounds.
constexpr size_t kRedSmem = sizeof(float) * kAccs * kPT;
constexpr size_t cache_smem(int rounds) {
  return ((size_t)rounds * kPR * kPT * kCachePointBytes + 15) & ~size_t(15);
}
constexpr size_t kPersistSmem = kRedSmem + cache_smem(kMaxCacheRounds);
static_assert(kPersistSmem + sizeof(LoopShared) + 8192 <= 227 * 1024,
              "the persistent kernel's shared memory fits one block per SM");

// Blocks of the grid on the current device for kernel fn: the SMs times the
// resident blocks per SM (at most one, by the launch bounds), looked up once
// per device and kernel; 0 when the kernel does not fit.
int persist_capacity(PersistFn fn) {
  static std::mutex m;
  struct Entry {
    int dev;
    PersistFn fn;
    int blocks;
  };
  static Entry cache[64];
  static int used = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  std::lock_guard<std::mutex> lock(m);
  for (int k = 0; k < used; ++k)
    if (cache[k].dev == dev && cache[k].fn == fn) return cache[k].blocks;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kPersistSmem) != cudaSuccess)
    return -1;
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kPT, kPersistSmem) !=
      cudaSuccess)
    return -1;
  const int blocks = sms * (per_sm > 1 ? 1 : per_sm);
  if (used < 64) cache[used++] = Entry{dev, fn, blocks};
  return blocks;
}

unsigned g_test_spin_limit = 0;  // 0: the default
int g_test_phantom = 0;
std::mutex g_test_mutex;

}  // namespace

int launch_persistent(const Plan &p, Job job, cudaStream_t st) {
  const PersistFn fn = pick_persist(p);
  const int cap = persist_capacity(fn);
  if (cap < 0) return check_launch("stb_icp_estimate (persistent kernel set-up)");
  if (cap == 0)
    return fail(STB_ECUDA, "Cuda call error stb_icp_estimate: the persistent kernel does not "
                "fit an SM");
  // at most one block per workspace slot
  const int grid = cap < p.nblocks ? cap : p.nblocks;
  // rounds of the block with the most source chunks; the first
  // kMaxCacheRounds of them are cached in shared memory
  const long long nch = (p.n + kChunk - 1) / kChunk;
  const long long rounds = ((nch + grid - 1) / grid + kChunksPerRound - 1) / kChunksPerRound;
  job.src_cache_rounds = (int)(rounds < kMaxCacheRounds ? rounds : kMaxCacheRounds);
  {
    std::lock_guard<std::mutex> lock(g_test_mutex);
    job.spin_limit = g_test_spin_limit ? g_test_spin_limit : (1u << 24);
    job.bar_phantom = g_test_phantom;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kPT);
  cfg.dynamicSmemBytes = kRedSmem + cache_smem(job.src_cache_rounds);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t err = cudaLaunchKernelEx(&cfg, fn, job);
  if (err != cudaSuccess)
    return fail(STB_ECUDA, "Cuda call error stb_icp_estimate (persistent kernel): %s",
                cudaGetErrorString(err));
  return STB_OK;
}

int reset_persistent(const Job &job, cudaStream_t st) {
  // the barrier words start at zero for every call
  if (cudaMemsetAsync(reinterpret_cast<char *>(job.state) + offsetof(State, bar_count), 0,
                      2 * sizeof(unsigned), st) != cudaSuccess)
    return check_launch("cudaMemsetAsync");
  return STB_OK;
}

void set_persist_test_limits(unsigned spin_limit, int phantom) {
  std::lock_guard<std::mutex> lock(g_test_mutex);
  g_test_spin_limit = spin_limit;
  g_test_phantom = phantom;
}

}  // namespace fused

void wait_test_limits(unsigned *spin_limit, int *phantom) {
  std::lock_guard<std::mutex> lock(fused::g_test_mutex);
  *spin_limit = fused::g_test_spin_limit;
  *phantom = fused::g_test_phantom;
}

}  // namespace stb
