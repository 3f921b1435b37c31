// The phases of a persistent registration (association, reduction into
// block slots, the polled fold of the slots, the information sum) for the
// blocks that run one registration: the whole grid of the single-pair
// kernel (icp_persist.cu) or one group of the grouped batch kernel
// (icp_group.cu).  The phases are templates over the registration's
// parameters X (a Job, or a group's level), which provide the frames'
// pointers and sizes, the estimator's weights and gates, the key map, the
// slot buffers and the barrier words, and the functions rank_of(x) and
// size_of(x) (this block's rank among the size blocks that run it),
// bar_word(x) (their arrival counter) and err_word(x) (the error word).
#pragma once

#include <math.h>
#include <stddef.h>

#include "feature_term.cuh"
#include "fused_common.cuh"
#include "gn_solve.cuh"
#include "stb_common.cuh"

namespace stb {
namespace fused {

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

__device__ __forceinline__ Share share_of(long long total, int rank, int size) {
  const long long nch = (total + kChunk - 1) / kChunk, b = rank, G = size;
  const long long mine = nch > b ? (nch - 1 - b) / G + 1 : 0;
  return Share{total, (int)((mine + kChunksPerRound - 1) / kChunksPerRound)};
}

// Unit of this thread's k-th slot in round r of block `rank` of `size`
// (>= the total: no unit).
__device__ __forceinline__ long long unit_of(int r, int k, int rank, int size) {
  const long long slot =
      (long long)r * kChunksPerRound + k * (kPT / kChunk) + threadIdx.x / kChunk;
  return (rank + (long long)size * slot) * kChunk + (threadIdx.x % kChunk);
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
__device__ __forceinline__ void st_relaxed_u32(unsigned *p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void prefetch_l2(const void *p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ void red_add_release(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Barrier number `k` of the blocks running a registration (a grid, or a
// group of a grid; counted by every block alike), with a bounded wait.  The arrival counter only grows: barrier k is
// complete when it reaches (k + 1) x the expected arrivals, so an arrival is
// one release-add and a wait polls one word (no generation word to read
// first, no reset).  The release orders the block's writes before the
// barrier (key-map atomics, slot stores; made block-wide by the preceding
// __syncthreads), the acquiring poll orders the reads after it.
// `wait` false: arrive and return at once; only for the last barrier of a
// launch (a block that arrives without waiting and goes on to the next
// barrier would count there before the others arrived here).  Returns
// false when a wait gave up (here or in another block).
template <class X>
__device__ __forceinline__ bool group_barrier(const X &J, unsigned k, bool wait) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned *count = bar_word(J), *err = err_word(J);
    const unsigned target = (k + 1) * ((unsigned)size_of(J) + (unsigned)J.bar_phantom);
    red_add_release(count, 1u);
    bool ok = true;
    if (wait) {
      unsigned spins = 0;
      while (ld_acquire(count) < target) {
        if (++spins > J.spin_limit) {
          atomicOr(err, 1u);
          ok = false;
          break;
        }
        // another block's wait gave up: checked every 64 polls
        if ((spins & 63u) == 0 && ld_relaxed(err)) {
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
template <class X>
__device__ __forceinline__ void associate(const X &J, const Pose32 &P, Share sh,
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
        const long long i = unit_of(r, k, rank_of(J), size_of(J));
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
      const long long i = unit_of(r, k, rank_of(J), size_of(J));
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
      const long long i = unit_of(r, k, rank_of(J), size_of(J));
      const float dx = fsub(q[k][0], Tp[k].x), dy = fsub(q[k][1], Tp[k].y),
                  dz = fsub(q[k][2], Tp[k].z);
      const float sq = dot3(dx, dy, dz, dx, dy, dz);
      if (sq > J.thr2) continue;
      const float3 Tn = transform_normal(P.nm, snrm[k][0], snrm[k][1], snrm[k][2]);
      if (normal_angle_rejects(Tn, m[k][0], m[k][1], m[k][2], J.cos_max)) continue;
      atomicMin(keys + pix[k],
                tag | ((unsigned long long)__float_as_uint(__fsqrt_rn(sq)) << 24) |
                    (unsigned long long)i);
    }
  }
}

// Unit of thread t's k-th slot in round r of block `rank` of `size` (as
// unit_of, for another thread of the block).
__device__ __forceinline__ long long unit_of_thread(int r, int k, int t, int rank, int size) {
  const long long slot = (long long)r * kChunksPerRound + k * (kPT / kChunk) + t / kChunk;
  return (rank + (long long)size * slot) * kChunk + (t % kChunk);
}

// Per-thread partials of the normal equations over this block's share of
// the target pixels at epoch e.
//
// Only the pixels whose key carries the epoch's tag (about one in ten at
// 640x480) contribute, and they are scattered over the warp's lanes: a
// warp that ran the residual and Jacobian on its own lanes' pixels would
// execute them for almost every pixel slot with a few lanes active.  So a
// round first reads the keys of the warp's kPR x 32 pixels, packs the
// matched ones (their slot and winning source index) into a per-warp list
// in ballot order, and then the warp's lanes take the list's entries in
// turn: the target point, normal and source point loads of all of a lane's
// entries are issued before the first use, and the arithmetic runs with
// full lanes.  The list order is fixed, so the sums are deterministic.
template <typename FT, bool kGeom, bool kFeat, bool kHWC, class X>
__device__ __forceinline__ void reduce_pixels(const X &J, const Pose32 &P, Share sh, int e,
                                              float *acc) {
  __shared__ unsigned s_list[kPW][kPR * 32];  // (source index << 8) | (slot << 5) | lane
  const unsigned tag = 254u - (unsigned)e;
  const int H = J.H, W = J.W;
  const long long npix = (long long)H * W;
  const unsigned long long *__restrict__ keys = J.keys;
  const float *__restrict__ sp = J.sp;
  const float *__restrict__ tp = J.tp;
  const float *__restrict__ tn = J.tn;
  const bool unit_w = J.wg1 == 1.f && J.wg2 == 1.f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rank = rank_of(J), size = size_of(J);
  unsigned *list = s_list[warp];
  for (int r = 0; r < sh.rounds; ++r) {
    unsigned long long key[kPR];
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      const long long pix = unit_of(r, k, rank, size);
      key[k] = pix < npix ? __ldcg(keys + pix) : 0ull;
    }
    int count = 0;
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      const bool match = (unsigned)(key[k] >> 56) == tag;
      const unsigned bal = __ballot_sync(0xffffffffu, match);
      if (match)
        list[count + __popc(bal & ((1u << lane) - 1u))] =
            ((unsigned)(key[k] & 0xffffffull) << 8) | ((unsigned)k << 5) | (unsigned)lane;
      count += __popc(bal);
    }
    __syncwarp();
    const int rounds = (count + 31) >> 5;  // warp-uniform, at most kPR
    int src[kPR];  // the entry's winning source point, -1 past the list
    float q[kPR][3], m[kPR][3], s[kPR][3];
#pragma unroll
    for (int j = 0; j < kPR; ++j) {
      if (j >= rounds) break;
      const int d = lane + 32 * j;
      const unsigned ent = d < count ? list[d] : 0u;
      const long long pc =
          d < count ? unit_of_thread(r, (ent >> 5) & 7u, warp * 32 + (ent & 31u), rank, size) : 0;
      src[j] = d < count ? (int)(ent >> 8) : -1;
      const long long ic = ent >> 8;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        q[j][c] = kGeom ? __ldg(tp + 3 * pc + c) : 0.f;
        m[j][c] = kGeom ? __ldg(tn + 3 * pc + c) : 0.f;
        s[j][c] = __ldg(sp + 3 * ic + c);
      }
    }
#pragma unroll
    for (int j = 0; j < kPR; ++j) {
      if (j >= rounds) break;
      if (src[j] < 0) continue;
      const long long i = src[j];
      const float3 Tp = transform_point(P.rt, s[j][0], s[j][1], s[j][2]);
      if (kGeom) {
        const float nx = m[j][0], ny = m[j][1], nz = m[j][2];
        const float rr = dot3(fsub(q[j][0], Tp.x), fsub(q[j][1], Tp.y), fsub(q[j][2], Tp.z), nx,
                              ny, nz);
        const float Jv[6] = {nx, ny, nz, fsub(fmul(Tp.y, nz), fmul(Tp.z, ny)),
                             fsub(fmul(Tp.z, nx), fmul(Tp.x, nz)),
                             fsub(fmul(Tp.x, ny), fmul(Tp.y, nx))};
        if (unit_w) {
          // unit weights (geometric weight 1, the default): w x (a b) is a b,
          // so each term is one FMA into the partial (no rounding of the
          // product; the teacher-forced 1e-5 gate holds either way)
#pragma unroll
          for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int c = a; c < 6; ++c)
              acc[upper_index(a, c)] = fmaf(Jv[a], Jv[c], acc[upper_index(a, c)]);
#pragma unroll
          for (int a = 0; a < 6; ++a) acc[kJr + a] = fmaf(Jv[a], rr, acc[kJr + a]);
          acc[kR2] = fmaf(rr, rr, acc[kR2]);
        } else {
          accumulate_se3(acc, Jv, rr, J.wg1, J.wg2);
          acc[kR2] += J.wg1 * (rr * rr);
        }
        acc[kCountGeom] += 1.f;
      }
      if (kFeat && J.use_feat) {
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
    __syncwarp();  // the list is rewritten by the next round
  }
}

// Information partials G^T G over this block's share of the target pixels
// at epoch e.
template <class X>
__device__ __forceinline__ void info_pixels(const X &J, Share sh, int e, float *acc) {
  const unsigned tag = 254u - (unsigned)e;
  const unsigned long long *__restrict__ keys = J.keys;
  const float *__restrict__ tp = J.tp;
  for (int slot = 0; slot < sh.rounds * kPR; ++slot) {
    const long long pix = unit_of(slot / kPR, slot % kPR, rank_of(J), size_of(J));
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

template <class X>
__device__ __forceinline__ float2 *slot_of(const X &J, int buf, int block) {
  return J.part + ((size_t)buf * size_of(J) + block) * kSlotAccs;
}

template <class X>
__device__ __forceinline__ void poison_slot(const X &J, int buf) {
  if (threadIdx.x < kSlotAccs)
    st_relaxed_f2(slot_of(J, buf, rank_of(J)) + threadIdx.x,
                  make_float2(__uint_as_float(kPoison), __uint_as_float(kPoison)));
}

// Totals of kN accumulators over the grid's slots of buffer buf into L.tot
// (FP64) and L.totw (double-words), in every block in the same order: warp
// w merges slots w, w + 16, ... with lane = accumulator, then the warps'
// sums are merged in warp order.  poll: the slots may still be arriving
// (reload a slot while any of its words holds kPoison, at most
// J.spin_limit times); otherwise a grid barrier has ordered them.  Returns
// false when a poll gave up (here or, seen on the error word, elsewhere).
template <int kN, class X>
__device__ __forceinline__ bool fold_slots(const X &J, LoopShared &L, int buf, bool poll) {
  __shared__ float2 wsum[kPW][32];
  __shared__ int s_fail[kPW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  CSum t = {0.f, 0.f};
  bool fail = false;
  // slots per warp in one round of loads: a grid of up to 192 blocks is
  // folded with every load in flight at once
  constexpr int kLoads = 12;
  for (int b0 = warp; b0 < size_of(J) && !fail; b0 += kPW * kLoads) {
    float2 v[kLoads];
#pragma unroll
    for (int k = 0; k < kLoads; ++k) {
      const int b = b0 + k * kPW;
      v[k] = (b < size_of(J) && lane < kN) ? ld_relaxed_f2(slot_of(J, buf, b) + lane)
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
          if (lane == 0) atomicOr(err_word(J), 1u);
          fail = true;
          break;
        }
        if ((spins & 63u) == 0 && ld_relaxed(err_word(J))) {
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

// Sums of kN (<= 32) per-thread partials over the warp, by a transposing
// butterfly: at the level of offset o each lane keeps half of its values
// (the upper half where lane bit o is set), sends the other half to lane
// ^ o and adds what it receives, so after five levels lane a holds the
// warp's sum of partial a: 31 exchanges a lane, where a reduction per
// partial costs 5 x kN.  The first two levels add in plain float32 (sums
// of four threads' partials, as a thread's own partial of kPR pixels); from
// the third level on the sums are compensated (TwoSum, the carried error
// exchanged with the sum), so lane a ends with the (sum, error) pair.
template <int kN>
__device__ __forceinline__ CSum warp_transpose_sum(const float *acc, int lane) {
  float v[32];
#pragma unroll
  for (int a = 0; a < 32; ++a) v[a] = a < kN ? acc[a] : 0.f;
#pragma unroll
  for (int o = 16, n = 32; o >= 8; o >>= 1, n >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int j = 0; j < n / 2; ++j) {
      const float send = up ? v[j] : v[j + n / 2];
      const float keep = up ? v[j + n / 2] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  // offset 4: 8 values -> 4 compensated pairs
  CSum c[4];
  {
    const bool up = (lane & 4) != 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float send = up ? v[j] : v[j + 4];
      const float keep = up ? v[j + 4] : v[j];
      two_sum(keep, __shfl_xor_sync(0xffffffffu, send, 4), c[j].s, c[j].c);
    }
  }
  // offsets 2 and 1: pairs merged with their errors
#pragma unroll
  for (int o = 2, n = 4; o >= 1; o >>= 1, n >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int j = 0; j < n / 2; ++j) {
      const CSum send = up ? c[j] : c[j + n / 2];
      CSum keep = up ? c[j + n / 2] : c[j];
      csum_merge(keep, __shfl_xor_sync(0xffffffffu, send.s, o),
                 __shfl_xor_sync(0xffffffffu, send.c, o));
      c[j] = keep;
    }
  }
  return c[0];
}

// This block's sums of kN per-thread partials into its slot of buffer buf:
// each warp's compensated totals by warp_transpose_sum, then the kPW warp
// totals of a partial merged in warp order.
template <int kN, class X>
__device__ __forceinline__ void write_slot(const X &J, const float *acc, int buf) {
  __shared__ float2 wtot[kPW][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const CSum w = warp_transpose_sum<kN>(acc, lane);
  wtot[warp][lane] = make_float2(w.s, w.c);
  __syncthreads();
  if (threadIdx.x < kN) {
    CSum t = {wtot[0][threadIdx.x].x, wtot[0][threadIdx.x].y};
#pragma unroll
    for (int k = 1; k < kPW; ++k) csum_merge(t, wtot[k][threadIdx.x].x, wtot[k][threadIdx.x].y);
    st_relaxed_f2(slot_of(J, buf, rank_of(J)) + threadIdx.x, make_float2(t.s, t.c));
  }
}


}  // namespace fused
}  // namespace stb
