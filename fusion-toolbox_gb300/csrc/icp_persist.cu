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

#include "persist_phases.cuh"
#include "stb_host.hpp"

namespace stb {
namespace fused {

// The single-pair kernel's blocks are the grid; its barrier words are in
// the workspace's State.
__device__ __forceinline__ int rank_of(const Job &) { return blockIdx.x; }
__device__ __forceinline__ int size_of(const Job &) { return gridDim.x; }
__device__ __forceinline__ unsigned *bar_word(const Job &J) { return &J.state->bar_count; }
__device__ __forceinline__ unsigned *err_word(const Job &J) { return &J.state->bar_err; }

namespace {

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

extern __shared__ __align__(16) float s_dyn_p[];

template <typename FT, bool kGeom, bool kFeat, bool kHWC>
__global__ void __launch_bounds__(kPT, 1) k_persist(const __grid_constant__ Job J) {
  __shared__ LoopShared L;
  const int lane = threadIdx.x & 31;
  const long long n = J.n, npix = (long long)J.H * J.W;
  const long long G = gridDim.x, b = blockIdx.x;
  const long long pc = (npix + G - 1) / G;
  const long long p0 = min(npix, b * pc), p1 = min(npix, p0 + pc);
  const Share src = share_of(n, blockIdx.x, gridDim.x);
  const Share tgt = share_of(npix, blockIdx.x, gridDim.x);
  SrcCache C;
  C.rounds = min(J.src_cache_rounds, src.rounds);
  C.cap = J.src_cache_rounds * kPR * kPT;
  C.f = s_dyn_p;
  C.m = reinterpret_cast<uint8_t *>(C.f + 6 * C.cap);

  // set-up: the initial pose in every block; this block's key-map range
  // cleared (a key of an earlier registration may carry a current tag);
  // its source points copied to the cache; its slots of both buffers
  // poisoned
  for (int r = 0; r < C.rounds; ++r) {
#pragma unroll
    for (int k = 0; k < kPR; ++k) {
      const long long i = unit_of(r, k, blockIdx.x, gridDim.x);
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
  // this block's range of the target frame into L2 (128-byte lines): the
  // first association's gathers then hit L2 instead of memory
  if (p1 > p0) {
    const char *pt = reinterpret_cast<const char *>(J.tp + 3 * p0);
    const char *pn = reinterpret_cast<const char *>(J.tn + 3 * p0);
    const long long nb = 12 * (p1 - p0);
    for (long long off = 128ll * threadIdx.x; off < nb; off += 128ll * kPT) {
      prefetch_l2(pt + off);
      prefetch_l2(pn + off);
    }
    for (long long off = 128ll * threadIdx.x; off < p1 - p0; off += 128ll * kPT)
      prefetch_l2(J.tm + p0 + off);
  }
  unsigned nbar = 0;  // grid barriers passed
  bool alive = group_barrier(J, nbar++, true);

  int used = 0;  // iterations that wrote and folded their slots
  for (int iter = 0; alive && iter < J.iters; ++iter) {
    associate(J, L.P, src, C, iter);
    if (!(alive = group_barrier(J, nbar++, true))) break;
    float acc[kAccs];
#pragma unroll
    for (int a = 0; a < kAccs; ++a) acc[a] = 0.f;
    reduce_pixels<FT, kGeom, kFeat, kHWC>(J, L.P, tgt, iter, acc);
    // every block has folded the previous iteration's buffer (it passed the
    // barrier above after its fold): poisoned again for the next iteration
    if (iter > 0) poison_slot(J, (iter + 1) & 1);
    write_slot<kAccs>(J, acc, iter & 1);
    if (!(alive = fold_slots<kAccs>(J, L, iter & 1, true))) break;
    ++used;
    if (threadIdx.x < 32) persist_step(J, L, iter, lane);
    __syncthreads();
    if (!L.ok) break;  // a failed solve ends the loop (icp.py:241-242 `except: break`)
  }

  // the association at the final pose and the information sum
  if (alive) {
    associate(J, L.P, src, C, J.iters);
    alive = group_barrier(J, nbar++, true);
  }
  // the information sums go to the slot buffer the next iteration would
  // have used: poisoned (at the set-up, or after the last iteration's
  // association barrier), so block 0 folds them as they land and no block
  // waits at a last barrier
  if (alive) {
    float acc[kInfoAccs];
#pragma unroll
    for (int a = 0; a < kInfoAccs; ++a) acc[a] = 0.f;
    info_pixels(J, tgt, J.iters, acc);
    write_slot<kInfoAccs>(J, acc, used & 1);
  }
  if (blockIdx.x != 0) return;
  double *R = J.result;
  if (alive) alive = fold_slots<kInfoAccs>(J, L, used & 1, true);
  if (alive) {
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

// Dynamic shared memory: the source-point cache of Job::src_cache_rounds
// rounds.
constexpr size_t cache_smem(int rounds) {
  return ((size_t)rounds * kPR * kPT * kCachePointBytes + 15) & ~size_t(15);
}
constexpr size_t kPersistSmem = cache_smem(kMaxCacheRounds);
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
  cfg.dynamicSmemBytes = cache_smem(job.src_cache_rounds);
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
