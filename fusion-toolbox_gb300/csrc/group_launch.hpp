// Host-side interface of the grouped batch kernel (icp_group.cu), called by
// stb_icp_estimate_batch (icp_batch.cu) when STB_OPT_GROUPS is set.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "slamtb_gb300.h"

namespace stb {
namespace fused {

constexpr int kGroupMaxLevels = 4;
// Most groups of one launch (the barrier words of the workspace's sync
// region have room for this many).
constexpr int kMaxGroups = 96;
// Most blocks of one grouped launch: the slot buffers of the workspace are
// sized for this many.
constexpr int kGroupMaxBlocks = 1024;

// One level's estimator, in the kernels' float32 terms.
struct GroupLevelParams {
  int iters, use_geom, use_feat;
  float wg1, wg2, wf1, wf2, thr2, cos_max, feat_thr2;
};

struct GroupLaunch {
  const stb_level *levels;
  int B, L, C, dtype, mode, total_iters, solve_dw;
  GroupLevelParams lp[kGroupMaxLevels];
  const double *init;
  double *results, *history;
  unsigned spin_limit;
  int bar_phantom;
  unsigned *sync;          // 16 KB of barrier words, zeroed before the launch
  long long *key_off;      // [B + 1]
  int *order;              // [B]
  float2 *part;            // [kGroupMaxBlocks][2][kSlotAccs] float2
  unsigned long long *keys;
  long long keys_cap;
  int groups;              // requested groups (1 .. kMaxGroups)
};

// Enqueues the grouped kernel and the status pass on st.
int launch_grouped(const GroupLaunch &g, cudaStream_t st);

}  // namespace fused
}  // namespace stb
