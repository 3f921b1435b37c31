// Read-back of the registration kernels' per-pixel key maps in the
// reference's correspondence-map layout.
//
// The fused, batched and loss kernels keep one 64-bit key per target pixel:
//   bits 56..63  epoch tag (254 - the association's step; older steps' keys
//                read as empty, so a map is cleared once per call)
//   bits 24..54  float32 bits of the distance (non-negative, 31 bits)
//   bits  0..23  source index
// and a 64-bit atomicMin keeps the lexicographic (distance, index) minimum.
// The reference's map (slamtb/registration/correspondence_map.py:5,66-70,
// src/merge_map.hpp:54-98) holds (source index << 32) | distance bits, with
// 0x0fffffff7f800000 for a pixel without a correspondence.
#pragma once

#include <stdint.h>

namespace stb {
namespace {

constexpr long long kEmptyMergeEntry = 0x0fffffff7f800000ll;

// out[k] = the reference-layout entry of keys[base + k] for k < n, where
// base = *key_base (a device word) when key_base is given, else 0; keys of
// another tag than `tag` read as empty.
__global__ void k_keys_to_merge_map(const unsigned long long *__restrict__ keys,
                                    const long long *key_base, long long n, unsigned tag,
                                    long long *__restrict__ out) {
  const long long base = key_base ? *key_base : 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += stride) {
    const unsigned long long key = keys[base + k];
    long long v = kEmptyMergeEntry;
    if ((unsigned)(key >> 56) == tag) {
      const long long idx = (long long)(key & 0xffffffull);
      const long long dist = (long long)((key >> 24) & 0x7fffffffull);
      v = (idx << 32) | dist;
    }
    out[k] = v;
  }
}

inline unsigned keys_grid(long long n) {
  long long b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)b;
}

}  // namespace
}  // namespace stb
