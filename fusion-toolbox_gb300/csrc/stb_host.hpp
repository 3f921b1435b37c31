// Host-side helpers shared by the C-ABI translation units: the per-thread
// error message, argument checks and launch checks.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "slamtb_gb300.h"

namespace stb {

// Records a printf-style message for stb_last_error() and returns `code`.
int fail(int code, const char *fmt, ...);

// Clears the message (start of every entry point).
void clear_error();

// STB_EDEVICE unless `p` is device (or managed) memory of the current device.
// Messages keep the reference's wording: "Check failed: <where>: Expected a
// gpu tensor" (include/slamtb/error.hpp:12-37).
int check_device_ptr(const void *p, const char *name, bool allow_null = false);

// For small inputs whose values a call reads on the host (intrinsics, an
// initial pose): device memory of the current device (*on_host = false), or
// host memory, pinned or pageable (*on_host = true).
int check_small_input(const void *p, const char *name, bool allow_null, bool *on_host);

// STB_ECUDA with the CUDA error string if the last launch failed.
int check_launch(const char *what);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// The test limits of the kernels' bounded grid-barrier waits set by
// stb_set_wait_test_limits: polls before a wait gives up (0: the kernel's
// default) and phantom arrivals (0: none).
void wait_test_limits(unsigned *spin_limit, int *phantom);

inline unsigned blocks_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

}  // namespace stb

#define STB_TRY(expr)            \
  do {                           \
    const int _rc = (expr);      \
    if (_rc != STB_OK) return _rc; \
  } while (0)
