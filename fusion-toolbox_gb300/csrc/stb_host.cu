// Error state and argument checks of the C ABI.
#include <stdarg.h>
#include <stdio.h>

#include "stb_host.hpp"

namespace stb {

static thread_local char g_message[512];

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_message, sizeof(g_message), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() { g_message[0] = '\0'; }

// Recently validated device pointers of this thread (a tracker passes the
// same buffers every frame): a hit skips cudaPointerGetAttributes.  Only pointers
// that passed as device memory of the current device are remembered, so a
// host pointer is always queried and refused.
struct PtrCacheEntry {
  const void *p;
  int dev;
};
static thread_local PtrCacheEntry g_ptr_cache[32];
static thread_local int g_ptr_next = 0;

int check_device_ptr(const void *p, const char *name, bool allow_null) {
  if (p == nullptr) {
    if (allow_null) return STB_OK;
    return fail(STB_EINVAL, "Check failed: %s: null pointer", name);
  }
  int dev = -1;
  cudaGetDevice(&dev);
  for (const PtrCacheEntry &e : g_ptr_cache)
    if (e.p == p && e.dev == dev) return STB_OK;
  cudaPointerAttributes attr;
  const cudaError_t err = cudaPointerGetAttributes(&attr, p);
  if (err != cudaSuccess) {
    cudaGetLastError();
    return fail(STB_EDEVICE, "Check failed: %s: Expected a gpu tensor (%s)", name,
                cudaGetErrorString(err));
  }
  if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
    return fail(STB_EDEVICE, "Check failed: %s: Expected a gpu tensor", name);
  if (attr.device != dev)
    return fail(STB_EDEVICE,
                "Check failed: %s: Expected a tensor on cuda:%d, got cuda:%d", name,
                dev, attr.device);
  g_ptr_cache[g_ptr_next] = PtrCacheEntry{p, dev};
  g_ptr_next = (g_ptr_next + 1) % 32;
  return STB_OK;
}

int check_small_input(const void *p, const char *name, bool allow_null, bool *on_host) {
  *on_host = false;
  if (p == nullptr) return allow_null ? STB_OK : fail(STB_EINVAL, "Check failed: %s: null pointer", name);
  int dev = -1;
  cudaGetDevice(&dev);
  for (const PtrCacheEntry &e : g_ptr_cache)
    if (e.p == p && e.dev == dev) return STB_OK;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return fail(STB_EDEVICE, "Check failed: %s: not a host or device address", name);
  }
  if (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeUnregistered) {
    *on_host = true;
    return STB_OK;
  }
  return check_device_ptr(p, name, false);
}

int check_launch(const char *what) {
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess)
    return fail(STB_ECUDA, "Cuda call error %s: %s", what, cudaGetErrorString(err));
  return STB_OK;
}

}  // namespace stb

extern "C" const char *stb_last_error(void) { return stb::g_message; }

extern "C" const char *stb_version(void) { return "slamtb_gb300 0.1 (sm_103a)"; }
