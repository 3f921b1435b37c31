// RegistrationVerifier (slamtb/registration/result.py:49-95) for many
// result blocks on the device: a registration is accepted when
//   residual <= residual_thresh,
//   no eigenvalue of information^-1 exceeds covariance_max_thresh, and
//   matches / num_source >= match_ratio_thresh
// (the reference's tests in its order; a NaN residual passes the first, as
// there).  The covariance test needs no eigen-decomposition: for the
// symmetric positive semi-definite information matrix A, an eigenvalue of
// A^-1 above c means an eigenvalue of A below 1 / c, that is A - I / c is
// not positive definite, which an LDL^T factorisation of A - I / c in FP64
// decides (a pivot that is not > 0 rejects).  An eigenvalue exactly at the
// threshold, where the reference accepts, rejects here.
#include <math.h>

#include "stb_common.cuh"
#include "stb_host.hpp"
#include "slamtb_gb300.h"

namespace stb {
namespace {

// A - s I positive definite, for a symmetric 6x6 A (row-major), by LDL^T.
__device__ bool shifted_positive_definite(const double *A, double s) {
  double L[6][6], d[6];
  for (int j = 0; j < 6; ++j) {
    double v = A[j * 6 + j] - s;
    for (int k = 0; k < j; ++k) v -= L[j][k] * L[j][k] * d[k];
    if (!(v > 0.0)) return false;  // also NaN
    d[j] = v;
    for (int i = j + 1; i < 6; ++i) {
      double w = A[i * 6 + j];
      for (int k = 0; k < j; ++k) w -= L[i][k] * L[j][k] * d[k];
      L[i][j] = w / v;
    }
  }
  return true;
}

__global__ void k_verify(const double *__restrict__ results, const int64_t *__restrict__ num_source,
                         int n, double match_ratio_thresh, double covariance_max_thresh,
                         double residual_thresh, int32_t *__restrict__ verdict) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const double *R = results + (size_t)p * STB_RES_SIZE;
  bool ok = !(R[STB_RES_RESIDUAL] > residual_thresh);
  if (ok) {
    // a threshold <= 0 is below every eigenvalue of the inverse of a
    // positive definite information matrix
    double A[36];
    for (int k = 0; k < 36; ++k) A[k] = R[STB_RES_INFO + k];
    ok = covariance_max_thresh > 0.0 &&
         shifted_positive_definite(A, 1.0 / covariance_max_thresh);
  }
  if (ok) {
    const double ratio = R[STB_RES_MATCHES] / (double)num_source[p];
    ok = !(ratio < match_ratio_thresh);
  }
  verdict[p] = ok ? 1 : 0;
}

}  // namespace
}  // namespace stb

using namespace stb;

extern "C" int stb_verify_registrations(const double *results, const int64_t *num_source,
                                        int32_t num_results, double match_ratio_thresh,
                                        double covariance_max_thresh, double residual_thresh,
                                        int32_t *verdict, void *stream) {
  clear_error();
  if (num_results <= 0)
    return fail(STB_EINVAL, "Check failed: num_results must be positive, got %d", num_results);
  STB_TRY(check_device_ptr(results, "results"));
  STB_TRY(check_device_ptr(num_source, "num_source"));
  STB_TRY(check_device_ptr(verdict, "verdict"));
  k_verify<<<(num_results + 127) / 128, 128, 0, as_stream(stream)>>>(
      results, num_source, num_results, match_ratio_thresh, covariance_max_thresh,
      residual_thresh, verdict);
  return check_launch("stb_verify_registrations");
}
