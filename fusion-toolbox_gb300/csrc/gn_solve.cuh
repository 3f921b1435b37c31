// Gauss-Newton step on the device: 6x6 LDL^T solve, SE(3) exponential,
// left pose update, and the float32 pose view for the next association.
// Replaces the host code of the reference loop
// (slamtb/registration/icp.py:236-256: torch.cholesky + cholesky_solve on
// the CPU, tenviz SE3.exp, transform = update @ transform).
#pragma once

#include "stb_common.cuh"

namespace stb {

// Coefficients of the SE(3) exponential, A = sin t / t, B = (1 - cos t) / t^2,
// C = (t - sin t) / t^3, of t2 = t^2.  Below t = 0.5 (every Gauss-Newton
// update of a registration that converges) they are their Maclaurin series in
// t^2 through t^14, evaluated by Horner's rule: 7 dependent FMAs instead of
// sincos and three divisions; the first omitted term is below
// 0.5^16 / 17! < 5e-20 of the sum.  Above, the closed forms.
__device__ __forceinline__ void se3_coeffs(double t2, double &A, double &B, double &C) {
  if (t2 < 0.25) {
    // A_k = (-1)^k / (2k+1)!, B_k = (-1)^k / (2k+2)!, C_k = (-1)^k / (2k+3)!
    double a = -1.0 / 1307674368000.0, b = -1.0 / 20922789888000.0,
           c = -1.0 / 355687428096000.0;
    a = fma(a, t2, 1.0 / 6227020800.0);
    b = fma(b, t2, 1.0 / 87178291200.0);
    c = fma(c, t2, 1.0 / 1307674368000.0);
    a = fma(a, t2, -1.0 / 39916800.0);
    b = fma(b, t2, -1.0 / 479001600.0);
    c = fma(c, t2, -1.0 / 6227020800.0);
    a = fma(a, t2, 1.0 / 362880.0);
    b = fma(b, t2, 1.0 / 3628800.0);
    c = fma(c, t2, 1.0 / 39916800.0);
    a = fma(a, t2, -1.0 / 5040.0);
    b = fma(b, t2, -1.0 / 40320.0);
    c = fma(c, t2, -1.0 / 362880.0);
    a = fma(a, t2, 1.0 / 120.0);
    b = fma(b, t2, 1.0 / 720.0);
    c = fma(c, t2, 1.0 / 5040.0);
    a = fma(a, t2, -1.0 / 6.0);
    b = fma(b, t2, -1.0 / 24.0);
    c = fma(c, t2, -1.0 / 120.0);
    A = fma(a, t2, 1.0);
    B = fma(b, t2, 0.5);
    C = fma(c, t2, 1.0 / 6.0);
    return;
  }
  const double t = sqrt(t2);
  double s, c;
  sincos(t, &s, &c);
  A = s / t;
  B = (1.0 - c) / t2;
  C = (t - s) / (t2 * t);
}

// SE(3) exponential of a twist [v; w] (translation first, the order fixed by
// the Jacobian J = [n; p x n]): R = I + A W + B W^2, t = (I + B W + C W^2) v
// with the coefficients of se3_coeffs.  Writes a row-major 4x4.
__device__ inline void se3_exp(const double xi[6], double E[16]) {
  const double wx = xi[3], wy = xi[4], wz = xi[5];
  const double t2 = wx * wx + wy * wy + wz * wz;
  double A, B, C;
  se3_coeffs(t2, A, B, C);
  // W = hat(w), W2 = W W
  const double W[9] = {0.0, -wz, wy, wz, 0.0, -wx, -wy, wx, 0.0};
  double W2[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      W2[i * 3 + j] = W[i * 3 + 0] * W[0 * 3 + j] + W[i * 3 + 1] * W[1 * 3 + j] +
                      W[i * 3 + 2] * W[2 * 3 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double id = (i == j) ? 1.0 : 0.0;
      E[i * 4 + j] = id + A * W[i * 3 + j] + B * W2[i * 3 + j];
      t += (id + B * W[i * 3 + j] + C * W2[i * 3 + j]) * xi[j];
    }
    E[i * 4 + 3] = t;
  }
  E[12] = 0.0;
  E[13] = 0.0;
  E[14] = 0.0;
  E[15] = 1.0;
}

// Out = E * T for row-major 4x4 rigid transforms (last row 0 0 0 1).
__device__ inline void compose(const double E[16], const double T[16], double Out[16]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double s = E[i * 4 + 0] * T[0 * 4 + j] + E[i * 4 + 1] * T[1 * 4 + j] +
                 E[i * 4 + 2] * T[2 * 4 + j];
      if (j == 3) s += E[i * 4 + 3];
      Out[i * 4 + j] = s;
    }
  }
  Out[12] = 0.0;
  Out[13] = 0.0;
  Out[14] = 0.0;
  Out[15] = 1.0;
}

// float32 view of an FP64 pose: the cast transform.to(float32) of
// icp.py:53,61 and the normal matrix of RigidTransform's constructor.
__device__ inline void refresh_pose32(Pose32 &P, const double T[16]) {
#pragma unroll
  for (int k = 0; k < 12; ++k) P.rt[k] = __double2float_rn(T[k]);
  inverse_transpose(P.rt, P.nm);
}

// Upper-triangle index of (a, b), a <= b, in the 21-entry packed J^T J.
__host__ __device__ constexpr int upper_index(int a, int b) {
  return a * 6 - a * (a - 1) / 2 + (b - a);
}

}  // namespace stb

// ---------------------------------------------------------------------------
// Gauss-Newton step by one warp, in double-word arithmetic on the FP32 pipes
// (opt-in, STB_OPT_DW_SOLVE; the default is the FP64 step further below).
//
// On this part every FP64 warp instruction (arithmetic, comparisons and
// conversions alike) occupies the FP64 pipe of its SM sub-partition for 64
// cycles whatever its lanes, and independent FP64 instructions of one warp
// do not overlap, so a step written in FP64 costs its FP64 instruction
// count (~55 of them: ~3 us at the end of every iteration).  A double-word value is the unevaluated
// sum hi + lo of two float32 with |lo| <= ulp(hi) / 2: ~48 significant bits
// from float32 additions, multiplications and FMAs at 4 cycles each.  The
// error-free transforms are Fast2Sum (Dekker), 2Sum (Knuth) and 2Prod by
// FMA; the sum and the product are Algorithm 6 (AccurateDWPlusDW, relative
// error <= 3u^2) and Algorithm 12 (DWTimesDW3, <= 4u^2) of Joldes, Muller
// and Popescu, "Tight and rigorous error bounds for basic building blocks
// of double-word arithmetic", ACM TOMS 44(2), 2017, u = 2^-24.
// ---------------------------------------------------------------------------
namespace stb {

struct dw {
  float hi, lo;
};

// s + t = a + b exactly, for |a| >= |b| (or a == 0).
__device__ __forceinline__ dw fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dw two_sum_dw(float a, float b) {
  dw r;
  two_sum(a, b, r.hi, r.lo);
  return r;
}

// Normalised double-word of a compensated sum (s, c).
__device__ __forceinline__ float2 dw_of_csum(float s, float c) {
  const dw r = two_sum_dw(s, c);
  return make_float2(r.hi, r.lo);
}

__device__ __forceinline__ dw dw_add(dw x, dw y) {
  const dw s = two_sum_dw(x.hi, y.hi), t = two_sum_dw(x.lo, y.lo);
  const dw v = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}

__device__ __forceinline__ dw dw_mul(dw x, dw y) {
  const float ch = __fmul_rn(x.hi, y.hi);
  const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
  const float tl1 = __fmaf_rn(x.hi, y.lo, __fmul_rn(x.lo, y.lo));
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
  return fast_two_sum(ch, __fadd_rn(cl1, cl2));
}

// x - y z
__device__ __forceinline__ dw dw_sub_mul(dw x, dw y, dw z) {
  const dw p = dw_mul(y, z);
  return dw_add(x, dw{-p.hi, -p.lo});
}

// 1 / d for d > 0: rcp.approx.ftz.f32 (relative error ~2^-23) and one
// Newton-Raphson step y (1 + e), e = 1 - d y formed exactly enough (d.hi y
// by 2Prod; 1 - ph is exact, ph being within a factor 2 of 1), which
// squares the error to ~2^-46.  A subnormal d.hi flushes to an infinite
// reciprocal, which turns the solution into NaN (flagged by the caller).
__device__ __forceinline__ dw dw_rcp(dw d) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(d.hi));
  const float ph = __fmul_rn(d.hi, y);
  const float pl = __fmaf_rn(d.hi, y, -ph);
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, ph), pl), __fmul_rn(d.lo, y));
  return fast_two_sum(y, __fmul_rn(y, e));
}

__device__ __forceinline__ dw shfl_dw(dw v, int src) {
  return {__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

// d > 0 on the integer bits (false for +-0, negatives and NaN; +inf
// passes, as the comparison does).  For a normalised double-word the sign
// and finiteness of hi are those of the value.
__device__ __forceinline__ bool positive_bits(float d) {
  const int b = __float_as_int(d);
  return b > 0 && b <= 0x7f800000;
}

// Lane of entry (i, k), k <= i, of the 6x6 lower triangle stored column by
// column (column k starts at 6k - k(k-1)/2); right-hand side entry i is on
// lane 21 + i.
__host__ __device__ constexpr int tri_lane(int i, int k) { return 6 * k - k * (k - 1) / 2 + (i - k); }

// Maclaurin coefficient n (in t^2) of A = sin t / t (which = 0),
// B = (1 - cos t) / t^2 (1) or C = (t - sin t) / t^3 (2): (-1)^n / (2n + 1 +
// which)!, n < 8, as a double-word constant (hi = the float32 rounding, lo =
// the float32 rounding of the remainder).  n is a compile-time constant,
// which a per-lane select.
template <int n>
__device__ __forceinline__ dw se3_series_coeff_dw(int which) {
  constexpr double f[18] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0, 40320.0, 362880.0,
                            3628800.0, 39916800.0, 479001600.0, 6227020800.0, 87178291200.0,
                            1307674368000.0, 20922789888000.0, 355687428096000.0};
  constexpr double s = (n & 1) ? -1.0 : 1.0;
  constexpr double c[3] = {s / f[2 * n + 1], s / f[2 * n + 2], s / f[2 * n + 3]};
  constexpr float h0 = (float)c[0], h1 = (float)c[1], h2 = (float)c[2];
  constexpr float l0 = (float)(c[0] - (double)h0), l1 = (float)(c[1] - (double)h1),
                  l2 = (float)(c[2] - (double)h2);
  return which == 0 ? dw{h0, l0} : (which == 1 ? dw{h1, l1} : dw{h2, l2});
}

// FP64 value -> normalised double-word.
__device__ __forceinline__ float2 dw_of_double(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}

// One Gauss-Newton update by one warp (all 32 lanes call it), in
// double-words: the opt-in variant of warp_gn_update below.
//   up: the 21 packed upper-triangle entries of J^T J and bv: J^T r (6),
//       normalised double-words (hi, lo) in shared memory;
//   T: the current pose as double-words (16, row-major, shared).
// Solves J^T J x = J^T r by LDL^T with the failure rule of LAPACK potrf (a
// pivot that is not > 0, or NaN, fails: the LDL^T pivots are the squares of
// the Cholesky pivots), one lane per triangle entry and one per right-hand
// side entry, so that a column step is one product and one difference for
// all entries.  Then Tn = exp(x) T, also in double-words: within ~1e-14 of
// the FP64 update, so the float32 view of the pose (its high words) is
// that of the FP64 pose.  Returns the solve status (warp-uniform); on success lanes
// 0..15 hold Tn's entries in tn_out (lane k -> entry k), and every lane
// holds x rounded to float32 in xs (for the finiteness test).
__device__ inline bool warp_gn_update_dw(const float2 *up, const float2 *bv, const float2 *T,
                                         float *xs, float2 &tn_out, int lane) {
  // this lane's entry (i, k); k == 6 marks the right-hand side
  int ei = 0, ek = 0;
  if (lane < 21) {
    int k = 0, first = 0;
    while (lane >= first + (6 - k)) {
      first += 6 - k;
      ++k;
    }
    ek = k;
    ei = k + (lane - first);
  } else if (lane < 27) {
    ei = lane - 21;
    ek = 6;
  }
  const bool is_rhs = (lane >= 21 && lane < 27);
  const bool is_tri = lane < 21;
  dw v = {0.f, 0.f};
  if (is_tri) {
    const float2 a = up[upper_index(ek, ei)];
    v = {a.x, a.y};
  }
  if (is_rhs) {
    const float2 b = bv[ei];
    v = {b.x, b.y};
  }
  bool ok = true;
  // forward: LDL^T factorisation with L z = b and y = D^-1 z fused in
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const dw piv = shfl_dw(v, tri_lane(j, j));
    ok = ok && positive_bits(piv.hi);
    const dw inv = dw_rcp(piv);
    const int src_i = (ei >= j) ? tri_lane(ei, j) : 0;
    const int src_k = is_rhs ? 21 + j : ((ek >= j && ek < 6) ? tri_lane(ek, j) : 0);
    const dw aij = shfl_dw(v, src_i);
    const dw akj = shfl_dw(v, src_k);
    const bool own_y = is_rhs && ei == j;
    const dw t = dw_mul(own_y ? v : aij, inv);  // L_ij, or y_j on the rhs lane j
    const bool upd = (is_tri && ek > j && ei >= ek) || (is_rhs && ei > j);
    const dw nv = dw_sub_mul(v, t, akj);
    if (upd) v = nv;
    if ((is_tri && ek == j && ei > j) || own_y) v = t;
  }
  if (!ok) return false;
  // backward: L^T x = y; rhs lane i ends with x_i
#pragma unroll
  for (int j = 5; j >= 0; --j) {
    const dw xj = shfl_dw(v, 21 + j);
    xs[j] = xj.hi;
    if (j > 0) {
      const int src = (is_rhs && ei < j) ? tri_lane(j, ei) : 0;
      const dw lji = shfl_dw(v, src);
      const dw nv = dw_sub_mul(v, lji, xj);
      if (is_rhs && ei < j) v = nv;
    }
  }
  dw x[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) x[k] = shfl_dw(v, 21 + k);
  // exp(x).  Below t = 0.5 the coefficients A = sin t / t, B = (1 - cos t) /
  // t^2, C = (t - sin t) / t^3 are their Maclaurin series in t^2 through
  // t^12 (the first omitted term is below 0.5^14 / 15! < 5e-17), the three
  // at once on three lane groups by Horner's rule: the terms from t^8 on in
  // float32 (each below 6e-16 of its rounding), the rest in double-words.
  // Above, the FP64 closed forms.
  const dw wx = x[3], wy = x[4], wz = x[5];
  const dw t2 = dw_add(dw_add(dw_mul(wx, wx), dw_mul(wy, wy)), dw_mul(wz, wz));
  dw A, B, C;
  if (t2.hi < 0.25f) {
    const int which = lane < 10 ? 0 : (lane < 20 ? 1 : 2);
    const float th = t2.hi;
    const float tail = __fmaf_rn(__fmaf_rn(se3_series_coeff_dw<6>(which).hi, th,
                                           se3_series_coeff_dw<5>(which).hi),
                                 th, se3_series_coeff_dw<4>(which).hi);
    dw coef = {tail, 0.f};
    coef = dw_add(dw_mul(coef, t2), se3_series_coeff_dw<3>(which));
    coef = dw_add(dw_mul(coef, t2), se3_series_coeff_dw<2>(which));
    coef = dw_add(dw_mul(coef, t2), se3_series_coeff_dw<1>(which));
    coef = dw_add(dw_mul(coef, t2), se3_series_coeff_dw<0>(which));
    A = shfl_dw(coef, 0);
    B = shfl_dw(coef, 10);
    C = shfl_dw(coef, 20);
  } else {
    double Ad, Bd, Cd;
    se3_coeffs((double)t2.hi + (double)t2.lo, Ad, Bd, Cd);
    const float2 a2 = dw_of_double(Ad), b2 = dw_of_double(Bd), c2 = dw_of_double(Cd);
    A = {a2.x, a2.y};
    B = {b2.x, b2.y};
    C = {c2.x, c2.y};
  }
  // lanes 0..8 hold R_ac = I + A W + B W^2, lanes 9..17 V_ac = I + B W + C W^2
  const int e = lane < 9 ? lane : (lane < 18 ? lane - 9 : 0);
  const int ea = e / 3, ec = e % 3;
  const dw wa = ea == 0 ? wx : (ea == 1 ? wy : wz);
  const dw wc = ec == 0 ? wx : (ec == 1 ? wy : wz);
  // W = hat(w): W_01 = -wz, W_02 = wy, W_10 = wz, W_12 = -wx, W_20 = -wy, W_21 = wx
  const dw nwx = {-wx.hi, -wx.lo}, nwy = {-wy.hi, -wy.lo}, nwz = {-wz.hi, -wz.lo};
  const dw zero = {0.f, 0.f};
  const dw Wac = e == 1 ? nwz : e == 2 ? wy : e == 3 ? wz : e == 5 ? nwx : e == 6 ? nwy
               : e == 7 ? wx : zero;
  const bool diag = (ea == ec);
  const dw ww = dw_mul(wa, wc);
  const dw W2ac = diag ? dw_add(ww, dw{-t2.hi, -t2.lo}) : ww;  // W^2 = w w^T - |w|^2 I
  const bool isR = lane < 9;
  dw val = dw_add(dw_mul(isR ? A : B, Wac), dw_mul(isR ? B : C, W2ac));
  if (diag) val = dw_add(val, dw{1.f, 0.f});
  // t_a = sum_c V_ac x_c (V row a on lanes 9 + 3a ...)
  const dw v0 = shfl_dw(val, 9 + 3 * ea), v1 = shfl_dw(val, 10 + 3 * ea),
           v2 = shfl_dw(val, 11 + 3 * ea);
  const dw ta = dw_add(dw_add(dw_mul(v0, x[0]), dw_mul(v1, x[1])), dw_mul(v2, x[2]));
  // Tn = [R t] T: lane q = 4 row + col < 12
  const int row = lane < 12 ? (lane >> 2) : 0, col = lane & 3;
  const dw r0 = shfl_dw(val, 3 * row), r1 = shfl_dw(val, 3 * row + 1),
           r2 = shfl_dw(val, 3 * row + 2), tr = shfl_dw(ta, 3 * row);
  const float2 T0 = T[col], T1 = T[4 + col], T2 = T[8 + col];
  dw tn = dw_add(dw_add(dw_mul(r0, dw{T0.x, T0.y}), dw_mul(r1, dw{T1.x, T1.y})),
                 dw_mul(r2, dw{T2.x, T2.y}));
  if (col == 3) tn = dw_add(tn, tr);
  if (lane >= 12) tn = {(lane == 15) ? 1.f : 0.f, 0.f};
  tn_out = make_float2(tn.hi, tn.lo);
  return true;
}

// ---------------------------------------------------------------------------
// Gauss-Newton step by one warp in FP64: the default, as the reference's
// solve (torch.cholesky + cholesky_solve in float64, icp.py:236-251) and its
// SE(3) update (icp.py:244-247).
//
// Every FP64 warp instruction occupies its sub-partition's FP64 pipe for
// many cycles whatever its lanes, so the layout makes each instruction do
// the work of many lanes: one lane per entry of the 6x6 lower triangle plus
// one per right-hand-side entry, a division-free symmetric elimination
// whose column step is one multiply and one FMA for all entries (the six
// reciprocals taken at once at the end), and the three exponential
// coefficients at once on three lane groups.
// ---------------------------------------------------------------------------

// 1 / d for d > 0: rcp.approx.ftz.f64 (relative error below 2^-22) and one
// third-order correction: with e = 1 - d y, y (1 + e + e^2) = (1 - e^3) / d,
// a relative error below 2^-66 before the last rounding, so the result is
// within an ulp of the correctly rounded reciprocal.  Three FP64
// instructions (two Newton-Raphson steps take four).  A subnormal d flushes
// to an infinite reciprocal, which turns the solution into NaN (flagged by
// the caller).
__device__ __forceinline__ double rcp_fp64(double d) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
  const double e = fma(-d, y, 1.0);
  return fma(y, fma(e, e, e), y);
}

// Maclaurin coefficient n (in t^2) of A = sin t / t (which = 0),
// B = (1 - cos t) / t^2 (1) or C = (t - sin t) / t^3 (2): (-1)^n / (2n + 1 +
// which)!, n < 8.  n is a compile-time constant, which a per-lane select.
template <int n>
__device__ __forceinline__ double se3_series_coeff(int which) {
  constexpr double f[18] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0, 40320.0, 362880.0,
                            3628800.0, 39916800.0, 479001600.0, 6227020800.0, 87178291200.0,
                            1307674368000.0, 20922789888000.0, 355687428096000.0};
  constexpr double s = (n & 1) ? -1.0 : 1.0;
  constexpr double ca = s / f[2 * n + 1], cb = s / f[2 * n + 2], cc = s / f[2 * n + 3];
  return which == 0 ? ca : (which == 1 ? cb : cc);
}

// v * 2^-e on the bits (integer instructions only): exact for a normal v
// whose result stays normal; zeros, subnormals, infinities and NaN pass
// unchanged, a result below the normal range flushes to a signed zero and
// one above it becomes a signed infinity.
__device__ __forceinline__ double scale_pow2(double v, int e) {
  int hi = __double2hiint(v), lo = __double2loint(v);
  const int ef = (hi >> 20) & 0x7ff, nf = ef - e;
  if (ef != 0 && ef != 0x7ff) {
    if (nf <= 0) {
      hi &= (int)0x80000000u;
      lo = 0;
    } else if (nf >= 0x7ff) {
      hi = (hi & (int)0x80000000u) | 0x7ff00000;
      lo = 0;
    } else {
      hi -= e * (1 << 20);
    }
  }
  return __hiloint2double(hi, lo);
}

// One Gauss-Newton update by one warp (all 32 lanes call it), in FP64.
//   up: the 21 packed upper-triangle entries of J^T J, bv: J^T r (6),
//   T: the current pose (16, row-major); all in shared memory.
// Solves J^T J x = J^T r, then Tn = exp(x) T.  The solve is Gaussian
// elimination in its division-free symmetric form: column j replaces every
// later row i by p_j row_i - a_ij row_j (p_j the pivot), which keeps the
// trailing block symmetric (p_j times the Schur complement of LDL^T), and
// scales the block by the power of two nearest below p_j so its entries stay
// near the Schur complement's size.  So each column costs one multiply and
// one FMA, and the pivots differ from the LDL^T pivots (the squares of the
// Cholesky pivots) by positive factors only: the failure rule stays that of
// LAPACK potrf (a pivot that is not > 0, or NaN, fails; one below the
// normal range fails too).  The six rows are then divided by their pivots
// at once (one reciprocal for all), and back substitution runs on the unit
// upper triangle.  Returns the solve status (warp-uniform); on success
// lanes 0..15 hold Tn's entries in tn_out (lane k -> entry k), and every
// lane holds x in xs.
__device__ inline bool warp_gn_update(const double *up, const double *bv, const double *T,
                                      double *xs, double &tn_out, int lane) {
  const unsigned full = 0xffffffffu;
  // this lane's entry (i, k); k == 6 marks the right-hand side
  int ei = 0, ek = 0;
  if (lane < 21) {
    int k = 0, first = 0;
    while (lane >= first + (6 - k)) {
      first += 6 - k;
      ++k;
    }
    ek = k;
    ei = k + (lane - first);
  } else if (lane < 27) {
    ei = lane - 21;
    ek = 6;
  }
  const bool is_rhs = (lane >= 21 && lane < 27);
  const bool is_tri = lane < 21;
  double v = 0.0;
  if (is_tri) v = up[upper_index(ek, ei)];
  if (is_rhs) v = bv[ei];
  bool ok = true;
  // forward: division-free elimination of the lower triangle and the
  // right-hand side (column j's entries keep their values: they are row j of
  // the upper triangle)
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double piv = __shfl_sync(full, v, tri_lane(j, j));
    const long long pb = __double_as_longlong(piv);
    ok = ok && pb >= 0x0010000000000000ll && pb < 0x7ff0000000000000ll;
    if (j == 5) break;
    const int src_i = (ei >= j) ? tri_lane(ei, j) : 0;
    const int src_k = is_rhs ? 21 + j : ((ek >= j && ek < 6) ? tri_lane(ek, j) : 0);
    const double aij = __shfl_sync(full, v, src_i);
    const double akj = __shfl_sync(full, v, src_k);
    const bool upd = (is_tri && ek > j && ei >= ek) || (is_rhs && ei > j);
    // (piv v - aij akj) 2^-pe with piv in [2^pe, 2^(pe+1)): the pivot's
    // exponent field set to 1023 and aij scaled on the bits while the
    // multiply runs
    const int pe = (int)(pb >> 52) - 1023;
    const double pn = __longlong_as_double((pb & 0x000fffffffffffffll) | 0x3ff0000000000000ll);
    const double nv = fma(-scale_pow2(aij, pe), akj, pn * v);
    if (upd) v = nv;
  }
  if (!ok) return false;
  // rows to unit pivots: lane (i, k) of the triangle holds U_ki, the right-
  // hand-side lane i holds c_i; both divide by row k's (or i's) pivot
  {
    const double rr = rcp_fp64(v);  // meaningful on the diagonal lanes
    const int row = is_rhs ? ei : ek;
    const double r = __shfl_sync(full, rr, tri_lane(row, row));
    v *= r;
  }
  // backward: U x = c on the unit upper triangle; rhs lane i ends with x_i
#pragma unroll
  for (int j = 5; j >= 0; --j) {
    const double xj = __shfl_sync(full, v, 21 + j);
    xs[j] = xj;
    if (j > 0) {
      const int src = (is_rhs && ei < j) ? tri_lane(j, ei) : 0;
      const double lji = __shfl_sync(full, v, src);
      const double nv = fma(-lji, xj, v);
      if (is_rhs && ei < j) v = nv;
    }
  }
  // exp(x).  The coefficients A on lanes 0..9, B on 10..19, C on 20..31,
  // from their Maclaurin series in t^2: below t^2 = 2^-14 (a rotation
  // update under 0.45 degrees, the usual case after the first iterations)
  // through t^4 by Horner's rule, the series alternating and the first
  // omitted term (t^6 / 7!, t^6 / 8!, t^6 / 9!) below 2^-42 / 5040 < 4.6e-17,
  // under half an ulp of A, B and C (A near 1, B near 1/2, C near 1/6);
  // below t = 0.5 through t^14 by Estrin's scheme (the first omitted term
  // below 0.5^16 / 17! < 5e-20); above, the closed forms of se3_coeffs.
  const double wx = xs[3], wy = xs[4], wz = xs[5];
  const double t2 = fma(wx, wx, fma(wy, wy, wz * wz));
  double A, B, C;
  // the thresholds are tested on the bits (t2 >= 0; NaN takes the last
  // branch): an FP64 comparison would cost an FP64 instruction
  const long long t2b = __double_as_longlong(t2);
  if (t2b < 0x3F10000000000000ll) {  // t2 < 2^-14
    const int which = lane < 10 ? 0 : (lane < 20 ? 1 : 2);
    const double coef = fma(fma(se3_series_coeff<2>(which), t2, se3_series_coeff<1>(which)), t2,
                            se3_series_coeff<0>(which));
    A = __shfl_sync(full, coef, 0);
    B = __shfl_sync(full, coef, 10);
    C = __shfl_sync(full, coef, 20);
  } else if (t2b < 0x3FD0000000000000ll) {  // t2 < 0.25
    const int which = lane < 10 ? 0 : (lane < 20 ? 1 : 2);
    const double u2 = t2 * t2, u4 = u2 * u2;
    const double a01 = fma(se3_series_coeff<1>(which), t2, se3_series_coeff<0>(which));
    const double a23 = fma(se3_series_coeff<3>(which), t2, se3_series_coeff<2>(which));
    const double a45 = fma(se3_series_coeff<5>(which), t2, se3_series_coeff<4>(which));
    const double a67 = fma(se3_series_coeff<7>(which), t2, se3_series_coeff<6>(which));
    const double coef = fma(u4, fma(u2, a67, a45), fma(u2, a23, a01));
    A = __shfl_sync(full, coef, 0);
    B = __shfl_sync(full, coef, 10);
    C = __shfl_sync(full, coef, 20);
  } else {
    se3_coeffs(t2, A, B, C);
  }
  // lanes 0..8 hold R_ac = I + A W + B W^2, lanes 9..17 V_ac = I + B W + C W^2
  const int e = lane < 9 ? lane : (lane < 18 ? lane - 9 : 0);
  const int ea = e / 3, ec = e % 3;
  const double wa = ea == 0 ? wx : (ea == 1 ? wy : wz);
  const double wc = ec == 0 ? wx : (ec == 1 ? wy : wz);
  // W = hat(w): W_01 = -wz, W_02 = wy, W_10 = wz, W_12 = -wx, W_20 = -wy, W_21 = wx
  const double Wac = e == 1 ? -wz : e == 2 ? wy : e == 3 ? wz : e == 5 ? -wx : e == 6 ? -wy
                   : e == 7 ? wx : 0.0;
  const bool diag = (ea == ec);
  const double W2ac = fma(wa, wc, diag ? -t2 : 0.0);  // W^2 = w w^T - |w|^2 I
  const bool isR = lane < 9;
  const double val = fma(isR ? A : B, Wac, fma(isR ? B : C, W2ac, diag ? 1.0 : 0.0));
  // t_a = sum_c V_ac x_c (V row a on lanes 9 + 3a ...)
  const double v0 = __shfl_sync(full, val, 9 + 3 * ea), v1 = __shfl_sync(full, val, 10 + 3 * ea),
               v2 = __shfl_sync(full, val, 11 + 3 * ea);
  const double ta = fma(v0, xs[0], fma(v1, xs[1], v2 * xs[2]));
  // Tn = [R t] T: lane q = 4 row + col < 12
  const int row = lane < 12 ? (lane >> 2) : 0, col = lane & 3;
  const double r0 = __shfl_sync(full, val, 3 * row), r1 = __shfl_sync(full, val, 3 * row + 1),
               r2 = __shfl_sync(full, val, 3 * row + 2), tr = __shfl_sync(full, ta, 3 * row);
  double tn = fma(r0, T[col], fma(r1, T[4 + col], fma(r2, T[8 + col], col == 3 ? tr : 0.0)));
  if (lane >= 12) tn = (lane == 15) ? 1.0 : 0.0;
  tn_out = tn;
  return true;
}

}  // namespace stb
