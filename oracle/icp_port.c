/*
 * C/OpenMP restatement of fusion-toolbox's CPU ICP path.
 *
 * TEST INFRASTRUCTURE ONLY: the CPU baseline that bench.py times (cpu_baseline
 * kind "port", and the --impl reference arm) and a second CPU oracle that
 * the tests check against the numpy oracle.  Never linked into the product.
 *
 * It keeps the reference CPU path's structure (the reference itself cannot
 * be built here: its native module needs Eigen, which is absent):
 *   per iteration (slamtb/registration/icp.py:210-256)
 *     - association, one OpenMP loop over source points
 *       (src/correspondence_map.cu:39-61, Launch1DKernelCPU of
 *       include/slamtb/kernel.hpp:58-72) with every map write under one
 *       global mutex, as MergeMap<kCPU>::Set (src/merge_map.hpp:37-50);
 *     - per-point partials JtJ[N,6,6], Jtr[N,6], r^2[N] written for every
 *       source point (src/icp_jacobian_geometric.cu:54-85,
 *       src/icp_jacobian_feature.cu:58-109), the association rebuilt for
 *       each term as _JacobianStep does (icp.py:49-55);
 *     - the sums of icp.py:78-80 (an OpenMP reduction);
 *     - the 6x6 Cholesky solve, SE(3) exponential and left update in double.
 * Float32 arithmetic follows the reference's operation order; build with
 * -ffp-contract=off so no multiply-add is fused (bit-exact with the numpy
 * oracle).  Deterministic tie rule on the map: (distance, index)
 * lexicographic, as the numpy oracle and the GPU path.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EMPTY_ENTRY 0x0FFFFFFF7F800000LL

typedef struct {
  float rt[12], nm[9], fx, fy, cx, cy;
} pose32_t;

static pthread_mutex_t g_merge_mutex = PTHREAD_MUTEX_INITIALIZER;

static inline uint32_t f2u(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}
static inline float u2f(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

/* InverseTranspose, include/slamtb/camera.hpp:99-116 */
static void inverse_transpose(const float *A, float *r) {
#define E(i, j) A[(i)*4 + (j)]
  float det = E(0, 0) * (E(1, 1) * E(2, 2) - E(2, 1) * E(1, 2)) -
              E(0, 1) * (E(1, 0) * E(2, 2) - E(1, 2) * E(2, 0)) +
              E(0, 2) * (E(1, 0) * E(2, 1) - E(1, 1) * E(2, 0));
  float inv = 1.0f / det;
  r[0] = (E(1, 1) * E(2, 2) - E(2, 1) * E(1, 2)) * inv;
  r[3] = -(E(0, 1) * E(2, 2) - E(0, 2) * E(2, 1)) * inv;
  r[6] = (E(0, 1) * E(1, 2) - E(0, 2) * E(1, 1)) * inv;
  r[1] = -(E(1, 0) * E(2, 2) - E(1, 2) * E(2, 0)) * inv;
  r[4] = (E(0, 0) * E(2, 2) - E(0, 2) * E(2, 0)) * inv;
  r[7] = -(E(0, 0) * E(1, 2) - E(1, 0) * E(0, 2)) * inv;
  r[2] = (E(1, 0) * E(2, 1) - E(2, 0) * E(1, 1)) * inv;
  r[5] = -(E(0, 0) * E(2, 1) - E(2, 0) * E(0, 1)) * inv;
  r[8] = (E(0, 0) * E(1, 1) - E(1, 0) * E(0, 1)) * inv;
#undef E
}

static void make_pose(const double *T, const float *kcam, pose32_t *P) {
  for (int k = 0; k < 12; ++k) P->rt[k] = (float)T[k];
  inverse_transpose(P->rt, P->nm);
  P->fx = kcam[0];
  P->cx = kcam[2];
  P->fy = kcam[4];
  P->cy = kcam[5];
}

static inline void xform(const float *m, float x, float y, float z, float *o) {
  o[0] = m[0] * x + m[1] * y + m[2] * z + m[3];
  o[1] = m[4] * x + m[5] * y + m[6] * z + m[7];
  o[2] = m[8] * x + m[9] * y + m[10] * z + m[11];
}

static inline int project_round(const pose32_t *P, const float *p, int W, int H, float *u,
                                float *v, int *ui, int *vi) {
  *u = P->fx * p[0] / p[2] + P->cx;
  *v = P->fy * p[1] / p[2] + P->cy;
  const float ru = roundf(*u), rv = roundf(*v);
  if (!(ru >= 0.0f && ru < (float)W && rv >= 0.0f && rv < (float)H)) return 0;
  *ui = (int)ru;
  *vi = (int)rv;
  return 1;
}

/* Eigen's dot / squaredNorm of 3-vectors: its unrolled redux
 * (Eigen/src/Core/Redux.h, redux_novec_unroller) splits three terms at one,
 * a0 b0 + (a1 b1 + a2 b2). */
static inline float dot3(const float *a, const float *b) {
  return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]);
}

static float angle_cos_max(double angle) {
  const float th = (float)angle;
  if (isnan(th) || (double)th >= M_PI) return -INFINITY;
  const double c = (th <= 0.0f) ? 1.0 : cos((double)th);
  float f = (float)c;
  if ((double)f > c) f = nextafterf(f, -INFINITY);
  return f;
}

static void associate(const pose32_t *P, const float *sp, const float *sn, const uint8_t *sm,
                      int64_t n, const float *tp, const float *tn, const uint8_t *tm, int H,
                      int W, float thr2, float cos_max, int64_t *map) {
  for (int64_t k = 0; k < (int64_t)H * W; ++k) map[k] = EMPTY_ENTRY;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    if (!sm[i]) continue;
    float p[3], nn[3], u, v;
    int ui, vi;
    xform(P->rt, sp[3 * i], sp[3 * i + 1], sp[3 * i + 2], p);
    if (!project_round(P, p, W, H, &u, &v, &ui, &vi)) continue;
    const int64_t pix = (int64_t)vi * W + ui;
    if (!tm[pix]) continue;
    const float d[3] = {tp[3 * pix] - p[0], tp[3 * pix + 1] - p[1], tp[3 * pix + 2] - p[2]};
    const float sq = dot3(d, d);
    if (sq > thr2) continue;
    const float *nmx = P->nm;
    const float x = sn[3 * i], y = sn[3 * i + 1], z = sn[3 * i + 2];
    nn[0] = nmx[0] * x + nmx[1] * y + nmx[2] * z;
    nn[1] = nmx[3] * x + nmx[4] * y + nmx[5] * z;
    nn[2] = nmx[6] * x + nmx[7] * y + nmx[8] * z;
    const float *nq = tn + 3 * pix;
    const float c = dot3(nn, nq) / (sqrtf(dot3(nn, nn)) * sqrtf(dot3(nq, nq)));
    if (c >= -1.0f && c <= cos_max) continue;
    const float dist = sqrtf(sq);
    pthread_mutex_lock(&g_merge_mutex);
    const uint64_t cur = (uint64_t)map[pix];
    const float cur_d = u2f((uint32_t)(cur & 0xffffffffu));
    const int32_t cur_i = (int32_t)(cur >> 32);
    if (dist < cur_d || (dist == cur_d && (int32_t)i < cur_i))
      map[pix] = (int64_t)(((uint64_t)(uint32_t)i << 32) | f2u(dist));
    pthread_mutex_unlock(&g_merge_mutex);
  }
}

static inline void write_partials(float *JtJ, float *Jr, const float *J, float r) {
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 6; ++b) JtJ[a * 6 + b] = J[b] * J[a];
  for (int k = 0; k < 6; ++k) Jr[k] = J[k] * r;
}

/* GeometricJacobianKernel, per-point partials; returns the match count */
static int64_t geometric_partials(const pose32_t *P, const float *sp, const uint8_t *sm,
                                  int64_t n, const float *tp, const float *tn, int H, int W,
                                  const int64_t *map, float *JtJ, float *Jr, float *r2) {
  int64_t count = 0;
#pragma omp parallel for schedule(static) reduction(+ : count)
  for (int64_t i = 0; i < n; ++i) {
    memset(JtJ + 36 * i, 0, 36 * sizeof(float));
    memset(Jr + 6 * i, 0, 6 * sizeof(float));
    r2[i] = 0.0f;
    if (!sm[i]) continue;
    float p[3], u, v;
    int ui, vi;
    xform(P->rt, sp[3 * i], sp[3 * i + 1], sp[3 * i + 2], p);
    if (!project_round(P, p, W, H, &u, &v, &ui, &vi)) continue;
    const int64_t pix = (int64_t)vi * W + ui;
    if ((int32_t)(map[pix] >> 32) != (int32_t)i) continue;
    const float *q = tp + 3 * pix, *nq = tn + 3 * pix;
    const float d[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
    const float r = dot3(d, nq);
    const float J[6] = {nq[0], nq[1], nq[2], p[1] * nq[2] - p[2] * nq[1],
                        p[2] * nq[0] - p[0] * nq[2], p[0] * nq[1] - p[1] * nq[0]};
    write_partials(JtJ + 36 * i, Jr + 6 * i, J, r);
    r2[i] = r * r;
    ++count;
  }
  return count;
}

static inline float bilinear(const float *f, int H, int W, float u, float v) {
  const int ui = (int)u, vi = (int)v;
  const float ur = u - (float)ui, vr = v - (float)vi;
  const float v00 = f[(int64_t)vi * W + ui];
  const float v10 = (ui + 1 < W) ? f[(int64_t)vi * W + ui + 1] : 0.f;
  const float v01 = (vi + 1 < H) ? f[(int64_t)(vi + 1) * W + ui] : 0.f;
  const float v11 = (ui + 1 < W && vi + 1 < H) ? f[(int64_t)(vi + 1) * W + ui + 1] : 0.f;
  const float a0 = v00 * (1 - ur) + v10 * ur;
  const float a1 = v01 * (1 - ur) + v11 * ur;
  return a0 * (1 - vr) + a1 * vr;
}

/* FeatureJacobianKernel (SE3), per-point partials; returns the match count */
static int64_t feature_partials(const pose32_t *P, const float *sp, const float *sf,
                                const uint8_t *sm, int64_t n, const float *tf, int C, int H,
                                int W, const int64_t *map, float thresh, float *JtJ, float *Jr,
                                float *r2) {
  int64_t count = 0;
  const float h = 0.05f, div = 1.0f / (2.0f * h);
#pragma omp parallel for schedule(static) reduction(+ : count)
  for (int64_t i = 0; i < n; ++i) {
    memset(JtJ + 36 * i, 0, 36 * sizeof(float));
    memset(Jr + 6 * i, 0, 6 * sizeof(float));
    r2[i] = 0.0f;
    if (!sm[i]) continue;
    float p[3], u, v;
    int ui, vi;
    xform(P->rt, sp[3 * i], sp[3 * i + 1], sp[3 * i + 2], p);
    if (!project_round(P, p, W, H, &u, &v, &ui, &vi)) continue;
    const int64_t pix = (int64_t)vi * W + ui;
    if ((int32_t)(map[pix] >> 32) != (int32_t)i) continue;
    const float zz = p[2] * p[2];
    const float j00 = P->fx / p[2], j02 = -p[0] * P->fx / zz;
    const float j11 = P->fy / p[2], j12 = -p[1] * P->fy / zz;
    const float uu0 = u + h, uu1 = fmaxf(u - h, 0.f), vv0 = v + h, vv1 = fmaxf(v - h, 0.f);
    float sq = 0.f, r = 0.f, J[6];
    for (int c = 0; c < C; ++c) {
      const float *fc = tf + (int64_t)c * H * W;
      r = bilinear(fc, H, W, u, v) - sf[(int64_t)c * n + i];
      const float du = (bilinear(fc, H, W, uu0, v) - bilinear(fc, H, W, uu1, v)) * div;
      const float dv = (bilinear(fc, H, W, u, vv0) - bilinear(fc, H, W, u, vv1)) * div;
      const float g[3] = {du * j00, dv * j11, du * j02 + dv * j12};
      J[0] = g[0];
      J[1] = g[1];
      J[2] = g[2];
      J[3] = p[1] * g[2] - p[2] * g[1];
      J[4] = p[2] * g[0] - p[0] * g[2];
      J[5] = p[0] * g[1] - p[1] * g[0];
      sq += r * r;
    }
    if (sq > thresh * thresh) continue;
    write_partials(JtJ + 36 * i, Jr + 6 * i, J, r);
    r2[i] = sq;
    ++count;
  }
  return count;
}

/* torch.sum(0) of the partials (icp.py:78-80) */
static void sum_partials(int64_t n, const float *JtJ, const float *Jr, const float *r2,
                         double *sJtJ, double *sJr, double *sr2) {
  double a[36] = {0}, b[6] = {0}, c = 0.0;
#pragma omp parallel
  {
    double la[36] = {0}, lb[6] = {0}, lc = 0.0;
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < 36; ++k) la[k] += JtJ[36 * i + k];
      for (int k = 0; k < 6; ++k) lb[k] += Jr[6 * i + k];
      lc += r2[i];
    }
#pragma omp critical
    {
      for (int k = 0; k < 36; ++k) a[k] += la[k];
      for (int k = 0; k < 6; ++k) b[k] += lb[k];
      c += lc;
    }
  }
  memcpy(sJtJ, a, sizeof(a));
  memcpy(sJr, b, sizeof(b));
  *sr2 = c;
}

static int cholesky_solve6(const double *A, const double *b, double *x) {
  double L[36] = {0}, y[6];
  for (int j = 0; j < 6; ++j) {
    double d = A[j * 6 + j];
    for (int k = 0; k < j; ++k) d -= L[j * 6 + k] * L[j * 6 + k];
    if (!(d > 0.0)) return 0;
    L[j * 6 + j] = sqrt(d);
    for (int i = j + 1; i < 6; ++i) {
      double s = A[i * 6 + j];
      for (int k = 0; k < j; ++k) s -= L[i * 6 + k] * L[j * 6 + k];
      L[i * 6 + j] = s / L[j * 6 + j];
    }
  }
  for (int i = 0; i < 6; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[i * 6 + k] * y[k];
    y[i] = s / L[i * 6 + i];
  }
  for (int i = 5; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < 6; ++k) s -= L[k * 6 + i] * x[k];
    x[i] = s / L[i * 6 + i];
  }
  return 1;
}

static void se3_exp(const double *xi, double *E) {
  const double wx = xi[3], wy = xi[4], wz = xi[5];
  const double t2 = wx * wx + wy * wy + wz * wz;
  double A, B, C;
  if (t2 < 1e-4) {
    const double t4 = t2 * t2, t6 = t4 * t2;
    A = 1.0 - t2 / 6.0 + t4 / 120.0 - t6 / 5040.0;
    B = 0.5 - t2 / 24.0 + t4 / 720.0 - t6 / 40320.0;
    C = 1.0 / 6.0 - t2 / 120.0 + t4 / 5040.0 - t6 / 362880.0;
  } else {
    const double t = sqrt(t2);
    A = sin(t) / t;
    B = (1.0 - cos(t)) / t2;
    C = (t - sin(t)) / (t2 * t);
  }
  const double W[9] = {0.0, -wz, wy, wz, 0.0, -wx, -wy, wx, 0.0};
  double W2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      W2[i * 3 + j] = W[i * 3] * W[j] + W[i * 3 + 1] * W[3 + j] + W[i * 3 + 2] * W[6 + j];
  for (int i = 0; i < 3; ++i) {
    double t = 0.0;
    for (int j = 0; j < 3; ++j) {
      const double id = (i == j) ? 1.0 : 0.0;
      E[i * 4 + j] = id + A * W[i * 3 + j] + B * W2[i * 3 + j];
      t += (id + B * W[i * 3 + j] + C * W2[i * 3 + j]) * xi[j];
    }
    E[i * 4 + 3] = t;
  }
  E[12] = E[13] = E[14] = 0.0;
  E[15] = 1.0;
}

static void compose(const double *E, const double *T, double *O) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = E[i * 4] * T[j] + E[i * 4 + 1] * T[4 + j] + E[i * 4 + 2] * T[8 + j];
      if (j == 3) s += E[i * 4 + 3];
      O[i * 4 + j] = s;
    }
  O[12] = O[13] = O[14] = 0.0;
  O[15] = 1.0;
}

/*
 * ICPOdometry.estimate (icp.py:152-262).  src_feats [C, n] / tgt_feats
 * [C, H, W] may be NULL.  Outputs: final transform (16), information (36),
 * residual, match ratio, successful iterations.  Returns 0.
 */
int icp_port_estimate(const float *kcam, const float *sp, const float *sn, const uint8_t *sm,
                      int64_t n, const float *sf, const float *tp, const float *tn,
                      const uint8_t *tm, int H, int W, const float *tf, int C,
                      const double *init, int iters, double wg, double wf, double dist,
                      double angle, double feat_thresh, int threads, double *out_T,
                      double *out_info, double *out_residual, double *out_ratio,
                      int *out_iters) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  const float thr2 = (float)(dist * dist), cos_max = angle_cos_max(angle);
  const int use_feat = wf > 0.0 && sf && tf, use_geom = wg > 0.0;
  int64_t *map = (int64_t *)malloc(sizeof(int64_t) * (size_t)H * W);
  float *JtJ = (float *)malloc(sizeof(float) * 36 * (size_t)n);
  float *Jr = (float *)malloc(sizeof(float) * 6 * (size_t)n);
  float *r2 = (float *)malloc(sizeof(float) * (size_t)n);
  double T[16];
  for (int k = 0; k < 16; ++k) T[k] = init ? init[k] : ((k % 5) == 0 ? 1.0 : 0.0);
  *out_iters = 0;
  *out_residual = INFINITY;
  *out_ratio = 0.0;
  for (int it = 0; it < iters; ++it) {
    pose32_t P;
    make_pose(T, kcam, &P);
    double A[36] = {0}, b[6] = {0}, res = 0.0, sJ[36], sb[6], sr;
    int64_t count = 0;
    if (use_feat) {
      associate(&P, sp, sn, sm, n, tp, tn, tm, H, W, thr2, cos_max, map);
      count = feature_partials(&P, sp, sf, sm, n, tf, C, H, W, map, (float)feat_thresh, JtJ,
                               Jr, r2);
      sum_partials(n, JtJ, Jr, r2, sJ, sb, &sr);
      for (int k = 0; k < 36; ++k) A[k] = sJ[k] * wf * wf;
      for (int k = 0; k < 6; ++k) b[k] = sb[k] * -wf;
      res = sr * wf;
    }
    if (use_geom) {
      associate(&P, sp, sn, sm, n, tp, tn, tm, H, W, thr2, cos_max, map);
      const int64_t gc = geometric_partials(&P, sp, sm, n, tp, tn, H, W, map, JtJ, Jr, r2);
      sum_partials(n, JtJ, Jr, r2, sJ, sb, &sr);
      for (int k = 0; k < 36; ++k) A[k] += sJ[k] * wg * wg;
      for (int k = 0; k < 6; ++k) b[k] += sb[k] * wg;
      res += sr * wg;
      if (gc > count) count = gc;
    }
    double x[6], E[16], Tn[16];
    if (!cholesky_solve6(A, b, x)) break;
    se3_exp(x, E);
    compose(E, T, Tn);
    memcpy(T, Tn, sizeof(T));
    memcpy(out_T, T, sizeof(T));
    *out_residual = res / (double)count;
    *out_ratio = (double)count / (double)n;
    *out_iters = it + 1;
  }
  /* information matrix at the final pose (icp.py:84-108, 258-261) */
  {
    pose32_t P;
    make_pose(T, kcam, &P);
    associate(&P, sp, sn, sm, n, tp, tn, tm, H, W, thr2, cos_max, map);
    double info[36] = {0};
#pragma omp parallel
    {
      double li[36] = {0};
#pragma omp for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        if (!sm[i]) continue;
        float p[3], u, v;
        int ui, vi;
        xform(P.rt, sp[3 * i], sp[3 * i + 1], sp[3 * i + 2], p);
        if (!project_round(&P, p, W, H, &u, &v, &ui, &vi)) continue;
        const int64_t pix = (int64_t)vi * W + ui;
        if ((int32_t)(map[pix] >> 32) != (int32_t)i) continue;
        const float *q = tp + 3 * pix;
        const float G[3][6] = {{0.f, q[2], -q[1], 1.f, 0.f, 0.f},
                               {-q[2], 0.f, q[0], 0.f, 1.f, 0.f},
                               {q[1], -q[0], 0.f, 0.f, 0.f, 1.f}};
        for (int a = 0; a < 6; ++a)
          for (int c = 0; c < 6; ++c)
            li[a * 6 + c] += G[0][a] * G[0][c] + G[1][a] * G[1][c] + G[2][a] * G[2][c];
      }
#pragma omp critical
      for (int k = 0; k < 36; ++k) info[k] += li[k];
    }
    memcpy(out_info, info, sizeof(info));
  }
  free(map);
  free(JtJ);
  free(Jr);
  free(r2);
  return 0;
}

int icp_port_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
