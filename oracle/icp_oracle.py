"""numpy restatement of fusion-toolbox's ICP registration path.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Parity with the
reference's own binaries is unpinned (the reference cannot be built or
imported here); the oracle is pinned by the known-answer poses of the
reference's ``test-data/rgbd/sample2`` frames.

Two precisions, on purpose:

* ``*32`` functions restate the reference's float32 kernels operation by
  operation (no fused multiply-add, correctly rounded ``/`` and ``sqrt``).
  They are the bit-exact gate for correspondence indices, validity masks
  and the per-point partials of the ``_cslamtb``-compatible entry points.
* ``*64`` functions take the reference's float32 geometry (the float32 cast
  of the pose, the float32 transformed point, the float32 projection and
  sample coordinates, the float32 gates) and evaluate all value arithmetic
  (residuals, Jacobians, products, sums, the 6x6 solve and the SE(3)
  exponential) in float64.  They are the 1e-5 error reference for the
  reduced normal equations and the per-iteration pose.

Deterministic tie rule: the reference's z-buffer keeps the first writer on
equal distance (``src/merge_map.hpp:71-79``, nondeterministic on the GPU);
here and in the CUDA path the winner of a target pixel is the lexicographic
minimum of (distance, source index).

Normal-angle gate: the reference rejects when ``acosf(c) >= theta``
(``src/correspondence.hpp:85-86``, ``include/slamtb/math.hpp:14-18``) with
``c`` the float32 cosine.  ``acosf`` is not bit-reproducible across libms,
so both sides evaluate the exact-arithmetic form of the same test: reject
when ``-1 <= c <= cos(theta)``, with ``cos(theta)`` rounded down to float32
on the host (``angle_cos_threshold``).  A NaN cosine is accepted, as in
the reference.
"""
import math

import numpy as np

F32 = np.float32
F64 = np.float64

# correspondence_map.py:5 -- index 0x0fffffff ("empty") over +inf distance
CORRESP_EMPTY = 0x0FFFFFFF7F800000
EMPTY_INDEX = 0x0FFFFFFF
FEATURE_FD_STEP = F32(0.05)          # feature_map.hpp:57 default h
FEATURE_FD_DIV = F32(1) / (F32(2) * FEATURE_FD_STEP)   # feature_map.hpp:59


# ---------------------------------------------------------------------------
# camera / pose primitives (include/slamtb/camera.hpp)
# ---------------------------------------------------------------------------

def pose_rt32(transform):
    """``transform.to(float32)`` (icp.py:53,61) read as the 3x4
    ``RigidTransform::rt_matrix`` (camera.hpp:123-125)."""
    t = np.asarray(transform, dtype=F64)
    return np.ascontiguousarray(t[:3, :4].astype(F32))


def normal_matrix32(a):
    """``InverseTranspose`` (camera.hpp:99-116), float32, same op order."""
    A = np.asarray(a, dtype=F32)

    def e(i, j):
        return A[i, j]

    det = ((e(0, 0) * (e(1, 1) * e(2, 2) - e(2, 1) * e(1, 2))
            - e(0, 1) * (e(1, 0) * e(2, 2) - e(1, 2) * e(2, 0)))
           + e(0, 2) * (e(1, 0) * e(2, 1) - e(1, 1) * e(2, 0)))
    inv = F32(1) / det
    r = np.empty((3, 3), dtype=F32)
    r[0, 0] = (e(1, 1) * e(2, 2) - e(2, 1) * e(1, 2)) * inv
    r[1, 0] = -(e(0, 1) * e(2, 2) - e(0, 2) * e(2, 1)) * inv
    r[2, 0] = (e(0, 1) * e(1, 2) - e(0, 2) * e(1, 1)) * inv
    r[0, 1] = -(e(1, 0) * e(2, 2) - e(1, 2) * e(2, 0)) * inv
    r[1, 1] = (e(0, 0) * e(2, 2) - e(0, 2) * e(2, 0)) * inv
    r[2, 1] = -(e(0, 0) * e(1, 2) - e(1, 0) * e(0, 2)) * inv
    r[0, 2] = (e(1, 0) * e(2, 1) - e(2, 0) * e(1, 1)) * inv
    r[1, 2] = -(e(0, 0) * e(2, 1) - e(2, 0) * e(0, 1)) * inv
    r[2, 2] = (e(0, 0) * e(1, 1) - e(1, 0) * e(0, 1)) * inv
    return r


def transform32(rt, p):
    """``RigidTransform::Transform`` (camera.hpp:134-145), float32."""
    p = np.asarray(p, dtype=F32)
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    out = np.empty_like(p)
    for k in range(3):
        out[:, k] = ((rt[k, 0] * x + rt[k, 1] * y) + rt[k, 2] * z) + rt[k, 3]
    return out


def transform_normal32(nm, n):
    """``RigidTransform::TransformNormal`` (camera.hpp:150-165), float32."""
    n = np.asarray(n, dtype=F32)
    x, y, z = n[:, 0], n[:, 1], n[:, 2]
    out = np.empty_like(n)
    for k in range(3):
        out[:, k] = (nm[k, 0] * x + nm[k, 1] * y) + nm[k, 2] * z
    return out


def project32(kcam, p):
    """``KCamera::Project`` (camera.hpp:53-60): ``fx * x / z + cx``."""
    k = np.asarray(kcam, dtype=F32)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        u = (k[0, 0] * p[:, 0]) / p[:, 2] + k[0, 2]
        v = (k[1, 1] * p[:, 1]) / p[:, 2] + k[1, 2]
    return u.astype(F32), v.astype(F32)


def round_away(x):
    """C ``round`` (half away from zero) of float32 values, as float64
    (exact: ``x + 0.5`` cannot round in float64 for a float32 ``x``)."""
    x = np.asarray(x, dtype=F64)
    with np.errstate(invalid="ignore"):
        return np.where(x >= 0, np.floor(x + 0.5), np.ceil(x - 0.5))


def pixel_of(kcam, tp, width, height):
    """Projection, rounding and bounds test shared by every kernel of the
    path (correspondence_map.cu:53-54, icp_jacobian_geometric.cu:63-68,
    icp_jacobian_feature.cu:68-74).  Returns (u, v, ui, vi, inside); NaN
    projections and projections beyond the int range are outside."""
    u, v = project32(kcam, tp)
    ur, vr = round_away(u), round_away(v)
    with np.errstate(invalid="ignore"):
        inside = (ur >= 0) & (ur < width) & (vr >= 0) & (vr < height)
    ui = np.where(inside, ur, 0).astype(np.int64)
    vi = np.where(inside, vr, 0).astype(np.int64)
    return u, v, ui, vi, inside


def sqnorm32(d):
    """Eigen's ``squaredNorm`` of float32 3-vectors: the unrolled redux of
    Eigen/src/Core/Redux.h (``redux_novec_unroller``) splits the three
    terms at one, so the sum is ``d0^2 + (d1^2 + d2^2)``."""
    return d[:, 0] * d[:, 0] + (d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])


def dot32(a, b):
    """Eigen's ``dot`` of float32 3-vectors, ``a0 b0 + (a1 b1 + a2 b2)``
    (the redux order of ``sqnorm32``)."""
    return a[:, 0] * b[:, 0] + (a[:, 1] * b[:, 1] + a[:, 2] * b[:, 2])


def cross32(a, b):
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1)


def distance_threshold_sq(distance_thresh):
    """``RobustCorrespondence`` stores ``d * d`` computed in double and
    narrowed to float (correspondence.hpp:170)."""
    return F32(float(distance_thresh) * float(distance_thresh))


def angle_cos_threshold(angle_thresh):
    """float32 ``c_max`` such that, for a float32 cosine ``c`` in [-1, 1],
    ``acos(c) >= float32(angle_thresh)`` exactly when ``c <= c_max``.
    Returns -inf when no cosine is rejected (threshold NaN or >= pi)."""
    th = float(F32(angle_thresh))
    if math.isnan(th) or th >= math.pi:
        return F32(-np.inf)
    c = 1.0 if th <= 0.0 else math.cos(th)
    f = F32(c)
    if float(f) > c:
        f = np.nextafter(f, F32(-np.inf), dtype=F32)
    return F32(f)


# ---------------------------------------------------------------------------
# association (correspondence_map.cu:39-61, correspondence.hpp:173-193)
# ---------------------------------------------------------------------------

class Association:
    """Result of the projective association.

    ``winner`` is the (H, W) int64 source index per target pixel, -1 where
    no source point won; ``ref_map`` is the same in the reference layout
    (high 32 bits index, low 32 bits float32 distance, empty =
    ``CORRESP_EMPTY``)."""

    def __init__(self, winner, dist, ref_map):
        self.winner = winner
        self.dist = dist
        self.ref_map = ref_map

    @property
    def count(self):
        return int((self.winner >= 0).sum())


def associate32(src_points, src_normals, src_mask, rt, tgt_points,
                tgt_normals, tgt_mask, kcam, distance_thresh, angle_thresh):
    """Projective data association (float32, op by op).

    ``src_mask`` of length 1 disables the source mask, as the reference's
    size test at correspondence_map.cu:40-41.
    """
    sp = np.asarray(src_points, dtype=F32).reshape(-1, 3)
    sn = np.asarray(src_normals, dtype=F32).reshape(-1, 3)
    sm = np.asarray(src_mask, dtype=bool).reshape(-1)
    tp_img = np.asarray(tgt_points, dtype=F32)
    tn_img = np.asarray(tgt_normals, dtype=F32)
    tm = np.asarray(tgt_mask, dtype=bool)
    h, w = tm.shape
    n = sp.shape[0]
    rt = np.asarray(rt, dtype=F32)
    nm = normal_matrix32(rt)

    valid = sm if sm.size == n else np.ones(n, dtype=bool)
    Tp = transform32(rt, sp)
    Tn = transform_normal32(nm, sn)
    _, _, ui, vi, inside = pixel_of(kcam, Tp, w, h)
    cand = np.nonzero(valid & inside)[0]
    ui, vi = ui[cand], vi[cand]
    keep = tm[vi, ui]
    cand, ui, vi = cand[keep], ui[keep], vi[keep]

    q = tp_img[vi, ui]
    with np.errstate(invalid="ignore", over="ignore"):
        d = q - Tp[cand]
        sq = sqnorm32(d)
        keep = ~(sq > distance_threshold_sq(distance_thresh))
    cand, ui, vi, sq = cand[keep], ui[keep], vi[keep], sq[keep]

    a = Tn[cand]
    b = tn_img[vi, ui]
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        c = dot32(a, b) / (np.sqrt(sqnorm32(a)) * np.sqrt(sqnorm32(b)))
        reject = (c >= F32(-1)) & (c <= angle_cos_threshold(angle_thresh))
    keep = ~reject
    cand, ui, vi, sq = cand[keep], ui[keep], vi[keep], sq[keep]
    dist = np.sqrt(sq).astype(F32)

    # z-buffer: lexicographic minimum of (distance bits, index); a NaN
    # distance sorts above +inf and never wins.
    empty_key = np.uint64((0x7F800000 << 32) | 0xFFFFFFFF)
    keys = np.full(h * w, empty_key, dtype=np.uint64)
    key = (dist.view(np.uint32).astype(np.uint64) << np.uint64(32)) | cand.astype(np.uint64)
    np.minimum.at(keys, vi * w + ui, key)
    won = keys != empty_key
    winner = np.where(won, (keys & np.uint64(0xFFFFFFFF)).astype(np.int64), -1)
    dbits = (keys >> np.uint64(32)).astype(np.uint32)
    dist_img = np.where(won, dbits.view(F32), F32(np.inf)).astype(F32)
    ref = np.where(won, (winner << 32) | dbits.astype(np.int64), np.int64(CORRESP_EMPTY))
    return Association(winner.reshape(h, w), dist_img.reshape(h, w),
                       ref.astype(np.int64).reshape(h, w))


def winners_from_ref_map(ref_map):
    """Source index per target pixel of a reference-layout map
    (``MergeMapAccessor``, merge_map.hpp:91-93): ``map >> 32``."""
    return (np.asarray(ref_map, dtype=np.int64) >> 32).astype(np.int64)


# ---------------------------------------------------------------------------
# per-point partials, float32 (the _cslamtb.ICPJacobian entry points)
# ---------------------------------------------------------------------------

def _matched_sources(src_points, src_mask, rt, kcam, ref_map, width, height):
    """Source points whose projection's map entry names them
    (icp_jacobian_geometric.cu:58-73)."""
    sp = np.asarray(src_points, dtype=F32).reshape(-1, 3)
    sm = np.asarray(src_mask, dtype=bool).reshape(-1)
    n = sp.shape[0]
    Tp = transform32(np.asarray(rt, dtype=F32), sp)
    u, v, ui, vi, inside = pixel_of(kcam, Tp, width, height)
    owner = winners_from_ref_map(ref_map)
    ok = sm & inside
    idx = np.nonzero(ok)[0]
    own = owner[vi[idx], ui[idx]]
    matched = idx[own == idx]
    return Tp, u, v, ui, vi, matched, n


def geometric_partials32(src_points, src_mask, rt, tgt_points, tgt_normals,
                         kcam, ref_map):
    """``GeometricJacobianKernel`` (icp_jacobian_geometric.cu:54-85) with
    ``SE3ICPJacobian::Compute`` (icp_jacobian_common.hpp:37-61).

    Returns (JtJ[N,6,6], Jtr[N,6], r2[N], match_count), float32."""
    tpi = np.asarray(tgt_points, dtype=F32)
    tni = np.asarray(tgt_normals, dtype=F32)
    h, w = tpi.shape[:2]
    Tp, _, _, ui, vi, m, n = _matched_sources(src_points, src_mask, rt, kcam,
                                              ref_map, w, h)
    JtJ = np.zeros((n, 6, 6), dtype=F32)
    Jtr = np.zeros((n, 6), dtype=F32)
    r2 = np.zeros(n, dtype=F32)
    p = Tp[m]
    q = tpi[vi[m], ui[m]]
    nq = tni[vi[m], ui[m]]
    r = dot32(q - p, nq)
    J = np.concatenate([nq, cross32(p, nq)], axis=1)
    Jtr[m] = J * r[:, None]
    JtJ[m] = J[:, None, :] * J[:, :, None]
    r2[m] = r * r
    return JtJ, Jtr, r2, int(m.size)


def _bilinear32(fmap, u, v):
    """``BilinearInterp`` (feature_map.hpp:15-27,29-41), float32: truncating
    ``int(u)``, taps beyond the right/bottom edge read as 0.  Returns
    (C, M)."""
    c, h, w = fmap.shape
    ui = np.trunc(u).astype(np.int64)
    vi = np.trunc(v).astype(np.int64)
    ur = (u - ui.astype(F32)).astype(F32)
    vr = (v - vi.astype(F32)).astype(F32)
    r_ok = ui + 1 < w
    d_ok = vi + 1 < h
    u1 = np.minimum(ui + 1, w - 1)
    v1 = np.minimum(vi + 1, h - 1)
    z = F32(0)
    v00 = fmap[:, vi, ui]
    v10 = np.where(r_ok[None], fmap[:, vi, u1], z)
    v01 = np.where(d_ok[None], fmap[:, v1, ui], z)
    v11 = np.where((r_ok & d_ok)[None], fmap[:, v1, u1], z)
    one = F32(1)
    a0 = v00 * (one - ur) + v10 * ur
    a1 = v01 * (one - ur) + v11 * ur
    return (a0 * (one - vr) + a1 * vr).astype(F32)


def _bilinear64(fmap, u, v):
    """Same sampling as ``_bilinear32`` (float32 coordinates and weights),
    value arithmetic in float64."""
    c, h, w = fmap.shape
    ui = np.trunc(u).astype(np.int64)
    vi = np.trunc(v).astype(np.int64)
    ur = (u - ui.astype(F32)).astype(F64)
    vr = (v - vi.astype(F32)).astype(F64)
    r_ok = ui + 1 < w
    d_ok = vi + 1 < h
    u1 = np.minimum(ui + 1, w - 1)
    v1 = np.minimum(vi + 1, h - 1)
    f = fmap.astype(F64)
    v00 = f[:, vi, ui]
    v10 = np.where(r_ok[None], f[:, vi, u1], 0.0)
    v01 = np.where(d_ok[None], f[:, v1, ui], 0.0)
    v11 = np.where((r_ok & d_ok)[None], f[:, v1, u1], 0.0)
    a0 = v00 * (1.0 - ur) + v10 * ur
    a1 = v01 * (1.0 - ur) + v11 * ur
    return a0 * (1.0 - vr) + a1 * vr


def _fd_positions(u, v):
    """Sample positions of ``BilinearInterpGrad`` (feature_map.hpp:50-57),
    float32: (u+h, v), (max(u-h,0), v), (u, v+h), (u, max(v-h,0))."""
    h = FEATURE_FD_STEP
    z = F32(0)
    return ((u + h).astype(F32), v), (np.maximum(u - h, z).astype(F32), v), \
        (u, (v + h).astype(F32)), (u, np.maximum(v - h, z).astype(F32))


def _feature_matches(src_points, src_mask, rt, tgt_feats, kcam, ref_map):
    tf = np.asarray(tgt_feats, dtype=F32)
    c, h, w = tf.shape
    Tp, u, v, ui, vi, m, n = _matched_sources(src_points, src_mask, rt, kcam,
                                              ref_map, w, h)
    return tf, Tp, u, v, m, n


def _dx_project(kcam, p, dtype):
    """``KCamera::Dx_Project`` (camera.hpp:65-78)."""
    k = np.asarray(kcam, dtype=F32).astype(dtype)
    fx, fy = k[0, 0], k[1, 1]
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    zz = z * z
    return fx / z, (-x * fx) / zz, fy / z, (-y * fy) / zz


def feature_partials32(src_points, src_feats, src_mask, rt, tgt_feats, kcam,
                       ref_map, residual_thresh):
    """``FeatureJacobianKernel`` (icp_jacobian_feature.cu:58-109), float32.

    Reference quirk kept: ``SE3ICPJacobian::Compute`` assigns the partials,
    so with several channels only the last channel's J and J*r survive,
    while the squared residual sums all channels.

    Returns (JtJ[N,6,6], Jtr[N,6], r2[N], match_count, passed_mask[N])."""
    tf, Tp, u, v, m, n = _feature_matches(src_points, src_mask, rt,
                                          tgt_feats, kcam, ref_map)
    sf = np.asarray(src_feats, dtype=F32).reshape(tf.shape[0], -1)
    JtJ = np.zeros((n, 6, 6), dtype=F32)
    Jtr = np.zeros((n, 6), dtype=F32)
    r2 = np.zeros(n, dtype=F32)
    passed = np.zeros(n, dtype=bool)
    if m.size == 0:
        return JtJ, Jtr, r2, 0, passed
    p = Tp[m]
    um, vm = u[m], v[m]
    val = _bilinear32(tf, um, vm)
    (pu0, pu1, pv0, pv1) = _fd_positions(um, vm)
    g_u0 = _bilinear32(tf, *pu0)
    g_u1 = _bilinear32(tf, *pu1)
    g_v0 = _bilinear32(tf, *pv0)
    g_v1 = _bilinear32(tf, *pv1)
    j00, j02, j11, j12 = _dx_project(kcam, p, F32)
    sq = np.zeros(m.size, dtype=F32)
    J = None
    r = None
    for ch in range(tf.shape[0]):
        r = (val[ch] - sf[ch, m]).astype(F32)
        du = (g_u0[ch] - g_u1[ch]) * FEATURE_FD_DIV
        dv = (g_v0[ch] - g_v1[ch]) * FEATURE_FD_DIV
        gk = np.stack([du * j00, dv * j11, du * j02 + dv * j12], axis=1).astype(F32)
        J = np.concatenate([gk, cross32(p, gk)], axis=1)
        sq = (sq + r * r).astype(F32)
    thr = F32(residual_thresh)
    ok = ~(sq > thr * thr)
    mm = m[ok]
    Jtr[mm] = (J * r[:, None])[ok]
    JtJ[mm] = (J[:, None, :] * J[:, :, None])[ok]
    r2[mm] = sq[ok]
    passed[mm] = True
    return JtJ, Jtr, r2, int(ok.sum()), passed


def information_partials32(src_points, src_mask, rt, tgt_points, kcam, ref_map):
    """``InformationMatrixKernel`` (icp_jacobian_geometric.cu:118-158),
    float32: G^T G with G built from the matched target point."""
    tpi = np.asarray(tgt_points, dtype=F32)
    h, w = tpi.shape[:2]
    Tp, _, _, ui, vi, m, n = _matched_sources(src_points, src_mask, rt, kcam,
                                              ref_map, w, h)
    out = np.zeros((n, 6, 6), dtype=F32)
    q = tpi[vi[m], ui[m]]
    G = _info_rows(q, F32)
    gtg = G[0][:, :, None] * G[0][:, None, :]
    gtg = gtg + G[1][:, :, None] * G[1][:, None, :]
    gtg = gtg + G[2][:, :, None] * G[2][:, None, :]
    out[m] = gtg
    return out


def _info_rows(q, dtype):
    z = np.zeros(q.shape[0], dtype=dtype)
    o = np.ones(q.shape[0], dtype=dtype)
    q = q.astype(dtype)
    r0 = np.stack([z, q[:, 2], -q[:, 1], o, z, z], axis=1)
    r1 = np.stack([-q[:, 2], z, q[:, 0], z, o, z], axis=1)
    r2 = np.stack([q[:, 1], -q[:, 0], z, z, z, o], axis=1)
    return r0, r1, r2


# ---------------------------------------------------------------------------
# reduced normal equations, float64 value arithmetic
# ---------------------------------------------------------------------------

class Terms:
    """Reduced normal equations of one term: JtJ (6x6), Jtr (6), the sum
    of squared residuals, the match count, and ``scale`` = sum of
    |J_i| * |r_i| (the magnitude against which Jtr errors are measured,
    since Jtr itself cancels towards 0 at convergence)."""

    def __init__(self, JtJ, Jtr, r2, count, scale):
        self.JtJ, self.Jtr, self.r2, self.count, self.scale = JtJ, Jtr, r2, count, scale


def _winner_geometry(assoc, src_points, rt):
    win = assoc.winner.reshape(-1)
    pix = np.nonzero(win >= 0)[0]
    idx = win[pix]
    sp = np.asarray(src_points, dtype=F32).reshape(-1, 3)
    Tp = transform32(np.asarray(rt, dtype=F32), sp[idx])
    return pix, idx, Tp


def geometric_terms64(assoc, src_points, rt, tgt_points, tgt_normals):
    """Point-to-plane normal equations summed over the association's
    winners: r = (q - Tp).n, J = [n; Tp x n] (icp_jacobian_geometric.cu:82,
    icp_jacobian_common.hpp:41-48)."""
    pix, idx, Tp = _winner_geometry(assoc, src_points, rt)
    q = np.asarray(tgt_points, dtype=F32).reshape(-1, 3)[pix].astype(F64)
    nq = np.asarray(tgt_normals, dtype=F32).reshape(-1, 3)[pix].astype(F64)
    p = Tp.astype(F64)
    r = ((q - p) * nq).sum(axis=1)
    J = np.concatenate([nq, np.cross(p, nq)], axis=1)
    return Terms(J.T @ J, J.T @ r, float((r * r).sum()), int(pix.size),
                 float((np.linalg.norm(J, axis=1) * np.abs(r)).sum()))


def feature_terms64(assoc, src_points, src_feats, rt, tgt_feats, kcam,
                    residual_thresh, channel_mode="last"):
    """Feature-term normal equations over the association's winners
    (icp_jacobian_feature.cu:58-109).

    The float32 gate ``sum_c r_c^2 > thresh^2`` is decided exactly as the
    reference (float32 bilinear values, float32 sum), everything else is
    float64.  ``channel_mode`` "last" reproduces the reference's
    last-channel-wins partials; "sum" sums J_c J_c^T and J_c r_c over the
    channels."""
    tf = np.asarray(tgt_feats, dtype=F32)
    C = tf.shape[0]
    sf = np.asarray(src_feats, dtype=F32).reshape(C, -1)
    pix, idx, Tp = _winner_geometry(assoc, src_points, rt)
    if pix.size == 0:
        z6 = np.zeros(6)
        return Terms(np.zeros((6, 6)), z6, 0.0, 0, 0.0)
    u, v = project32(kcam, Tp)
    # float32 gate (bit-exact with the reference's decision)
    val32 = _bilinear32(tf, u, v)
    sq = np.zeros(pix.size, dtype=F32)
    for ch in range(C):
        r32 = (val32[ch] - sf[ch, idx]).astype(F32)
        sq = (sq + r32 * r32).astype(F32)
    thr = F32(residual_thresh)
    ok = ~(sq > thr * thr)

    val = _bilinear64(tf, u, v)
    (pu0, pu1, pv0, pv1) = _fd_positions(u, v)
    g_u0 = _bilinear64(tf, *pu0)
    g_u1 = _bilinear64(tf, *pu1)
    g_v0 = _bilinear64(tf, *pv0)
    g_v1 = _bilinear64(tf, *pv1)
    p = Tp.astype(F64)
    j00, j02, j11, j12 = _dx_project(kcam, p, F64)
    div = float(FEATURE_FD_DIV)
    JtJ = np.zeros((6, 6))
    Jtr = np.zeros(6)
    scale = 0.0
    r2 = np.zeros(pix.size)
    Js, rs = [], []
    for ch in range(C):
        r = val[ch] - sf[ch, idx].astype(F64)
        du = (g_u0[ch] - g_u1[ch]) * div
        dv = (g_v0[ch] - g_v1[ch]) * div
        gk = np.stack([du * j00, dv * j11, du * j02 + dv * j12], axis=1)
        J = np.concatenate([gk, np.cross(p, gk)], axis=1)
        r2 += r * r
        Js.append(J)
        rs.append(r)
    chans = [C - 1] if channel_mode == "last" else range(C)
    for ch in chans:
        J = Js[ch][ok]
        r = rs[ch][ok]
        JtJ += J.T @ J
        Jtr += J.T @ r
        scale += float((np.linalg.norm(J, axis=1) * np.abs(r)).sum())
    return Terms(JtJ, Jtr, float(r2[ok].sum()), int(ok.sum()), scale)


def information64(assoc, tgt_points):
    """Information matrix sum_i G_i^T G_i over the winners
    (icp_jacobian_geometric.cu:118-158 summed as icp.py:108)."""
    win = assoc.winner.reshape(-1)
    pix = np.nonzero(win >= 0)[0]
    q = np.asarray(tgt_points, dtype=F32).reshape(-1, 3)[pix]
    G = _info_rows(q, F64)
    out = np.zeros((6, 6))
    for g in G:
        out += g.T @ g
    return out


# ---------------------------------------------------------------------------
# FP64 6x6 Cholesky solve and SE(3) exponential / logarithm
# ---------------------------------------------------------------------------

def cholesky_solve6(JtJ, Jr):
    """``torch.cholesky`` + ``cholesky_solve`` (icp.py:236-240) restated:
    lower Cholesky with LAPACK potrf's failure rule (a pivot that is not
    > 0, or NaN).  Returns (ok, x)."""
    A = np.asarray(JtJ, dtype=F64)
    b = np.asarray(Jr, dtype=F64).reshape(-1)
    n = A.shape[0]
    L = np.zeros_like(A)
    for j in range(n):
        d = A[j, j] - np.dot(L[j, :j], L[j, :j])
        if not d > 0.0:
            return False, None
        L[j, j] = math.sqrt(d)
        for i in range(j + 1, n):
            L[i, j] = (A[i, j] - np.dot(L[i, :j], L[j, :j])) / L[j, j]
    y = np.zeros(n)
    for i in range(n):
        y[i] = (b[i] - np.dot(L[i, :i], y[:i])) / L[i, i]
    x = np.zeros(n)
    for i in reversed(range(n)):
        x[i] = (y[i] - np.dot(L[i + 1:, i], x[i + 1:])) / L[i, i]
    return True, x


def _hat(w):
    return np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])


def se3_coeffs(theta2):
    """A = sin t / t, B = (1 - cos t) / t^2, C = (t - sin t) / t^3, with
    Taylor series below t = 1e-2 (truncation < 1e-18)."""
    if theta2 < 1e-4:
        t2, t4, t6 = theta2, theta2 * theta2, theta2 * theta2 * theta2
        A = 1.0 - t2 / 6.0 + t4 / 120.0 - t6 / 5040.0
        B = 0.5 - t2 / 24.0 + t4 / 720.0 - t6 / 40320.0
        C = 1.0 / 6.0 - t2 / 120.0 + t4 / 5040.0 - t6 / 362880.0
        return A, B, C
    t = math.sqrt(theta2)
    s, c = math.sin(t), math.cos(t)
    return s / t, (1.0 - c) / theta2, (t - s) / (theta2 * t)


def se3_exp(xi):
    """Exact SE(3) exponential of a twist ordered [v (translation); w
    (rotation)] -- the order fixed by the Jacobian J = [n; p x n]
    (icp_jacobian_common.hpp:41-48).  The reference calls
    ``tenviz.pose.SE3.exp`` (icp.py:245), which is not available; this is
    the closed form R = I + A W + B W^2, t = (I + B W + C W^2) v."""
    xi = np.asarray(xi, dtype=F64).reshape(6)
    v, w = xi[:3], xi[3:]
    W = _hat(w)
    W2 = W @ W
    A, B, C = se3_coeffs(float(w @ w))
    T = np.eye(4)
    T[:3, :3] = np.eye(3) + A * W + B * W2
    T[:3, 3] = (np.eye(3) + B * W + C * W2) @ v
    return T


def se3_log(T):
    """Inverse of ``se3_exp`` for rotation angles below pi."""
    T = np.asarray(T, dtype=F64)
    R, t = T[:3, :3], T[:3, 3]
    c = min(1.0, max(-1.0, (np.trace(R) - 1.0) * 0.5))
    theta = math.acos(c)
    if theta < 1e-5:
        w = 0.5 * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    else:
        w = theta / (2.0 * math.sin(theta)) * np.array(
            [R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    W = _hat(w)
    A, B, C = se3_coeffs(float(w @ w))
    V = np.eye(3) + B * W + C * (W @ W)
    v = np.linalg.solve(V, t)
    return np.concatenate([v, w])


# ---------------------------------------------------------------------------
# Gauss-Newton loop (icp.py:152-262) and multiscale wrapper (multiscale.py)
# ---------------------------------------------------------------------------

class Result:
    """``RegistrationResult`` fields plus the per-iteration history used by
    the parity tests."""

    def __init__(self):
        self.transform = None
        self.information = None
        self.residual = math.inf
        self.match_ratio = 0.0
        self.JtJ = None
        self.history = []


def gn_step(T, kcam, src_points, src_normals, src_mask, tgt_points, tgt_normals,
            tgt_mask, src_feats=None, tgt_feats=None, geom_weight=1.0, feat_weight=1.0,
            distance_threshold=0.5, normals_angle_thresh=math.pi / 4,
            feat_residual_thresh=2.75, channel_mode="last"):
    """One Gauss-Newton iteration of ``ICPOdometry.estimate`` at pose ``T``
    (icp.py:211-253): association at the float32 cast of ``T``, the
    weighted normal equations (JtJ by w^2, Jtr by +w for the geometric and
    -w for the feature term, residual by w; icp.py:216-235), the Cholesky
    solve (icp.py:236-242) and the left update T <- exp(x) T
    (icp.py:245-247).  Returns a dict; ``ok`` is False when the solve
    failed (the reference's ``break``)."""
    sp = np.asarray(src_points, dtype=F32).reshape(-1, 3)
    sn = np.asarray(src_normals, dtype=F32).reshape(-1, 3)
    sm = np.asarray(src_mask, dtype=bool).reshape(-1)
    T = np.asarray(T, dtype=F64)
    use_geom = geom_weight > 0
    use_feat = feat_weight > 0 and src_feats is not None and tgt_feats is not None
    rt = pose_rt32(T)
    assoc = associate32(sp, sn, sm, rt, tgt_points, tgt_normals, tgt_mask, kcam,
                        distance_threshold, normals_angle_thresh)
    JtJ = np.zeros((6, 6))
    Jr = np.zeros(6)
    residual = 0.0
    count = 0
    scale = 0.0
    geom_count = feat_count = 0
    if use_feat:
        f = feature_terms64(assoc, sp, src_feats, rt, tgt_feats, kcam,
                            feat_residual_thresh, channel_mode)
        JtJ = f.JtJ * feat_weight * feat_weight
        Jr = f.Jtr * -feat_weight
        residual = f.r2 * feat_weight
        count = feat_count = f.count
        scale += f.scale * feat_weight
    if use_geom:
        g = geometric_terms64(assoc, sp, rt, tgt_points, tgt_normals)
        JtJ = JtJ + g.JtJ * geom_weight * geom_weight
        Jr = Jr + g.Jtr * geom_weight
        residual = residual + g.r2 * geom_weight
        geom_count = g.count
        count = max(g.count, count)
        scale += g.scale * geom_weight
    ok, update = cholesky_solve6(JtJ, Jr)
    out = dict(ok=ok, JtJ=JtJ, Jr=Jr, r2=residual, count=count, geom_count=geom_count,
               feat_count=feat_count, Jr_scale=scale, update=update, assoc=assoc)
    if ok:
        out["transform"] = se3_exp(update) @ T
        out["residual"] = residual / count
    return out


def icp_estimate(kcam, src_points, src_normals, src_mask, tgt_points,
                 tgt_normals, tgt_mask, src_feats=None, tgt_feats=None,
                 num_iters=10, geom_weight=1.0, feat_weight=1.0,
                 distance_threshold=0.5, normals_angle_thresh=math.pi / 4,
                 feat_residual_thresh=2.75, transform=None,
                 channel_mode="last"):
    """``ICPOdometry.estimate`` (icp.py:152-262) in float64 on the CPU:
    ``gn_step`` until ``num_iters`` or a failed solve, then the information
    matrix at the last pose (icp.py:258-261)."""
    sp = np.asarray(src_points, dtype=F32).reshape(-1, 3)
    n = sp.shape[0]
    T = np.eye(4) if transform is None else np.asarray(transform, dtype=F64).copy()
    kw = dict(src_feats=src_feats, tgt_feats=tgt_feats, geom_weight=geom_weight,
              feat_weight=feat_weight, distance_threshold=distance_threshold,
              normals_angle_thresh=normals_angle_thresh,
              feat_residual_thresh=feat_residual_thresh, channel_mode=channel_mode)
    res = Result()
    for _ in range(num_iters):
        st = gn_step(T, kcam, sp, src_normals, src_mask, tgt_points, tgt_normals, tgt_mask,
                     **kw)
        if not st["ok"]:
            break
        T = st["transform"]
        res.transform = T.copy()
        res.JtJ = st["JtJ"]
        res.residual = st["residual"]
        res.match_ratio = st["count"] / n
        st.pop("assoc")
        res.history.append(st)
    assoc = associate32(sp, src_normals, src_mask, pose_rt32(T), tgt_points, tgt_normals,
                        tgt_mask, kcam, distance_threshold, normals_angle_thresh)
    res.information = information64(assoc, tgt_points)
    return res


def multiscale_estimate(levels, estimators, transform=None):
    """``MultiscaleRegistration.estimate_frame`` (multiscale.py:30-67).

    ``levels`` are coarsest-first dicts with the ``icp_estimate`` tensor
    arguments; ``estimators`` are the per-level keyword dicts, listed finest
    first as the reference's estimator list (multiscale.py:52-55 reverses
    it).  Reference quirk kept: a result is always truthy, so a level whose
    first iteration fails hands ``transform=None`` (identity) to the next
    level (multiscale.py:64-65)."""
    result = None
    for level, est in zip(levels, estimators[::-1]):
        result = icp_estimate(transform=transform, **level, **est)
        transform = result.transform
    return result


# ---------------------------------------------------------------------------
# point-to-plane loss with frozen correspondences (the differentiable form
# of icp_jacobian_geometric.cu:82; J convention icp_jacobian_common.hpp:41-48)
# ---------------------------------------------------------------------------

class LossMatches:
    """Frozen correspondences of an association: source index ``idx``,
    target point ``q`` and normal ``n`` (float64 of the float32 inputs),
    and the matched target pixel ``pix``."""

    def __init__(self, assoc, tgt_points, tgt_normals):
        win = assoc.winner.reshape(-1)
        self.pix = np.nonzero(win >= 0)[0]
        self.idx = win[self.pix]
        self.q = np.asarray(tgt_points, dtype=F32).reshape(-1, 3)[self.pix].astype(F64)
        self.n = np.asarray(tgt_normals, dtype=F32).reshape(-1, 3)[self.pix].astype(F64)


def loss_residuals64(T, src_points, m):
    """r = (q - (R s + t)).n in float64 at a float64 pose."""
    T = np.asarray(T, dtype=F64)
    s = np.asarray(src_points, dtype=F32).reshape(-1, 3)[m.idx].astype(F64)
    p = s @ T[:3, :3].T + T[:3, 3]
    return ((m.q - p) * m.n).sum(axis=1)


def point_to_plane_loss64(T, src_points, m):
    r = loss_residuals64(T, src_points, m)
    return float((r * r).sum())


def loss_twist_grad_fd(T0, twist, src_points, m, h=1e-6):
    """Central differences of L(exp(twist) T0) over the six twist
    components (float64)."""
    twist = np.asarray(twist, dtype=F64)
    g = np.zeros(6)
    for k in range(6):
        e = np.zeros(6)
        e[k] = h
        lp = point_to_plane_loss64(se3_exp(twist + e) @ T0, src_points, m)
        lm = point_to_plane_loss64(se3_exp(twist - e) @ T0, src_points, m)
        g[k] = (lp - lm) / (2.0 * h)
    return g


def loss_twist_grad64(T, src_points, m):
    """Analytic left-perturbation gradient -2 sum r J, J = [n; Tp x n]
    (float64), and the scale sum 2 |J| |r| its errors are measured against."""
    T = np.asarray(T, dtype=F64)
    s = np.asarray(src_points, dtype=F32).reshape(-1, 3)[m.idx].astype(F64)
    p = s @ T[:3, :3].T + T[:3, 3]
    r = ((m.q - p) * m.n).sum(axis=1)
    J = np.concatenate([m.n, np.cross(p, m.n)], axis=1)
    return -2.0 * (J.T @ r), float(2.0 * (np.linalg.norm(J, axis=1) * np.abs(r)).sum())


def loss_depth_grad_fd(T, src_points, m, kcam, width, pixels, h=1e-6):
    """Central differences of L with respect to the depth of the source
    pixels ``pixels`` (flat indices): the source point moves along its
    back-projection ray d = ((u - cx)/fx, (v - cy)/fy, 1)
    (slamtb/camera.py:127-149).  Returns (grad, r, a) with a = dr/dz, 0
    for pixels without a correspondence."""
    fx, fy, cx, cy = (float(kcam[0][0]), float(kcam[1][1]), float(kcam[0][2]),
                      float(kcam[1][2]))
    T = np.asarray(T, dtype=F64)
    R, t = T[:3, :3], T[:3, 3]
    sp = np.asarray(src_points, dtype=F32).reshape(-1, 3).astype(F64)
    where = {int(i): k for k, i in enumerate(m.idx)}
    out = np.zeros(len(pixels))
    rr = np.zeros(len(pixels))
    aa = np.zeros(len(pixels))
    for j, i in enumerate(pixels):
        k = where.get(int(i))
        if k is None:
            continue
        u, v = i % width, i // width
        d = np.array([(u - cx) / fx, (v - cy) / fy, 1.0])

        def r_of(dz):
            p = R @ (sp[i] + dz * d) + t
            return float((m.q[k] - p) @ m.n[k])

        out[j] = (r_of(h) ** 2 - r_of(-h) ** 2) / (2.0 * h)
        rr[j] = r_of(0.0)
        aa[j] = -float((R.T @ m.n[k]) @ d)
    return out, rr, aa


def se3_left_jacobian_fd(xi, h=1e-6):
    """Columns log(exp(xi + h e_k) exp(xi)^-1) by central differences:
    the SE(3) left Jacobian, exp(xi + d) = exp(J d) exp(xi) + O(|d|^2)."""
    xi = np.asarray(xi, dtype=F64)
    Einv = np.linalg.inv(se3_exp(xi))
    J = np.zeros((6, 6))
    for k in range(6):
        e = np.zeros(6)
        e[k] = h
        J[:, k] = (se3_log(se3_exp(xi + e) @ Einv) - se3_log(se3_exp(xi - e) @ Einv)) / (2 * h)
    return J
