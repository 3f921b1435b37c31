"""Self-tests of the CPU oracle (no GPU): SE(3) algebra, the Jacobian sign
conventions against finite differences, the 6x6 solve, hand-built
association cases (ties, bounds, thresholds, NaN angle), and the vectorised
association and the geometric, feature and information partials against
literal per-point loops of the reference's steps."""
import math

import numpy as np
import pytest
import scipy.linalg

from oracle import icp_oracle as io
from oracle import frame_prep as fp


def _twist_matrix(xi):
    v, w = xi[:3], xi[3:]
    M = np.zeros((4, 4))
    M[:3, :3] = [[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]]
    M[:3, 3] = v
    return M


@pytest.mark.parametrize("scale", [1e-9, 1e-4, 5e-3, 0.05, 0.8, 2.5])
def test_se3_exp_matches_matrix_exponential(scale):
    rng = np.random.default_rng(1)
    for _ in range(5):
        xi = rng.normal(size=6) * scale
        np.testing.assert_allclose(io.se3_exp(xi), scipy.linalg.expm(_twist_matrix(xi)),
                                   rtol=0, atol=1e-13)


def test_se3_log_roundtrip():
    rng = np.random.default_rng(2)
    for s in (1e-7, 1e-3, 0.3, 2.0):
        xi = rng.normal(size=6) * s
        np.testing.assert_allclose(io.se3_log(io.se3_exp(xi)), xi, rtol=1e-9, atol=1e-12)


def test_cholesky_solve6():
    rng = np.random.default_rng(3)
    A = rng.normal(size=(6, 6))
    A = A @ A.T + 0.1 * np.eye(6)
    b = rng.normal(size=6)
    ok, x = io.cholesky_solve6(A, b)
    assert ok
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-10)
    assert not io.cholesky_solve6(np.zeros((6, 6)), b)[0]
    B = A.copy()
    B[2, 2] = -1.0
    assert not io.cholesky_solve6(B, b)[0]
    C = A.copy()
    C[0, 0] = np.nan
    assert not io.cholesky_solve6(C, b)[0]


def test_geometric_jacobian_is_minus_residual_derivative():
    """J = [n; p x n] (icp_jacobian_common.hpp:41-48) equals -dr/dxi for the
    left update T <- exp(xi) T, so the reference's update +solve(JtJ, Jtr)
    (icp.py:233-240) is a Gauss-Newton step."""
    rng = np.random.default_rng(4)
    p = rng.normal(size=3) + [0, 0, 2]
    q = p + rng.normal(size=3) * 0.01
    n = rng.normal(size=3)
    n /= np.linalg.norm(n)

    def r(xi):
        tp = (io.se3_exp(xi) @ np.append(p, 1.0))[:3]
        return (q - tp) @ n

    J = np.concatenate([n, np.cross(p, n)])
    eps = 1e-6
    fd = np.array([(r(eps * e) - r(-eps * e)) / (2 * eps) for e in np.eye(6)])
    np.testing.assert_allclose(fd, -J, rtol=1e-6, atol=1e-9)


def test_feature_jacobian_is_plus_residual_derivative():
    """J_f = [g; p x g] with g = grad(f) dpi/dp equals +dr/dxi for
    r = f(pi(exp(xi) p)) - f_s, hence the reference's -w_f J^T r
    (icp.py:222).  Checked on a linear intensity ramp."""
    k = np.array([[525, 0, 319.5], [0, 525, 239.5], [0, 0, 1]], dtype=np.float64)
    gu, gv = 0.013, -0.007
    p = np.array([0.2, -0.1, 2.0])

    def f(uv):
        return gu * uv[0] + gv * uv[1]

    def proj(x):
        return np.array([k[0, 0] * x[0] / x[2] + k[0, 2], k[1, 1] * x[1] / x[2] + k[1, 2]])

    def r(xi):
        return f(proj((io.se3_exp(xi) @ np.append(p, 1.0))[:3]))

    fx, fy, z = k[0, 0], k[1, 1], p[2]
    g = np.array([gu * fx / z, gv * fy / z, -gu * p[0] * fx / z ** 2 - gv * p[1] * fy / z ** 2])
    J = np.concatenate([g, np.cross(p, g)])
    eps = 1e-6
    fd = np.array([(r(eps * e) - r(-eps * e)) / (2 * eps) for e in np.eye(6)])
    np.testing.assert_allclose(fd, J, rtol=1e-6, atol=1e-9)


def _grid(h=4, w=5, z=2.0):
    pts = np.zeros((h, w, 3), np.float32)
    k = np.array([[100, 0, 2], [0, 100, 1.5], [0, 0, 1]], np.float32)
    for v in range(h):
        for u in range(w):
            pts[v, u] = [(u - k[0, 2]) * z / k[0, 0], (v - k[1, 2]) * z / k[1, 1], z]
    nrm = np.zeros_like(pts)
    nrm[..., 2] = -1
    return pts, nrm, np.ones((h, w), bool), k


def test_association_tie_goes_to_smaller_index():
    pts, nrm, mask, k = _grid()
    # two identical sources land on the same pixel at the same distance
    src = np.stack([pts[1, 2], pts[1, 2]]).astype(np.float32)
    a = io.associate32(src, np.stack([nrm[1, 2]] * 2), np.ones(2, bool), io.pose_rt32(np.eye(4)),
                       pts, nrm, mask, k, 0.1, math.pi / 4)
    assert a.winner[1, 2] == 0 and a.count == 1
    assert (a.ref_map[1, 2] >> 32) == 0
    assert a.ref_map[0, 0] == io.CORRESP_EMPTY


def test_association_bounds_and_rounding():
    pts, nrm, mask, k = _grid()
    # u in [-0.5, 0) rounds to column 0 (kept); u = -0.5 rounds to -1 (dropped)
    z = np.float32(2.0)
    def at_u(u):
        return np.array([[(u - k[0, 2]) * z / k[0, 0], 0.0, z]], np.float32)
    keep = io.associate32(at_u(-0.4), nrm[:1, 0], np.ones(1, bool), io.pose_rt32(np.eye(4)),
                          pts, nrm, mask, k, 10.0, math.pi)
    drop = io.associate32(at_u(-0.5), nrm[:1, 0], np.ones(1, bool), io.pose_rt32(np.eye(4)),
                          pts, nrm, mask, k, 10.0, math.pi)
    assert keep.count == 1 and drop.count == 0


def test_association_thresholds_and_nan_angle():
    pts, nrm, mask, k = _grid()
    src = pts[2, 3][None].copy()
    far = src.copy()
    far[0, 2] += 0.2
    eye = io.pose_rt32(np.eye(4))
    one = np.ones(1, bool)
    assert io.associate32(far, nrm[2, 3][None], one, eye, pts, nrm, mask, k, 0.1, math.pi).count == 0
    tilted = np.array([[0.0, math.sin(0.5), -math.cos(0.5)]], np.float32)  # 0.5 rad off
    assert io.associate32(src, tilted, one, eye, pts, nrm, mask, k, 0.1, 0.4).count == 0
    assert io.associate32(src, tilted, one, eye, pts, nrm, mask, k, 0.1, 0.6).count == 1
    # a zero normal gives a NaN cosine, which the reference accepts
    zero = np.zeros((1, 3), np.float32)
    assert io.associate32(src, zero, one, eye, pts, nrm, mask, k, 0.1, 0.1).count == 1
    # masked target pixel
    m2 = mask.copy()
    m2[2, 3] = False
    assert io.associate32(src, nrm[2, 3][None], one, eye, pts, nrm, m2, k, 0.1, math.pi).count == 0


def test_angle_threshold_rounding():
    for th in (0.1, math.pi / 9, math.pi / 4, 1.0, 3.0):
        c = io.angle_cos_threshold(th)
        assert float(c) <= math.cos(float(np.float32(th)))
        assert float(np.nextafter(c, np.float32(1))) > math.cos(float(np.float32(th)))
    assert io.angle_cos_threshold(math.pi) == -np.inf


def test_partials_sum_to_terms():
    """The float32 per-point partials (the _cslamtb contract) sum to the
    float64 reduced terms within float32 accuracy."""
    from _helpers import synthetic_pair
    d = synthetic_pair(5, width=160, height=120, feature_channels=0)
    s, t = d["src"], d["tgt"]
    rt = io.pose_rt32(np.eye(4))
    a = io.associate32(s["points"], s["normals"], s["mask"], rt, t["points"], t["normals"],
                       t["mask"], d["kcam"], 0.1, math.radians(20))
    JtJ, Jtr, r2, cnt = io.geometric_partials32(s["points"], s["mask"], rt, t["points"],
                                                t["normals"], d["kcam"], a.ref_map)
    g = io.geometric_terms64(a, s["points"], rt, t["points"], t["normals"])
    assert cnt == g.count == a.count > 100
    np.testing.assert_allclose(JtJ.astype(np.float64).sum(0), g.JtJ, rtol=1e-5,
                               atol=1e-5 * np.abs(g.JtJ).max())
    np.testing.assert_allclose(Jtr.astype(np.float64).sum(0), g.Jtr, rtol=0, atol=1e-5 * g.scale)
    JtJ, Jtr, r2, cnt, passed = io.feature_partials32(
        s["points"], d["src_feats"], s["mask"], rt, d["tgt_feats"], d["kcam"], a.ref_map, 2.75)
    f = io.feature_terms64(a, s["points"], d["src_feats"], rt, d["tgt_feats"], d["kcam"], 2.75)
    assert cnt == f.count
    np.testing.assert_allclose(JtJ.astype(np.float64).sum(0), f.JtJ, rtol=1e-4,
                               atol=1e-4 * np.abs(f.JtJ).max())


def test_erode_quirk_ignores_row_below():
    m = np.ones((5, 5), bool)
    m[3, 2] = False  # the pixel below (2, 2)
    e = fp.erode_mask(m)
    assert e[2, 2]  # reference neighbourhood never looks down (erode_mask.cu:24)
    assert not e[4, 2]  # looks up
    assert not e[3, 1] and not e[3, 3]  # left / right


def test_normals_of_a_plane():
    k = np.array([[300, 0, 31.5], [0, 300, 23.5], [0, 0, 1]], np.float32)
    v, u = np.mgrid[0:48, 0:64].astype(np.float32)
    n = np.array([0.2, -0.3, -1.0])
    n /= np.linalg.norm(n)
    # plane n.x = d  ->  z = d / (n . ((u-cx)/fx, (v-cy)/fy, 1))
    rays = np.stack([(u - k[0, 2]) / k[0, 0], (v - k[1, 2]) / k[1, 1], np.ones_like(u)], -1)
    z = (-2.0 / (rays @ n)).astype(np.float32)
    pts = fp.depth_to_points(z, k)
    nr = fp.estimate_normals(pts, np.ones(z.shape, bool))
    inner = nr[1:-1, 1:-1].reshape(-1, 3)
    dots = np.abs(inner @ n)
    assert dots.min() > 0.999


def _ad(xi):
    A = np.zeros((6, 6))
    A[:3, :3] = io._hat(xi[3:])
    A[:3, 3:] = io._hat(xi[:3])
    A[3:, 3:] = io._hat(xi[3:])
    return A


@pytest.mark.parametrize("scale", [0.0, 1e-4, 0.3, 1.5])
def test_se3_left_jacobian_series(scale):
    """The power series sum ad^n / (n+1)! that stb_se3_twist_grad sums is
    the left Jacobian of the oracle's exp (central differences of log)."""
    rng = np.random.default_rng(int(scale * 10) + 3)
    xi = rng.normal(size=6) * scale
    S, term = np.eye(6), np.eye(6)
    for n in range(1, 60):
        term = term @ _ad(xi) / (n + 1)
        S = S + term
    np.testing.assert_allclose(io.se3_left_jacobian_fd(xi), S, atol=1e-8)


def test_loss_gradients_fd_vs_analytic():
    """Oracle self-check of the loss gradients on a small synthetic pair:
    the analytic -2 sum r J and dr/dz against central differences."""
    from _helpers import synthetic_pair
    d = synthetic_pair(3, width=80, height=60)
    s, t = d["src"], d["tgt"]
    T = io.se3_exp([0.004, -0.003, 0.002, 0.003, -0.002, 0.001])
    a = io.associate32(s["points"], s["normals"], s["mask"], io.pose_rt32(T), t["points"],
                       t["normals"], t["mask"], d["kcam"], 0.1, math.radians(20))
    m = io.LossMatches(a, t["points"], t["normals"])
    assert m.idx.size > 500
    an, scale = io.loss_twist_grad64(T, s["points"], m)
    fd = io.loss_twist_grad_fd(T, np.zeros(6), s["points"], m)
    assert np.abs(an - fd).max() <= 1e-7 * scale
    pix = m.idx[:16]
    g, r, dr = io.loss_depth_grad_fd(T, s["points"], m, d["kcam"], 80, pix)
    np.testing.assert_allclose(g, 2 * r * dr, rtol=1e-6, atol=1e-12)


def test_registration_verifier_rules():
    """RegistrationVerifier (slamtb/registration/result.py:49-95): a result
    passes when its residual, the largest covariance eigenvalue (inverse of
    the information matrix) and its match ratio are all within bounds."""
    import torch
    from slamtb_gb300.registration import RegistrationResult, RegistrationVerifier

    def res(residual, info_scale, ratio):
        return RegistrationResult(torch.eye(4, dtype=torch.float64),
                                  torch.eye(6, dtype=torch.float32) * info_scale, residual, ratio)
    v = RegistrationVerifier()
    assert v(res(1e-5, 1e6, 0.9))
    assert not v(res(1e-3, 1e6, 0.9))     # residual above 1e-4
    assert not v(res(1e-5, 1e2, 0.9))     # covariance eigenvalue 1e-2 above 1e-4
    assert not v(res(1e-5, 1e6, 0.1))     # match ratio below 0.6


def test_bilateral_oracle_matches_literal_loop():
    """The vectorised restatement of BilateralDepthFilterKernel
    (src/bilateral_depth_filter.cu:37-71) against a literal per-pixel loop
    of the same float32 operations, on a small image with masked pixels."""
    F = np.float32
    rng = np.random.default_rng(0)
    d = (rng.random((9, 11)) * 3000).astype(np.int32)
    d[2, 3] = 0
    d[5, :] = 0
    m = d > 0
    out = fp.bilateral_depth_filter(d, m, 5, 4.5, 29.99, 1.0)
    hw = 2
    isc = F(1.0 / float(F(F(4.5) * F(4.5))))
    iss = F(1.0 / float(F(F(29.99) * F(29.99))))
    ref = np.zeros_like(d)
    for r in range(9):
        for c in range(11):
            if not m[r, c]:
                continue
            z, cs, ws = F(d[r, c]), F(0), F(0)
            for y in range(-hw, hw + 1):
                for x in range(-hw, hw + 1):
                    kr, kc = r + y, c + x
                    if not (0 <= kr < 9 and 0 <= kc < 11) or not m[kr, kc]:
                        continue
                    cz = F(d[kr, kc])
                    sp = F(F(F(-x) * F(-x)) + F(F(-y) * F(-y)))
                    dc = F(z - cz)
                    wt = F(np.exp(F(F(-0.5) * F(F(sp * iss) + F(F(dc * dc) * isc)))))
                    cs, ws = F(cs + F(cz * wt)), F(ws + wt)
            ref[r, c] = int(np.trunc(F(cs / ws)))
    np.testing.assert_array_equal(out, ref)


def test_exp_rt_oracle_is_a_rotation_with_the_twist_axis():
    from oracle import autograd_oracle as ao
    rng = np.random.default_rng(5)
    for w in [np.zeros(3), np.array([1e-9, 0, 0]), rng.normal(size=3) * 0.1,
              rng.normal(size=3) * 1.2]:
        R = ao.rotation64(w)
        np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-14)
        assert abs(np.linalg.det(R) - 1.0) < 1e-13
        np.testing.assert_allclose(R @ w, w, atol=1e-14)
        np.testing.assert_allclose(np.trace(R), 1 + 2 * np.cos(np.linalg.norm(w)), atol=1e-13)


def test_exp_rt_backward_oracle_matches_finite_differences():
    """The Gallego-Yezzi restatement against central differences of the
    forward, including angles near the 1e-12 switch."""
    from oracle import autograd_oracle as ao
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.normal(size=(6, 3)), rng.normal(size=(6, 3))], axis=1)
    x[1, 3:] *= 1e-3
    x[2, 3:] *= 2.5 / np.linalg.norm(x[2, 3:])
    x[3, 3:] = 0.0
    g = rng.normal(size=(6, 3, 4))
    an = ao.exp_rt_to_matrix_backward64(g, x)
    fd = ao.exp_rt_to_matrix_fd64(g, x)
    np.testing.assert_allclose(an, fd, rtol=1e-7, atol=1e-8)


def test_matrix_to_exp_rt_oracle_round_trip():
    from oracle import autograd_oracle as ao
    rng = np.random.default_rng(7)
    x = rng.normal(size=(8, 6))
    x[:, 3:] *= (rng.uniform(0.01, 3.0, size=8) / np.linalg.norm(x[:, 3:], axis=1))[:, None]
    np.testing.assert_allclose(ao.matrix_to_exp_rt64(ao.exp_rt_to_matrix64(x)), x, atol=1e-10)


def test_fpcl_matcher_oracle_matches_literal_loops():
    """The vectorised matcher restatement against per-point loops of the
    same float32 operations (fpcl_matcher.cu:46-80 and :150-189)."""
    from oracle import autograd_oracle as ao
    F = np.float32
    rng = np.random.default_rng(8)
    h, w, c = 6, 7, 2
    kcam = np.array([[5.0, 0, 3.1], [0, 5.0, 2.6], [0, 0, 1]], F)
    tp = rng.normal(size=(h, w, 3)).astype(F)
    tn = rng.normal(size=(h, w, 3)).astype(F)
    tf = rng.normal(size=(c, h, w)).astype(F)
    sp = np.stack([rng.uniform(-0.8, 0.8, 12), rng.uniform(-0.6, 0.6, 12),
                   rng.uniform(1.0, 2.0, 12)], 1).astype(F)
    ref = np.full((h, w), 0x0FFFFFFF7F800000, np.int64)
    for i, p in enumerate(sp):      # every point wins its own pixel when free
        uu = (kcam[0, 0] * p[0]) / p[2] + kcam[0, 2]
        vv = (kcam[1, 1] * p[1]) / p[2] + kcam[1, 2]
        r, q = int(np.floor(vv + 0.5)), int(np.floor(uu + 0.5))
        if 0 <= r < h and 0 <= q < w and (ref[r, q] >> 32) == 0x0FFFFFFF:
            ref[r, q] = np.int64(i) << 32
    pts, nrm, fts, mask = ao.fpcl_forward32(tp, tn, tf, sp, kcam, ref)
    dl = rng.normal(size=(c, 12)).astype(F)
    dx = ao.fpcl_backward32(tf, sp, mask, dl, kcam, 0.005)

    def bil(ch, u, v):
        ui, vi = int(np.trunc(u)), int(np.trunc(v))
        ur, vr = F(u - F(ui)), F(v - F(vi))
        f = tf[ch]
        v00 = f[vi, ui]
        v10 = f[vi, ui + 1] if ui + 1 < w else F(0)
        v01 = f[vi + 1, ui] if vi + 1 < h else F(0)
        v11 = f[vi + 1, ui + 1] if (ui + 1 < w and vi + 1 < h) else F(0)
        a0 = F(F(v00 * F(F(1) - ur)) + F(v10 * ur))
        a1 = F(F(v01 * F(F(1) - ur)) + F(v11 * ur))
        return F(F(a0 * F(F(1) - vr)) + F(a1 * vr))

    for i, p in enumerate(sp):
        u = F(F(F(kcam[0, 0] * p[0]) / p[2]) + kcam[0, 2])
        v = F(F(F(kcam[1, 1] * p[1]) / p[2]) + kcam[1, 2])
        q, r = int(np.floor(float(u) + 0.5)), int(np.floor(float(v) + 0.5))
        ok = 0 <= q < w and 0 <= r < h and (ref[r, q] >> 32) == i
        assert mask[i] == ok
        if not ok:
            assert not pts[i].any() and not dx[i].any()
            continue
        np.testing.assert_array_equal(pts[i], tp[r, q])
        for ch in range(c):
            assert fts[ch, i] == bil(ch, u, v)
        hh = F(0.005)
        dv = F(F(1) / F(F(2) * hh))
        gu = gv = F(0)
        for ch in range(c):
            du = F(F(bil(ch, F(u + hh), v) - bil(ch, max(F(u - hh), F(0)), v)) * dv)
            dvv = F(F(bil(ch, u, F(v + hh)) - bil(ch, u, max(F(v - hh), F(0)))) * dv)
            gu = F(gu + F(du * dl[ch, i]))
            gv = F(gv + F(dvv * dl[ch, i]))
        z2 = F(p[2] * p[2])
        j00, j02 = F(kcam[0, 0] / p[2]), F(F(-p[0] * kcam[0, 0]) / z2)
        j11, j12 = F(kcam[1, 1] / p[2]), F(F(-p[1] * kcam[1, 1]) / z2)
        np.testing.assert_array_equal(dx[i], [F(j00 * gu), F(j11 * gv),
                                              F(F(j02 * gu) + F(j12 * gv))])
    assert mask.sum() >= 4


def _round_half_away(x):
    """C ``round`` on a float32 value (exact in float64)."""
    return int(math.copysign(math.floor(abs(float(x)) + 0.5), float(x)))


def _associate_literal(sp, sn, sm, rt, tp, tn, tm, kcam, dist_th, angle_th):
    """Per source point, in index order, the reference's own steps in
    float32 scalars: ``CorrespondenceMapKernel`` (correspondence_map.cu:39-61)
    -> ``RigidTransform::Transform/TransformNormal`` (camera.hpp:134-165) ->
    ``RobustCorrespondence::Match`` (correspondence.hpp:69-89: project,
    round, bounds, target mask, squared distance, ``GetVectorsAngle``,
    math.hpp:14-18) -> ``MergeMap::Set`` (merge_map.hpp:37-50: replace when
    the distance is smaller, so a tie keeps the first, smaller index)."""
    f = np.float32
    h, w = tm.shape
    nm = io.normal_matrix32(rt)
    d2 = f(float(dist_th) * float(dist_th))
    ath = f(angle_th)
    fx, cx, fy, cy = f(kcam[0, 0]), f(kcam[0, 2]), f(kcam[1, 1]), f(kcam[1, 2])
    best = {}
    for i in range(sp.shape[0]):
        if sm.size == sp.shape[0] and not sm[i]:
            continue
        p = [((rt[k, 0] * sp[i, 0] + rt[k, 1] * sp[i, 1]) + rt[k, 2] * sp[i, 2]) + rt[k, 3]
             for k in range(3)]
        n = [(nm[k, 0] * sn[i, 0] + nm[k, 1] * sn[i, 1]) + nm[k, 2] * sn[i, 2] for k in range(3)]
        u = (fx * p[0]) / p[2] + cx
        v = (fy * p[1]) / p[2] + cy
        ui, vi = _round_half_away(u), _round_half_away(v)
        if ui < 0 or ui >= w or vi < 0 or vi >= h or not tm[vi, ui]:
            continue
        q, m = tp[vi, ui], tn[vi, ui]
        d = [q[k] - p[k] for k in range(3)]
        sq = d[0] * d[0] + (d[1] * d[1] + d[2] * d[2])  # Eigen squaredNorm
        if sq > d2:
            continue
        dot = n[0] * m[0] + (n[1] * m[1] + n[2] * m[2])  # Eigen dot, norm
        na = np.sqrt(n[0] * n[0] + (n[1] * n[1] + n[2] * n[2]))
        nb = np.sqrt(m[0] * m[0] + (m[1] * m[1] + m[2] * m[2]))
        with np.errstate(invalid="ignore"):
            angle = abs(np.arccos(dot / (na * nb)))
        if angle >= ath:
            continue
        dist = np.sqrt(sq)
        if (vi, ui) not in best or dist < best[(vi, ui)][0]:
            best[(vi, ui)] = (dist, i)
    return best


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_association_matches_the_reference_steps_point_by_point(seed):
    """The vectorised float32 association (the bit-exact gate of the GPU
    kernels) equals a literal per-point loop of the reference's steps:
    winners, distance bits and the int64 map layout (index << 32 | distance
    bits, empty = 0x0fffffff7f800000), with duplicated source points so
    that distance ties occur."""
    rng = np.random.default_rng(seed)
    h, w = 18, 24
    kcam = np.array([[30.0, 0, 11.5], [0, 30.0, 8.5], [0, 0, 1]], dtype=np.float32)
    vv, uu = np.mgrid[0:h, 0:w].astype(np.float32)
    z = (1.2 + 0.3 * uu / w + 0.2 * vv / h + rng.normal(0, 0.005, size=(h, w))).astype(np.float32)
    tp = np.stack([(uu - kcam[0, 2]) * z / kcam[0, 0], (vv - kcam[1, 2]) * z / kcam[1, 1], z],
                  axis=-1).astype(np.float32)
    tn = rng.normal(size=(h, w, 3)).astype(np.float32)
    tn[..., 2] = -np.abs(tn[..., 2]) - 0.5
    tm = rng.random((h, w)) > 0.15
    sp = (tp.reshape(-1, 3) + rng.normal(0, 0.03, size=(h * w, 3))).astype(np.float32)
    sn = (tn.reshape(-1, 3) + rng.normal(0, 0.1, size=(h * w, 3))).astype(np.float32)
    dup = rng.choice(h * w, size=40, replace=False)
    sp[dup[20:]], sn[dup[20:]] = sp[dup[:20]], sn[dup[:20]]  # ties
    sm = rng.random(h * w) > 0.1
    ang = 0.02 * seed
    rt = np.array([[math.cos(ang), -math.sin(ang), 0, 0.01], [math.sin(ang), math.cos(ang), 0, 0],
                   [0, 0, 1, 0.005], [0, 0, 0, 1]], dtype=np.float32)
    dth, ath = 0.1, math.radians(30)
    a = io.associate32(sp, sn, sm, rt, tp, tn, tm, kcam, dth, ath)
    best = _associate_literal(sp, sn, sm, rt, tp, tn, tm, kcam, dth, ath)
    assert len(best) > 100
    winners = np.full((h, w), -1, dtype=np.int64)
    dist = np.full((h, w), np.inf, dtype=np.float32)
    for (vi, ui), (d, i) in best.items():
        winners[vi, ui], dist[vi, ui] = i, d
    np.testing.assert_array_equal(a.winner, winners)
    np.testing.assert_array_equal(a.dist.view(np.uint32), dist.view(np.uint32))
    ref = np.where(winners >= 0, (winners << 32) | dist.view(np.uint32).astype(np.int64),
                   np.int64(io.CORRESP_EMPTY))
    np.testing.assert_array_equal(a.ref_map, ref)
    # ties: both copies of a duplicated point valid, so both reach the same
    # pixel at the same distance; the smaller index holds it
    won = set(winners[winners >= 0].tolist())
    ties = [(a, b) for a, b in zip(dup[:20].tolist(), dup[20:].tolist())
            if sm[a] and sm[b] and (a in won or b in won)]
    assert ties and all(min(a, b) in won and max(a, b) not in won for a, b in ties)


def _feature_partials_literal(sp, sf, sm, rt, tf, kcam, ref_map, thresh):
    """Per source point, the reference's ``FeatureJacobianKernel``
    (icp_jacobian_feature.cu:58-109) in float32 scalars: ``BilinearInterp``
    with C truncation and zero taps past the right / bottom edge,
    ``BilinearInterpGrad`` at (u + h, v), (max(u - h, 0), v), ... with the
    divisor 1 / (2h) (feature_map.hpp:15-63), ``Dx_Project`` (camera.hpp:
    65-78) and ``SE3ICPJacobian::Compute`` assigning the partials per
    channel (icp_jacobian_common.hpp:37-61)."""
    f = np.float32
    c, h, w = tf.shape
    n = sp.shape[0]
    JtJ = np.zeros((n, 6, 6), f)
    Jtr = np.zeros((n, 6), f)
    r2 = np.zeros(n, f)
    fx, cx, fy, cy = f(kcam[0, 0]), f(kcam[0, 2]), f(kcam[1, 1]), f(kcam[1, 2])
    step = f(0.05)
    div = f(1) / (f(2) * step)
    count = 0

    def interp(ch, u, v):
        ui, vi = int(u), int(v)  # truncation toward zero, as int(scalar_t)
        ur, vr = u - f(ui), v - f(vi)
        m = tf[ch]
        v00 = m[vi, ui]
        v10 = m[vi, ui + 1] if ui + 1 < w else f(0)
        v01 = m[vi + 1, ui] if vi + 1 < h else f(0)
        v11 = m[vi + 1, ui + 1] if ui + 1 < w and vi + 1 < h else f(0)
        a0 = v00 * (f(1) - ur) + v10 * ur
        a1 = v01 * (f(1) - ur) + v11 * ur
        return a0 * (f(1) - vr) + a1 * vr

    for i in range(n):
        if not sm[i]:
            continue
        p = [((rt[k, 0] * sp[i, 0] + rt[k, 1] * sp[i, 1]) + rt[k, 2] * sp[i, 2]) + rt[k, 3]
             for k in range(3)]
        u = (fx * p[0]) / p[2] + cx
        v = (fy * p[1]) / p[2] + cy
        ui, vi = _round_half_away(u), _round_half_away(v)
        if ui < 0 or ui >= w or vi < 0 or vi >= h or (int(ref_map[vi, ui]) >> 32) != i:
            continue
        z2 = p[2] * p[2]
        j00, j02 = fx / p[2], (-p[0] * fx) / z2
        j11, j12 = fy / p[2], (-p[1] * fy) / z2
        sq = f(0)
        for ch in range(c):
            r = interp(ch, u, v) - sf[ch, i]
            du = (interp(ch, u + step, v) - interp(ch, max(u - step, f(0)), v)) * div
            dv = (interp(ch, u, v + step) - interp(ch, u, max(v - step, f(0)))) * div
            g = [du * j00, dv * j11, du * j02 + dv * j12]
            J = g + [p[1] * g[2] - p[2] * g[1], p[2] * g[0] - p[0] * g[2],
                     p[0] * g[1] - p[1] * g[0]]
            for a in range(6):
                Jtr[i, a] = J[a] * r
                for b in range(6):
                    JtJ[i, a, b] = J[b] * J[a]
            sq = sq + r * r
        if sq > f(thresh) * f(thresh):
            JtJ[i], Jtr[i] = 0, 0
            continue
        r2[i] = sq
        count += 1
    return JtJ, Jtr, r2, count


@pytest.mark.parametrize("seed", [0, 1])
def test_feature_partials_match_the_reference_steps_point_by_point(seed):
    """The vectorised float32 feature partials equal a literal per-point loop
    of the reference's kernel bit for bit, on 2 channels (only the last
    channel's J survives), with projections at the image borders (negative
    bilinear weights left of column 0, zero taps past the right and bottom
    edges) and a residual threshold that rejects some matches."""
    rng = np.random.default_rng(seed)
    h, w, c = 14, 20, 2
    kcam = np.array([[24.0, 0, 9.5], [0, 24.0, 6.5], [0, 0, 1]], dtype=np.float32)
    vv, uu = np.mgrid[0:h, 0:w].astype(np.float32)
    z = (1.3 + 0.2 * uu / w + 0.1 * vv / h).astype(np.float32)
    tp = np.stack([(uu - kcam[0, 2]) * z / kcam[0, 0], (vv - kcam[1, 2]) * z / kcam[1, 1], z],
                  axis=-1).astype(np.float32)
    tn = np.broadcast_to(np.array([0, 0, -1], np.float32), (h, w, 3)).copy()
    tm = np.ones((h, w), bool)
    sp = (tp.reshape(-1, 3) + rng.normal(0, 0.02, size=(h * w, 3))).astype(np.float32)
    sn = tn.reshape(-1, 3).copy()
    sm = rng.random(h * w) > 0.05
    rt = np.eye(4, dtype=np.float32)
    tf = rng.random((c, h, w)).astype(np.float32)
    sf = rng.random((c, h * w)).astype(np.float32)
    thresh = 0.6
    ref_map = io.associate32(sp, sn, sm, rt, tp, tn, tm, kcam, 0.1, math.radians(30)).ref_map
    JtJ, Jtr, r2, cnt, passed = io.feature_partials32(sp, sf, sm, rt, tf, kcam, ref_map, thresh)
    lJtJ, lJtr, lr2, lcnt = _feature_partials_literal(sp, sf, sm, rt, tf, kcam, ref_map, thresh)
    assert cnt == lcnt > 50
    np.testing.assert_array_equal(Jtr.view(np.uint32), lJtr.view(np.uint32))
    np.testing.assert_array_equal(JtJ.view(np.uint32), lJtJ.view(np.uint32))
    np.testing.assert_array_equal(r2.view(np.uint32), lr2.view(np.uint32))
    # the border and threshold cases occurred
    T = io.transform32(rt, sp)
    u, v = io.project32(kcam, T)
    winners = set(io.winners_from_ref_map(ref_map)[ref_map != io.CORRESP_EMPTY].tolist())
    won = np.array(sorted(winners))
    assert np.any(u[won] < 0) or np.any(v[won] < 0)
    assert np.any(u[won] + np.float32(0.05) >= w - 1) or np.any(v[won] + np.float32(0.05) >= h - 1)
    assert cnt < len(won)  # the threshold rejected some matches


def test_geometric_and_information_partials_match_the_reference_steps():
    """``GeometricJacobianKernel`` and ``InformationMatrixKernel``
    (icp_jacobian_geometric.cu:54-85,118-158) as literal per-point loops in
    float32 scalars equal the vectorised partials bit for bit: r = (q - Tp).n,
    J = [n; Tp x n] with the partials assigned by
    ``SE3ICPJacobian::Compute``, and G^T G summed row by row from the
    matched target point."""
    f = np.float32
    rng = np.random.default_rng(4)
    h, w = 16, 22
    kcam = np.array([[26.0, 0, 10.5], [0, 26.0, 7.5], [0, 0, 1]], dtype=np.float32)
    vv, uu = np.mgrid[0:h, 0:w].astype(np.float32)
    z = (1.1 + 0.3 * uu / w + 0.2 * vv / h).astype(np.float32)
    tp = np.stack([(uu - kcam[0, 2]) * z / kcam[0, 0], (vv - kcam[1, 2]) * z / kcam[1, 1], z],
                  axis=-1).astype(np.float32)
    tn = rng.normal(size=(h, w, 3)).astype(np.float32)
    tn[..., 2] = -np.abs(tn[..., 2]) - 1.0
    tm = rng.random((h, w)) > 0.1
    sp = (tp.reshape(-1, 3) + rng.normal(0, 0.02, size=(h * w, 3))).astype(np.float32)
    sn = (tn.reshape(-1, 3) + rng.normal(0, 0.05, size=(h * w, 3))).astype(np.float32)
    sm = rng.random(h * w) > 0.05
    rt = np.array([[1, -0.01, 0, 0.004], [0.01, 1, 0, -0.002], [0, 0, 1, 0.003], [0, 0, 0, 1]],
                  dtype=np.float32)
    ref_map = io.associate32(sp, sn, sm, rt, tp, tn, tm, kcam, 0.1, math.radians(30)).ref_map
    JtJ, Jtr, r2, cnt = io.geometric_partials32(sp, sm, rt, tp, tn, kcam, ref_map)
    GtG = io.information_partials32(sp, sm, rt, tp, kcam, ref_map)

    n = sp.shape[0]
    lJtJ, lJtr, lr2, lG = (np.zeros((n, 6, 6), f), np.zeros((n, 6), f), np.zeros(n, f),
                           np.zeros((n, 6, 6), f))
    lcnt = 0
    fx, cx, fy, cy = f(kcam[0, 0]), f(kcam[0, 2]), f(kcam[1, 1]), f(kcam[1, 2])
    for i in range(n):
        if not sm[i]:
            continue
        p = [((rt[k, 0] * sp[i, 0] + rt[k, 1] * sp[i, 1]) + rt[k, 2] * sp[i, 2]) + rt[k, 3]
             for k in range(3)]
        ui = _round_half_away((fx * p[0]) / p[2] + cx)
        vi = _round_half_away((fy * p[1]) / p[2] + cy)
        if ui < 0 or ui >= w or vi < 0 or vi >= h or (int(ref_map[vi, ui]) >> 32) != i:
            continue
        q, m = tp[vi, ui], tn[vi, ui]
        lcnt += 1
        d = [q[k] - p[k] for k in range(3)]
        r = d[0] * m[0] + (d[1] * m[1] + d[2] * m[2])  # Eigen dot
        J = [m[0], m[1], m[2], p[1] * m[2] - p[2] * m[1], p[2] * m[0] - p[0] * m[2],
             p[0] * m[1] - p[1] * m[0]]
        for a in range(6):
            lJtr[i, a] = J[a] * r
            for b in range(6):
                lJtJ[i, a, b] = J[b] * J[a]
        lr2[i] = r * r
        rows = ([f(0), q[2], -q[1], f(1), f(0), f(0)], [-q[2], f(0), q[0], f(0), f(1), f(0)],
                [q[1], -q[0], f(0), f(0), f(0), f(1)])
        for a in range(6):
            for b in range(6):
                lG[i, a, b] = (rows[0][a] * rows[0][b] + rows[1][a] * rows[1][b]) + \
                    rows[2][a] * rows[2][b]
    assert cnt == lcnt > 100
    for x, y in ((JtJ, lJtJ), (Jtr, lJtr), (r2, lr2), (GtG, lG)):
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


def test_normals_and_xyz_downsample_match_the_reference_steps():
    """``CentralDifferencesKernel`` (normals.cu:27-100) and the
    nearest-to-mean XYZ downsample (downsample.cu:25-72) as literal
    per-pixel loops in float32 scalars equal the vectorised restatements
    bit for bit, on a surface with depth jumps (both ratio branches) and
    masked pixels."""
    f = np.float32
    rng = np.random.default_rng(5)
    h, w = 12, 15
    k = np.array([[20.0, 0, 7.0], [0, 20.0, 5.5], [0, 0, 1]], dtype=np.float32)
    depth = (1.0 + 0.05 * rng.random((h, w))).astype(np.float32)
    depth[:, 9:] += f(0.4)  # a step: one-sided differences next to it
    depth[4, 3] += f(0.2)
    xyz = fp.depth_to_points(depth, k)
    mask = rng.random((h, w)) > 0.15

    def v3(r, c):
        return [xyz[r, c, 0], xyz[r, c, 1], xyz[r, c, 2]]

    def sub(a, b):
        return [a[0] - b[0], a[1] - b[1], a[2] - b[2]]

    def sq(a):  # Eigen squaredNorm
        return a[0] * a[0] + (a[1] * a[1] + a[2] * a[2])

    zero = [f(0), f(0), f(0)]
    normals = np.zeros((h, w, 3), f)
    for r in range(h):
        for c in range(w):
            if not mask[r, c]:
                continue
            ce = v3(r, c)
            le = v3(r, c - 1) if c > 0 and mask[r, c - 1] else zero
            ri = v3(r, c + 1) if c < w - 1 and mask[r, c + 1] else zero
            to = v3(r - 1, c) if r > 0 and mask[r - 1, c] else zero
            bo = v3(r + 1, c) if r < h - 1 and mask[r + 1, c] else zero
            t2 = f(2.0) * f(2.0)
            with np.errstate(divide="ignore", invalid="ignore"):
                lds, rds = sq(sub(le, ce)), sq(sub(ri, ce))
                ratio = lds / rds
                if ratio < t2 and ratio > f(1.0) / t2:
                    l2r = sub(ri, le)
                elif lds < rds:
                    l2r = sub(ce, le)
                else:
                    l2r = sub(ri, ce)
                bds, tds = sq(sub(bo, ce)), sq(sub(to, ce))
                ratio = bds / tds
                if ratio < t2 and ratio > f(1.0) / t2:
                    b2t = sub(to, bo)
                elif bds < tds:
                    b2t = sub(ce, bo)
                else:
                    b2t = sub(to, ce)
            n = [l2r[1] * b2t[2] - l2r[2] * b2t[1], l2r[2] * b2t[0] - l2r[0] * b2t[2],
                 l2r[0] * b2t[1] - l2r[1] * b2t[0]]
            length = np.sqrt(sq(n))
            normals[r, c] = [f(0), f(0), f(-1)] if not length > f(1e-6) else \
                [n[0] / length, n[1] / length, n[2] / length]
    np.testing.assert_array_equal(fp.estimate_normals(xyz, mask).view(np.uint32),
                                  normals.view(np.uint32))

    scale = 0.5
    inv = f(1) / f(scale)
    dh, dw = int(h * scale), int(w * scale)
    down = np.zeros((dh, dw, 3), f)
    taps = ((0, 0), (0, 1), (1, 0), (1, 1))
    for r in range(dh):
        for c in range(dw):
            r0, c0 = int(f(r) * inv), int(f(c) * inv)
            valid = [(r0 + a, c0 + b) for a, b in taps
                     if c0 + b < w and r0 + a < h and mask[r0 + a, c0 + b]]
            mean = zero
            for rr, cc in valid:
                mean = [mean[0] + xyz[rr, cc, 0], mean[1] + xyz[rr, cc, 1],
                        mean[2] + xyz[rr, cc, 2]]
            with np.errstate(divide="ignore", invalid="ignore"):
                cnt = f(len(valid))
                mean = [mean[0] / cnt, mean[1] / cnt, mean[2] / cnt]
            best = f(np.inf)
            for rr, cc in valid:
                d = sq(sub(v3(rr, cc), mean))
                if d < best:
                    best, down[r, c] = d, xyz[rr, cc]
    np.testing.assert_array_equal(fp.downsample_xyz_nearest(xyz, mask, scale).view(np.uint32),
                                  down.view(np.uint32))
    assert mask.sum() > 100
    assert not np.any(np.all(normals == 0, axis=-1) & mask)  # every valid pixel has a normal


@pytest.mark.parametrize("scale", [0.5, 0.6])
def test_feature_and_mask_downsample_match_the_reference_steps(scale):
    """``DownsampleFeatureKernel`` (downsample.cu:133-168: the taps' sum in
    order, divided by their count) and the nearest mask downsample
    (downsample.cu:85-116) as literal loops equal the restatements bit for
    bit, at an odd width and a scale that is not a power of two."""
    f = np.float32
    rng = np.random.default_rng(6)
    c, h, w = 3, 10, 13
    feats = rng.random((c, h, w)).astype(np.float32)
    mask = rng.random((h, w)) > 0.3
    inv = f(1) / f(scale)
    dh, dw = int(h * scale), int(w * scale)
    down = np.zeros((c, dh, dw), f)
    dmask = np.zeros((dh, dw), bool)
    for r in range(dh):
        for col in range(dw):
            r0, c0 = int(f(r) * inv), int(f(col) * inv)
            dmask[r, col] = mask[r0, c0]
            for ch in range(c):
                total, n = f(0), 0
                for a, b in ((0, 0), (0, 1), (1, 0), (1, 1)):
                    if c0 + b >= w:
                        continue
                    total = total + feats[ch, r0 + a, c0 + b]
                    n += 1
                down[ch, r, col] = total / f(n)
    got = fp.downsample_features(feats, scale)
    np.testing.assert_array_equal(got.view(np.uint32), down.view(np.uint32))
    np.testing.assert_array_equal(fp.downsample_mask(mask, scale), dmask)


def test_erosion_matches_the_reference_steps():
    """``ErodeMaskKernel`` (erode_mask.cu:18-39) as a literal loop over its
    neighbourhood table {-1,0}, {0,1}, {0,-1}, {0,1} (the row below never
    checked; neighbours outside the image ignored) equals the restatement."""
    rng = np.random.default_rng(7)
    mask = rng.random((17, 23)) > 0.2
    table = ((-1, 0), (0, 1), (0, -1), (0, 1))
    out = np.zeros_like(mask)
    h, w = mask.shape
    for r in range(h):
        for c in range(w):
            out[r, c] = bool(mask[r, c]) and all(
                not (0 <= r + dr < h and 0 <= c + dc < w) or mask[r + dr, c + dc]
                for dr, dc in table)
    np.testing.assert_array_equal(fp.erode_mask(mask), out)
    assert out.sum() > 50
