"""numpy restatement of the reference's differentiable registration layer:
``ExpRtToMatrixOp`` / ``MatrixToExpRtOp`` (src/exp_rt_to_matrix.cu,
src/matrix_to_exp_rt.cu, src/exp_rt.hpp) and ``FPCLMatcherOp``
(src/fpcl_matcher.cu, src/feature_map.hpp).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Parity with the
reference's binaries is unpinned (they cannot be built here).  The twist
map is pinned by mathematics instead: the FP64 matrix is checked to be a
rotation with the twist's axis and angle, the Gallego-Yezzi backward
against central differences of the forward, and the inverse map by round
trips.  The matcher restates the float32 kernels operation by operation
(the bit-exact gate), on the same correspondence map as the GPU.
"""
import numpy as np

from .icp_oracle import F32, F64, _bilinear32, _dx_project, project32, round_away

# ---------------------------------------------------------------------------
# ExpRt
# ---------------------------------------------------------------------------


def _hat(w):
    return np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])


def rotation64(w):
    """R(w) = cos(a) I + sin(a) [k]x + (1 - cos(a)) k k^T, a = |w|, k = w / a
    (exp_rt.hpp:27-32 with Eigen's AngleAxis rotation matrix), FP64."""
    w = np.asarray(w, dtype=F64)
    a = np.linalg.norm(w)
    k = w / a if a > 0 else w
    return np.cos(a) * np.eye(3) + np.sin(a) * _hat(k) + (1.0 - np.cos(a)) * np.outer(k, k)


def exp_rt_to_matrix64(x):
    """[B, 6] twists [t; w] -> [B, 3, 4] matrices [R(w) | t]
    (exp_rt_to_matrix.cu:22-36)."""
    x = np.asarray(x, dtype=F64).reshape(-1, 6)
    out = np.zeros((x.shape[0], 3, 4))
    for i, xi in enumerate(x):
        out[i, :, :3] = rotation64(xi[3:])
        out[i, :, 3] = xi[:3]
    return out


def exp_rt_to_matrix_backward64(d_matrix, x):
    """d loss / d twist from d loss / d matrix (exp_rt_to_matrix.cu:69-97,
    exp_rt.hpp:90-138): dM/dt_r is the unit at (r, 3); dR/dw_k = [u_k]x R,
    u_k = (w w_k + w x ((I - R) e_k)) / |w|^2 (Gallego and Yezzi, JMIV 2015),
    u_k = e_k when |w|^2 <= 1e-12."""
    g = np.asarray(d_matrix, dtype=F64).reshape(-1, 3, 4)
    x = np.asarray(x, dtype=F64).reshape(-1, 6)
    out = np.zeros_like(x)
    for i, xi in enumerate(x):
        w = xi[3:]
        R = rotation64(w)
        out[i, :3] = g[i, :, 3]
        vn = w @ w
        for k in range(3):
            if vn > 1e-12:
                e = (np.eye(3) - R)[:, k]
                u = (w * w[k] + np.cross(w, e)) / vn
            else:
                u = np.eye(3)[k]
            out[i, 3 + k] = np.sum((_hat(u) @ R) * g[i, :, :3])
    return out


def exp_rt_to_matrix_fd64(d_matrix, x, step=1e-6):
    """Central differences of sum(d_matrix * M(x)) with respect to x."""
    g = np.asarray(d_matrix, dtype=F64).reshape(-1, 3, 4)
    x = np.asarray(x, dtype=F64).reshape(-1, 6)
    out = np.zeros_like(x)
    for i in range(x.shape[0]):
        for j in range(6):
            xp, xm = x[i].copy(), x[i].copy()
            xp[j] += step
            xm[j] -= step
            out[i, j] = np.sum(g[i] * (exp_rt_to_matrix64(xp)[0] - exp_rt_to_matrix64(xm)[0])) \
                / (2 * step)
    return out


def matrix_to_exp_rt64(m):
    """[B, 3, 4] -> [B, 6] (matrix_to_exp_rt.cu:20-32) by the rotation
    angle from the trace and the axis from the antisymmetric part (an
    independent route from the kernel's quaternion); rotations below pi -
    1e-3 only."""
    m = np.asarray(m, dtype=F64).reshape(-1, 3, 4)
    out = np.zeros((m.shape[0], 6))
    for i, mi in enumerate(m):
        R = mi[:, :3]
        out[i, :3] = mi[:, 3]
        c = np.clip((np.trace(R) - 1.0) / 2.0, -1.0, 1.0)
        a = np.arccos(c)
        s = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2.0
        out[i, 3:] = s * (a / np.sin(a)) if a > 1e-8 else s
    return out


# ---------------------------------------------------------------------------
# FPCLMatcher
# ---------------------------------------------------------------------------


def fpcl_forward32(tgt_points, tgt_normals, tgt_feats, src_points, kcam, ref_map):
    """FPCLMatcherOp forward (fpcl_matcher.cu:46-80), float32: point i
    matches when its rounded projection is inside the image and the map's
    winner there (``map >> 32``) is i; matches take the target point and
    normal at the pixel and the bilinear samples at the unrounded
    projection.  Non-matches are zero.  Returns (points, normals, feats
    [C, N], mask)."""
    sp = np.asarray(src_points, dtype=F32).reshape(-1, 3)
    tp = np.asarray(tgt_points, dtype=F32)
    tn = np.asarray(tgt_normals, dtype=F32)
    tf = np.asarray(tgt_feats, dtype=F32)
    h, w = tp.shape[:2]
    n = sp.shape[0]
    u, v = project32(kcam, sp)
    ur, vr = round_away(u), round_away(v)
    with np.errstate(invalid="ignore"):
        inside = (ur >= 0) & (ur < w) & (vr >= 0) & (vr < h)
    ui = np.where(inside, ur, 0).astype(np.int64)
    vi = np.where(inside, vr, 0).astype(np.int64)
    winner = (np.asarray(ref_map, dtype=np.int64) >> 32).astype(np.int32).astype(np.int64)
    mask = inside & (winner[vi, ui] == np.arange(n))
    points = np.zeros((n, 3), F32)
    normals = np.zeros((n, 3), F32)
    feats = np.zeros((tf.shape[0], n), F32)
    idx = np.nonzero(mask)[0]
    points[idx] = tp[vi[idx], ui[idx]]
    normals[idx] = tn[vi[idx], ui[idx]]
    if tf.shape[0] > 0 and idx.size:
        feats[:, idx] = _bilinear32(tf, u[idx], v[idx])
    return points, normals, feats, mask


def fpcl_backward32(tgt_feats, src_points, mask, dl_feats, kcam, grad_precision):
    """FPCLMatcherOp backward (fpcl_matcher.cu:150-189), float32: central
    differences of the bilinear sample with step h, the lower sample clamped
    at 0 (feature_map.hpp:45-63), contracted with dl over the channels in
    channel order, then the projection's Jacobian (camera.hpp:64-77)."""
    tf = np.asarray(tgt_feats, dtype=F32)
    sp = np.asarray(src_points, dtype=F32).reshape(-1, 3)
    dl = np.asarray(dl_feats, dtype=F32)
    idx = np.nonzero(np.asarray(mask, dtype=bool))[0]
    dx = np.zeros_like(sp)
    if idx.size == 0:
        return dx
    p = sp[idx]
    u, v = project32(kcam, p)
    hh = F32(grad_precision)
    div = F32(1) / (F32(2) * hh)
    z = F32(0)
    up, um = (u + hh).astype(F32), np.maximum(u - hh, z).astype(F32)
    vp, vm = (v + hh).astype(F32), np.maximum(v - hh, z).astype(F32)
    gu = np.zeros(idx.size, F32)
    gv = np.zeros(idx.size, F32)
    if tf.shape[0] > 0:
        du = (_bilinear32(tf, up, v) - _bilinear32(tf, um, v)) * div
        dv = (_bilinear32(tf, u, vp) - _bilinear32(tf, u, vm)) * div
        for c in range(tf.shape[0]):
            gu = gu + du[c] * dl[c, idx]
            gv = gv + dv[c] * dl[c, idx]
    j00, j02, j11, j12 = _dx_project(kcam, p, F32)
    dx[idx, 0] = j00 * gu
    dx[idx, 1] = j11 * gv
    dx[idx, 2] = j02 * gu + j12 * gv
    return dx
