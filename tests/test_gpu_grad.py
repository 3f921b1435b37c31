"""Differentiable point-to-plane loss (PointToPlaneLoss -> stb_icp_loss_forward
/ _backward / stb_se3_twist_grad) against the FP64 oracle.

Each pair is registered for 5 Gauss-Newton iterations first; the loss and its
gradients are taken at that pose, rounded to float32 so that the kernels'
float32 pose is the oracle's pose exactly.  Tolerances (all written below):

* loss: 1e-5 relative to the FP64 sum of squares over the same (bit-exact)
  correspondences;
* twist gradient: per component within 1e-5 of sum 2 |J| |r| (the scale of
  the Jacobian-residual products, the Jtr gate of the registration tests)
  against FP64 central differences (step 1e-6) and against -2 J^T r summed
  from the reference-layout per-point partials of ICPJacobian;
* depth gradient at 64 sampled matched pixels per pair: within
  1e-5 |dL/dz| + 2 |dr/dz| * 8 eps32 (|q| + |Tp|), the float32 rounding
  bound of the residual r = (q - Tp).n, against FP64 central differences
  (step 1e-6); exactly 0 at pixels without a correspondence.
"""
import math

import numpy as np
import pytest
import torch

from oracle import icp_oracle as io
from _helpers import synthetic_pair

pytestmark = pytest.mark.gpu

DIST = 0.1
ANGLE = math.radians(20)
EPS32 = 2.0 ** -24


def _t(x, dev, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    return t if dtype is None else t.to(dtype)


def _batch(cuda, seeds, w, h):
    from slamtb_gb300.registration import ICPOdometry
    icp = ICPOdometry(5, geom_weight=1.0, feat_weight=0.0, distance_threshold=DIST,
                      normals_angle_thresh=ANGLE)
    pairs, poses = [], []
    for seed in seeds:
        d = synthetic_pair(seed, width=w, height=h)
        s, t = d["src"], d["tgt"]
        res = icp.estimate(_t(d["kcam"], cuda), _t(s["points"], cuda), _t(s["normals"], cuda),
                           _t(s["mask"], cuda), target_points=_t(t["points"], cuda),
                           target_normals=_t(t["normals"], cuda), target_mask=_t(t["mask"], cuda))
        T0 = res.transform.numpy().astype(np.float32).astype(np.float64)
        pairs.append(d)
        poses.append(T0)
    return pairs, np.stack(poses)


def _inputs(cuda, pairs):
    st = lambda key, part: torch.stack([_t(d[part][key], cuda) for d in pairs])
    depth = torch.stack([_t(d["src_fpcl"].points[..., 2], cuda) for d in pairs])
    return dict(source_depth=depth, source_normals=st("normals", "src"),
                source_mask=st("mask", "src"), target_points=st("points", "tgt"),
                target_normals=st("normals", "tgt"), target_mask=st("mask", "tgt"))


def _kcam_params(K):
    return (float(K[0][0]), float(K[1][1]), float(K[0][2]), float(K[1][2]))


def _oracle(d, T0):
    s, t = d["src"], d["tgt"]
    a = io.associate32(s["points"], s["normals"], s["mask"], io.pose_rt32(T0), t["points"],
                       t["normals"], t["mask"], d["kcam"], DIST, ANGLE)
    return a, io.LossMatches(a, t["points"], t["normals"])


@pytest.fixture(scope="module")
def batch(cuda):
    pairs, poses = _batch(cuda, [70, 71, 72], 320, 240)
    return pairs, poses


def _run(cuda, pairs, poses, twist=None):
    from slamtb_gb300.registration import point_to_plane_loss
    B = len(pairs)
    inp = _inputs(cuda, pairs)
    inp["source_depth"].requires_grad_(True)
    if twist is None:
        twist = np.zeros((B, 6))
    tw = torch.tensor(twist, dtype=torch.float64, device=cuda, requires_grad=True)
    loss = point_to_plane_loss(tw, kcam=_kcam_params(pairs[0]["kcam"]),
                               poses=torch.from_numpy(poses).to(cuda), distance_threshold=DIST,
                               normals_angle_thresh=ANGLE, **inp)
    loss.sum().backward()
    return loss.detach().cpu().numpy(), tw.grad.cpu().numpy(), \
        inp["source_depth"].grad.cpu().numpy()


def test_source_points_match_oracle_backprojection(cuda, batch):
    """The loss back-projects the source depth on the device; the points
    must be the oracle's float32 points bit for bit."""
    from slamtb_gb300 import processing
    pairs, _ = batch
    d = pairs[0]
    depth = _t(d["src_fpcl"].points[..., 2], cuda)
    pts, _ = processing.depth_to_points(depth, torch.tensor(d["kcam"], dtype=torch.float32))
    np.testing.assert_array_equal(pts.cpu().numpy(), d["src"]["points"])


def test_loss_matches_fp64_oracle(cuda, batch):
    pairs, poses = batch
    loss, _, _ = _run(cuda, pairs, poses)
    for p, d in enumerate(pairs):
        _, m = _oracle(d, poses[p])
        assert m.idx.size > 1000
        ref = io.point_to_plane_loss64(poses[p], d["src"]["points"], m)
        assert loss[p] == pytest.approx(ref, rel=1e-5)


def test_twist_grad_vs_fd_and_reference_jacobian(cuda, batch):
    from slamtb_gb300._cslamtb import CorrespondenceMap, ICPJacobian
    pairs, poses = batch
    _, gtw, _ = _run(cuda, pairs, poses)
    for p, d in enumerate(pairs):
        _, m = _oracle(d, poses[p])
        sp = d["src"]["points"]
        fd = io.loss_twist_grad_fd(poses[p], np.zeros(6), sp, m, h=1e-6)
        an, scale = io.loss_twist_grad64(poses[p], sp, m)
        assert np.abs(fd - an).max() <= 1e-7 * scale      # the oracle against itself
        assert np.abs(gtw[p] - fd).max() <= 1e-5 * scale
        # -2 J^T r from the reference-layout per-point partials
        s, t = d["src"], d["tgt"]
        h, w = t["mask"].shape
        cmap = torch.full((h, w), io.CORRESP_EMPTY, dtype=torch.int64, device=cuda)
        rt = _t(poses[p], cuda, torch.float32)
        CorrespondenceMap.compute_correspondence_map(
            _t(s["points"], cuda).view(-1, 3), _t(s["normals"], cuda).view(-1, 3),
            _t(s["mask"], cuda).view(-1), rt, _t(t["points"], cuda), _t(t["normals"], cuda),
            _t(t["mask"], cuda), _t(d["kcam"], cuda), cmap, DIST, ANGLE)
        n = h * w
        JtJ = torch.zeros(n, 6, 6, device=cuda)
        Jr = torch.zeros(n, 6, device=cuda)
        r2 = torch.zeros(n, device=cuda)
        cnt = ICPJacobian.estimate_geometric(
            _t(s["points"], cuda).view(-1, 3), _t(s["mask"], cuda).view(-1), rt,
            _t(t["points"], cuda), _t(t["normals"], cuda), _t(d["kcam"], cuda), cmap, JtJ, Jr, r2)
        assert cnt == m.idx.size
        ref = -2.0 * Jr.double().sum(0).cpu().numpy()
        assert np.abs(gtw[p] - ref).max() <= 1e-5 * scale


def test_depth_grad_vs_fd(cuda, batch):
    pairs, poses = batch
    _, _, gz = _run(cuda, pairs, poses)
    rng = np.random.default_rng(5)
    for p, d in enumerate(pairs):
        _, m = _oracle(d, poses[p])
        h, w = d["tgt"]["mask"].shape
        g = gz[p].reshape(-1)
        unmatched = np.ones(h * w, dtype=bool)
        unmatched[m.idx] = False
        assert np.all(g[unmatched] == 0.0)
        pix = rng.choice(m.idx, size=64, replace=False)
        fd, r, a = io.loss_depth_grad_fd(poses[p], d["src"]["points"], m, d["kcam"], w, pix,
                                         h=1e-6)
        sp = d["src"]["points"].reshape(-1, 3)[pix].astype(np.float64)
        tp = sp @ poses[p][:3, :3].T + poses[p][:3, 3]
        where = {int(i): k for k, i in enumerate(m.idx)}
        q = m.q[[where[int(i)] for i in pix]]
        bound = 1e-5 * np.abs(fd) + 2.0 * np.abs(a) * 8 * EPS32 * (
            np.abs(q).sum(1) + np.abs(tp).sum(1))
        assert np.all(np.abs(g[pix] - fd) <= bound)
        assert np.all(fd != 0.0)


def test_twist_grad_maps_through_left_jacobian(cuda):
    """stb_se3_twist_grad against the central-difference left Jacobian of the
    oracle's exp / log."""
    from slamtb_gb300 import _native as N
    rng = np.random.default_rng(9)
    xi = np.concatenate([rng.normal(0, 0.3, (8, 3)), rng.normal(0, 0.5, (8, 3))], axis=1)
    xi[0] = 0.0
    xi[1, 3:] = [1e-9, 0.0, 0.0]
    g = rng.normal(size=(8, 6))
    txi, tg = _t(xi, cuda), _t(g, cuda)
    out = torch.empty_like(tg)
    N.check(N.lib().stb_se3_twist_grad(N.ptr(txi), N.ptr(tg), N.ptr(out), 8, N.stream_of(cuda)))
    out = out.cpu().numpy()
    np.testing.assert_array_equal(out[0], g[0])
    for k in range(8):
        J = io.se3_left_jacobian_fd(xi[k])
        np.testing.assert_allclose(out[k], J.T @ g[k], rtol=1e-6, atol=1e-7 * np.abs(g[k]).sum())


def test_nonzero_twist_grad_vs_fd(cuda, batch):
    """At twist != 0 the kernels run at the float32 cast of exp(twist) T0:
    the gradient agrees with FP64 central differences of L(exp(twist) T0)
    up to that cast (tolerance 1e-3 of the scale)."""
    pairs, poses = batch
    twist = np.tile([[2e-3, -1e-3, 1.5e-3, 1e-3, 2e-3, -1.5e-3]], (len(pairs), 1))
    _, gtw, _ = _run(cuda, pairs, poses, twist)
    for p, d in enumerate(pairs):
        T = io.se3_exp(twist[p]) @ poses[p]
        _, m = _oracle(d, T)
        fd = io.loss_twist_grad_fd(poses[p], twist[p], d["src"]["points"], m, h=1e-6)
        _, scale = io.loss_twist_grad64(T, d["src"]["points"], m)
        assert np.abs(gtw[p] - fd).max() <= 1e-3 * scale


def test_loss_is_zero_without_correspondences(cuda, batch):
    pairs, poses = batch
    d = dict(pairs[0])
    d["tgt"] = dict(d["tgt"])
    d["tgt"]["mask"] = np.zeros_like(d["tgt"]["mask"])
    loss, gtw, gz = _run(cuda, [d, pairs[1]], poses[:2])
    assert loss[0] == 0.0 and np.all(gtw[0] == 0.0) and np.all(gz[0] == 0.0)
    assert loss[1] > 0.0


def test_full_size_32_pairs_640x480(cuda):
    """The loss at its full size (32 pairs of 640x480, poses after 5 Gauss-
    Newton iterations): for every pair the twist gradient equals -2 J^T r
    from the reference-layout partials of ICPJacobian (same correspondences,
    1e-5 of sum 2|J||r|), the depth gradient vanishes off the
    correspondences, and one pair's twist gradient matches FP64 central
    differences."""
    from slamtb_gb300 import synthetic
    from slamtb_gb300._cslamtb import CorrespondenceMap, ICPJacobian
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    from slamtb_gb300.registration import BatchRegistration, ICPOdometry, point_to_plane_loss
    B = 32
    src, tgt, kc = [], [], None
    for k in range(B):
        p = synthetic.make_pair(200 + k, width=640, height=480, device=cuda)
        kc = KCamera(p["kcam"])
        src.append(FramePointCloud.from_frame(Frame(FrameInfo(kc), p["source_depth"]), cuda))
        tgt.append(FramePointCloud.from_frame(Frame(FrameInfo(kc), p["target_depth"]), cuda))
    br = BatchRegistration([(1.0, ICPOdometry(5, geom_weight=1.0, feat_weight=0.0,
                                              distance_threshold=DIST,
                                              normals_angle_thresh=ANGLE))])
    res = br.estimate_pyramids([[s] for s in src], [[t] for t in tgt])
    poses = torch.stack([r.transform.double().float().double() for r in res]).to(cuda)
    st = lambda f: torch.stack([f(k) for k in range(B)]).contiguous()  # noqa: E731
    depth = st(lambda k: src[k].points[..., 2]).requires_grad_(True)
    twist = torch.zeros(B, 6, dtype=torch.float64, device=cuda, requires_grad=True)
    loss = point_to_plane_loss(twist, depth, st(lambda k: src[k].normals),
                               st(lambda k: src[k].mask), st(lambda k: tgt[k].points),
                               st(lambda k: tgt[k].normals), st(lambda k: tgt[k].mask),
                               kc.params(), poses, DIST, ANGLE)
    loss.sum().backward()
    gtw = twist.grad.cpu().numpy()
    assert torch.isfinite(loss).all() and bool((loss > 0).all())
    h, w = 480, 640
    for k in range(B):
        s, t = src[k], tgt[k]
        cmap = torch.full((h, w), io.CORRESP_EMPTY, dtype=torch.int64, device=cuda)
        rt = poses[k].float()
        CorrespondenceMap.compute_correspondence_map(
            s.points.view(-1, 3), s.normals.view(-1, 3), s.mask.view(-1), rt, t.points,
            t.normals, t.mask, torch.as_tensor(kc.matrix, device=cuda), cmap, DIST, ANGLE)
        JtJ = torch.zeros(h * w, 6, 6, device=cuda)
        Jr = torch.zeros(h * w, 6, device=cuda)
        r2 = torch.zeros(h * w, device=cuda)
        ICPJacobian.estimate_geometric(s.points.view(-1, 3), s.mask.view(-1), rt, t.points,
                                       t.normals, torch.as_tensor(kc.matrix, device=cuda), cmap,
                                       JtJ, Jr, r2)
        ref = -2.0 * Jr.double().sum(0).cpu().numpy()
        Jn = torch.linalg.norm(JtJ.double().diagonal(dim1=1, dim2=2).sqrt(), dim=1)
        scale = float(2.0 * (Jn * r2.double().sqrt()).sum())
        assert np.abs(gtw[k] - ref).max() <= 1e-5 * scale, k
        matched = (cmap.cpu().numpy() >> 32).reshape(-1)
        matched = matched[matched != (io.CORRESP_EMPTY >> 32)]
        gz = depth.grad[k].reshape(-1).cpu().numpy()
        off = np.ones(h * w, dtype=bool)
        off[matched] = False
        assert np.all(gz[off] == 0.0), k
    # FP64 central differences of the twist gradient, pair 0
    d0 = dict(src=dict(points=src[0].points.cpu().numpy(), normals=src[0].normals.cpu().numpy(),
                       mask=src[0].mask.cpu().numpy()),
              tgt=dict(points=tgt[0].points.cpu().numpy(), normals=tgt[0].normals.cpu().numpy(),
                       mask=tgt[0].mask.cpu().numpy()),
              kcam=kc.matrix.numpy())
    T0 = poses[0].cpu().numpy()
    _, m = _oracle(d0, T0)
    fd = io.loss_twist_grad_fd(T0, np.zeros(6), d0["src"]["points"], m, h=1e-6)
    _, sc = io.loss_twist_grad64(T0, d0["src"]["points"], m)
    assert np.abs(gtw[0] - fd).max() <= 1e-5 * sc


def _abi_args(cuda, pairs, poses):
    """The dense C-ABI arguments of a batch (inputs, sizes, intrinsics, poses)."""
    inp = _inputs(cuda, pairs)
    ins = [inp[k].contiguous() for k in ("source_depth", "source_normals", "source_mask",
                                         "target_points", "target_normals", "target_mask")]
    ins[2], ins[5] = ins[2].to(torch.uint8), ins[5].to(torch.uint8)
    B, H, W = ins[0].shape
    return ins, (B, H, W), _kcam_params(pairs[0]["kcam"]), torch.from_numpy(poses).to(cuda)


def test_fused_adjoint_equals_the_separate_adjoint(cuda, batch):
    """stb_icp_loss_forward_adjoint (loss and adjoint in one pass) against
    stb_icp_loss_forward + stb_icp_loss_backward on the same batch: the loss,
    the tangent gradient and the depth gradient are the same bits at
    grad_loss = 1.  After stb_icp_loss_scale_adjoint with other output
    gradients (one of them 0), where the separate adjoint rounds g r in
    float32 in every term and the scale multiplies the FP64 sum once: the
    tangent gradient within 1e-6 of sum 2 |g| |J| |r|, and the depth gradient
    within 2^-22 relative (four float32 roundings) of the separate
    adjoint's."""
    from slamtb_gb300 import _native as N
    pairs, poses = batch
    ins, (B, H, W), k, T = _abi_args(cuda, pairs, poses)
    lib, st = N.lib(), N.stream_of(cuda)
    need = int(lib.stb_icp_loss_workspace_bytes(B, H, W))
    ws1 = torch.empty(need, dtype=torch.uint8, device=cuda)
    ws2 = torch.empty(need, dtype=torch.uint8, device=cuda)
    loss1 = torch.empty(B, dtype=torch.float64, device=cuda)
    loss2 = torch.empty(B, dtype=torch.float64, device=cuda)
    tangent = torch.empty(B, 6, dtype=torch.float64, device=cuda)
    dadj = torch.full((B, H, W), float("nan"), dtype=torch.float32, device=cuda)
    p = [N.ptr(x) for x in ins]
    N.check(lib.stb_icp_loss_forward(*p, B, H, W, *k, N.ptr(T), DIST, ANGLE, N.ptr(ws1), need,
                                     N.ptr(loss1), st))
    N.check(lib.stb_icp_loss_forward_adjoint(*p, B, H, W, *k, N.ptr(T), DIST, ANGLE,
                                             N.ptr(ws2), need, N.ptr(loss2), N.ptr(tangent),
                                             N.ptr(dadj), st))
    assert torch.equal(loss1, loss2)
    for g in ([1.0] * B, [0.5, -3.0, 0.0][:B]):
        gl = torch.tensor(g, dtype=torch.float64, device=cuda)
        gt1 = torch.empty(B, 6, dtype=torch.float64, device=cuda)
        gz1 = torch.empty(B, H, W, dtype=torch.float32, device=cuda)
        N.check(lib.stb_icp_loss_backward(*p, B, H, W, *k, N.ptr(T), N.ptr(gl), N.ptr(ws1),
                                          need, N.ptr(gt1), N.ptr(gz1), st))
        gt2 = torch.empty(B, 6, dtype=torch.float64, device=cuda)
        gz2 = torch.empty(B, H, W, dtype=torch.float32, device=cuda)
        N.check(lib.stb_icp_loss_scale_adjoint(N.ptr(gl), N.ptr(tangent), N.ptr(dadj), B, H, W,
                                               N.ptr(gt2), N.ptr(gz2), st))
        a1, a2 = gt1.cpu().numpy(), gt2.cpu().numpy()
        z1, z2 = gz1.cpu().numpy(), gz2.cpu().numpy()
        if g[0] == 1.0:
            np.testing.assert_array_equal(a1, a2)
            np.testing.assert_array_equal(z1, z2)
            assert np.count_nonzero(z2) > 1000
            continue
        for q in range(B):
            _, m = _oracle(pairs[q], poses[q])
            _, scale = io.loss_twist_grad64(poses[q], pairs[q]["src"]["points"], m)
            assert np.abs(a1[q] - a2[q]).max() <= 1e-6 * abs(g[q]) * scale
        np.testing.assert_allclose(z2, z1, rtol=2.0 ** -22, atol=0.0)
    # only the tangent: a NULL depth adjoint and a NULL depth gradient
    gt3 = torch.empty(B, 6, dtype=torch.float64, device=cuda)
    N.check(lib.stb_icp_loss_forward_adjoint(*p, B, H, W, *k, N.ptr(T), DIST, ANGLE,
                                             N.ptr(ws2), need, N.ptr(loss2), N.ptr(gt3), None,
                                             st))
    assert torch.equal(gt3, tangent)
    N.check(lib.stb_icp_loss_scale_adjoint(N.ptr(torch.ones(B, dtype=torch.float64,
                                                             device=cuda)),
                                           N.ptr(gt3), None, B, H, W, N.ptr(gt2), None, st))
    assert torch.equal(gt2, tangent)


def test_loss_without_gradients_equals_the_fused_forward(cuda, batch):
    """With no input needing a gradient the forward runs the loss alone
    (stb_icp_loss_forward); its values are the fused forward's bits, and a
    gradient only for the twist leaves the depth without one."""
    from slamtb_gb300.registration import point_to_plane_loss
    pairs, poses = batch
    B = len(pairs)
    kw = dict(kcam=_kcam_params(pairs[0]["kcam"]), poses=torch.from_numpy(poses).to(cuda),
              distance_threshold=DIST, normals_angle_thresh=ANGLE, **_inputs(cuda, pairs))
    with torch.no_grad():
        plain = point_to_plane_loss(torch.zeros(B, 6, dtype=torch.float64, device=cuda), **kw)
    tw = torch.zeros(B, 6, dtype=torch.float64, device=cuda, requires_grad=True)
    fused = point_to_plane_loss(tw, **kw)
    assert torch.equal(plain, fused.detach())
    fused.sum().backward()
    loss, gtw, _ = _run(cuda, pairs, poses)
    np.testing.assert_array_equal(tw.grad.cpu().numpy(), gtw)
    assert kw["source_depth"].grad is None


def test_graph_captured_loss_equals_eager(cuda, batch):
    """PointToPlaneLoss captured as CUDA graphs (torch.cuda.make_graphed_
    callables over twist and depth, as the benchmark runs it): two replays
    at different twists give the eager call's loss and gradients bit for
    bit."""
    from slamtb_gb300.registration import point_to_plane_loss
    pairs, poses = batch
    B = len(pairs)
    inp = _inputs(cuda, pairs)
    depth = inp.pop("source_depth").clone().requires_grad_(True)
    kw = dict(kcam=_kcam_params(pairs[0]["kcam"]), poses=torch.from_numpy(poses).to(cuda),
              distance_threshold=DIST, normals_angle_thresh=ANGLE, **inp)

    def fn(tw, z):
        return point_to_plane_loss(tw, z, **kw)

    tw = torch.zeros(B, 6, dtype=torch.float64, device=cuda, requires_grad=True)
    graphed = torch.cuda.make_graphed_callables(fn, (tw, depth))
    for scale in (0.0, 1e-3):
        twist = torch.full((B, 6), scale, dtype=torch.float64, device=cuda)
        t1 = twist.clone().requires_grad_(True)
        z1 = depth.detach().clone().requires_grad_(True)
        e = fn(t1, z1)
        e.sum().backward()
        t2 = twist.clone().requires_grad_(True)
        z2 = depth.detach().clone().requires_grad_(True)
        g = graphed(t2, z2)
        g.sum().backward()
        torch.cuda.synchronize(cuda)
        assert torch.equal(e.detach(), g.detach())
        assert torch.equal(t1.grad, t2.grad)
        assert torch.equal(z1.grad, z2.grad)
