"""The differentiable registration layer of AutogradICP on the GPU:
ExpRtToMatrix / MatrixToExpRt (twist <-> [R | t]) against the FP64
oracle and autograd's gradcheck, the frame point-cloud matcher's forward
and backward bit for bit against the float32 restatement (on a
correspondence map that is itself checked bit for bit), and the
AutogradICP optimisation loop on a synthetic pair."""
import math

import numpy as np
import pytest
import torch

from oracle import autograd_oracle as ao
from oracle import icp_oracle as io
from _helpers import rel_pose, synthetic_pair

pytestmark = pytest.mark.gpu

DIST, ANGLE = 0.1, math.radians(30)


def _twists(rng, n, max_angle=3.0):
    x = rng.normal(size=(n, 6))
    ang = rng.uniform(0.0, max_angle, size=n)
    x[:, 3:] *= (ang / np.linalg.norm(x[:, 3:], axis=1))[:, None]
    x[0, 3:] = 0.0
    x[1, 3:] = [1e-7, 0.0, 0.0]      # |w|^2 below the derivative's 1e-12 switch
    x[2, 3:] = [2e-6, -1e-6, 0.0]    # just above it
    return x


def test_exp_rt_to_matrix_forward(cuda):
    from slamtb_gb300.registration import ExpRtToMatrix
    rng = np.random.default_rng(1)
    x = _twists(rng, 64)
    m64 = ExpRtToMatrix.apply(torch.from_numpy(x).to(cuda)).cpu().numpy()
    np.testing.assert_allclose(m64, ao.exp_rt_to_matrix64(x), rtol=0, atol=1e-13)
    x32 = x.astype(np.float32)
    m32 = ExpRtToMatrix.apply(torch.from_numpy(x32).to(cuda)).cpu().numpy()
    np.testing.assert_allclose(m32, ao.exp_rt_to_matrix64(x32), rtol=0, atol=2e-6)
    one = ExpRtToMatrix.apply(torch.from_numpy(x[5]).to(cuda))
    assert one.shape == (3, 4)
    np.testing.assert_array_equal(one.cpu().numpy(), m64[5])


def test_exp_rt_to_matrix_backward(cuda):
    from slamtb_gb300.registration import ExpRtToMatrix
    rng = np.random.default_rng(2)
    x = _twists(rng, 32)
    g = rng.normal(size=(32, 3, 4))
    xt = torch.from_numpy(x).to(cuda).requires_grad_(True)
    (ExpRtToMatrix.apply(xt) * torch.from_numpy(g).to(cuda)).sum().backward()
    np.testing.assert_allclose(xt.grad.cpu().numpy(), ao.exp_rt_to_matrix_backward64(g, x),
                               rtol=1e-10, atol=1e-12)
    # the analytic derivative against autograd's own central differences
    xs = torch.from_numpy(x[3:9]).to(cuda).requires_grad_(True)
    assert torch.autograd.gradcheck(ExpRtToMatrix.apply, (xs,), eps=1e-6, atol=1e-6)
    # float32: same formula, float32 rounding
    x32 = torch.from_numpy(x.astype(np.float32)).to(cuda).requires_grad_(True)
    (ExpRtToMatrix.apply(x32) * torch.from_numpy(g).float().to(cuda)).sum().backward()
    np.testing.assert_allclose(x32.grad.cpu().numpy(),
                               ao.exp_rt_to_matrix_backward64(g, x.astype(np.float32)),
                               rtol=1e-4, atol=1e-4)


def test_matrix_to_exp_rt_round_trip(cuda):
    from slamtb_gb300.registration import ExpRtToMatrix, MatrixToExpRt
    rng = np.random.default_rng(3)
    x = _twists(rng, 64, max_angle=3.1)
    x[1:3, 3:] = [0.01, 0.0, 0.0]
    m = ao.exp_rt_to_matrix64(x)
    back = MatrixToExpRt.apply(torch.from_numpy(m).to(cuda)).cpu().numpy()
    np.testing.assert_allclose(back, x, rtol=0, atol=1e-10)
    sel = np.linalg.norm(x[:, 3:], axis=1) < 3.0
    np.testing.assert_allclose(back[sel], ao.matrix_to_exp_rt64(m[sel]), rtol=0, atol=1e-10)
    m32 = ExpRtToMatrix.apply(torch.from_numpy(x).float().to(cuda))
    np.testing.assert_allclose(MatrixToExpRt.apply(m32).cpu().numpy(), x, rtol=0, atol=2e-5)
    single = MatrixToExpRt.apply(torch.from_numpy(m[4]).to(cuda))
    assert single.shape == (6,)


@pytest.fixture(scope="module")
def fpair():
    d = synthetic_pair(3, width=320, height=240, feature_channels=3)
    gt = d["gt"].astype(np.float32)
    s = d["src"]
    m = s["mask"].reshape(-1)
    sp = s["points"].reshape(-1, 3)[m]
    sn = s["normals"].reshape(-1, 3)[m]
    d["tsp"] = (sp @ gt[:3, :3].T + gt[:3, 3]).astype(np.float32)
    d["tsn"] = (sn @ gt[:3, :3].T).astype(np.float32)
    return d


def _target(d, cuda):
    from slamtb_gb300.frame import KCamera
    from slamtb_gb300.spatial import FPCLMatcherOp
    t = d["tgt"]
    return FPCLMatcherOp.Target(
        torch.from_numpy(t["points"]).to(cuda), torch.from_numpy(t["normals"]).to(cuda),
        torch.from_numpy(t["mask"]).to(cuda), torch.from_numpy(d["tgt_feats"]).to(cuda),
        KCamera(d["kcam"]), DIST, ANGLE)


def _oracle_map(d):
    t = d["tgt"]
    return io.associate32(d["tsp"], d["tsn"], np.ones(1, bool), np.eye(4, dtype=np.float32),
                          t["points"], t["normals"], t["mask"], d["kcam"], DIST, ANGLE).ref_map


def test_fpcl_matcher_forward_is_bit_exact(cuda, fpair):
    from slamtb_gb300.registration import CorrespondenceMap
    from slamtb_gb300.spatial import FPCLMatcherOp
    d = fpair
    target = _target(d, cuda)
    sp = torch.from_numpy(d["tsp"]).to(cuda)
    sn = torch.from_numpy(d["tsn"]).to(cuda)
    gmap = CorrespondenceMap(DIST, ANGLE)(
        sp, sn, torch.ones(1, dtype=torch.bool, device=cuda),
        torch.eye(4, dtype=torch.float32, device=cuda), target.points, target.normals,
        target.mask, torch.from_numpy(d["kcam"]).to(cuda))
    omap = _oracle_map(d)
    np.testing.assert_array_equal(gmap.cpu().numpy(), omap)
    match = FPCLMatcherOp.Match()
    feats = FPCLMatcherOp.apply(sp, sn, target, match)
    t = d["tgt"]
    op, on, of, om = ao.fpcl_forward32(t["points"], t["normals"], d["tgt_feats"], d["tsp"],
                                       d["kcam"], omap)
    assert om.sum() > 5000
    np.testing.assert_array_equal(match.mask.cpu().numpy(), om)
    np.testing.assert_array_equal(match.points.cpu().numpy(), op)
    np.testing.assert_array_equal(match.normals.cpu().numpy(), on)
    np.testing.assert_array_equal(feats.detach().cpu().numpy(), of)


@pytest.mark.parametrize("grad_precision", [None, 0.02])
def test_fpcl_matcher_backward_is_bit_exact(cuda, fpair, grad_precision):
    from slamtb_gb300.spatial import FPCLMatcherOp
    d = fpair
    target = _target(d, cuda)
    sp = torch.from_numpy(d["tsp"]).to(cuda).requires_grad_(True)
    sn = torch.from_numpy(d["tsn"]).to(cuda)
    match = FPCLMatcherOp.Match()
    args = (sp, sn, target, match) + (() if grad_precision is None else (grad_precision,))
    feats = FPCLMatcherOp.apply(*args)
    rng = np.random.default_rng(9)
    dl = rng.normal(size=feats.shape).astype(np.float32)
    feats.backward(torch.from_numpy(dl).to(cuda))
    h = 0.005 if grad_precision is None else grad_precision
    ref = ao.fpcl_backward32(d["tgt_feats"], d["tsp"], match.mask.cpu().numpy(), dl, d["kcam"], h)
    np.testing.assert_array_equal(sp.grad.cpu().numpy(), ref)
    assert np.abs(ref).sum() > 0


def test_frame_point_cloud_matcher(cuda, fpair):
    from slamtb_gb300.frame import KCamera
    from slamtb_gb300.spatial import FramePointCloudMatcher
    d = fpair
    t = d["tgt"]
    matcher = FramePointCloudMatcher(
        torch.from_numpy(t["points"]).to(cuda), torch.from_numpy(t["normals"]).to(cuda),
        torch.from_numpy(t["mask"]).to(cuda), torch.from_numpy(d["tgt_feats"]).to(cuda),
        KCamera(d["kcam"]), DIST, ANGLE)
    pts, nrm, feats, mask = matcher.find_correspondences(
        torch.from_numpy(d["tsp"]).to(cuda), torch.from_numpy(d["tsn"]).to(cuda))
    k = int(mask.sum())
    assert pts.shape == (k, 3) and nrm.shape == (k, 3) and feats.shape == (3, k)
    _, _, _, om = ao.fpcl_forward32(t["points"], t["normals"], d["tgt_feats"], d["tsp"],
                                    d["kcam"], _oracle_map(d))
    assert k == int(om.sum())


def _agicp_inputs(cuda, d):
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)  # noqa: E731
    s, t = d["src"], d["tgt"]
    return dict(source_points=dev(s["points"].reshape(-1, 3)),
                source_normals=dev(s["normals"].reshape(-1, 3)),
                source_mask=dev(s["mask"].reshape(-1)), target_points=dev(t["points"]),
                target_mask=dev(t["mask"]), target_normals=dev(t["normals"]))


def test_autograd_icp_geometric(cuda):
    """The reference's optimiser, depth only, on a pair 2 deg / 2 cm apart:
    the pose it returns is closer to the ground truth than the start."""
    from slamtb_gb300.frame import KCamera
    from slamtb_gb300.registration import AutogradICP
    d = synthetic_pair(4, width=320, height=240, max_rot_deg=2.0, max_trans=0.02)
    icp = AutogradICP(20, geom_weight=1.0, feat_weight=0.0, distance_threshold=DIST,
                      normals_angle_thresh=ANGLE)
    res = icp.estimate(KCamera(d["kcam"]), **_agicp_inputs(cuda, d))
    assert res.transform.shape == (4, 4) and np.isfinite(res.residual)
    err = rel_pose(res.transform.numpy().astype(np.float64), d["gt"])
    assert err < 0.9, err


def test_autograd_icp_features(cuda):
    """Features only (as the reference's rgb tests: geometric weight 0,
    feature weight 1, learning rate 0.1), through the matcher's backward.
    The features are image coordinates (u / W, v / H): smooth everywhere,
    and each source point carries those of its true projection, so the
    feature residual is a reprojection error with its minimum at the ground
    truth.  (On high-frequency textures, or features that jump at depth
    edges, the finite-difference feature gradient of the reference is
    dominated by points straddling the jumps and BFGS cannot descend.)"""
    from slamtb_gb300.frame import KCamera
    from slamtb_gb300.registration import AutogradICP
    d = synthetic_pair(4, width=320, height=240, max_rot_deg=2.0, max_trans=0.02)
    s, t = d["src"], d["tgt"]
    gt = d["gt"].astype(np.float32)
    k = d["kcam"].astype(np.float32)
    h, w = t["mask"].shape
    q = (s["points"].reshape(-1, 3) @ gt[:3, :3].T + gt[:3, 3]).astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        uq = k[0, 0] * q[:, 0] / q[:, 2] + k[0, 2]
        vq = k[1, 1] * q[:, 1] / q[:, 2] + k[1, 2]
    src_feats = np.nan_to_num(np.stack([uq / w, vq / h])).astype(np.float32)
    vv, uu = np.mgrid[0:h, 0:w].astype(np.float32)
    tgt_feats = np.stack([uu / w, vv / h]).astype(np.float32)
    icp = AutogradICP(50, learning_rate=0.1, geom_weight=0.0, feat_weight=1.0,
                      distance_threshold=DIST, normals_angle_thresh=math.pi / 4)
    res = icp.estimate(KCamera(d["kcam"]), **_agicp_inputs(cuda, d),
                       target_feats=torch.from_numpy(tgt_feats).to(cuda),
                       source_feats=torch.from_numpy(src_feats).to(cuda))
    err = rel_pose(res.transform.numpy().astype(np.float64), d["gt"])
    assert err < 0.1, err


def test_reference_se3_cases(cuda):
    """The cases of slamtb/registration/_test/test_se3.py:16-50: the forward
    of its twist, gradcheck of ExpRtToMatrix on rand(1, 6) doubles (seed 10,
    eps 1e-6, atol 1e-4), and the round trip of its MatrixToExpRt case (a
    rotation given to 4 decimals, so the tolerance is 1e-3)."""
    from slamtb_gb300.registration import ExpRtToMatrix, MatrixToExpRt
    a = torch.tensor([1.9295e-03, 8.0992e-05, -7.9066e-04, -3.2908e-05, 7.6515e-03,
                      1.2822e-03], dtype=torch.float32)
    A = ExpRtToMatrix.apply(a.to(cuda)).cpu().numpy()
    np.testing.assert_allclose(A, ao.exp_rt_to_matrix64(a.numpy())[0], rtol=0, atol=1e-6)
    torch.manual_seed(10)
    inp = torch.rand(1, 6, dtype=torch.double, device=cuda, requires_grad=True)
    assert torch.autograd.gradcheck(ExpRtToMatrix.apply, (inp,), eps=1e-6, atol=1e-4,
                                    raise_exception=True)
    matrix = torch.tensor([[0.7350, 0.3997, -0.5477, -0.2654],
                           [-0.4502, 0.8917, 0.0464, 0.3553],
                           [0.5069, 0.2125, 0.8354, -0.3161]], device=cuda)
    matrix2 = ExpRtToMatrix.apply(MatrixToExpRt.apply(matrix))
    np.testing.assert_allclose(matrix2.cpu().numpy(), matrix.cpu().numpy(), rtol=0, atol=1e-3)
