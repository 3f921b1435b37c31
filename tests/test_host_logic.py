"""Host-side logic of the package that needs no GPU: the rigid transform and
Huber loss of AutogradICP's cost, the small host inputs handed to the C
entry by value, the unpacking of the FP64 result block, BatchRegistration's
level table and argument checks, MultiscaleRegistration's level loop, and
ICPOdometry's defaults and refusals."""
import math

import numpy as np
import pytest
import torch


def test_rigid_transform_points_and_normals():
    """camera.py:310-408: R p + t for points, (R^-1)^T n for normals."""
    from slamtb_gb300.camera import RigidTransform
    rng = np.random.default_rng(0)
    a = rng.normal(size=3)
    a *= 0.7 / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = np.eye(3) + np.sin(0.7) / 0.7 * K + (1 - np.cos(0.7)) / 0.49 * K @ K
    T = np.eye(4)
    T[:3, :3] = R * 1.5  # a non-rigid scale shows the inverse transpose at work
    T[:3, 3] = [0.1, -0.2, 0.3]
    p = rng.normal(size=(7, 3))
    n = rng.normal(size=(7, 3))
    rt = RigidTransform(torch.from_numpy(T))
    np.testing.assert_allclose((rt @ torch.from_numpy(p)).numpy(), p @ T[:3, :3].T + T[:3, 3],
                               atol=1e-12)
    np.testing.assert_allclose(rt.transform_normals(torch.from_numpy(n)).numpy(),
                               n @ np.linalg.inv(T[:3, :3]), atol=1e-12)


def test_huber_loss_matches_the_reference_formula():
    """autogradicp.py:60-90: mean of the residuals below alpha plus the mean
    of alpha |r| - alpha over the rest (either part may be empty)."""
    from slamtb_gb300.registration.autogradicp import robust_feature_cost
    r = torch.tensor([0.5, 1.0, 3.0, 5.0])
    assert float(robust_feature_cost(r, 2.0)) == pytest.approx(
        0.75 + ((2 * 3 - 2) + (2 * 5 - 2)) / 2)
    assert float(robust_feature_cost(torch.tensor([0.1, 0.3]), 2.0)) == pytest.approx(0.2)
    assert float(robust_feature_cost(torch.tensor([3.0, 5.0]), 2.0)) == pytest.approx(6.0)
    assert robust_feature_cost(torch.tensor([]), 2.0) == 0
    # alpha <= 0: the plain mean (autogradicp.py:183-186)
    assert float(robust_feature_cost(r, 0.0)) == pytest.approx(float(r.mean()))


def test_small_host_inputs_are_passed_by_value():
    """Intrinsics and initial poses held on the host reach the C entry as
    contiguous float32 / float64 arrays of the right size."""
    from slamtb_gb300.registration.icp import _small_input
    k = torch.tensor([[500.0, 0, 320], [0, 510, 240], [0, 0, 1]], dtype=torch.float64)
    arr, ptr = _small_input(k, torch.device("cuda", 0), torch.float32, np.float32, 9, "kcam")
    assert arr.dtype == np.float32 and arr.flags["C_CONTIGUOUS"] and ptr.value == arr.ctypes.data
    np.testing.assert_array_equal(arr.reshape(3, 3), k.numpy().astype(np.float32))
    T = np.eye(4)[:, ::-1]  # a non-contiguous view
    arr, _ = _small_input(T, torch.device("cuda", 0), torch.float64, np.float64, 16, "transform")
    assert arr.flags["C_CONTIGUOUS"]
    np.testing.assert_array_equal(arr, T)
    with pytest.raises(RuntimeError, match="16 entries"):
        _small_input(np.eye(3), torch.device("cuda", 0), torch.float64, np.float64, 16,
                     "transform")


def test_result_block_unpacking():
    """The FP64 result block (STB_RES_* layout) -> RegistrationResult, as
    icp.py:249-262: the transform and information as tensors that do not
    alias the (reused) block, the residual, and matches over source points;
    an empty result (information only) when no iteration succeeded."""
    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration.icp import ICPOdometry
    out = torch.zeros(N.RES_SIZE, dtype=torch.float64)
    T = torch.arange(16, dtype=torch.float64)
    out[N.RES_TRANSFORM:N.RES_TRANSFORM + 16] = T
    out[N.RES_INFO:N.RES_INFO + 36] = torch.arange(36, dtype=torch.float64) * 0.5
    out[N.RES_RESIDUAL] = 0.25
    out[N.RES_MATCHES] = 300.0
    out[N.RES_ITERS] = 10.0
    res = ICPOdometry._result(out, 1200, torch.float32)
    np.testing.assert_array_equal(res.transform.numpy(), T.view(4, 4).numpy())
    assert res.information.dtype == torch.float32 and res.information.shape == (6, 6)
    assert res.residual == 0.25 and res.match_ratio == 0.25
    out[N.RES_TRANSFORM] = 99.0
    assert res.transform[0, 0] == 0.0  # a copy
    out[N.RES_ITERS] = 0.0
    empty = ICPOdometry._result(out, 1200, torch.float32)
    assert empty.transform is None and empty.information is not None
    assert math.isinf(empty.residual)


def test_batch_registration_levels_and_argument_checks():
    """BatchRegistration takes the multiscale estimator list finest first (as
    MultiscaleRegistration, multiscale.py:11-67) and hands the kernel the
    levels coarsest first (the order they run, multiscale.py:52-55), each
    with its own estimator's parameters; bad arguments raise before any
    device work."""
    from slamtb_gb300.registration import BatchRegistration, ICPOdometry
    b = BatchRegistration([(1.0, ICPOdometry(10, feat_weight=0.1)), (0.5, ICPOdometry(5)),
                           (0.5, ICPOdometry(3, distance_threshold=0.2))])
    assert b.scales == [1.0, 0.5, 0.5]
    params, total = b._params()
    assert total == 18
    assert [(p.num_iters, p.distance_thresh, p.feat_weight) for p in params] == [
        (3, pytest.approx(0.2), 1.0), (5, pytest.approx(0.5), 1.0), (10, pytest.approx(0.5), 0.1)]
    with pytest.raises(ValueError, match="1 to 4 levels"):
        BatchRegistration([])
    with pytest.raises(ValueError, match="1 to 4 levels"):
        BatchRegistration([(1.0, ICPOdometry(1))] * 5)
    with pytest.raises(TypeError):
        BatchRegistration([(1.0, object())])
    with pytest.raises(ValueError, match="feat_channel_mode"):
        BatchRegistration([(1.0, ICPOdometry(1))], feat_channel_mode="mean")
    with pytest.raises(ValueError, match="non-empty"):
        b.prepare([], [])


def test_batch_schedule_encoding(monkeypatch):
    """BatchRegistration.run passes the lock-step schedules (0..5) as the
    entry's tile_config and the grouped ones (GROUPED + g) as
    STB_OPT_GROUPS in channel_mode with g groups; the tuned default covers
    both kinds."""
    import types

    import torch

    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration import BatchRegistration, ICPOdometry
    from slamtb_gb300.registration import batch as bmod
    calls = []

    class FakeLib:
        def stb_icp_estimate_batch(self, *args):
            calls.append(args)
            return 0

    monkeypatch.setattr(N, "lib", lambda: FakeLib())
    monkeypatch.setattr(N, "stream_of", lambda device: None)
    monkeypatch.setattr(torch.cuda, "device", lambda d: __import__("contextlib").nullcontext())
    b = BatchRegistration([(1.0, ICPOdometry(3))])
    plan = types.SimpleNamespace(
        device="cuda:0", levels=None, B=2, L=1, params=b._params()[0], channels=0, code=0,
        mode=1, init=None, total_px=100, ws=torch.empty(1), results=None, history=None)
    b.run(plan, 3)
    b.run(plan, bmod.GROUPED + 8)
    assert calls[0][6] == 1 and calls[0][13] == 3
    assert calls[1][6] == 1 | N.OPT_GROUPS and calls[1][13] == 8
    assert any(c < bmod.GROUPED for c in bmod.TUNE_CONFIGS)
    assert any(c > bmod.GROUPED for c in bmod.TUNE_CONFIGS)


def test_multiscale_level_loop_hands_transforms_coarse_to_fine():
    """MultiscaleRegistration.estimate_pyramid (multiscale.py:52-67): the
    estimators, listed finest first, run on the pyramid coarsest first; each
    level starts from the previous level's transform, and a level that
    failed (transform None) hands None -- the identity -- to the next, as
    the reference does."""
    from slamtb_gb300.registration import MultiscaleRegistration
    from slamtb_gb300.registration.result import RegistrationResult

    calls = []

    class Fake:
        def __init__(self, name, out):
            self.name, self.out = name, out

        def estimate_frame(self, source, target, source_feats=None, target_feats=None,
                           transform=None, device=None):
            calls.append((self.name, source, target, source_feats, transform))
            return RegistrationResult(self.out)

    T1 = torch.eye(4, dtype=torch.float64) * 2
    ms = MultiscaleRegistration([(1.0, Fake("fine", "T_fine")), (0.5, Fake("mid", None)),
                                 (0.5, Fake("coarse", T1))])
    res = ms.estimate_pyramid(["s_coarse", "s_mid", "s_fine"], ["t_coarse", "t_mid", "t_fine"],
                              transform="T0")
    assert [c[0] for c in calls] == ["coarse", "mid", "fine"]
    assert [(c[1], c[2]) for c in calls] == [("s_coarse", "t_coarse"), ("s_mid", "t_mid"),
                                              ("s_fine", "t_fine")]
    assert calls[0][4] == "T0" and calls[1][4] is T1 and calls[2][4] is None
    assert all(c[3] is None for c in calls)
    assert res.transform == "T_fine"


def test_icp_odometry_constructor_checks():
    """ICPOdometry keeps the reference's keyword defaults (icp.py:137-139)
    and refuses what it cannot run: so3=True (the reference's rotation-only
    path fails with a TypeError, icp.py:71-76), more iterations than the
    key map's epoch tags, and unknown channel modes, layouts or solve
    precisions; the solve is FP64 unless asked otherwise."""
    from slamtb_gb300.registration import ICPOdometry
    icp = ICPOdometry(10)
    assert (icp.geom_weight, icp.feat_weight, icp.so3) == (1.0, 1.0, False)
    assert icp.distance_threshold == 0.5
    assert icp.normals_angle_thresh == pytest.approx(math.pi / 4)
    assert icp.feat_residual_thresh == 2.75
    with pytest.raises(NotImplementedError, match="so3"):
        ICPOdometry(10, so3=True)
    with pytest.raises(ValueError, match="254"):
        ICPOdometry(255)
    with pytest.raises(ValueError, match="feat_channel_mode"):
        ICPOdometry(10, feat_channel_mode="max")
    with pytest.raises(ValueError, match="feat_layout"):
        ICPOdometry(10, feat_layout="hwc")
    assert icp.solve_precision == "fp64"
    with pytest.raises(ValueError, match="solve_precision"):
        ICPOdometry(10, solve_precision="fp32")


def test_point_to_plane_loss_argument_checks():
    """PointToPlaneLoss refuses host tensors before any device work (it
    checks every per-pixel input's dtype, device and (B, H, W[, 3]) shape)."""
    from slamtb_gb300.registration import point_to_plane_loss
    B, H, W = 2, 6, 8
    depth = torch.rand(B, H, W)
    pts = torch.rand(B, H, W, 3)
    mask = torch.ones(B, H, W, dtype=torch.bool)
    poses = torch.eye(4, dtype=torch.float64).expand(B, 4, 4)
    twist = torch.zeros(B, 6, dtype=torch.float64)
    args = [twist, depth, pts, mask, pts, pts, mask, (50.0, 50.0, 4.0, 3.0), poses, 0.1, 0.5]
    with pytest.raises(RuntimeError, match="source_depth must be a float32 CUDA tensor"):
        point_to_plane_loss(*args)
