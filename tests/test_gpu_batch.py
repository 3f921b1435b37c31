"""Persistent batched path (BatchRegistration -> stb_icp_estimate_batch).

Every pair's every iteration is checked against the oracle step at the
GPU's own previous pose (teacher forcing, the 1e-5 gate of
``_helpers.compare_forced``), for uneven resolutions, three levels and the
hybrid geometric + feature term; failures stay inside their pair; the
reference's level hand-over (identity after a failed first iteration,
multiscale.py:64-65) is reproduced.  Each check runs under four schedules:
the lock-step kernel, and the grouped kernel with one group (the whole
grid on each pair in turn), three groups (so that the grid's blocks past
the last whole group stay idle) and 76 groups of two blocks (more groups
than pairs).
"""
import math

import numpy as np
import pytest
import torch

from oracle import frame_prep as fp
from slamtb_gb300 import synthetic
from _helpers import compare_forced, rel_pose

pytestmark = pytest.mark.gpu

SCALES = [1.0, 0.5, 0.5]
ITERS = [6, 4, 3]  # finest first
SCHEDULES = [0, 101, 103, 176]  # lock-step (8192-pixel work items); grouped, 1, 3 and 76 groups


def _kw(n, wf, wg=1.0):
    return dict(num_iters=n, geom_weight=wg, feat_weight=wf, distance_threshold=0.1,
                normals_angle_thresh=math.radians(20))


def _estimators(wf, iters=ITERS, scales=SCALES, wg=1.0):
    from slamtb_gb300.registration import ICPOdometry
    return [(s, ICPOdometry(n, **{k: v for k, v in _kw(n, wf, wg).items() if k != "num_iters"}))
            for s, n in zip(scales, iters)]


def _device_levels(cuda, pyr):
    from slamtb_gb300.frame import FramePointCloud, KCamera
    out = []
    for lv in pyr:
        out.append(FramePointCloud(None, torch.from_numpy(lv.mask).to(cuda), KCamera(lv.kcam),
                                   points=torch.from_numpy(lv.points).to(cuda),
                                   normals=torch.from_numpy(lv.normals).to(cuda)))
    return out


def _pair(cuda, seed, w, h, feats, scales=SCALES, channels=0, dtype=torch.float32, **kw):
    from slamtb_gb300.processing import feature_pyramid
    p = synthetic.make_pair(seed, width=w, height=h, feature_channels=channels if feats else None,
                            **kw)
    spyr = fp.FramePointCloud.from_depth(p["source_depth"], p["kcam"]).pyramid(scales)
    tpyr = fp.FramePointCloud.from_depth(p["target_depth"], p["kcam"]).pyramid(scales)
    out = dict(spyr=spyr, tpyr=tpyr, src=_device_levels(cuda, spyr),
               tgt=_device_levels(cuda, tpyr))
    if feats:
        out["sf"] = feature_pyramid(torch.from_numpy(p["source_feats"]).to(cuda, dtype), scales)
        out["tf"] = feature_pyramid(torch.from_numpy(p["target_feats"]).to(cuda, dtype), scales)
    return out


def _check_pair(hist, pair, wf, iters=ITERS, init=None, channel_mode="last", wg=1.0):
    """Teacher-forced check of one pair's history, level by level."""
    from slamtb_gb300 import _native as N
    off = 0
    T = init
    for level, n in enumerate(iters[::-1]):
        s, t = pair["spyr"][level], pair["tpyr"][level]
        d = dict(kcam=s.kcam, src=dict(points=s.points, normals=s.normals, mask=s.mask),
                 tgt=dict(points=t.points, normals=t.normals, mask=t.mask))
        x = {}
        if wf > 0:
            x = dict(sf=pair["sf"][level].reshape(pair["sf"][level].size(0), -1),
                     tf=pair["tf"][level])
        h = hist[off:off + n]
        ok = h[:, N.HIST_OK].numpy()
        compare_forced(h, d, x, _kw(n, wf, wg), init=T, channel_mode=channel_mode)
        done = int(ok.sum()) if ok.all() else int(np.argmin(ok))
        if done > 0:
            T = h[done - 1, N.HIST_TRANSFORM:N.HIST_TRANSFORM + 16].view(4, 4).numpy()
        else:
            T = np.eye(4)  # the reference hands transform=None to the next level
        off += n


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_single_pair_single_level_matches_icpodometry(cuda, schedule):
    from slamtb_gb300.registration import BatchRegistration, ICPOdometry
    pair = _pair(cuda, 31, 640, 480, False, scales=[1.0])
    br = BatchRegistration(_estimators(0.0, iters=[10], scales=[1.0]), record_history=True)
    br.tile_config = schedule
    res = br.estimate_pyramids([pair["src"]], [pair["tgt"]])[0]
    icp = ICPOdometry(10, geom_weight=1.0, feat_weight=0.0, distance_threshold=0.1,
                      normals_angle_thresh=math.radians(20))
    s, t = pair["src"][0], pair["tgt"][0]
    ref = icp.estimate(s.kcam, s.points, s.normals, s.mask, target_points=t.points,
                       target_mask=t.mask, target_normals=t.normals)
    assert rel_pose(res.transform.numpy(), ref.transform.numpy()) <= 1e-5
    assert res.match_ratio == ref.match_ratio
    assert res.residual == pytest.approx(ref.residual, rel=1e-5)
    np.testing.assert_allclose(res.information.numpy(), ref.information.numpy(), rtol=1e-5)
    _check_pair(br.last_history[0], pair, 0.0, iters=[10])


@pytest.mark.parametrize("wf", [0.0, 0.1])
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_uneven_multiscale_batch_teacher_forced(cuda, wf, schedule):
    from slamtb_gb300.registration import BatchRegistration
    sizes = [(320, 240), (160, 120), (424, 240)]
    pairs = [_pair(cuda, 40 + k, w, h, wf > 0) for k, (w, h) in enumerate(sizes)]
    br = BatchRegistration(_estimators(wf), record_history=True)
    br.tile_config = schedule
    res = br.estimate_pyramids([p["src"] for p in pairs], [p["tgt"] for p in pairs],
                               [p["sf"] for p in pairs] if wf > 0 else None,
                               [p["tf"] for p in pairs] if wf > 0 else None)
    assert len(res) == 3
    for k, pair in enumerate(pairs):
        assert res[k].transform is not None
        _check_pair(br.last_history[k], pair, wf)


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_failed_pair_stays_isolated(cuda, schedule):
    from slamtb_gb300.registration import BatchRegistration
    good = _pair(cuda, 50, 320, 240, False)
    bad = _pair(cuda, 51, 320, 240, False)
    for lv in bad["tgt"]:
        lv.mask = torch.zeros_like(lv.mask)
    for lv in bad["tpyr"]:
        lv.mask = np.zeros_like(lv.mask)
    br = BatchRegistration(_estimators(0.0), record_history=True)
    br.tile_config = schedule
    res = br.estimate_pyramids([good["src"], bad["src"]], [good["tgt"], bad["tgt"]])
    assert res[1].transform is None and res[1].match_ratio == 0
    assert res[0].transform is not None
    _check_pair(br.last_history[0], good, 0.0)
    _check_pair(br.last_history[1], bad, 0.0)


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_level_handover_after_failed_first_iteration(cuda, schedule):
    """The coarsest level of pair 0 cannot match (empty target mask): the
    next level starts from the identity, not from the initial transform."""
    from slamtb_gb300.registration import BatchRegistration
    from oracle import icp_oracle as io
    pair = _pair(cuda, 52, 320, 240, False)
    pair["tgt"][0].mask = torch.zeros_like(pair["tgt"][0].mask)
    pair["tpyr"][0].mask = np.zeros_like(pair["tpyr"][0].mask)
    init = io.se3_exp([0.01, 0.0, 0.0, 0.0, 0.0, 0.0])
    br = BatchRegistration(_estimators(0.0), record_history=True)
    br.tile_config = schedule
    br.estimate_pyramids([pair["src"]], [pair["tgt"]], transforms=[torch.from_numpy(init)])
    _check_pair(br.last_history[0], pair, 0.0, init=init)


@pytest.mark.parametrize("mode", ["last", "sum"])
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_bf16_sixteen_channel_four_level_batch(cuda, mode, schedule):
    """The high-resolution feature workload at reduced size: 16:9 pairs
    (480x270), 16 BF16 feature channels normalised per pixel, 4 levels
    with iterations [10, 8, 5, 3], rotation up to 10 degrees and
    translation up to 10 cm; the oracle sees the same BF16 values as
    float32.  Weights are the reference preset's (geometric 10, feature 1,
    slamtb/registration/preset.py:10): with 16 channels a feature weight of
    0.1 makes the reference's weighting (J^T r by w, J^T J by w^2) overshoot
    and the normal equations ill-conditioned (the FP64 oracle's own
    Cholesky fails), where no float32 pose can meet a 1e-5 gate."""
    from slamtb_gb300.registration import BatchRegistration
    scales, iters = [1.0, 0.5, 0.5, 0.5], [10, 8, 5, 3]
    pairs = [_pair(cuda, 60 + k, 480, 270, True, scales=scales, channels=16,
                   dtype=torch.bfloat16, max_rot_deg=10.0, max_trans=0.1) for k in range(2)]
    assert pairs[0]["tf"][0].dtype == torch.bfloat16 and pairs[0]["tf"][0].size(0) == 16
    br = BatchRegistration(_estimators(1.0, iters=iters, scales=scales, wg=10.0),
                           feat_channel_mode=mode, record_history=True)
    br.tile_config = schedule
    res = br.estimate_pyramids([p["src"] for p in pairs], [p["tgt"] for p in pairs],
                               [p["sf"] for p in pairs], [p["tf"] for p in pairs])
    for k, pair in enumerate(pairs):
        assert res[k].transform is not None
        _check_pair(br.last_history[k], pair, 1.0, iters=iters, channel_mode=mode, wg=10.0)


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_bounded_waits_give_up_with_a_timeout_status(cuda, schedule):
    """With stb_set_wait_test_limits making every grid barrier expect one
    block more than the cooperative grid has, no barrier completes: each
    wait gives up after its poll limit, every pair's status gets
    STB_ST_TIMEOUT and BatchRegistration.results raises.  Nothing hangs; the
    next run (limits restored) succeeds."""
    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration import BatchRegistration
    pairs = [_pair(cuda, 53 + k, 160, 120, False) for k in range(2)]
    br = BatchRegistration(_estimators(0.0))
    br.tile_config = schedule
    srcs, tgts = [p["src"] for p in pairs], [p["tgt"] for p in pairs]
    try:
        N.check(N.lib().stb_set_wait_test_limits(1 << 10, 1))
        _, _, plan = br.launch(srcs, tgts)
        status = plan.results[:, N.RES_STATUS].cpu().numpy().astype(np.int64)
        with pytest.raises(RuntimeError, match="stopped early"):
            br.results(plan)
    finally:
        N.check(N.lib().stb_set_wait_test_limits(0, 0))
    assert ((status & N.ST_TIMEOUT) != 0).all()
    res = br.estimate_pyramids(srcs, tgts)
    assert all(r.transform is not None for r in res)


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_graph_replay_equals_direct(cuda, schedule):
    """BatchRegistration.run(graph=True) captures the launch sequence once
    per schedule and replays it: every replay gives the direct launch's
    result block bit for bit."""
    from slamtb_gb300.registration import BatchRegistration
    pairs = [_pair(cuda, 90 + k, w, h, False) for k, (w, h) in enumerate([(320, 240), (160, 120)])]
    br = BatchRegistration(_estimators(0.0))
    br.tile_config = schedule
    plan = br.prepare([p["src"] for p in pairs], [p["tgt"] for p in pairs])
    direct = br.run(plan)[0].clone()
    for _ in range(2):
        replay = br.run(plan, graph=True)[0]
        torch.cuda.synchronize()
        assert torch.equal(replay, direct)
    assert list(plan.graphs) == [schedule]
