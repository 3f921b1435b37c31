"""Multiscale registration (three levels 640/320/160 with 10/5/3
iterations) against the oracle on the same pyramids: every level's
iterations teacher-forced within the 1e-5 gate (geometric-only and hybrid
geometric + intensity term with w_f = 0.1), and the geometric-only run
free-running within 1e-3 of the pose and of the match ratio (18 iterations
over three levels accumulate the ~1e-7 per-step float32 differences)."""
import math

import numpy as np
import pytest
import torch

from oracle import frame_prep as fp
from oracle import icp_oracle as io
from slamtb_gb300 import synthetic
from _helpers import compare_forced, rel_pose

pytestmark = pytest.mark.gpu

ITERS = [10, 5, 3]  # finest first, as the reference's estimator lists
SCALES = [1.0, 0.5, 0.5]


def _kw(wf):
    return dict(geom_weight=1.0, feat_weight=wf, distance_threshold=0.1,
                normals_angle_thresh=math.radians(20))


def _run(cuda, p, wf):
    from slamtb_gb300.frame import Frame, FrameInfo, KCamera
    from slamtb_gb300.registration import ICPOdometry, MultiscaleICPOdometry
    k = KCamera(p["kcam"])
    ests = [ICPOdometry(n, record_history=True, **_kw(wf)) for n in ITERS]
    ms = MultiscaleICPOdometry(list(zip(SCALES, ests)))
    sf = torch.from_numpy(p["source_feats"]).to(cuda)
    tf = torch.from_numpy(p["target_feats"]).to(cuda)
    res = ms.estimate_frame(Frame(FrameInfo(k), p["source_depth"]),
                            Frame(FrameInfo(k), p["target_depth"]),
                            source_feats=sf if wf > 0 else None,
                            target_feats=tf if wf > 0 else None, device=cuda)
    return res, ests, sf, tf


def _levels(p):
    spyr = fp.FramePointCloud.from_depth(p["source_depth"], p["kcam"]).pyramid(SCALES)
    tpyr = fp.FramePointCloud.from_depth(p["target_depth"], p["kcam"]).pyramid(SCALES)
    return spyr, tpyr


@pytest.mark.parametrize("wf", [0.0, 0.1])
def test_multiscale_levels_teacher_forced(cuda, wf):
    from slamtb_gb300.processing import feature_pyramid
    p = synthetic.make_pair(1, feature_channels=0)
    res, ests, sf, tf = _run(cuda, p, wf)
    spyr, tpyr = _levels(p)
    sfp = feature_pyramid(sf, SCALES)
    tfp = feature_pyramid(tf, SCALES)
    init = None
    for level, (s, t, a, b, est) in enumerate(zip(spyr, tpyr, sfp, tfp, ests[::-1])):
        d = dict(kcam=s.kcam, src=dict(points=s.points, normals=s.normals, mask=s.mask),
                 tgt=dict(points=t.points, normals=t.normals, mask=t.mask))
        x = dict(sf=a.reshape(a.size(0), -1), tf=b) if wf > 0 else {}
        compare_forced(est.last_history, d, x, dict(num_iters=est.num_iters, **_kw(wf)),
                       init=init)
        from slamtb_gb300 import _native as N
        init = est.last_history[-1, N.HIST_TRANSFORM:N.HIST_TRANSFORM + 16].view(4, 4).numpy()
    np.testing.assert_array_equal(res.transform.numpy(), init)


def test_multiscale_geometric_free_running(cuda):
    p = synthetic.make_pair(1, feature_channels=0)
    res, _, _, _ = _run(cuda, p, 0.0)
    spyr, tpyr = _levels(p)
    levels = [dict(kcam=s.kcam, src_points=s.points, src_normals=s.normals, src_mask=s.mask,
                   tgt_points=t.points, tgt_normals=t.normals, tgt_mask=t.mask)
              for s, t in zip(spyr, tpyr)]
    ores = io.multiscale_estimate(levels, [dict(num_iters=n, **_kw(0.0)) for n in ITERS])
    # free-running: float32 sums against the oracle's FP64 ones move each
    # pose by ~1e-7 relative, which flips a few correspondences of later
    # iterations (a dozen of the ~30,700 matches at the final pose; how many
    # depends on the order of the float32 sums, not on a defect); the
    # per-iteration gate is the teacher-forced one above
    assert rel_pose(res.transform.numpy(), ores.transform) <= 1e-3
    assert res.match_ratio == pytest.approx(ores.match_ratio, rel=1e-3)
