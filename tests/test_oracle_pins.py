"""Known-answer pins of the oracle on the reference's own test data.

The reference's ICP tests hold no golden vectors; their fixtures hold
ground-truth camera poses.  The synthetic pair of
slamtb/registration/_test/test_icp.py:19-27 (sample2 frames 0 -> 3, run
by ``depth_synthetic`` with ICPOdometry(15, geom_weight=1, feat_weight=0,
distance_threshold=0.1, normals_angle_thresh=pi/4)) must recover the
ground-truth relative pose."""
import math

import numpy as np

from oracle import icp_oracle as io
from _helpers import sample2_pair, pose_error


def test_sample2_depth_synthetic_recovers_ground_truth():
    d = sample2_pair(0, 3)
    s, t = d["src"], d["tgt"]
    res = io.icp_estimate(d["kcam"], s["points"], s["normals"], s["mask"], t["points"],
                          t["normals"], t["mask"], num_iters=15, geom_weight=1,
                          feat_weight=0, distance_threshold=0.1,
                          normals_angle_thresh=math.pi / 4)
    gt_t, gt_r = pose_error(np.eye(4), d["gt"])
    err_t, err_r = pose_error(res.transform, d["gt"])
    assert gt_r > 5e-3  # the pair has a real motion (~0.48 degrees)
    assert err_r < 0.1 * gt_r
    assert err_t < 1e-3
    assert res.match_ratio > 0.9
    assert len(res.history) == 15
    info = res.information
    assert np.allclose(info, info.T) and np.all(np.linalg.eigvalsh(info) > 0)


def test_sample2_correspondence_map_fixture_pair():
    """The pair of test_correspondence_map.py:16-19 (frames 0 and 13,
    CorrespondenceMap(10, 10) at identity): every winner's stored distance
    is the float32 distance of its pair and no source wins twice."""
    d = sample2_pair(0, 13)
    s, t = d["src"], d["tgt"]
    a = io.associate32(s["points"], s["normals"], s["mask"], io.pose_rt32(np.eye(4)),
                       t["points"], t["normals"], t["mask"], d["kcam"], 10, 10)
    won = a.winner[a.winner >= 0]
    assert won.size > 0.9 * s["mask"].sum() * 0.5
    assert np.unique(won).size == won.size
    pix = np.nonzero(a.winner.reshape(-1) >= 0)[0]
    q = t["points"].reshape(-1, 3)[pix]
    p = s["points"].reshape(-1, 3)[a.winner.reshape(-1)[pix]]
    dist = np.sqrt(io.sqnorm32((q - p).astype(np.float32)))
    np.testing.assert_array_equal(dist, a.dist.reshape(-1)[pix])
