"""Multiscale hybrid registration (geometric + intensity term, three
levels 640/320/160 with 10/5/3 iterations, w_g = 1, w_f = 0.1) against the
oracle's multiscale loop on the same pyramids."""
import math

import numpy as np
import pytest
import torch

from oracle import frame_prep as fp
from oracle import icp_oracle as io
from slamtb_gb300 import synthetic

pytestmark = pytest.mark.gpu

LEVEL_KW = dict(geom_weight=1.0, feat_weight=0.1, distance_threshold=0.1,
                normals_angle_thresh=math.radians(20))
ITERS = [10, 5, 3]  # finest first, as the reference's estimator lists


def test_multiscale_hybrid_matches_oracle(cuda):
    from slamtb_gb300.frame import Frame, FrameInfo, KCamera
    from slamtb_gb300.registration import ICPOdometry, MultiscaleICPOdometry
    p = synthetic.make_pair(1, feature_channels=0)
    k = KCamera(p["kcam"])
    ms = MultiscaleICPOdometry([(1.0, ICPOdometry(ITERS[0], **LEVEL_KW)),
                                (0.5, ICPOdometry(ITERS[1], **LEVEL_KW)),
                                (0.5, ICPOdometry(ITERS[2], **LEVEL_KW))])
    sf = torch.from_numpy(p["source_feats"]).to(cuda)
    tf = torch.from_numpy(p["target_feats"]).to(cuda)
    res = ms.estimate_frame(Frame(FrameInfo(k), p["source_depth"]),
                            Frame(FrameInfo(k), p["target_depth"]),
                            source_feats=sf, target_feats=tf, device=cuda)

    # oracle on the same pyramids (the blur is float32 on the device and
    # float64 in the oracle, so the device feature pyramid is read back)
    from slamtb_gb300.processing import feature_pyramid
    scales = [1.0, 0.5, 0.5]
    spyr = fp.FramePointCloud.from_depth(p["source_depth"], p["kcam"]).pyramid(scales)
    tpyr = fp.FramePointCloud.from_depth(p["target_depth"], p["kcam"]).pyramid(scales)
    sfp = [f.cpu().numpy() for f in feature_pyramid(sf, scales)]
    tfp = [f.cpu().numpy() for f in feature_pyramid(tf, scales)]
    levels = [dict(kcam=s.kcam, src_points=s.points, src_normals=s.normals, src_mask=s.mask,
                   tgt_points=t.points, tgt_normals=t.normals, tgt_mask=t.mask,
                   src_feats=a, tgt_feats=b) for s, t, a, b in zip(spyr, tpyr, sfp, tfp)]
    ests = [dict(num_iters=n, **LEVEL_KW) for n in ITERS]
    ores = io.multiscale_estimate(levels, ests)
    d = io.se3_log(np.linalg.inv(ores.transform) @ res.transform.numpy())
    scale = max(np.linalg.norm(io.se3_log(ores.transform)), 1e-3)
    assert np.linalg.norm(d) <= 1e-5 * scale
    assert res.match_ratio == pytest.approx(ores.match_ratio, rel=1e-4)
