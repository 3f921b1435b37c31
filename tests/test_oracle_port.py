"""The C/OpenMP port (the timed CPU baseline) agrees with the numpy oracle."""
import math

import numpy as np

from oracle import icp_oracle as io
from oracle import port
from _helpers import synthetic_pair


def _rel(a, b):
    d = io.se3_log(np.linalg.inv(b) @ a)
    return np.linalg.norm(d) / max(np.linalg.norm(io.se3_log(b)), 1e-3)


import pytest


@pytest.mark.parametrize("iters,wf", [(6, 0.0), (1, 0.1)])
def test_port_matches_numpy_oracle(iters, wf):
    """Free-running over 6 iterations for the geometric term; one iteration
    with the feature term (its float32 evaluation in the port, as in the
    reference, differs from the oracle's float64 one by ~1e-6 per step,
    which feature-driven iterations can amplify)."""
    d = synthetic_pair(6, width=320, height=240, feature_channels=0)
    s, t = d["src"], d["tgt"]
    kw = dict(num_iters=iters, geom_weight=1.0, feat_weight=wf, distance_threshold=0.1,
              normals_angle_thresh=math.radians(20))
    o = io.icp_estimate(d["kcam"], s["points"], s["normals"], s["mask"], t["points"],
                        t["normals"], t["mask"], src_feats=d["src_feats"],
                        tgt_feats=d["tgt_feats"], **kw)
    p = port.icp_estimate(d["kcam"], s["points"], s["normals"], s["mask"], t["points"],
                          t["normals"], t["mask"], src_feats=d["src_feats"],
                          tgt_feats=d["tgt_feats"], threads=4, **kw)
    assert p["iters"] == len(o.history) == iters
    assert _rel(p["transform"], o.transform) < 1e-5
    assert p["match_ratio"] == o.match_ratio
    np.testing.assert_allclose(p["information"], o.information, rtol=1e-6)
