"""The C/OpenMP port (the timed CPU baseline) agrees with the numpy oracle."""
import math

import numpy as np
import pytest

from oracle import icp_oracle as io
from oracle import port
from _helpers import synthetic_pair


def _rel(a, b):
    d = io.se3_log(np.linalg.inv(b) @ a)
    return np.linalg.norm(d) / max(np.linalg.norm(io.se3_log(b)), 1e-3)


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


@pytest.mark.parametrize("empty", ["source", "target"])
def test_port_and_oracle_without_matches(empty):
    """No valid source (or target) pixel: the first solve fails (JᵀJ = 0), so
    both stop before any update (icp.py:236-242 `break`) and report no
    transform, zero match ratio, an infinite residual and a zero
    information matrix, as the GPU path's empty result does."""
    d = synthetic_pair(6, width=64, height=48, feature_channels=0)
    s, t = d["src"], d["tgt"]
    sm = np.zeros_like(s["mask"]) if empty == "source" else s["mask"]
    tm = np.zeros_like(t["mask"]) if empty == "target" else t["mask"]
    kw = dict(num_iters=3, geom_weight=1.0, feat_weight=0.0, distance_threshold=0.1,
              normals_angle_thresh=math.radians(20))
    o = io.icp_estimate(d["kcam"], s["points"], s["normals"], sm, t["points"], t["normals"],
                        tm, **kw)
    p = port.icp_estimate(d["kcam"], s["points"], s["normals"], sm, t["points"], t["normals"],
                          tm, threads=2, **kw)
    assert o.transform is None and p["transform"] is None
    assert len(o.history) == p["iters"] == 0
    assert o.match_ratio == p["match_ratio"] == 0.0
    assert math.isinf(o.residual) and math.isinf(p["residual"])
    assert not np.any(o.information) and not np.any(p["information"])


def _levels(d, scales):
    """Coarsest-first level dicts of a pair's pyramids (normals per level)."""
    out = []
    for s, t in zip(d["src_fpcl"].pyramid(scales), d["tgt_fpcl"].pyramid(scales)):
        out.append(dict(kcam=s.kcam, src_points=s.points, src_normals=s.normals,
                        src_mask=s.mask, tgt_points=t.points, tgt_normals=t.normals,
                        tgt_mask=t.mask))
    return out


def test_port_multiscale_follows_the_oracle_hand_over():
    """port.multiscale_estimate runs the levels coarsest first with the
    estimators listed finest first, each level starting at the previous
    level's transform, as icp_oracle.multiscale_estimate; on a short
    geometric schedule the two agree within 1e-5 of the motion, and a level
    whose first solve fails hands identity to the next in both."""
    d = synthetic_pair(8, width=320, height=240)
    levels = _levels(d, [1.0, 0.5])
    ests = [dict(num_iters=n, geom_weight=1.0, feat_weight=0.0, distance_threshold=0.1,
                 normals_angle_thresh=math.radians(20)) for n in (3, 2)]
    o = io.multiscale_estimate(levels, ests)
    p = port.multiscale_estimate(levels, ests, threads=2)
    assert p["iters"] == len(o.history) == 3
    assert _rel(p["transform"], o.transform) < 1e-5
    # the coarse level without a valid source pixel: no transform from it,
    # and the fine level starts from identity in both
    dead = [dict(levels[0], src_mask=np.zeros_like(levels[0]["src_mask"])), levels[1]]
    o2 = io.multiscale_estimate(dead, ests)
    p2 = port.multiscale_estimate(dead, ests, threads=2)
    single = port.icp_estimate(**levels[1], **ests[0], threads=2)
    assert _rel(p2["transform"], o2.transform) < 1e-5
    np.testing.assert_array_equal(p2["transform"], single["transform"])
    with pytest.raises(ValueError):
        port.multiscale_estimate(levels, [dict(e, channel_mode="sum") for e in ests])


def test_bench_accuracy_tables_on_cpu():
    """The benchmark's accuracy rows run without a GPU: the FP64 oracle's
    free-running registrations (spawned processes), the error table of a set
    of final poses against them (the oracle's own poses give 0 up to the
    rounding of the rotation angle; a failed pair counts as infinite), and the port's registrations of the same jobs
    (the reference CPU arithmetic), within 1e-3 of the motion here."""
    import bench
    jobs = []
    for seed in (3, 4):
        d = synthetic_pair(seed, width=160, height=120)
        ests = [dict(num_iters=n, geom_weight=1.0, feat_weight=0.0, distance_threshold=0.1,
                     normals_angle_thresh=math.radians(20)) for n in (3, 2)]
        jobs.append((_levels(d, [1.0, 0.5]), ests, "last"))
    outs = bench._oracle_runs(jobs, 1)
    assert all(T is not None and np.isfinite(c) for T, c in outs)
    own = bench._error_table([T for T, _ in outs], outs)
    assert own["max"] < 1e-12 and own["within_1e-5"] == 1.0
    assert all(e < 1e-12 for e in own["per_pair"])
    failed = bench._error_table([outs[0][0], None], outs)
    assert failed["per_pair"][1] == math.inf
    ref = bench._reference_arithmetic(jobs, outs, 2)
    assert ref["pairs"] == 2 and ref["max"] < 1e-3
