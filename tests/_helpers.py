"""Input preparation shared by the tests: seeded synthetic pairs and the
reference's sample2 frames, prepared by the oracle's restatement of
FramePointCloud (erosion, back-projection, central-difference normals)."""
import math
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

from oracle import frame_prep as fp  # noqa: E402
from slamtb_gb300 import synthetic  # noqa: E402

ANGLE_20 = math.radians(20.0)


def frame_arrays(fpcl):
    return dict(points=fpcl.points, normals=fpcl.normals, mask=fpcl.mask, kcam=fpcl.kcam)


def synthetic_pair(seed, width=640, height=480, feature_channels=None, **kw):
    p = synthetic.make_pair(seed, width=width, height=height,
                            feature_channels=feature_channels, **kw)
    tgt = fp.FramePointCloud.from_depth(p["target_depth"], p["kcam"])
    src = fp.FramePointCloud.from_depth(p["source_depth"], p["kcam"])
    out = dict(src=frame_arrays(src), tgt=frame_arrays(tgt), kcam=p["kcam"], gt=p["gt"],
               src_fpcl=src, tgt_fpcl=tgt)
    if feature_channels is not None:
        out["src_feats"] = p["source_feats"]
        out["tgt_feats"] = p["target_feats"]
    return out


def sample2_pair(target=0, source=3):
    from make_golden import load_sample2
    d = load_sample2()

    def fpcl(i):
        depth = (d[i]["depth"].astype(np.float32) * np.float32(d[i]["depth_scale"])
                 + np.float32(d[i]["depth_bias"]))
        return fp.FramePointCloud.from_depth(depth, d[i]["kcam"])

    tgt, src = fpcl(target), fpcl(source)
    gt = np.linalg.inv(d[target]["rt_cam"]) @ d[source]["rt_cam"]
    return dict(src=frame_arrays(src), tgt=frame_arrays(tgt), kcam=src.kcam, gt=gt,
                src_fpcl=src, tgt_fpcl=tgt)


def pose_error(a, b):
    """(translation distance, rotation angle) of a^-1 b."""
    D = np.linalg.inv(np.asarray(a, dtype=np.float64)) @ np.asarray(b, dtype=np.float64)
    c = min(1.0, max(-1.0, (np.trace(D[:3, :3]) - 1.0) / 2.0))
    return float(np.linalg.norm(D[:3, 3])), math.acos(c)


def rel_pose(a, b):
    """||log(b^-1 a)|| / max(||log b||, 1e-3)."""
    from oracle import icp_oracle as io
    d = io.se3_log(np.linalg.inv(b) @ a)
    return np.linalg.norm(d) / max(np.linalg.norm(io.se3_log(b)), 1e-3)


def compare_forced(hist, d, x, kw, init=None, channel_mode="last", tol=1e-5, step_tol=1e-11):
    """Teacher-forced comparison of a GPU history (``ICPOdometry.last_history``)
    with the oracle's step evaluated at the GPU's previous pose; ``x`` holds
    the device feature maps as used (``sf``/``tf``).  Each iteration's device
    solve and update are also checked on their own inputs: the oracle's FP64
    Cholesky solve and exponential of the device's recorded J^T J and J^T r,
    applied to the device's previous pose, must give the device's pose within
    ``step_tol`` (largest entry difference over the largest entry).  Returns
    the worst pose error."""
    from oracle import icp_oracle as io
    from slamtb_gb300 import _native as N
    s, t = d["src"], d["tgt"]
    sf = x["sf"].float().cpu().numpy() if "sf" in x else None
    tf = x["tf"].float().cpu().numpy() if "tf" in x else None
    step_kw = {k: v for k, v in kw.items() if k != "num_iters"}
    h = hist.numpy()
    T_prev = np.eye(4) if init is None else np.asarray(init, dtype=np.float64)
    worst = 0.0
    for k in range(kw["num_iters"]):
        g = h[k]
        o = io.gn_step(T_prev, d["kcam"], s["points"], s["normals"], s["mask"], t["points"],
                       t["normals"], t["mask"], src_feats=sf, tgt_feats=tf,
                       channel_mode=channel_mode, **step_kw)
        assert g[N.HIST_OK] == float(o["ok"]), k
        if not o["ok"]:
            break
        assert g[N.HIST_GEOM_COUNT] == o["geom_count"], k
        assert g[N.HIST_FEAT_COUNT] == o["feat_count"], k
        A = g[N.HIST_JTJ:N.HIST_JTJ + 36].reshape(6, 6)
        b = g[N.HIST_JR:N.HIST_JR + 6]
        T = g[N.HIST_TRANSFORM:N.HIST_TRANSFORM + 16].reshape(4, 4)
        assert np.linalg.norm(A - o["JtJ"]) <= tol * np.linalg.norm(o["JtJ"]), k
        assert np.linalg.norm(b - o["Jr"]) <= tol * o["Jr_scale"], k
        assert abs(g[N.HIST_R2] - o["r2"]) <= tol * o["r2"], k
        err = rel_pose(T, o["transform"])
        assert err <= tol, (k, err)
        ok_own, x_own = io.cholesky_solve6(A, b)
        assert ok_own, k
        T_own = io.se3_exp(x_own) @ T_prev
        step_err = np.abs(T - T_own).max() / np.abs(T_own).max()
        assert step_err <= step_tol, (k, step_err)
        worst = max(worst, err)
        T_prev = T
    return worst


