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
