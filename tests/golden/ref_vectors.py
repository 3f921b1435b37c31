"""Known-answer vectors from the reference's own code: cases, digests and
loader of ``ref_vectors.npz`` (written by ``make_ref_vectors.py`` from the
reference build of ``oracle/build_ref.py``).

Every case is a pair of the reference's sample2 frames (``sample2.npz``),
prepared by the oracle's restatement of FramePointCloud, so the inputs are
the same on any machine.  The feature term reads one float32 channel made
from each frame's raw depth, ``(depth mod 1021) / 1021``.  The vectors are
SHA-256 digests of the reference's outputs (correspondence map, geometric,
feature and information partials) and their match counts.
"""
import hashlib
import math
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
PATH = HERE / "ref_vectors.npz"
FEAT_RESIDUAL_THRESH = 2.75


def _gt(d):
    return d["gt"]


CASES = [
    dict(name="s2_03_identity", target=0, source=3, pose=lambda d: np.eye(4), dist=0.1,
         angle=math.radians(20)),
    dict(name="s2_03_truth", target=0, source=3, pose=_gt, dist=0.1, angle=math.radians(20)),
    dict(name="s2_03_wide", target=0, source=3, pose=lambda d: np.eye(4), dist=0.5,
         angle=math.pi / 4),
    dict(name="s2_0_13", target=0, source=13, pose=lambda d: np.eye(4), dist=10.0, angle=10.0),
]


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.astype(a.dtype.newbyteorder("<")).tobytes()).hexdigest()


def case_pair(case):
    """The prepared frames of a case, with one-channel features."""
    from _helpers import sample2_pair
    from make_golden import load_sample2
    d = sample2_pair(case["target"], case["source"])
    raw = load_sample2()

    def feat(i):
        return ((raw[i]["depth"].astype(np.int32) % 1021).astype(np.float32)
                / np.float32(1021))[None]

    d["tgt_feats"] = feat(case["target"])
    d["src_feats"] = feat(case["source"]).reshape(1, -1)
    return d


def oracle_outputs(case, d):
    """The case's vectors computed by the oracle."""
    from oracle import icp_oracle as io
    s, t = d["src"], d["tgt"]
    rt = io.pose_rt32(case["pose"](d))
    m = io.associate32(s["points"], s["normals"], s["mask"], rt, t["points"], t["normals"],
                       t["mask"], d["kcam"], case["dist"], case["angle"]).ref_map
    gj, gr, gs, gc = io.geometric_partials32(s["points"], s["mask"], rt, t["points"],
                                             t["normals"], d["kcam"], m)
    fj, fr, fs, fc, _ = io.feature_partials32(s["points"], d["src_feats"], s["mask"], rt,
                                              d["tgt_feats"], d["kcam"], m,
                                              FEAT_RESIDUAL_THRESH)
    info = io.information_partials32(s["points"], s["mask"], rt, t["points"], d["kcam"], m)
    return pack(m, (gj, gr, gs, gc), (fj, fr, fs, fc), info)


def pack(ref_map, geom, feat, info):
    out = {"map": digest(np.asarray(ref_map, np.int64)),
           "map_count": str(int((np.asarray(ref_map) != 0x0fffffff7f800000).sum()))}
    for name, (j, r, s, c) in (("geom", geom), ("feat", feat)):
        out[f"{name}_JtJ"] = digest(np.asarray(j, np.float32))
        out[f"{name}_Jr"] = digest(np.asarray(r, np.float32))
        out[f"{name}_r2"] = digest(np.asarray(s, np.float32))
        out[f"{name}_count"] = str(int(c))
    out["info"] = digest(np.asarray(info, np.float32))
    return out


def load():
    z = np.load(PATH)
    return {k: str(z[k]) for k in z.files}
