"""Writes ``ref_vectors.npz``: the reference's own outputs on the cases of
``ref_vectors.py``, from the build of ``oracle/build_ref.py`` (run where the
reference tree is available, its root in $SLAMTB_REFERENCE):

    SLAMTB_REFERENCE=<reference root> python tests/golden/make_ref_vectors.py
"""
import pathlib
import sys

import numpy as np
import torch

HERE = pathlib.Path(__file__).resolve().parent
for p in (HERE, HERE.parent, HERE.parent.parent, HERE.parent.parent / "fusion-toolbox_gb300"):
    sys.path.insert(0, str(p))

import ref_vectors as rv  # noqa: E402
from oracle import build_ref  # noqa: E402
from oracle import icp_oracle as io  # noqa: E402


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a))


def reference_outputs(ref, case, d):
    s, t = d["src"], d["tgt"]
    n = s["mask"].size
    rt = _t(io.pose_rt32(case["pose"](d)))
    sp, sm = _t(s["points"]).view(-1, 3), _t(s["mask"]).view(-1)
    mm = torch.full(t["mask"].shape, io.CORRESP_EMPTY, dtype=torch.int64)
    ref.compute_correspondence_map(sp, _t(s["normals"]).view(-1, 3), sm, rt, _t(t["points"]),
                                   _t(t["normals"]), _t(t["mask"]), _t(d["kcam"]), mm,
                                   case["dist"], case["angle"])
    geom = [torch.zeros(n, 6, 6), torch.zeros(n, 6), torch.zeros(n)]
    gc = ref.estimate_geometric(sp, sm, rt, _t(t["points"]), _t(t["normals"]), _t(d["kcam"]),
                                mm, *geom)
    feat = [torch.zeros(n, 6, 6), torch.zeros(n, 6), torch.zeros(n)]
    fc = ref.estimate_feature(sp, _t(d["src_feats"]), sm, rt, _t(d["tgt_feats"]),
                              _t(d["kcam"]), mm, rv.FEAT_RESIDUAL_THRESH, *feat)
    info = torch.zeros(n, 6, 6)
    ref.get_information_matrix(sp, sm, rt, _t(t["points"]), _t(d["kcam"]), mm, info)
    return rv.pack(mm.numpy(), [x.numpy() for x in geom] + [gc],
                   [x.numpy() for x in feat] + [fc], info.numpy())


def main():
    ref = build_ref.load()
    if ref is None:
        sys.exit("no reference build: set SLAMTB_REFERENCE to the reference root")
    out = {}
    for case in rv.CASES:
        d = rv.case_pair(case)
        for key, value in reference_outputs(ref, case, d).items():
            out[f"{case['name']}/{key}"] = np.array(value)
    np.savez_compressed(rv.PATH, **out)
    print("wrote", rv.PATH, len(out), "vectors")


if __name__ == "__main__":
    main()
