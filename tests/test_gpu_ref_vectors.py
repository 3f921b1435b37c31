"""The GPU kernels against the reference's own outputs.

``tests/golden/ref_vectors.npz`` holds SHA-256 digests of what the
reference's code (built by ``oracle/build_ref.py``) computes on its sample2
frames: correspondence maps, per-point geometric, feature and information
partials, match counts.  The ``_cslamtb``-compatible kernels must reproduce
every digest, and the fused registration's association (read back with
``stb_icp_correspondences`` after a zero-iteration registration, which
associates once at the initial pose) must reproduce the map's.
"""
import numpy as np
import pytest
import torch

from oracle import icp_oracle as io
import _helpers  # noqa: F401  (puts tests/golden on the path)
import ref_vectors as rv

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _compat_outputs(cuda, case, d):
    from slamtb_gb300._cslamtb import CorrespondenceMap, ICPJacobian
    s, t = d["src"], d["tgt"]
    n = s["mask"].size
    rt = _t(io.pose_rt32(case["pose"](d)), cuda)
    sp, sm = _t(s["points"], cuda).view(-1, 3), _t(s["mask"], cuda).view(-1)
    tp, tn, tm = _t(t["points"], cuda), _t(t["normals"], cuda), _t(t["mask"], cuda)
    kcam = _t(d["kcam"], cuda)
    mm = torch.full(t["mask"].shape, io.CORRESP_EMPTY, dtype=torch.int64, device=cuda)
    CorrespondenceMap.compute_correspondence_map(sp, _t(s["normals"], cuda).view(-1, 3), sm, rt,
                                                 tp, tn, tm, kcam, mm, case["dist"],
                                                 case["angle"])
    z = lambda *shape: torch.full(shape, 7.0, device=cuda)  # noqa: E731
    geom = [z(n, 6, 6), z(n, 6), z(n)]
    gc = ICPJacobian.estimate_geometric(sp, sm, rt, tp, tn, kcam, mm, *geom)
    feat = [z(n, 6, 6), z(n, 6), z(n)]
    fc = ICPJacobian.estimate_feature(sp, _t(d["src_feats"], cuda), sm, rt,
                                      _t(d["tgt_feats"], cuda), kcam, mm,
                                      rv.FEAT_RESIDUAL_THRESH, *feat)
    info = z(n, 6, 6)
    ICPJacobian.get_information_matrix(sp, sm, rt, tp, kcam, mm, info)
    torch.cuda.synchronize(cuda)
    return rv.pack(mm.cpu().numpy(), [x.cpu().numpy() for x in geom] + [gc],
                   [x.cpu().numpy() for x in feat] + [fc], info.cpu().numpy())


@pytest.mark.parametrize("case", rv.CASES, ids=[c["name"] for c in rv.CASES])
def test_compat_kernels_reproduce_reference_vectors(cuda, case):
    golden = rv.load()
    d = rv.case_pair(case)
    for key, value in _compat_outputs(cuda, case, d).items():
        assert golden[f"{case['name']}/{key}"] == value, (case["name"], key)


@pytest.mark.parametrize("case", rv.CASES, ids=[c["name"] for c in rv.CASES])
def test_fused_association_reproduces_reference_map(cuda, case):
    from slamtb_gb300 import _native as N
    lib = N.lib()
    d = rv.case_pair(case)
    s, t = d["src"], d["tgt"]
    h, w = t["mask"].shape
    sp = _t(s["points"], cuda).view(-1, 3)
    args = [_t(d["kcam"], cuda), sp, _t(s["normals"], cuda).view(-1, 3),
            _t(s["mask"], cuda).view(-1)]
    tgt = [_t(t["points"], cuda), _t(t["normals"], cuda), _t(t["mask"], cuda)]
    init = np.ascontiguousarray(case["pose"](d), np.float64)
    ws_bytes = lib.stb_icp_workspace_bytes(sp.size(0), h, w)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    res = torch.empty(N.RES_SIZE, dtype=torch.float64, device=cuda)
    stream = N.stream_of(cuda)
    N.check(lib.stb_icp_estimate(
        *[N.ptr(x) for x in args], sp.size(0), None, *[N.ptr(x) for x in tgt], h, w, None, 0,
        N.STB_F32, init.ctypes.data, 0, 1.0, 0.0, case["dist"], case["angle"], 2.75, 0,
        N.ptr(ws), ws_bytes, N.ptr(res), None, 0, stream))
    m = torch.empty(h, w, dtype=torch.int64, device=cuda)
    N.check(lib.stb_icp_correspondences(N.ptr(ws), h, w, 0, N.ptr(m), stream))
    torch.cuda.synchronize(cuda)
    golden = rv.load()
    assert rv.digest(m.cpu().numpy()) == golden[f"{case['name']}/map"]
