"""The allocation-free registration entry point, ``stb_icp_estimate_static``.

It serves callers that cannot allocate device memory while they track (C or
FFI hosts without a CUDA allocator, fixed-budget real-time applications);
its scratch is a fixed array inside the library instead of a caller
workspace.  Called through the C ABI, twice in a row (the array keeps the
previous call's contents, which must not leak into the next result), it
must give what ``stb_icp_estimate`` gives on the same inputs, within the
1e-5 gate of the path.  This file is collected last on purpose.
"""
import ctypes
import math

import numpy as np
import pytest
import torch

from oracle import icp_oracle as io
from _helpers import synthetic_pair

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _inputs(cuda, seed):
    d = synthetic_pair(seed, feature_channels=0)
    s, t = d["src"], d["tgt"]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)  # noqa: E731
    return dict(kcam=dev(d["kcam"]), sp=dev(s["points"]).view(-1, 3),
                sn=dev(s["normals"]).view(-1, 3), sm=dev(s["mask"]).view(-1),
                tp=dev(t["points"]), tn=dev(t["normals"]), tm=dev(t["mask"]),
                sf=dev(d["src_feats"]).view(1, -1), tf=dev(d["tgt_feats"]))


def _args(x, iters):
    from slamtb_gb300 import _native as N
    h, w = x["tm"].shape
    return [N.ptr(x["kcam"]), N.ptr(x["sp"]), N.ptr(x["sn"]), N.ptr(x["sm"]), x["sp"].size(0),
            N.ptr(x["sf"]), N.ptr(x["tp"]), N.ptr(x["tn"]), N.ptr(x["tm"]), h, w,
            N.ptr(x["tf"]), 1, N.STB_F32, None, iters, 1.0, 0.1, 0.1, math.radians(20), 2.75, 0]


def _check_close(a_res, b_res, a_hist, b_hist):
    from slamtb_gb300 import _native as N
    a, b = a_res.cpu().numpy(), b_res.cpu().numpy()
    assert a[N.RES_ITERS] == b[N.RES_ITERS] > 0
    assert a[N.RES_MATCHES] == b[N.RES_MATCHES]
    Ta = a[N.RES_TRANSFORM:N.RES_TRANSFORM + 16].reshape(4, 4)
    Tb = b[N.RES_TRANSFORM:N.RES_TRANSFORM + 16].reshape(4, 4)
    d = io.se3_log(np.linalg.inv(Tb) @ Ta)
    assert np.linalg.norm(d) <= TOL * max(np.linalg.norm(io.se3_log(Tb)), 1e-3)
    for off in (N.RES_JTJ, N.RES_INFO):
        A, B = a[off:off + 36], b[off:off + 36]
        assert np.linalg.norm(A - B) <= TOL * np.linalg.norm(B)
    assert abs(a[N.RES_RESIDUAL] - b[N.RES_RESIDUAL]) <= TOL * abs(b[N.RES_RESIDUAL])
    # fields 0..61 of a history record are written; 62..63 are padding
    ha, hb = a_hist.cpu().numpy()[:, :N.HIST_OK + 1], b_hist.cpu().numpy()[:, :N.HIST_OK + 1]
    assert np.isfinite(ha).all() and np.isfinite(hb).all()
    np.testing.assert_allclose(ha, hb, rtol=TOL, atol=TOL * np.abs(hb).max())


def test_static_entry_point_matches_workspace_entry_point(cuda):
    from slamtb_gb300 import _native as N
    lib = N.lib()
    iters = 6
    stream = N.stream_of(cuda)
    ws_bytes = lib.stb_icp_workspace_bytes(640 * 480, 480, 640)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    # two different pairs, each registered by both entry points, back to back
    for seed in (21, 22):
        x = _inputs(cuda, seed)
        ref_res = torch.empty(N.RES_SIZE, dtype=torch.float64, device=cuda)
        ref_hist = torch.empty(iters, N.HIST_SIZE, dtype=torch.float64, device=cuda)
        N.check(lib.stb_icp_estimate(*_args(x, iters), N.ptr(ws), ws_bytes, N.ptr(ref_res),
                                     N.ptr(ref_hist), 0, stream))
        for _ in range(2):
            res = torch.full((N.RES_SIZE,), float("nan"), dtype=torch.float64, device=cuda)
            hist = torch.full((iters, N.HIST_SIZE), float("nan"), dtype=torch.float64,
                              device=cuda)
            N.check(lib.stb_icp_estimate_static(*_args(x, iters), N.ptr(res), N.ptr(hist),
                                                stream))
            torch.cuda.synchronize(cuda)
            _check_close(res, ref_res, hist, ref_hist)


def test_static_entry_point_rejects_oversized_frames(cuda):
    from slamtb_gb300 import _native as N
    lib = N.lib()
    x = _inputs(cuda, 23)
    args = _args(x, 2)
    args[9], args[10] = 1025, 1024  # 1,049,600 target pixels > 1,048,576
    res = torch.empty(N.RES_SIZE, dtype=torch.float64, device=cuda)
    rc = lib.stb_icp_estimate_static(*args, N.ptr(res), None, N.stream_of(cuda))
    assert rc == 1
    assert b"at most 1048576 target pixels" in lib.stb_last_error()
