"""The allocation-free registration entry point, ``stb_icp_estimate_static``.

It serves callers that cannot allocate device memory while they track (C or
FFI hosts without a CUDA allocator, fixed-budget real-time applications);
its scratch is a fixed array inside the library instead of a caller
workspace.  It runs the same launch sequence as ``stb_icp_estimate``, so,
called through the C ABI twice in a row (the array keeps the previous
call's contents, which must not leak into the next result), it must give
exactly what ``stb_icp_estimate`` gives on the same inputs: at 640x480 and
at its documented limit of 1,048,576 target pixels (1024x1024).  One pixel
row past the limit is refused.  This file is collected last on purpose.
"""
import math

import numpy as np
import pytest
import torch

from _helpers import synthetic_pair

pytestmark = pytest.mark.gpu


def _inputs(cuda, seed, width=640, height=480):
    d = synthetic_pair(seed, width=width, height=height, feature_channels=0)
    s, t = d["src"], d["tgt"]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)  # noqa: E731
    return dict(kcam=dev(d["kcam"]), sp=dev(s["points"]).view(-1, 3),
                sn=dev(s["normals"]).view(-1, 3), sm=dev(s["mask"]).view(-1),
                tp=dev(t["points"]), tn=dev(t["normals"]), tm=dev(t["mask"]),
                sf=dev(d["src_feats"]).view(1, -1), tf=dev(d["tgt_feats"]))


def _args(x, iters, opts=0):
    from slamtb_gb300 import _native as N
    h, w = x["tm"].shape
    return [N.ptr(x["kcam"]), N.ptr(x["sp"]), N.ptr(x["sn"]), N.ptr(x["sm"]), x["sp"].size(0),
            N.ptr(x["sf"]), N.ptr(x["tp"]), N.ptr(x["tn"]), N.ptr(x["tm"]), h, w,
            N.ptr(x["tf"]), 1, N.STB_F32, None, iters, 1.0, 0.1, 0.1, math.radians(20), 2.75,
            opts]


def _check_equal(a_res, b_res, a_hist, b_hist):
    from slamtb_gb300 import _native as N
    a, b = a_res.cpu().numpy(), b_res.cpu().numpy()
    assert a[N.RES_ITERS] == b[N.RES_ITERS] > 0
    # fields 0..91 of the result block are written; the rest is padding
    np.testing.assert_array_equal(a[:N.RES_STATUS + 1], b[:N.RES_STATUS + 1])
    # fields 0..61 of a history record are written; 62..63 are padding
    ha, hb = a_hist.cpu().numpy()[:, :N.HIST_OK + 1], b_hist.cpu().numpy()[:, :N.HIST_OK + 1]
    assert np.isfinite(ha).all()
    np.testing.assert_array_equal(ha, hb)


@pytest.mark.parametrize("width,height,launch", [(640, 480, "single"), (640, 480, "multi"),
                                                 (1024, 1024, "single")])
def test_static_entry_point_matches_workspace_entry_point(cuda, width, height, launch):
    """Both launch modes (the default single launch and STB_OPT_MULTI_LAUNCH)."""
    from slamtb_gb300 import _native as N
    lib = N.lib()
    opts = N.OPT_MULTI_LAUNCH if launch == "multi" else 0
    iters = 6
    stream = N.stream_of(cuda)
    ws_bytes = lib.stb_icp_workspace_bytes(width * height, height, width)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    # two different pairs, each registered by both entry points, back to back
    for seed in (21, 22):
        x = _inputs(cuda, seed, width, height)
        ref_res = torch.empty(N.RES_SIZE, dtype=torch.float64, device=cuda)
        ref_hist = torch.empty(iters, N.HIST_SIZE, dtype=torch.float64, device=cuda)
        N.check(lib.stb_icp_estimate(*_args(x, iters, opts), N.ptr(ws), ws_bytes, N.ptr(ref_res),
                                     N.ptr(ref_hist), 0, stream))
        for _ in range(2):
            res = torch.full((N.RES_SIZE,), float("nan"), dtype=torch.float64, device=cuda)
            hist = torch.full((iters, N.HIST_SIZE), float("nan"), dtype=torch.float64,
                              device=cuda)
            N.check(lib.stb_icp_estimate_static(*_args(x, iters, opts), N.ptr(res), N.ptr(hist),
                                                stream))
            torch.cuda.synchronize(cuda)
            _check_equal(res, ref_res, hist, ref_hist)


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
