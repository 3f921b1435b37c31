"""The single-launch registration (the default of stb_icp_estimate) and the
launch machinery around it.

* The single cooperative launch is deterministic (bit-equal histories run to
  run) and agrees with the two-launches-per-iteration sequence within the
  1e-5 gate; both are held to the oracle iteration by iteration in
  test_gpu_icp.py.
* Frames with fewer workspace slots than the GPU has SMs run with a smaller
  grid.
* Its bounded waits: with stb_set_wait_test_limits making every grid
  barrier expect one block more than the grid has, no barrier completes,
  every wait gives up after its poll limit and the registration returns
  with STB_ST_TIMEOUT in its status (nothing hangs, the context stays
  usable: the next call succeeds).
* The CUDA-graph cache of the multi-launch sequence: one estimator
  registering pairs A, B, A, B (same size, different buffers) through its
  cached graph gives, for each call, the direct launches' result bit for
  bit.
"""
import math

import numpy as np
import pytest
import torch

from _helpers import ANGLE_20, rel_pose, synthetic_pair

pytestmark = pytest.mark.gpu

GEOM = dict(num_iters=10, geom_weight=1.0, feat_weight=0.0, distance_threshold=0.1,
            normals_angle_thresh=ANGLE_20)


def _dev(d, cuda):
    s, t = d["src"], d["tgt"]
    f = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)  # noqa: E731
    return dict(kcam=f(d["kcam"]), sp=f(s["points"]).view(-1, 3), sn=f(s["normals"]).view(-1, 3),
                sm=f(s["mask"]).view(-1), tp=f(t["points"]), tn=f(t["normals"]),
                tm=f(t["mask"]))


def _run(icp, x, transform=None):
    return icp.estimate(x["kcam"], x["sp"], x["sn"], x["sm"], target_points=x["tp"],
                        target_mask=x["tm"], target_normals=x["tn"], transform=transform)


@pytest.fixture(scope="module")
def pair0(cuda):
    return _dev(synthetic_pair(0, feature_channels=0), cuda)


def test_single_launch_is_deterministic(cuda, pair0):
    from slamtb_gb300.registration.icp import ICPOdometry
    outs = []
    for _ in range(3):
        icp = ICPOdometry(record_history=True, **GEOM)
        res = _run(icp, pair0)
        outs.append((res.transform.numpy().copy(), icp.last_history.numpy().copy(),
                     res.information.numpy().copy()))
    for T, H, I in outs[1:]:
        np.testing.assert_array_equal(T, outs[0][0])
        np.testing.assert_array_equal(H, outs[0][1])
        np.testing.assert_array_equal(I, outs[0][2])


def test_single_and_multi_launch_agree(cuda, pair0):
    from slamtb_gb300.registration.icp import ICPOdometry
    a = ICPOdometry(record_history=True, **GEOM)
    b = ICPOdometry(record_history=True, launch="multi", **GEOM)
    ra, rb = _run(a, pair0), _run(b, pair0)
    assert rel_pose(ra.transform.numpy(), rb.transform.numpy()) <= 1e-5
    assert ra.match_ratio == pytest.approx(rb.match_ratio, rel=1e-4)
    np.testing.assert_allclose(ra.information.double().numpy(), rb.information.double().numpy(),
                               rtol=1e-5, atol=1e-5 * float(rb.information.abs().max()))


@pytest.mark.parametrize("w,h", [(64, 48), (40, 30)])
def test_small_frames_use_a_smaller_grid(cuda, w, h):
    """64x48 has 3 workspace slots and 40x30 two: the grid shrinks to them;
    the result equals the multi-launch sequence's within the gate."""
    from slamtb_gb300.registration.icp import ICPOdometry
    x = _dev(synthetic_pair(6, width=w, height=h, feature_channels=0), cuda)
    kw = dict(GEOM, num_iters=5)
    ra = _run(ICPOdometry(**kw), x)
    rb = _run(ICPOdometry(launch="multi", **kw), x)
    assert (ra.transform is None) == (rb.transform is None)
    if ra.transform is not None:
        assert rel_pose(ra.transform.numpy(), rb.transform.numpy()) <= 1e-5


def test_bounded_waits_give_up_with_a_timeout_status(cuda, pair0):
    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration.icp import ICPOdometry
    lib = N.lib()
    icp = ICPOdometry(**GEOM)
    try:
        N.check(lib.stb_set_wait_test_limits(1 << 12, 1))
        res, _, _, _ = icp.launch(pair0["kcam"], pair0["sp"], pair0["sn"], pair0["sm"],
                                  target_points=pair0["tp"], target_mask=pair0["tm"],
                                  target_normals=pair0["tn"])
        out = res.cpu().numpy()
    finally:
        N.check(lib.stb_set_wait_test_limits(0, 0))
    status = int(out[N.RES_STATUS])
    assert status & N.ST_TIMEOUT
    assert out[N.RES_ITERS] == 0
    # the context is usable and the limits are back to their defaults
    res = _run(icp, pair0)
    assert res.transform is not None and res.match_ratio > 0


def test_graph_cache_serves_different_pairs(cuda):
    """One estimator, one cached graph, pairs A, B, A, B of the same size in
    different buffers: each result equals the direct launches' bit for bit."""
    from slamtb_gb300.registration.icp import ICPOdometry
    pa = _dev(synthetic_pair(31, width=320, height=240, feature_channels=0), cuda)
    pb = _dev(synthetic_pair(32, width=320, height=240, feature_channels=0), cuda)
    kw = dict(GEOM, num_iters=6)
    direct = {}
    for name, x in (("A", pa), ("B", pb)):
        icp = ICPOdometry(launch="multi", use_graph=False, record_history=True, **kw)
        res = _run(icp, x)
        direct[name] = (res.transform.numpy().copy(), icp.last_history.numpy().copy())
    assert not np.array_equal(direct["A"][0], direct["B"][0])
    icp = ICPOdometry(launch="multi", use_graph=True, record_history=True, **kw)
    for name, x in (("A", pa), ("B", pb), ("A", pa), ("B", pb)):
        res = _run(icp, x)
        np.testing.assert_array_equal(res.transform.numpy(), direct[name][0], err_msg=name)
        np.testing.assert_array_equal(icp.last_history.numpy(), direct[name][1], err_msg=name)


@pytest.mark.parametrize("launch,use_graph", [("single", False), ("multi", False),
                                               ("multi", True)])
def test_profile_hook_times_every_launch(cuda, pair0, launch, use_graph):
    """stb_profile_* brackets the launches of a call with CUDA events: one
    single-launch registration, or 10 associations + 10 reductions + the
    final association, information pass and set-up of the multi-launch
    sequence (direct or replayed as a graph)."""
    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration.icp import ICPOdometry
    icp = ICPOdometry(launch=launch, use_graph=use_graph, **GEOM)
    N.profile_enable(True)
    try:
        for _ in range(2):
            _run(icp, pair0)
        torch.cuda.synchronize(cuda)
        prof = N.profile_read()
    finally:
        N.profile_enable(False)
    counts = {k: c for k, (_, c) in prof.items()}
    if launch == "single":
        assert counts == {"association": 0, "reduction+solve": 0, "information": 0, "setup": 0,
                          "registration": 1}
    else:
        assert counts == {"association": 11, "reduction+solve": 10, "information": 1,
                          "setup": 1, "registration": 0}
    assert all(ms > 0 for ms, c in prof.values() if c)
