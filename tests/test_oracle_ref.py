"""The oracle against the reference's own code (CPU, no GPU).

``oracle/build_ref.py`` compiles the reference's registration sources
(``src/correspondence_map.cu``, ``src/icp_jacobian_geometric.cu``,
``src/icp_jacobian_feature.cu``, ``src/merge_map.cpp``) with the project's
Eigen subset into ``oracle/_ref/slamtb_ref``; its CPU path runs here on the
same float32 inputs as the oracle.  Correspondence maps (source index and
distance bits), per-point partials of the geometric, feature and information
kernels and match counts must be equal bit for bit.  The reference's CPU
loops run sequentially in that build, so its z-buffer keeps the first (the
smallest) source index among equal distances, the oracle's rule.

``tests/golden/ref_vectors.npz`` holds digests of the reference's outputs on
the sample2 frames (written by ``tests/golden/make_ref_vectors.py`` from this
build); the oracle is checked against them even where the reference build is
absent, and the GPU kernels are checked against them in
``test_gpu_ref_vectors.py``.
"""
import math

import numpy as np
import pytest
import torch

from oracle import build_ref
from oracle import icp_oracle as io
from _helpers import sample2_pair, synthetic_pair
import ref_vectors as rv

ANGLE_20 = math.radians(20)


@pytest.fixture(scope="module")
def ref():
    mod = build_ref.load()
    if mod is None:
        pytest.skip("the reference build (oracle/_ref) is absent and no reference tree is "
                    "given in $SLAMTB_REFERENCE")
    return mod


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a))


def _ref_map(ref, d, pose, dist, angle, src_mask=None):
    s, t = d["src"], d["tgt"]
    mm = torch.full(t["mask"].shape, io.CORRESP_EMPTY, dtype=torch.int64)
    ref.compute_correspondence_map(
        _t(s["points"]).view(-1, 3), _t(s["normals"]).view(-1, 3),
        _t(s["mask"] if src_mask is None else src_mask).view(-1),
        _t(io.pose_rt32(pose)), _t(t["points"]), _t(t["normals"]), _t(t["mask"]),
        _t(d["kcam"]), mm, dist, angle)
    return mm.numpy()


def _oracle_map(d, pose, dist, angle, src_mask=None):
    s, t = d["src"], d["tgt"]
    return io.associate32(s["points"], s["normals"],
                          s["mask"] if src_mask is None else src_mask, io.pose_rt32(pose),
                          t["points"], t["normals"], t["mask"], d["kcam"], dist, angle).ref_map


POSE_B = io.se3_exp([0.01, -0.02, 0.015, 0.02, -0.01, 0.03])


@pytest.fixture(scope="module")
def pair0():
    return synthetic_pair(0, feature_channels=3)


@pytest.mark.parametrize("pose", [np.eye(4), POSE_B], ids=["identity", "moved"])
@pytest.mark.parametrize("dist,angle", [(0.1, ANGLE_20), (0.5, math.pi / 4), (1.5, math.pi),
                                        (10.0, 10.0)])
def test_correspondence_map_equals_reference(ref, pair0, pose, dist, angle):
    m = _ref_map(ref, pair0, pose, dist, angle)
    assert (m != io.CORRESP_EMPTY).sum() > 1000
    np.testing.assert_array_equal(_oracle_map(pair0, pose, dist, angle), m)


def test_correspondence_map_mask_disabled_equals_reference(ref, pair0):
    one = np.ones(1, bool)
    np.testing.assert_array_equal(_oracle_map(pair0, POSE_B, 0.1, ANGLE_20, one),
                                  _ref_map(ref, pair0, POSE_B, 0.1, ANGLE_20, one))


def test_correspondence_map_ties_and_nan_equal_reference(ref, pair0):
    """Duplicated source columns (equal distances: the reference's
    sequential CPU z-buffer keeps the first writer, the smaller index) and
    NaN source points."""
    s = {k: np.array(v, copy=True) for k, v in pair0["src"].items()}
    for key in ("points", "normals", "mask"):
        s[key][:, 1::2] = s[key][:, 0::2]
    s["points"][100:140] = np.nan
    s["mask"][100:140] = True
    d = dict(pair0, src=s)
    m = _ref_map(ref, d, POSE_B, 0.1, ANGLE_20)
    np.testing.assert_array_equal(_oracle_map(d, POSE_B, 0.1, ANGLE_20), m)
    win = (m[m != io.CORRESP_EMPTY] >> 32)
    assert win.size > 1000 and (win % 2 == 0).all()


def _ref_geometric(ref, d, pose, ref_map):
    s, t = d["src"], d["tgt"]
    n = s["mask"].size
    JtJ, Jr, r2 = torch.zeros(n, 6, 6), torch.zeros(n, 6), torch.zeros(n)
    cnt = ref.estimate_geometric(_t(s["points"]).view(-1, 3), _t(s["mask"]).view(-1),
                                 _t(io.pose_rt32(pose)), _t(t["points"]), _t(t["normals"]),
                                 _t(d["kcam"]), _t(ref_map), JtJ, Jr, r2)
    return JtJ.numpy(), Jr.numpy(), r2.numpy(), cnt


@pytest.mark.parametrize("pose", [np.eye(4), POSE_B], ids=["identity", "moved"])
def test_geometric_and_information_partials_equal_reference(ref, pair0, pose):
    s, t = pair0["src"], pair0["tgt"]
    m = _ref_map(ref, pair0, pose, 0.1, ANGLE_20)
    rj, rr, rs, rc = _ref_geometric(ref, pair0, pose, m)
    oj, orr, os_, oc = io.geometric_partials32(s["points"], s["mask"], io.pose_rt32(pose),
                                               t["points"], t["normals"], pair0["kcam"], m)
    assert rc == oc > 1000
    np.testing.assert_array_equal(oj, rj)
    np.testing.assert_array_equal(orr, rr)
    np.testing.assert_array_equal(os_, rs)
    n = s["mask"].size
    gtg = torch.zeros(n, 6, 6)
    ref.get_information_matrix(_t(s["points"]).view(-1, 3), _t(s["mask"]).view(-1),
                               _t(io.pose_rt32(pose)), _t(t["points"]), _t(pair0["kcam"]),
                               _t(m), gtg)
    np.testing.assert_array_equal(
        io.information_partials32(s["points"], s["mask"], io.pose_rt32(pose), t["points"],
                                  pair0["kcam"], m), gtg.numpy())


@pytest.mark.parametrize("channels", [1, 3])
@pytest.mark.parametrize("thresh", [2.75, 0.05])
def test_feature_partials_equal_reference(ref, pair0, channels, thresh):
    """FeatureJacobianKernel, the last-channel quirk included (only the last
    channel's J and J r survive with several channels)."""
    s, t = pair0["src"], pair0["tgt"]
    sf = np.ascontiguousarray(pair0["src_feats"][:channels]).reshape(channels, -1)
    tf = np.ascontiguousarray(pair0["tgt_feats"][:channels])
    m = _ref_map(ref, pair0, POSE_B, 0.1, ANGLE_20)
    n = s["mask"].size
    JtJ, Jr, r2 = torch.zeros(n, 6, 6), torch.zeros(n, 6), torch.zeros(n)
    cnt = ref.estimate_feature(_t(s["points"]).view(-1, 3), _t(sf), _t(s["mask"]).view(-1),
                               _t(io.pose_rt32(POSE_B)), _t(tf), _t(pair0["kcam"]), _t(m),
                               thresh, JtJ, Jr, r2)
    oj, orr, os_, oc, _ = io.feature_partials32(s["points"], sf, s["mask"],
                                                io.pose_rt32(POSE_B), tf, pair0["kcam"], m,
                                                thresh)
    assert cnt == oc > 100
    np.testing.assert_array_equal(oj, JtJ.numpy())
    np.testing.assert_array_equal(orr, Jr.numpy())
    np.testing.assert_array_equal(os_, r2.numpy())


def test_sample2_pairs_equal_reference(ref):
    """The reference's own test frames: 0 -> 3 at identity and at the
    float32 ground truth, and 0 / 13 with CorrespondenceMap(10, 10)
    (slamtb/registration/_test/test_correspondence_map.py:14-38)."""
    for case in rv.CASES:
        d = rv.case_pair(case)
        m = _ref_map(ref, d, case["pose"](d), case["dist"], case["angle"])
        np.testing.assert_array_equal(
            _oracle_map(d, case["pose"](d), case["dist"], case["angle"]), m,
            err_msg=case["name"])


def test_oracle_equals_committed_reference_vectors():
    """Digests of the reference's outputs (tests/golden/ref_vectors.npz)
    against the oracle's on the same inputs: no reference build needed."""
    golden = rv.load()
    for case in rv.CASES:
        d = rv.case_pair(case)
        out = rv.oracle_outputs(case, d)
        for key, value in out.items():
            assert golden[f"{case['name']}/{key}"] == value, (case["name"], key)


# ---------------------------------------------------------------------------
# frame preparation: src/normals.cu, src/downsample.cu, src/erode_mask.cu,
# src/bilateral_depth_filter.cu
# ---------------------------------------------------------------------------

def _frames():
    """Two prepared frames: sample2 frame 3 and the synthetic 640x480 one."""
    from oracle import frame_prep as fp
    from make_golden import load_sample2
    raw = load_sample2()[3]
    depth = raw["depth"].astype(np.float32) * np.float32(raw["depth_scale"])
    s2 = fp.FramePointCloud.from_depth(depth, raw["kcam"])
    syn = synthetic_pair(5, feature_channels=3)
    return [("sample2", s2, None), ("synthetic", syn["src_fpcl"], syn["src_feats"])]


def test_frame_preparation_equals_reference(ref):
    from oracle import frame_prep as fp
    for name, f, feats in _frames():
        pts, mask = f.points, f.mask
        h, w = mask.shape
        # erosion of the raw mask (depth > 0)
        raw_mask = pts[..., 2] > 0
        out = torch.zeros(h, w, dtype=torch.bool)
        ref.erode_mask(_t(raw_mask), out)
        np.testing.assert_array_equal(fp.erode_mask(raw_mask), out.numpy(), err_msg=name)
        # central-difference normals
        nrm = torch.zeros(h, w, 3)
        ref.estimate_normals_central_differences(_t(pts), _t(mask), nrm)
        np.testing.assert_array_equal(fp.estimate_normals(pts, mask), nrm.numpy(),
                                      err_msg=name)
        # one pyramid step at scale 0.5
        dh, dw = int(h * 0.5), int(w * 0.5)
        dxyz = torch.zeros(dh, dw, 3)
        ref.downsample_xyz_nearest(_t(pts), _t(mask), 0.5, dxyz, True)
        np.testing.assert_array_equal(fp.downsample_xyz_nearest(pts, mask, 0.5), dxyz.numpy(),
                                      err_msg=name)
        dmask = torch.zeros(dh, dw, dtype=torch.bool)
        ref.downsample_mask(_t(mask), 0.5, dmask)
        np.testing.assert_array_equal(fp.downsample_mask(mask, 0.5), dmask.numpy(),
                                      err_msg=name)
        if feats is not None:
            dfeat = torch.zeros(feats.shape[0], dh, dw)
            ref.downsample_features(_t(feats), 0.5, dfeat)
            np.testing.assert_array_equal(fp.downsample_features(feats, 0.5), dfeat.numpy(),
                                          err_msg=name)


def test_bilateral_filter_equals_reference(ref):
    """On the depth frame of the reference's processing tests
    (slamtb/_test/test_processing.py:24-45): float32 depth within 2e-6
    relative and int32 depth within one unit, with more than 99.9 %
    identical (numpy's and the C library's float32 exp may differ by an
    ulp)."""
    from oracle import frame_prep as fp
    from make_golden import load_frame_depth
    depth = load_frame_depth()
    mask = depth > 0
    for dtype in (np.float32, np.int32):  # the reference dispatches no uint16
        d = depth.astype(dtype)
        out = torch.zeros(d.shape, dtype=torch.from_numpy(d).dtype)
        # (input, mask, result, filter_width, sigma_color, sigma_space,
        # depth_scale): the definition's order, src/bilateral_depth_filter.cu:73-75
        ref.bilateral_depth_filter(_t(d), _t(mask), out, 6, 29.9999880000072, 4.50000000225,
                                   1.0)
        mine = fp.bilateral_depth_filter(d, mask, 6, 29.9999880000072, 4.50000000225, 1.0)
        r = out.numpy()
        if dtype == np.float32:
            np.testing.assert_allclose(mine, r, rtol=2e-6, atol=0)
        else:
            diff = np.abs(mine.astype(np.int64) - r.astype(np.int64))
            assert diff.max() <= 1 and (diff == 0).mean() > 0.999
