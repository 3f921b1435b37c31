"""_cslamtb-compatible entry points on the GPU against the float32 oracle:
correspondence maps, per-point partials and match counts must be bit-exact."""
import math

import numpy as np
import pytest
import torch

from oracle import icp_oracle as io
from _helpers import synthetic_pair, sample2_pair

pytestmark = pytest.mark.gpu

POSES = [np.eye(4), io.se3_exp([0.01, -0.02, 0.015, 0.02, -0.01, 0.03])]


@pytest.fixture(scope="module")
def pair():
    return synthetic_pair(0, feature_channels=0)


def _t(x, dev, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    return t if dtype is None else t.to(dtype)


def _gpu_map(cuda, d, pose, dist, angle, src_mask=None):
    from slamtb_gb300._cslamtb import CorrespondenceMap
    s, t = d["src"], d["tgt"]
    h, w = t["mask"].shape
    m = torch.full((h, w), io.CORRESP_EMPTY, dtype=torch.int64, device=cuda)
    CorrespondenceMap.compute_correspondence_map(
        _t(s["points"], cuda).view(-1, 3), _t(s["normals"], cuda).view(-1, 3),
        _t(s["mask"] if src_mask is None else src_mask, cuda).view(-1),
        _t(pose, cuda, torch.float32), _t(t["points"], cuda), _t(t["normals"], cuda),
        _t(t["mask"], cuda), _t(d["kcam"], cuda), m, dist, angle)
    return m


@pytest.mark.parametrize("pose_i", [0, 1])
@pytest.mark.parametrize("dist,angle", [(0.1, math.radians(20)), (0.5, math.pi / 4), (1.5, math.pi)])
def test_correspondence_map_bit_exact(cuda, pair, pose_i, dist, angle):
    d = pair
    pose = POSES[pose_i]
    m = _gpu_map(cuda, d, pose, dist, angle).cpu().numpy()
    s, t = d["src"], d["tgt"]
    a = io.associate32(s["points"], s["normals"], s["mask"], io.pose_rt32(pose), t["points"],
                       t["normals"], t["mask"], d["kcam"], dist, angle)
    assert a.count > 1000
    np.testing.assert_array_equal(m, a.ref_map)


def test_correspondence_map_mask_disabled(cuda, pair):
    """A length-1 source mask disables masking (correspondence_map.cu:40-41)."""
    d = pair
    m = _gpu_map(cuda, d, POSES[1], 0.1, math.radians(20), src_mask=np.ones(1, bool))
    s, t = d["src"], d["tgt"]
    a = io.associate32(s["points"], s["normals"], np.ones(1, bool), io.pose_rt32(POSES[1]),
                       t["points"], t["normals"], t["mask"], d["kcam"], 0.1, math.radians(20))
    np.testing.assert_array_equal(m.cpu().numpy(), a.ref_map)


def test_sample2_correspondence_map_bit_exact(cuda):
    """test_correspondence_map.py:14-38 (frames 0 and 13, CorrespondenceMap(10, 10)
    at identity), checked on the whole map, not only the distance bits."""
    d = sample2_pair(0, 13)
    m = _gpu_map(cuda, d, np.eye(4), 10, 10).cpu().numpy()
    s, t = d["src"], d["tgt"]
    a = io.associate32(s["points"], s["normals"], s["mask"], io.pose_rt32(np.eye(4)),
                       t["points"], t["normals"], t["mask"], d["kcam"], 10, 10)
    np.testing.assert_array_equal(m, a.ref_map)


def _partials(cuda, n):
    return (torch.full((n, 6, 6), 7.0, device=cuda), torch.full((n, 6), 7.0, device=cuda),
            torch.full((n,), 7.0, device=cuda))


@pytest.mark.parametrize("pose_i", [0, 1])
def test_geometric_partials_bit_exact(cuda, pair, pose_i):
    from slamtb_gb300._cslamtb import ICPJacobian
    d = pair
    pose = POSES[pose_i]
    m = _gpu_map(cuda, d, pose, 0.1, math.radians(20))
    s, t = d["src"], d["tgt"]
    n = s["mask"].size
    JtJ, Jr, r2 = _partials(cuda, n)
    cnt = ICPJacobian.estimate_geometric(
        _t(s["points"], cuda).view(-1, 3), _t(s["mask"], cuda).view(-1),
        _t(pose, cuda, torch.float32), _t(t["points"], cuda), _t(t["normals"], cuda),
        _t(d["kcam"], cuda), m, JtJ, Jr, r2)
    oJtJ, oJr, or2, ocnt = io.geometric_partials32(s["points"], s["mask"], io.pose_rt32(pose),
                                                   t["points"], t["normals"], d["kcam"],
                                                   m.cpu().numpy())
    assert cnt == ocnt > 1000
    np.testing.assert_array_equal(JtJ.cpu().numpy(), oJtJ)
    np.testing.assert_array_equal(Jr.cpu().numpy(), oJr)
    np.testing.assert_array_equal(r2.cpu().numpy(), or2)


@pytest.mark.parametrize("channels,dtype,so3", [(1, torch.float32, False), (3, torch.float32, False),
                                                (3, torch.bfloat16, False), (2, torch.float32, True)])
def test_feature_partials_bit_exact(cuda, pair, channels, dtype, so3):
    from slamtb_gb300._cslamtb import ICPJacobian
    d = pair
    pose = POSES[1]
    m = _gpu_map(cuda, d, pose, 0.1, math.radians(20))
    s, t = d["src"], d["tgt"]
    h, w = t["mask"].shape
    n = h * w
    rng = np.random.default_rng(7)
    tf = np.concatenate([d["tgt_feats"], rng.random((channels - 1, h, w), np.float32)])
    sf = np.concatenate([d["src_feats"], rng.random((channels - 1, h, w), np.float32)])
    tft = _t(tf, cuda, dtype)
    sft = _t(sf, cuda, dtype).view(channels, -1)
    tf32 = tft.float().cpu().numpy()
    sf32 = sft.float().cpu().numpy()
    JtJ, Jr, r2 = _partials(cuda, n)
    fn = ICPJacobian.estimate_feature_so3 if so3 else ICPJacobian.estimate_feature
    thresh = 0.35
    cnt = fn(_t(s["points"], cuda).view(-1, 3), sft, _t(s["mask"], cuda).view(-1),
             _t(pose, cuda, torch.float32), tft, _t(d["kcam"], cuda), m, thresh, JtJ, Jr, r2)
    oJtJ, oJr, or2, ocnt, passed = io.feature_partials32(
        s["points"], sf32, s["mask"], io.pose_rt32(pose), tf32, d["kcam"], m.cpu().numpy(), thresh)
    assert cnt == ocnt > 100
    if so3:
        # SO3ICPJacobian: J = Tp x g in the leading 3x3 block
        rot_jtj = oJtJ[:, 3:, 3:]
        rot_jr = oJr[:, 3:]
        oJtJ = np.zeros_like(oJtJ)
        oJr = np.zeros_like(oJr)
        oJtJ[:, :3, :3] = rot_jtj
        oJr[:, :3] = rot_jr
    np.testing.assert_array_equal(JtJ.cpu().numpy(), oJtJ)
    np.testing.assert_array_equal(Jr.cpu().numpy(), oJr)
    np.testing.assert_array_equal(r2.cpu().numpy(), or2)


def test_information_partials_bit_exact(cuda, pair):
    from slamtb_gb300._cslamtb import ICPJacobian
    d = pair
    pose = POSES[1]
    m = _gpu_map(cuda, d, pose, 0.1, math.radians(20))
    s, t = d["src"], d["tgt"]
    n = s["mask"].size
    G = torch.full((n, 6, 6), 3.0, device=cuda)
    ICPJacobian.get_information_matrix(
        _t(s["points"], cuda).view(-1, 3), _t(s["mask"], cuda).view(-1),
        _t(pose, cuda, torch.float32), _t(t["points"], cuda), _t(d["kcam"], cuda), m, G)
    o = io.information_partials32(s["points"], s["mask"], io.pose_rt32(pose), t["points"],
                                  d["kcam"], m.cpu().numpy())
    np.testing.assert_array_equal(G.cpu().numpy(), o)


def test_cpu_tensor_is_rejected(cuda, pair):
    from slamtb_gb300._cslamtb import CorrespondenceMap
    d = pair
    s, t = d["src"], d["tgt"]
    h, w = t["mask"].shape
    m = torch.full((h, w), io.CORRESP_EMPTY, dtype=torch.int64, device=cuda)
    with pytest.raises(RuntimeError, match="Expected a gpu tensor"):
        CorrespondenceMap.compute_correspondence_map(
            torch.from_numpy(s["points"]).view(-1, 3), _t(s["normals"], cuda).view(-1, 3),
            _t(s["mask"], cuda).view(-1), _t(np.eye(4), cuda, torch.float32),
            _t(t["points"], cuda), _t(t["normals"], cuda), _t(t["mask"], cuda),
            _t(d["kcam"], cuda), m, 0.1, 0.3)
