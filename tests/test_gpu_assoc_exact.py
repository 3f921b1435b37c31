"""The hot-path associations, bit for bit.

The kernels that run inside ``ICPOdometry`` (``k_assoc`` of the fused loop),
``BatchRegistration`` (the association phase of the persistent kernel) and
``PointToPlaneLoss`` (``k_g_assoc``) keep their correspondences in an
epoch-tagged key map.  ``stb_icp_correspondences``,
``stb_icp_batch_correspondences`` and ``stb_icp_loss_correspondences``
decode it into the reference's correspondence-map layout (source index in
the high word, distance bits in the low word, ``0x0fffffff7f800000`` empty:
``slamtb/registration/correspondence_map.py:5``, ``src/merge_map.hpp``).
Each map must equal, bit for bit, the float32 op-by-op oracle
``io.associate32`` at the pose the kernel associated at (the float32 cast of
the GPU's FP64 pose, as ``transform.to(float32)`` in ``icp.py:53,61``).

A registration of k iterations associates one last time at its final pose
(the information pass, ``icp.py:258-261``), so running k = 0, 1, ..., n
iterations exposes the association at every iteration's pose.  Covered:
the 640x480 synthetic pair under two threshold sets, the reference's sample2
frames (0 -> 3, and 0 / 13 with the thresholds of its
``test_correspondence_map.py``), a BF16 16-channel hybrid registration, ties
between duplicated source points (the smaller index wins), source points of
NaN depth (never match), three pairs of an uneven multiscale batch at every
level, a 1280x960 pair with more source rounds than the shared-memory
cache holds, and a batch of the differentiable loss.
"""
import math

import numpy as np
import pytest
import torch

from oracle import icp_oracle as io
from _helpers import sample2_pair, synthetic_pair

pytestmark = pytest.mark.gpu

ANGLE_20 = math.radians(20)


def _t(x, dev, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    return t if dtype is None else t.to(dtype)


def _oracle_map(d, pose, dist, angle):
    s, t = d["src"], d["tgt"]
    return io.associate32(s["points"], s["normals"], s["mask"], io.pose_rt32(pose), t["points"],
                          t["normals"], t["mask"], d["kcam"], dist, angle)


def _plain(cuda, d, iters, dist, angle, feats=None, wf=0.0, wg=1.0, init=None, opts=0):
    """Registers d's pair for `iters` iterations through the C ABI and reads
    the correspondences of the final association back; returns (map, pose
    it was taken at)."""
    from slamtb_gb300 import _native as N
    lib = N.lib()
    s, t = d["src"], d["tgt"]
    h, w = t["mask"].shape
    sp = _t(s["points"], cuda).view(-1, 3)
    sn = _t(s["normals"], cuda).view(-1, 3)
    sm = _t(s["mask"], cuda).view(-1)
    tp, tn, tm = _t(t["points"], cuda), _t(t["normals"], cuda), _t(t["mask"], cuda)
    kcam = _t(d["kcam"], cuda)
    sf = tf = None
    channels, code = 0, N.STB_F32
    if feats is not None:
        sf, tf = feats
        channels, code = tf.size(0), N.feat_dtype_code(tf)
    ws_bytes = lib.stb_icp_workspace_bytes(sp.size(0), h, w)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    res = torch.empty(N.RES_SIZE, dtype=torch.float64, device=cuda)
    init_t = None if init is None else _t(np.asarray(init, np.float64), cuda)
    stream = N.stream_of(cuda)
    N.check(lib.stb_icp_estimate(
        N.ptr(kcam), N.ptr(sp), N.ptr(sn), N.ptr(sm), sp.size(0), N.ptr(sf), N.ptr(tp),
        N.ptr(tn), N.ptr(tm), h, w, N.ptr(tf), channels, code, N.ptr(init_t), iters, wg, wf,
        dist, angle, 2.75, opts, N.ptr(ws), ws_bytes, N.ptr(res), None, 0, stream))
    m = torch.empty(h, w, dtype=torch.int64, device=cuda)
    N.check(lib.stb_icp_correspondences(N.ptr(ws), h, w, iters, N.ptr(m), stream))
    r = res.cpu().numpy()
    if r[N.RES_ITERS] > 0:
        pose = r[N.RES_TRANSFORM:N.RES_TRANSFORM + 16].reshape(4, 4)
    else:
        pose = np.eye(4) if init is None else np.asarray(init, np.float64)
    return m.cpu().numpy(), pose, int(r[N.RES_ITERS])


def _check_iterations(cuda, d, iters, dist, angle, **kw):
    done_prev = -1
    for k in iters:
        m, pose, done = _plain(cuda, d, k, dist, angle, **kw)
        a = _oracle_map(d, pose, dist, angle)
        assert a.count > 100, (k, a.count)
        np.testing.assert_array_equal(m, a.ref_map, err_msg=f"after {k} iterations")
        assert done >= done_prev
        done_prev = done


@pytest.fixture(scope="module")
def pair0():
    return synthetic_pair(0, feature_channels=0)


@pytest.mark.parametrize("launch", ["single", "multi"])
@pytest.mark.parametrize("dist,angle", [(0.1, ANGLE_20), (0.5, math.pi / 4)])
def test_fused_association_every_iteration(cuda, pair0, dist, angle, launch):
    """Both launch modes: the single cooperative launch (default) and the
    two-launches-per-iteration sequence (STB_OPT_MULTI_LAUNCH)."""
    from slamtb_gb300 import _native as N
    _check_iterations(cuda, pair0, range(0, 11), dist, angle,
                      opts=0 if launch == "single" else N.OPT_MULTI_LAUNCH)


def test_fused_association_from_an_initial_pose(cuda, pair0):
    init = io.se3_exp([0.01, -0.02, 0.015, 0.02, -0.01, 0.03])
    _check_iterations(cuda, pair0, [0, 1, 4], 0.1, ANGLE_20, init=init)


def test_fused_association_sample2(cuda):
    _check_iterations(cuda, sample2_pair(0, 3), range(0, 11), 0.1, ANGLE_20)
    # the thresholds of the reference's test_correspondence_map.py (10, 10)
    m, pose, _ = _plain(cuda, sample2_pair(0, 13), 0, 10, 10)
    np.testing.assert_array_equal(m, _oracle_map(sample2_pair(0, 13), pose, 10, 10).ref_map)


def test_fused_association_bf16_hybrid(cuda):
    """Sixteen BF16 channels with the reference preset's weights (geometric
    10, feature 1, slamtb/registration/preset.py:10): the association is the
    geometric one at poses that the feature term moved."""
    d = synthetic_pair(3, feature_channels=16)
    sf = _t(d["src_feats"], cuda, torch.bfloat16).reshape(16, -1)
    tf = _t(d["tgt_feats"], cuda, torch.bfloat16)
    _check_iterations(cuda, d, [1, 3, 6], 0.1, ANGLE_20, feats=(sf, tf), wf=1.0, wg=10.0)


def _with_duplicates_and_nans(d):
    """Copies of d whose source columns 2j+1 repeat columns 2j (equal points
    and normals: equal distances to every target pixel), and whose source
    rows 100..139 have NaN depth (NaN points) with the mask still set."""
    out = dict(d)
    s = {k: np.array(v, copy=True) for k, v in d["src"].items() if k != "kcam"}
    s["kcam"] = d["src"]["kcam"]
    for key in ("points", "normals", "mask"):
        s[key][:, 1::2] = s[key][:, 0::2]
    s["points"][100:140] = np.nan
    s["mask"][100:140] = True
    out["src"] = s
    return out


def test_fused_association_ties_and_nan_sources(cuda, pair0):
    d = _with_duplicates_and_nans(pair0)
    for k in (0, 2):
        m, pose, _ = _plain(cuda, d, k, 0.1, ANGLE_20)
        a = _oracle_map(d, pose, 0.1, ANGLE_20)
        np.testing.assert_array_equal(m, a.ref_map)
        win = io.winners_from_ref_map(m)
        win = win[m != io.CORRESP_EMPTY]
        w = d["tgt"]["mask"].shape[1]
        # every winner is the even (smaller) index of its duplicated pair,
        # and no NaN row wins
        assert win.size > 1000 and (win % 2 == 0).all()
        rows = win // w
        assert not ((rows >= 100) & (rows < 140)).any()


def test_fused_association_streamed_rounds(cuda):
    """1280x960 (1,228,800 source points, four rounds of 2048 points a block
    on 152 blocks): more rounds than the source cache holds, so the rounds
    past it read their source points from global memory; the maps at
    iterations 0, 1 and 3 against the oracle."""
    d = synthetic_pair(5, width=1280, height=960)
    _check_iterations(cuda, d, [0, 1, 3], 0.1, ANGLE_20)


# ---------------------------------------------------------------------------
# batched persistent kernel
# ---------------------------------------------------------------------------

SCALES = [1.0, 0.5, 0.5]
ITERS = [6, 4, 3]  # finest first


def _batch_pairs(cuda):
    from oracle import frame_prep as fp
    from slamtb_gb300 import synthetic
    from slamtb_gb300.frame import FramePointCloud, KCamera
    pairs = []
    for k, (w, h) in enumerate([(640, 480), (160, 120), (424, 240)]):
        p = synthetic.make_pair(70 + k, width=w, height=h)
        spyr = fp.FramePointCloud.from_depth(p["source_depth"], p["kcam"]).pyramid(SCALES)
        tpyr = fp.FramePointCloud.from_depth(p["target_depth"], p["kcam"]).pyramid(SCALES)
        dev = lambda pyr: [FramePointCloud(None, _t(lv.mask, cuda), KCamera(lv.kcam),  # noqa
                                           points=_t(lv.points, cuda),
                                           normals=_t(lv.normals, cuda)) for lv in pyr]
        pairs.append(dict(spyr=spyr, tpyr=tpyr, src=dev(spyr), tgt=dev(tpyr)))
    return pairs


@pytest.mark.parametrize("schedule", [0, 103, 176])
@pytest.mark.parametrize("levels", [1, 2, 3])
def test_batch_association_every_level(cuda, levels, schedule):
    """The coarsest `levels` levels of three uneven pairs in one batch; the
    last of them runs k iterations, so the final association is at that
    level's k-th pose.  Under the lock-step schedule and the grouped one
    (three groups of 50 blocks; 76 groups of 2, where a 640x480 level
    spans 75 rounds a block, past the source cache)."""
    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration import BatchRegistration, ICPOdometry
    pairs = _batch_pairs(cuda)
    iters_fine_first = ITERS[len(ITERS) - levels:]
    for k in sorted({0, 1, iters_fine_first[0]}):
        its = [k] + iters_fine_first[1:]
        ests = [(s, ICPOdometry(n, geom_weight=1.0, feat_weight=0.0, distance_threshold=0.1,
                                normals_angle_thresh=ANGLE_20))
                for s, n in zip(SCALES[len(SCALES) - levels:], its)]
        br = BatchRegistration(ests)
        br.tile_config = schedule
        srcs = [p["src"][:levels] for p in pairs]
        tgts = [p["tgt"][:levels] for p in pairs]
        res, _, plan = br.launch(srcs, tgts)
        out = res.cpu().numpy()
        for q, pair in enumerate(pairs):
            tl = pair["tpyr"][levels - 1]
            sl = pair["spyr"][levels - 1]
            h, w = tl.mask.shape
            m = torch.empty(h, w, dtype=torch.int64, device=cuda)
            N.check(N.lib().stb_icp_batch_correspondences(
                N.ptr(plan.ws), plan.B, plan.total_px, q, h, w, plan.total_iters, N.ptr(m),
                N.stream_of(cuda)))
            r = out[q]
            # the pose of the last level's association: the result's
            # transform when that level made a step, else its start pose
            # (the previous level's result, or identity)
            if r[N.RES_ITERS] > 0:
                pose = r[N.RES_TRANSFORM:N.RES_TRANSFORM + 16].reshape(4, 4)
            else:
                assert k == 0
                pose = _start_pose(cuda, pairs, q, levels, schedule)
            d = dict(kcam=sl.kcam, src=dict(points=sl.points, normals=sl.normals, mask=sl.mask),
                     tgt=dict(points=tl.points, normals=tl.normals, mask=tl.mask))
            a = _oracle_map(d, pose, 0.1, ANGLE_20)
            assert a.count > 50
            np.testing.assert_array_equal(m.cpu().numpy(), a.ref_map,
                                          err_msg=f"pair {q}, {levels} levels, {k} iterations")


def _start_pose(cuda, pairs, q, levels, schedule):
    """Pose pair q starts its `levels`-th level from: the result of the
    coarser levels' batch under the same schedule (identity for the
    coarsest level)."""
    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration import BatchRegistration, ICPOdometry
    if levels == 1:
        return np.eye(4)
    its = ITERS[len(ITERS) - levels + 1:]
    ests = [(s, ICPOdometry(n, geom_weight=1.0, feat_weight=0.0, distance_threshold=0.1,
                            normals_angle_thresh=ANGLE_20))
            for s, n in zip(SCALES[len(SCALES) - levels + 1:], its)]
    br = BatchRegistration(ests)
    br.tile_config = schedule
    res, _, _ = br.launch([p["src"][:levels - 1] for p in pairs],
                          [p["tgt"][:levels - 1] for p in pairs])
    r = res.cpu().numpy()[q]
    return r[N.RES_TRANSFORM:N.RES_TRANSFORM + 16].reshape(4, 4) if r[N.RES_ITERS] > 0 \
        else np.eye(4)


# ---------------------------------------------------------------------------
# differentiable loss
# ---------------------------------------------------------------------------

def test_loss_association(cuda):
    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration.grad import PointToPlaneLoss  # noqa: F401
    pairs = [synthetic_pair(seed, width=320, height=240) for seed in (80, 81, 82)]
    B, H, W = len(pairs), 240, 320
    poses = np.stack([io.se3_exp([0.004 * k, -0.003, 0.002, 0.003, 0.001 * k, -0.002])
                      for k in range(B)]).astype(np.float32).astype(np.float64)
    st = lambda key, part: torch.stack([_t(d[part][key], cuda) for d in pairs])  # noqa: E731
    depth = torch.stack([_t(d["src_fpcl"].points[..., 2], cuda) for d in pairs])
    ins = [depth, st("normals", "src"), st("mask", "src"), st("points", "tgt"),
           st("normals", "tgt"), st("mask", "tgt")]
    kc = pairs[0]["kcam"]
    fx, fy, cx, cy = float(kc[0, 0]), float(kc[1, 1]), float(kc[0, 2]), float(kc[1, 2])
    T = _t(poses, cuda)
    lib = N.lib()
    need = int(lib.stb_icp_loss_workspace_bytes(B, H, W))
    ws = torch.empty(need, dtype=torch.uint8, device=cuda)
    loss = torch.empty(B, dtype=torch.float64, device=cuda)
    stream = N.stream_of(cuda)
    N.check(lib.stb_icp_loss_forward(*[N.ptr(x.contiguous()) for x in ins], B, H, W, fx, fy, cx,
                                     cy, N.ptr(T), 0.1, ANGLE_20, N.ptr(ws), need, N.ptr(loss),
                                     stream))
    m = torch.empty(B, H, W, dtype=torch.int64, device=cuda)
    N.check(lib.stb_icp_loss_correspondences(N.ptr(ws), B, H, W, N.ptr(m), stream))
    m = m.cpu().numpy()
    for p, d in enumerate(pairs):
        a = _oracle_map(d, poses[p], 0.1, ANGLE_20)
        assert a.count > 1000
        np.testing.assert_array_equal(m[p], a.ref_map, err_msg=f"pair {p}")
