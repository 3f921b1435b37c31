"""The batched workloads at their full sizes, checked through properties that
do not need the oracle to run every pair:

* 256 pairs of uneven sizes (160x120 ... 1280x720), 3 levels [10, 5, 3]:
  every pair registers, the median error against the ground-truth motion is
  at the noise floor, and pairs of the smallest, a middle and the largest
  size pass the teacher-forced 1e-5 oracle gate (``compare_forced``) at
  every level and iteration of the full run;
* 16 pairs of 1920x1080 with 16 BF16 feature channels, 4 levels
  [10, 8, 5, 3]: every pair registers and pair 0 passes the gate on the
  three coarse levels and the first two iterations of the finest.

Both run under the lock-step schedule (BatchRegistration's default) and
under the grouped schedule the autotuner picks for each in the benchmark
(19 groups for the uneven pairs, 4 for the 1080p pairs).

Inputs are rendered and prepared on the device; the oracle sees the same
float32 point grids and the BF16 feature values as float32.
"""
import math

import numpy as np
import pytest
import torch

from _helpers import compare_forced, rel_pose

pytestmark = pytest.mark.gpu

DIST, ANGLE = 0.1, math.radians(20)


def _device_pair(cuda, seed, w, h, channels=None, **kw):
    from slamtb_gb300 import synthetic
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    p = synthetic.make_pair(seed, width=w, height=h, feature_channels=channels, device=cuda,
                            **kw)
    k = KCamera(p["kcam"])
    src = FramePointCloud.from_frame(Frame(FrameInfo(k), p["source_depth"]), cuda)
    tgt = FramePointCloud.from_frame(Frame(FrameInfo(k), p["target_depth"]), cuda)
    out = dict(src=src, tgt=tgt, gt=p["gt"])
    if channels is not None:
        out["sf"] = torch.from_numpy(p["source_feats"]).to(cuda, torch.bfloat16)
        out["tf"] = torch.from_numpy(p["target_feats"]).to(cuda, torch.bfloat16)
    return out


def _host_level(s, t):
    return dict(kcam=s.kcam.matrix.numpy(),
                src=dict(points=s.points.cpu().numpy(), normals=s.normals.cpu().numpy(),
                         mask=s.mask.cpu().numpy()),
                tgt=dict(points=t.points.cpu().numpy(), normals=t.normals.cpu().numpy(),
                         mask=t.mask.cpu().numpy()))


def _check(hist, spyr, tpyr, iters, kw, sfp=None, tfp=None, last_level_iters=None):
    """Teacher-forced gate of one pair's history, level by level (coarsest
    first), with the reference's hand-over of the level pose."""
    from slamtb_gb300 import _native as N
    off, T = 0, None
    levels = list(zip(range(len(iters)), iters[::-1]))
    for level, n in levels:
        d = _host_level(spyr[level], tpyr[level])
        x = {}
        if sfp is not None:
            x = dict(sf=sfp[level].reshape(sfp[level].size(0), -1), tf=tfp[level])
        h = hist[off:off + n]
        check = n if (last_level_iters is None or level < len(iters) - 1) else last_level_iters
        compare_forced(h[:check], d, x, dict(kw, num_iters=check), init=T)
        ok = h[:, N.HIST_OK].numpy()
        done = int(ok.sum()) if ok.all() else int(np.argmin(ok))
        T = h[done - 1, N.HIST_TRANSFORM:N.HIST_TRANSFORM + 16].view(4, 4).numpy() \
            if done > 0 else np.eye(4)
        off += n


def _estimators(iters, scales, wg, wf):
    from slamtb_gb300.registration import ICPOdometry
    return [(s, ICPOdometry(n, geom_weight=wg, feat_weight=wf, distance_threshold=DIST,
                            normals_angle_thresh=ANGLE)) for s, n in zip(scales, iters)]


@pytest.mark.parametrize("schedule", [0, 119])
def test_256_uneven_pairs_full_size(cuda, schedule):
    from slamtb_gb300.registration import BatchRegistration
    rng = np.random.default_rng(7)
    sizes = [(160, 120), (320, 240), (640, 480), (848, 480), (1280, 720)]
    pick = rng.integers(0, len(sizes), size=256)
    pairs = [_device_pair(cuda, 1000 + k, *sizes[i]) for k, i in enumerate(pick)]
    iters, scales = [10, 5, 3], [1.0, 0.5, 0.5]
    br = BatchRegistration(_estimators(iters, scales, 1.0, 0.0), record_history=True)
    br.tile_config = schedule
    spyrs = [p["src"].pyramid(scales) for p in pairs]
    tpyrs = [p["tgt"].pyramid(scales) for p in pairs]
    res = br.estimate_pyramids(spyrs, tpyrs)
    assert all(r.transform is not None for r in res)
    errs = [rel_pose(r.transform.numpy(), p["gt"]) for r, p in zip(res, pairs)]
    assert np.median(errs) < 0.2
    kw = dict(geom_weight=1.0, feat_weight=0.0, distance_threshold=DIST,
              normals_angle_thresh=ANGLE)
    for size in (0, 2, 4):
        k = int(np.nonzero(pick == size)[0][0])
        _check(br.last_history[k], spyrs[k], tpyrs[k], iters, kw)


@pytest.mark.parametrize("schedule", [0, 104])
def test_16_pairs_1080p_16_channel_bf16_full_size(cuda, schedule):
    from slamtb_gb300.processing import feature_pyramid
    from slamtb_gb300.registration import BatchRegistration
    iters, scales = [10, 8, 5, 3], [1.0, 0.5, 0.5, 0.5]
    pairs = [_device_pair(cuda, 2000 + k, 1920, 1080, channels=16, max_rot_deg=10.0,
                          max_trans=0.1) for k in range(16)]
    br = BatchRegistration(_estimators(iters, scales, 10.0, 1.0), record_history=True)
    br.tile_config = schedule
    spyrs = [p["src"].pyramid(scales) for p in pairs]
    tpyrs = [p["tgt"].pyramid(scales) for p in pairs]
    sfps = [feature_pyramid(p["sf"], scales) for p in pairs]
    tfps = [feature_pyramid(p["tf"], scales) for p in pairs]
    res = br.estimate_pyramids(spyrs, tpyrs, sfps, tfps)
    assert all(r.transform is not None for r in res)
    kw = dict(geom_weight=10.0, feat_weight=1.0, distance_threshold=DIST,
              normals_angle_thresh=ANGLE)
    _check(br.last_history[0], spyrs[0], tpyrs[0], iters, kw, sfps[0], tfps[0],
           last_level_iters=2)
