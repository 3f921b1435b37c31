"""numpy front end of the C/OpenMP port (test infrastructure)."""
import ctypes
import math

import numpy as np

from . import build_port

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        _LIB = build_port.load()
    return _LIB


def max_threads():
    return _lib().icp_port_max_threads()


def icp_estimate(kcam, src_points, src_normals, src_mask, tgt_points, tgt_normals, tgt_mask,
                 src_feats=None, tgt_feats=None, num_iters=10, geom_weight=1.0,
                 feat_weight=1.0, distance_threshold=0.5, normals_angle_thresh=math.pi / 4,
                 feat_residual_thresh=2.75, transform=None, threads=0):
    """Same arguments as ``icp_oracle.icp_estimate``; returns a dict with
    transform (or None), information, residual, match_ratio, iters."""
    def c(a, dt):
        return None if a is None else np.ascontiguousarray(a, dtype=dt)
    k = c(kcam, np.float32)
    sp = c(np.asarray(src_points).reshape(-1, 3), np.float32)
    sn = c(np.asarray(src_normals).reshape(-1, 3), np.float32)
    sm = c(np.asarray(src_mask).reshape(-1), np.uint8)
    tp, tn = c(tgt_points, np.float32), c(tgt_normals, np.float32)
    tm = c(tgt_mask, np.uint8)
    h, w = tm.shape
    tf = c(tgt_feats, np.float32)
    sf = None if src_feats is None else c(np.asarray(src_feats).reshape(tf.shape[0], -1),
                                          np.float32)
    init = c(transform, np.float64)
    T = np.zeros(16)
    info = np.zeros(36)
    res = ctypes.c_double()
    ratio = ctypes.c_double()
    iters = ctypes.c_int()
    p = (lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p))
    _lib().icp_port_estimate(
        p(k), p(sp), p(sn), p(sm), sp.shape[0], p(sf), p(tp), p(tn), p(tm), h, w, p(tf),
        0 if tf is None else tf.shape[0], p(init), num_iters, geom_weight,
        feat_weight if tf is not None else 0.0, distance_threshold, normals_angle_thresh,
        feat_residual_thresh, threads, p(T), p(info), ctypes.byref(res), ctypes.byref(ratio),
        ctypes.byref(iters))
    return dict(transform=T.reshape(4, 4) if iters.value else None,
                information=info.reshape(6, 6), residual=res.value, match_ratio=ratio.value,
                iters=iters.value)


def multiscale_estimate(levels, estimators, transform=None, threads=0):
    """``MultiscaleRegistration.estimate_frame`` (multiscale.py:30-67) on the
    port: ``levels`` coarsest first, ``estimators`` finest first, as
    ``icp_oracle.multiscale_estimate``, with the same hand-over (a level
    whose first iteration fails passes identity on, multiscale.py:64-65).
    The port computes the reference's float32 per-point partials, so its
    free-running result carries the reference's own arithmetic; the numpy
    oracle's FP64 terms are the error reference it is compared with.
    Returns the finest level's result dict."""
    result = None
    for level, est in zip(levels, estimators[::-1]):
        kw = {k: v for k, v in est.items() if k != "channel_mode"}
        if est.get("channel_mode", "last") != "last":
            raise ValueError("the port follows the reference's 'last' channel mode only")
        result = icp_estimate(transform=transform, threads=threads, **level, **kw)
        transform = result["transform"]
    return result
