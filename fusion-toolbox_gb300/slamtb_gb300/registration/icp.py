"""Pose estimation via iterative closest points, GB300 path.

Same interface as ``slamtb/registration/icp.py:111-310`` (``ICPOdometry``);
the Gauss-Newton loop runs on the device as one call into
``libslamtb_gb300`` (``stb_icp_estimate``), with one device-to-host copy of
the result at the end instead of the reference's ~8 synchronisations per
iteration.
"""
import ctypes
import math

import numpy as np
import torch

from .. import _native as N
from .. import processing
from .result import RegistrationResult


def _small_input(x, device, tdtype, ndtype, numel, name):
    """(keep-alive, pointer) of the intrinsics or the initial pose: a tensor
    on the device as it is, anything else as a host array that the library
    reads during the call (into the launch parameters: no copy, no wait)."""
    if isinstance(x, torch.Tensor) and x.device == device:
        a = x.to(dtype=tdtype).contiguous()
        ptr = N.ptr(a)
    else:
        if isinstance(x, torch.Tensor):
            x = x.detach().cpu().numpy()
        a = np.ascontiguousarray(x, dtype=ndtype)
        ptr = ctypes.c_void_p(a.ctypes.data)
    if (a.numel() if isinstance(a, torch.Tensor) else a.size) != numel:
        raise RuntimeError(f"Check failed: {name} must have {numel} entries")
    return a, ptr


class _Workspace:
    """Device scratch of ``stb_icp_estimate``, grown on demand and reused
    across calls (one per estimator: concurrent calls on several streams
    need several estimators)."""

    def __init__(self):
        self.buf = None
        self.result = None
        self.history = None
        self.result_host = None

    def host_result(self):
        """Pinned host copy of the result block (reused; the returned
        RegistrationResult never aliases it)."""
        if self.result_host is None:
            self.result_host = torch.empty(N.RES_SIZE, dtype=torch.float64, pin_memory=True)
        return self.result_host

    def get(self, device, num_source, height, width, num_iters, history):
        need = int(N.lib().stb_icp_workspace_bytes(num_source, height, width))
        if self.buf is None or self.buf.device != device or self.buf.numel() < need:
            self.buf = torch.empty(need, dtype=torch.uint8, device=device)
            self.result = torch.empty(N.RES_SIZE, dtype=torch.float64, device=device)
        hist = None
        if history:
            if (self.history is None or self.history.device != device
                    or self.history.size(0) < max(num_iters, 1)):
                self.history = torch.empty(max(num_iters, 1), N.HIST_SIZE,
                                           dtype=torch.float64, device=device)
            hist = self.history
        return self.buf, self.result, hist


class ICPOdometry:
    """Iterative closest points with the point-to-plane error and
    Gauss-Newton optimisation (``slamtb/registration/icp.py:111-150``).

    Args (as the reference):
        num_iters (int): Gauss-Newton iterations (at most 254).
        geom_weight (float): geometric term weight, 0 disables it.
        feat_weight (float): feature term weight, 0 disables it.
        so3 (bool): rotation-only optimisation; not supported (the
            reference's rotation-only call is broken: ``icp.py:71-76``
            passes 15 arguments to an 11-argument binding).
        distance_threshold (float): maximum matching distance.
        normals_angle_thresh (float): maximum normal angle (radians).
        feat_residual_thresh (float): maximum feature residual norm.

    Extra keyword arguments:
        feat_channel_mode (str): "last" (reference behaviour: with several
            feature channels only the last channel's Jacobian enters J^T J
            and J^T r) or "sum" (all channels).
        feat_layout (str): "auto" samples feature maps of several channels
            from texel-major copies (all channels of a pixel adjacent, built
            on the device per call); "planar" reads the (C, H, W) maps as
            given.  Results are identical.
        solve_precision (str): "fp64" (default: the 6x6 solve, the SE(3)
            exponential and the pose update in FP64, as the reference's
            float64 host solve) or "dw" (double-word float32, ~48 bits, on
            the FP32 pipes).
        launch (str): "single" (default: one cooperative launch runs the
            whole registration, phases separated by grid barriers) or
            "multi" (two launches per iteration).
        use_graph (bool): with launch="multi", replay the launch sequence
            as a CUDA graph.
        record_history (bool): keep per-iteration records in
            ``self.last_history`` (float64 (num_iters, 64) CPU tensor, layout
            ``STB_HIST_*`` of ``include/slamtb_gb300.h``).
    """

    def __init__(self, num_iters, geom_weight=1.0, feat_weight=1.0, so3=False,
                 distance_threshold=.5, normals_angle_thresh=math.pi / 4,
                 feat_residual_thresh=2.75, feat_channel_mode="last",
                 use_graph=True, record_history=False, feat_layout="auto",
                 solve_precision="fp64", launch="single"):
        if so3:
            raise NotImplementedError(
                "so3=True is not supported: the reference's rotation-only path "
                "cannot run (icp.py:71-76 calls estimate_feature_so3 with 15 "
                "arguments; the binding takes 11)")
        if num_iters > 254:
            raise ValueError("num_iters must be at most 254")
        if feat_channel_mode not in ("last", "sum"):
            raise ValueError("feat_channel_mode must be 'last' or 'sum'")
        if feat_layout not in ("auto", "planar"):
            raise ValueError("feat_layout must be 'auto' or 'planar'")
        if solve_precision not in ("fp64", "dw"):
            raise ValueError("solve_precision must be 'fp64' or 'dw'")
        if launch not in ("single", "multi"):
            raise ValueError("launch must be 'single' or 'multi'")
        self.num_iters = num_iters
        self.geom_weight = geom_weight
        self.feat_weight = feat_weight
        self.so3 = so3
        self.distance_threshold = distance_threshold
        self.normals_angle_thresh = normals_angle_thresh
        self.feat_residual_thresh = feat_residual_thresh
        self.feat_channel_mode = feat_channel_mode
        self.feat_layout = feat_layout
        self.solve_precision = solve_precision
        self.launch_mode = launch
        self.use_graph = use_graph
        self.record_history = record_history
        self.last_history = None
        self._ws = _Workspace()

    def estimate(self, kcam, source_points, source_normals, source_mask,
                 source_feats=None, target_points=None, target_mask=None,
                 target_normals=None, target_feats=None, transform=None):
        """Estimate the transform taking the source points onto the target
        point grid (``icp.py:152-262``).

        Args:
            kcam: intrinsics, a ``KCamera``-like object with ``.matrix`` or
                a (3, 3) tensor.
            source_points, source_normals: (N, 3) (or (H, W, 3)) float32.
            source_mask: (N,) bool.
            source_feats: (C, N) (or (C, H, W)) float32 / bfloat16, optional.
            target_points, target_normals: (H, W, 3) float32.
            target_mask: (H, W) bool.
            target_feats: (C, H, W) float32 / bfloat16, optional.
            transform: (4, 4) initial transform, optional.

        Returns:
            RegistrationResult
        """
        res, hist, n, dtype = self.launch(
            kcam, source_points, source_normals, source_mask, source_feats, target_points,
            target_mask, target_normals, target_feats, transform)
        out = self._ws.host_result()
        out.copy_(res, non_blocking=True)
        if hist is not None:
            self.last_history = hist[:self.num_iters].cpu()
        torch.cuda.current_stream(res.device).synchronize()
        return self._result(out, n, dtype)

    def launch(self, kcam, source_points, source_normals, source_mask, source_feats=None,
               target_points=None, target_mask=None, target_normals=None, target_feats=None,
               transform=None):
        """Enqueue the registration on the current stream without waiting.

        Returns (result, history, num_source, dtype): ``result`` is the
        float64 device result block (``STB_RES_*`` layout), ``history`` the
        per-iteration device records or None.  The block is reused by the
        next call of this estimator."""
        device = target_points.device
        if device.type != "cuda":
            raise RuntimeError("Check failed: target_points: Expected a gpu tensor "
                               "(slamtb_gb300 runs on CUDA devices only)")
        sp = source_points.reshape(-1, 3)
        sn = source_normals.reshape(-1, 3)
        sm = source_mask.reshape(-1)
        n = sp.size(0)
        for name, t in (("source_points", sp), ("source_normals", sn),
                        ("target_points", target_points), ("target_normals", target_normals)):
            if t.dtype != torch.float32:
                raise RuntimeError(f"Check failed: {name}: expected float32, got {t.dtype}")
            if t.device != device:
                raise RuntimeError(f"Check failed: {name}: Expected a gpu tensor on {device}")
        if sm.numel() != n:
            raise RuntimeError("Check failed: source_mask must have one entry per source point")
        sp, sn = sp.contiguous(), sn.contiguous()
        sm = sm.to(torch.bool).contiguous()
        tp = target_points.contiguous()
        tn = target_normals.contiguous()
        tm = target_mask.to(device=device, dtype=torch.bool).contiguous()
        h, w = tm.shape

        has_features = (source_feats is not None and target_feats is not None
                        and self.feat_weight > 0)
        sf = tf = None
        channels = 0
        code = N.STB_F32
        if has_features:
            tf = target_feats.to(device).contiguous()
            sf = source_feats.to(device).reshape(source_feats.size(0), -1).contiguous()
            code = N.feat_dtype_code(tf)
            if sf.dtype != tf.dtype:
                raise RuntimeError("Check failed: source and target features must share a dtype")
            channels = tf.size(0)
            if tf.shape[1:] != (h, w) or sf.size(1) != n:
                raise RuntimeError("Check failed: feature maps do not match the point grids")
            if channels > 1 and self.feat_layout == "auto":
                # texel-major copies: the kernels then read all channels of a
                # pixel from adjacent bytes (same values, same results)
                tf = processing.interleave_features(tf)
                sf = processing.interleave_features(sf)
                code += N.STB_F32_HWC
        m = kcam.matrix if hasattr(kcam, "matrix") else kcam
        k, kptr = _small_input(m, device, torch.float32, np.float32, 9, "kcam")
        init = iptr = None
        if transform is not None:
            init, iptr = _small_input(transform, device, torch.float64, np.float64, 16,
                                      "transform")
        ws, res, hist = self._ws.get(device, n, h, w, self.num_iters, self.record_history)
        with torch.cuda.device(device):
            N.check(N.lib().stb_icp_estimate(
                kptr, N.ptr(sp), N.ptr(sn), N.ptr(sm), n, N.ptr(sf), N.ptr(tp),
                N.ptr(tn), N.ptr(tm), h, w, N.ptr(tf), channels, code, iptr,
                self.num_iters, float(self.geom_weight),
                float(self.feat_weight if has_features else 0.0),
                float(self.distance_threshold), float(self.normals_angle_thresh),
                float(self.feat_residual_thresh),
                (0 if self.feat_channel_mode == "last" else 1)
                | (N.OPT_DW_SOLVE if self.solve_precision == "dw" else 0)
                | (N.OPT_MULTI_LAUNCH if self.launch_mode == "multi" else 0),
                N.ptr(ws), ws.numel(), N.ptr(res), N.ptr(hist), int(self.use_graph),
                N.stream_of(device)))
        del k, init  # kept alive through the call
        return res, hist, n, sp.dtype

    @staticmethod
    def _result(out, n, dtype):
        """RegistrationResult of one float64 result block (a CPU tensor);
        the returned tensors are copies."""
        o = out.numpy()
        info = torch.from_numpy(o[N.RES_INFO:N.RES_INFO + 36].reshape(6, 6).astype(
            np.float32 if dtype == torch.float32 else np.float64))
        if int(o[N.RES_ITERS]) == 0:
            return RegistrationResult(information=info)
        return RegistrationResult(
            torch.from_numpy(o[N.RES_TRANSFORM:N.RES_TRANSFORM + 16].reshape(4, 4).copy()),
            info, float(o[N.RES_RESIDUAL]), float(o[N.RES_MATCHES]) / n)

    def estimate_frame(self, source_frame, target_frame, source_feats=None,
                       target_feats=None, transform=None, device=None):
        """Estimate between two frames (``icp.py:264-310``).  Frames may be
        ``slamtb_gb300.frame.Frame`` or ``FramePointCloud``; ``device``
        defaults to the current CUDA device (a CPU device is refused)."""
        from ..frame import Frame, FramePointCloud, resolve_device
        device = resolve_device(device)
        if isinstance(source_frame, Frame):
            source_frame = FramePointCloud.from_frame(source_frame).to(device)
        if isinstance(target_frame, Frame):
            target_frame = FramePointCloud.from_frame(target_frame).to(device)
        return self.estimate(
            source_frame.kcam, source_frame.points, source_frame.normals,
            source_frame.mask, source_feats=source_feats,
            target_points=target_frame.points, target_normals=target_frame.normals,
            target_mask=target_frame.mask, target_feats=target_feats,
            transform=transform)
