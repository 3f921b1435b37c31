"""Many frame pairs, one multiscale schedule, one persistent launch.

``BatchRegistration`` runs ``MultiscaleRegistration.estimate_frame``
(``slamtb/registration/multiscale.py:30-67``) for a list of frame pairs at
once: ``stb_icp_estimate_batch`` advances every pair through every level
and Gauss-Newton iteration inside one cooperative kernel (grid barriers
between the association and reduction phases, a per-pair FP64 solve at the
end of each reduction), so a batch of uneven resolutions costs one launch.
"""
import ctypes

import torch

from .. import _native as N
from ..frame import Frame, FramePointCloud, resolve_device
from .. import processing
from ..processing import feature_pyramid
from .icp import ICPOdometry
from .result import RegistrationResult

# Schedules of stb_icp_estimate_batch as BatchRegistration numbers them:
# 0..5 the lock-step kernel's work-item sizes, GROUPED + g the grouped
# kernel with g groups.
GROUPED = 100
TUNE_CONFIGS = (0, 1, 2, 3, 4, 5, GROUPED + 1, GROUPED + 2, GROUPED + 4, GROUPED + 8,
                GROUPED + 19, GROUPED + 38, GROUPED + 76)


class BatchPlan:
    """A prepared batch (``BatchRegistration.prepare``): device level table,
    parameters, initial transforms, workspace and outputs."""


class BatchRegistration:
    """Args:
        estimators (list of (float, ICPOdometry)): scale and estimator per
            level, finest first, as ``MultiscaleRegistration``; at most 4
            levels and 253 iterations in total.
        feat_channel_mode (str): "last" (reference) or "sum".
        solve_precision (str): "fp64" (default: FP64 solve, exponential and
            pose update) or "dw" (double-word float32, ~48 bits).
        record_history (bool): keep per-iteration records in
            ``self.last_history`` ((pairs, total iterations, 64) float64 CPU,
            iterations numbered over the levels coarsest first).
    """

    def __init__(self, estimators, feat_channel_mode="last", record_history=False,
                 solve_precision="fp64"):
        if not 1 <= len(estimators) <= 4:
            raise ValueError("BatchRegistration takes 1 to 4 levels")
        for _, est in estimators:
            if not isinstance(est, ICPOdometry):
                raise TypeError("BatchRegistration levels must be ICPOdometry estimators")
        if feat_channel_mode not in ("last", "sum"):
            raise ValueError("feat_channel_mode must be 'last' or 'sum'")
        if solve_precision not in ("fp64", "dw"):
            raise ValueError("solve_precision must be 'fp64' or 'dw'")
        self.estimators = estimators
        self.solve_precision = solve_precision
        self.feat_channel_mode = feat_channel_mode
        self.record_history = record_history
        self.last_history = None
        # schedule: 0..5 the lock-step kernel with its largest work item
        # (0 -> 8192 pixels; 1..5 -> 512 ... 8192); GROUPED + g the grouped
        # kernel with g groups (stb_icp_estimate_batch, STB_OPT_GROUPS)
        self.tile_config = 0
        self.feat_layout = "auto"  # "auto": texel-major feature copies when C > 1; "planar"

    @property
    def scales(self):
        return [s for s, _ in self.estimators]

    def _params(self):
        levels = [est for _, est in self.estimators[::-1]]  # coarsest first
        arr = (N.StbLevelParams * len(levels))()
        for k, est in enumerate(levels):
            arr[k] = N.StbLevelParams(est.num_iters, float(est.geom_weight),
                                      float(est.feat_weight), float(est.distance_threshold),
                                      float(est.normals_angle_thresh),
                                      float(est.feat_residual_thresh))
        return arr, sum(est.num_iters for est in levels)

    def prepare(self, sources, targets, source_feats=None, target_feats=None,
                transforms=None):
        """Device description of a batch (``BatchPlan``): the level table,
        the initial transforms, the workspace and the result buffers.
        ``sources`` / ``targets``: per pair, the list of level
        ``FramePointCloud`` (coarsest first); ``*_feats``: per pair the list
        of (C, H, W) maps or None.  ``run(plan)`` launches it; the plan can
        be launched again while its tensors hold new data of the same
        shapes."""
        B, L = len(sources), len(self.estimators)
        if B == 0 or len(targets) != B:
            raise ValueError("sources and targets must be non-empty lists of equal length")
        device = targets[0][0].points.device
        use_feat = source_feats is not None and target_feats is not None
        keep = []
        lv = (N.StbLevel * (B * L))()
        total_px = 0
        channels, code = 0, N.STB_F32
        for p in range(B):
            if len(sources[p]) != L or len(targets[p]) != L:
                raise ValueError(f"pair {p}: expected {L} levels")
            biggest = 0
            for l in range(L):
                src, tgt = sources[p][l], targets[p][l]
                sp = src.points.reshape(-1, 3).contiguous()
                sn = src.normals.reshape(-1, 3).contiguous()
                sm = src.mask.reshape(-1).to(torch.bool).contiguous()
                tp, tn = tgt.points.contiguous(), tgt.normals.contiguous()
                tm = tgt.mask.to(torch.bool).contiguous()
                for t in (sp, sn, tp, tn):
                    if t.dtype != torch.float32 or t.device != device:
                        raise RuntimeError("Check failed: points and normals must be float32 "
                                           f"tensors on {device}")
                h, w = tm.shape
                sf = tf = None
                if use_feat and source_feats[p] is not None and target_feats[p] is not None:
                    tf = target_feats[p][l].to(device).contiguous()
                    sf = source_feats[p][l].to(device).reshape(tf.size(0), -1).contiguous()
                    channels = tf.size(0)
                    code = N.feat_dtype_code(tf)
                    if channels > 1 and self.feat_layout == "auto":
                        # texel-major copies, kept alive by the plan
                        tf = processing.interleave_features(tf)
                        sf = processing.interleave_features(sf)
                        code += N.STB_F32_HWC
                keep += [sp, sn, sm, tp, tn, tm, sf, tf]
                fx, fy, cx, cy = tgt.kcam.params()
                lv[p * L + l] = N.StbLevel(
                    sp.data_ptr(), sn.data_ptr(), sm.data_ptr(), sp.size(0),
                    sf.data_ptr() if sf is not None else None, tp.data_ptr(), tn.data_ptr(),
                    tm.data_ptr(), h, w, tf.data_ptr() if tf is not None else None,
                    fx, fy, cx, cy)
                biggest = max(biggest, h * w)
            total_px += biggest
        plan = BatchPlan()
        plan.B, plan.L, plan.device = B, L, device
        plan.graphs = {}  # schedule -> CUDA graph of its launch sequence
        plan.levels = torch.frombuffer(bytearray(bytes(lv)), dtype=torch.uint8).to(device)
        plan.params, plan.total_iters = self._params()
        plan.channels, plan.code, plan.total_px = channels, code, total_px
        plan.init = None
        if transforms is not None:
            plan.init = torch.stack([torch.eye(4, dtype=torch.float64) if t is None else
                                     torch.as_tensor(t, dtype=torch.float64).cpu()
                                     for t in transforms]).to(device).contiguous()
        need = int(N.lib().stb_icp_batch_workspace_bytes(B, total_px))
        plan.ws = torch.empty(need, dtype=torch.uint8, device=device)
        plan.results = torch.empty(B, N.RES_SIZE, dtype=torch.float64, device=device)
        plan.history = None
        if self.record_history:
            plan.history = torch.zeros(B, max(plan.total_iters, 1), N.HIST_SIZE,
                                       dtype=torch.float64, device=device)
        plan.num_source = [sources[p][-1].mask.numel() for p in range(B)]
        plan.keep = keep
        plan.mode = ((0 if self.feat_channel_mode == "last" else 1)
                     | (N.OPT_DW_SOLVE if self.solve_precision == "dw" else 0))
        return plan

    def run(self, plan, tile_config=None, graph=False):
        """Enqueue ``plan`` on the current stream (one cooperative launch);
        returns (results (B, 96) device tensor, history or None).
        ``tile_config``: the schedule (see ``self.tile_config``), default the
        tuned one.  ``graph``: replay the launch sequence (barrier-word
        memset, the persistent kernel with every level and Gauss-Newton
        iteration of every pair, the status pass) as a CUDA graph captured
        on the plan's first call with this schedule; the plan's buffers are
        the graph's, so the results are the same."""
        cfg = int(self.tile_config if tile_config is None else tile_config)
        if graph:
            g = plan.graphs.get(cfg)
            if g is None:
                g = torch.cuda.CUDAGraph()
                cur = torch.cuda.current_stream(plan.device)
                side = torch.cuda.Stream(plan.device)
                side.wait_stream(cur)
                with torch.cuda.stream(side), torch.cuda.graph(g, stream=side):
                    self._launch(plan, cfg)
                cur.wait_stream(side)
                plan.graphs[cfg] = g
            g.replay()
            return plan.results, plan.history
        self._launch(plan, cfg)
        return plan.results, plan.history

    def _launch(self, plan, cfg):
        mode, arg = plan.mode, cfg
        if cfg >= GROUPED:
            mode, arg = mode | N.OPT_GROUPS, cfg - GROUPED
        with torch.cuda.device(plan.device):
            N.check(N.lib().stb_icp_estimate_batch(
                N.ptr(plan.levels), plan.B, plan.L, ctypes.cast(plan.params, ctypes.c_void_p),
                plan.channels, plan.code, mode, N.ptr(plan.init), plan.total_px,
                N.ptr(plan.ws), plan.ws.numel(), N.ptr(plan.results), N.ptr(plan.history),
                arg, N.stream_of(plan.device)))

    def autotune(self, plan, configs=TUNE_CONFIGS, reps=3):
        """Times ``plan`` under each schedule (lock-step kernel with its
        largest work item 0 -> 8192, 1..5 -> 512 ... 8192 pixels; grouped
        kernel with GROUPED + g for g groups) with CUDA events and keeps the
        fastest in ``self.tile_config``.  Returns {config: ms}."""
        stream = torch.cuda.current_stream(plan.device)
        times = {}
        for cfg in configs:
            self.run(plan, cfg)  # warm-up
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record(stream)
            for _ in range(reps):
                self.run(plan, cfg)
            ev[1].record(stream)
            ev[1].synchronize()
            times[cfg] = ev[0].elapsed_time(ev[1]) / reps
        self.tile_config = min(times, key=times.get)
        return times

    def launch(self, sources, targets, source_feats=None, target_feats=None,
               transforms=None):
        """``prepare`` + ``run``: returns (results (B, 96) device tensor,
        history or None, the plan, which keeps the inputs alive)."""
        plan = self.prepare(sources, targets, source_feats, target_feats, transforms)
        results, hist = self.run(plan)
        return results, hist, plan

    def results(self, plan):
        """Host ``RegistrationResult`` list of a launched plan (synchronises);
        raises when the kernel stopped early."""
        out = plan.results.cpu()
        if plan.history is not None:
            self.last_history = plan.history.cpu()
        res = [ICPOdometry._result(out[p], plan.num_source[p], torch.float32)
               for p in range(plan.B)]
        status = out[:, N.RES_STATUS].to(torch.int64)
        if bool(((status & (N.ST_TIMEOUT | N.ST_CAPACITY)) != 0).any()):
            raise RuntimeError("stb_icp_estimate_batch stopped early "
                               f"(status bits {int(status.max())})")
        return res

    def estimate_pyramids(self, sources, targets, source_feats=None, target_feats=None,
                          transforms=None):
        """Register every pair; returns a list of ``RegistrationResult``
        (the finest level's, as ``MultiscaleRegistration``)."""
        _, _, plan = self.launch(sources, targets, source_feats, target_feats, transforms)
        return self.results(plan)

    def pyramids(self, frames, device=None):
        """Device pyramids (coarsest first) of a list of ``Frame`` or
        ``FramePointCloud``."""
        device = resolve_device(device)
        out = []
        for f in frames:
            if isinstance(f, Frame):
                f = FramePointCloud.from_frame(f, device)
            out.append(f.pyramid(self.scales))
        return out

    def estimate_frames(self, source_frames, target_frames, source_feats=None,
                        target_feats=None, transforms=None, device=None):
        """``MultiscaleRegistration.estimate_frame`` for lists of frame pairs."""
        sp = self.pyramids(source_frames, device)
        tp = self.pyramids(target_frames, device)
        sfp = tfp = None
        if source_feats is not None and target_feats is not None:
            sfp = [feature_pyramid(f.to(sp[0][0].points.device), self.scales)
                   for f in source_feats]
            tfp = [feature_pyramid(f.to(sp[0][0].points.device), self.scales)
                   for f in target_feats]
        return self.estimate_pyramids(sp, tp, sfp, tfp, transforms)
