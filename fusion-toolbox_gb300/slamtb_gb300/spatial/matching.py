"""Differentiable frame point-cloud matcher (``slamtb/spatial/matching.py:10-124``).

``FPCLMatcherOp`` matches source points (already in the target camera's
frame) against a target frame by projection: a point matches when it wins
its pixel of the correspondence map computed at the identity pose.  It
returns the bilinear feature samples of the matches; the backward pass
gives the gradient with respect to the source points (features' central
differences through the projection's Jacobian).  The target points and
normals of the matches are side outputs without gradient, as in the
reference.  Both passes are CUDA kernels of ``libslamtb_gb300``
(``stb_fpcl_match_forward`` / ``stb_fpcl_match_backward``); float32.
"""
import math

import torch

from .. import _native as N
from ..registration.correspondence_map import CorrespondenceMap


def _kcam(kcam, device):
    m = kcam.matrix if hasattr(kcam, "matrix") else kcam
    return torch.as_tensor(m).to(device=device, dtype=torch.float32).contiguous()


class FPCLMatcherOp(torch.autograd.Function):
    """``FPCLMatcherOp`` (``matching.py:10-87``)."""

    class Target:
        def __init__(self, points, normals, mask, features, kcam,
                     distance_threshold, normals_angle_thresh):
            self.points = points
            self.normals = normals
            self.mask = mask
            self.features = features
            self.kcam = kcam
            self.distance_threshold = distance_threshold
            self.normals_angle_thresh = normals_angle_thresh

    class Match:
        def __init__(self):
            self.points = None
            self.normals = None
            self.features = None
            self.mask = None

    @staticmethod
    def forward(ctx, source_points, source_normals, target, match, grad_precision=0.005):
        device = source_points.device
        if not source_points.is_cuda:
            raise RuntimeError("Check failed: source_points: Expected a gpu tensor "
                               "(slamtb_gb300 runs on CUDA devices only)")
        sp = source_points.detach().reshape(-1, 3).to(torch.float32).contiguous()
        size = sp.size(0)
        kcam = _kcam(target.kcam, device)
        corresp_map = CorrespondenceMap(target.distance_threshold, target.normals_angle_thresh)(
            sp, source_normals.detach().reshape(-1, 3).to(torch.float32),
            torch.ones(1, dtype=torch.bool, device=device),
            torch.eye(4, dtype=torch.float32, device=device),
            target.points, target.normals, target.mask, kcam)
        tf = target.features.to(device=device, dtype=torch.float32).contiguous()
        channels, h, w = tf.shape
        tp = target.points.to(torch.float32).contiguous()
        tn = target.normals.to(torch.float32).contiguous()
        match.points = torch.empty(size, 3, device=device, dtype=torch.float32)
        match.normals = torch.empty(size, 3, device=device, dtype=torch.float32)
        match.features = torch.empty(channels, size, device=device, dtype=torch.float32)
        match.mask = torch.empty(size, device=device, dtype=torch.bool)
        with torch.cuda.device(device):
            N.check(N.lib().stb_fpcl_match_forward(
                N.ptr(tp), N.ptr(tn), N.ptr(tf), channels, h, w, N.ptr(sp), size,
                N.ptr(kcam), N.ptr(corresp_map), N.ptr(match.points), N.ptr(match.normals),
                N.ptr(match.features), N.ptr(match.mask), N.STB_F32, N.stream_of(device)))
        ctx.target_features = tf
        ctx.kcam = kcam
        ctx.save_for_backward(sp, match.mask)
        ctx.grad_precision = float(grad_precision)
        return match.features

    @staticmethod
    def backward(ctx, dl_features):
        sp, mask = ctx.saved_tensors
        tf = ctx.target_features
        channels, h, w = tf.shape
        dl = dl_features.to(torch.float32).contiguous()
        dx = torch.empty(sp.size(0), 3, device=sp.device, dtype=torch.float32)
        with torch.cuda.device(sp.device):
            N.check(N.lib().stb_fpcl_match_backward(
                N.ptr(tf), channels, h, w, N.ptr(sp), sp.size(0), N.ptr(mask), N.ptr(dl),
                N.ptr(ctx.kcam), ctx.grad_precision, N.ptr(dx), N.STB_F32,
                N.stream_of(sp.device)))
        # one gradient per argument given to apply (grad_precision is optional)
        return (dx,) + (None,) * (len(ctx.needs_input_grad) - 1)


class FramePointCloudMatcher:
    """Differentiable layer matching points against an RGB-D frame
    (``matching.py:90-124``)."""

    def __init__(self, target_points, target_normals, target_mask, target_features, kcam,
                 distance_threshold=1.0, normals_angle_thresh=math.pi):
        self.target = FPCLMatcherOp.Target(
            target_points, target_normals, target_mask, target_features, kcam,
            distance_threshold, normals_angle_thresh)

    @classmethod
    def from_frame_pcl(cls, target_fpcl, features):
        return cls(target_fpcl.points, target_fpcl.normals, target_fpcl.mask, features,
                   target_fpcl.kcam)

    def find_correspondences(self, source_points, source_normals):
        """(target points, target normals, sampled features, mask) of the
        matched source points."""
        match = FPCLMatcherOp.Match()
        FPCLMatcherOp.apply(source_points, source_normals, self.target, match)
        return (match.points[match.mask, :], match.normals[match.mask, :],
                match.features[:, match.mask], match.mask)
