"""Pose estimation by autograd and BFGS, the reference's ``AutogradICP``
(``slamtb/registration/autogradicp.py:95-374``), on this package's kernels.

What is kept from the reference (its arguments, defaults and results):

* the pose is a twist ``x = [t; w]`` (``ExpRtToMatrix``);
* the cost is ``w_g * mean((n . (q - T s))^2)`` over the matched points plus
  ``w_f * robust(|f_t - f_s|)`` over the matched features whose squared norm
  is below ``feat_residual_thresh^2`` (``robust``: mean of the norms below
  ``huber_loss_alpha`` plus mean of ``alpha |r| - alpha`` above it, or the
  plain mean when ``huber_loss_alpha <= 0``), the matches being those of
  ``FramePointCloudMatcher`` at the current pose;
* scipy's BFGS minimises ``learning_rate * cost`` (``tol=1e-9``, at most
  ``num_iters`` iterations), then ``gradient_descent_iters`` plain gradient
  steps of size 0.1 on the unscaled cost start from the twist of BFGS's
  last evaluation and keep the twist of the lowest cost seen;
* the result: the 4x4 transform of the kept twist, the inverse of BFGS's
  inverse-Hessian estimate as information only when no descent steps run,
  the last cost evaluated as residual, match ratio 1.

How it is computed here: ``_TwistCost`` evaluates the cost and its
gradient on the device -- the twist map and its backward, the
correspondence map, the matcher forward and backward are kernels of
``libslamtb_gb300``; the loss terms are torch reductions -- and hands scipy
float64 numbers.  The descent refinement updates the twist in place.

Differences: CUDA tensors only (the reference evaluates the twist map on the
CPU); a registration without target features runs the geometric term alone
(the reference's matcher needs a feature map); the best-cost search starts
from +inf (the reference's sentinel is 5555, above any cost it meets);
``estimate_pcl`` needs the reference's k-d tree matcher, which is not part
of this package, and raises ``NotImplementedError``.
"""
import math

import numpy as np
import scipy.optimize
import torch

from ..camera import RigidTransform
from ..spatial.matching import FramePointCloudMatcher
from .result import RegistrationResult
from .se3 import ExpRtToMatrix, MatrixToExpRt


def robust_feature_cost(norms, alpha):
    """The reference's feature cost of residual norms (``autogradicp.py:60-90``):
    the mean of the norms below alpha plus the mean of alpha |r| - alpha over
    the others; a part with no element adds nothing (a plain 0 when both are
    empty)."""
    if alpha <= 0:
        return norms.mean()
    low = norms < alpha
    n_low = int(low.sum())
    n_high = norms.numel() - n_low
    cost = 0
    if n_low:
        cost = norms[low].sum() / n_low
    if n_high:
        cost = cost + (alpha * norms[~low].abs() - alpha).sum() / n_high
    return cost


class _TwistCost:
    """The registration cost of a twist on the device, for one source point
    set against one target frame."""

    def __init__(self, icp, points, normals, feats, matcher):
        self.icp = icp
        self.points, self.normals, self.feats = points, normals, feats
        self.matcher = matcher
        self.use_geom = icp.geom_weight > 0
        self.use_feat = icp.feat_weight > 0 and feats is not None
        self.last = math.inf   # the last cost evaluated (unscaled)
        self.last_x = None     # the twist it was evaluated at (float64 numpy)

    def __call__(self, twist):
        """Unscaled cost at ``twist`` (a (6,) tensor; differentiable), or a
        plain 0 when no term is enabled."""
        rigid = RigidTransform(ExpRtToMatrix.apply(twist))
        moved = rigid @ self.points
        q, n, f, hit = self.matcher.find_correspondences(moved,
                                                         rigid.transform_normals(self.normals))
        total = 0
        if self.use_geom:
            r = ((q - moved[hit]) * n).sum(dim=1)
            total = total + self.icp.geom_weight * (r * r).mean()
        if self.use_feat:
            norms = torch.linalg.vector_norm(f - self.feats[:, hit], dim=0)
            thr = self.icp.feat_residual_thresh
            if thr > 0:
                norms = norms[norms * norms < thr * thr]
            total = total + self.icp.feat_weight * robust_feature_cost(
                norms, self.icp.huber_loss_alpha)
        self.last = total
        self.last_x = twist.detach().double().cpu().numpy()
        return total

    def scaled_value_and_grad(self, x):
        """scipy's interface: (learning_rate * cost, its gradient) at the
        float64 twist x."""
        twist = torch.tensor(np.asarray(x, dtype=np.float64), dtype=self.points.dtype,
                             device=self.points.device, requires_grad=True)
        cost = self(twist)
        if not torch.is_tensor(cost):
            return 0.0, np.zeros(6)
        scaled = cost * self.icp.learning_rate
        scaled.backward()
        return float(scaled.detach()), twist.grad.double().cpu().numpy()


class AutogradICP:
    """ICP with the pose optimised by BFGS on autograd gradients
    (``autogradicp.py:95-140``; same arguments and defaults)."""

    def __init__(self, num_iters, learning_rate=0.01, geom_weight=0.5, feat_weight=0.5,
                 distance_threshold=0.1, normals_angle_thresh=math.pi / 8.0,
                 feat_residual_thresh=0.5, huber_loss_alpha=4.5, gradient_descent_iters=100):
        self.num_iters = num_iters
        self.geom_weight = geom_weight
        self.feat_weight = feat_weight
        self.learning_rate = learning_rate
        self.distance_threshold = distance_threshold
        self.normals_angle_thresh = normals_angle_thresh
        self.feat_residual_thresh = feat_residual_thresh
        self.huber_loss_alpha = huber_loss_alpha
        self.gradient_descent_iters = gradient_descent_iters

    def _register(self, cost, x0):
        """BFGS on the scaled cost from x0, then the descent refinement;
        returns (kept twist as a tensor, BFGS result or None, last cost)."""
        bfgs = scipy.optimize.minimize(cost.scaled_value_and_grad, x0, method="BFGS", jac=True,
                                       tol=1e-9, options=dict(disp=False,
                                                              maxiter=self.num_iters))
        dev, dt = cost.points.device, cost.points.dtype
        start = cost.last_x if cost.last_x is not None else np.asarray(x0, np.float64)
        x = torch.tensor(start, dtype=dt, device=dev)
        kept = x.clone()
        if self.gradient_descent_iters is None:
            return kept, bfgs, cost.last
        best = math.inf
        for _ in range(self.gradient_descent_iters):
            twist = x.clone().requires_grad_(True)
            value = cost(twist)
            if not torch.is_tensor(value):
                break
            value.backward()
            v = float(value.detach())
            if v < best:
                best, kept = v, x.clone()
            x = x - 0.1 * twist.grad
        return kept, None, cost.last

    def _estimate(self, source_points, source_normals, source_feats, target_matcher,
                  transform=None):
        dev, dt = source_points.device, source_points.dtype
        if transform is None:
            x0 = np.zeros(6)
        else:
            T = torch.as_tensor(transform).to(device=dev, dtype=dt)
            x0 = MatrixToExpRt.apply(T[:3, :4]).detach().double().cpu().numpy().reshape(6)
        cost = _TwistCost(self, source_points, source_normals, source_feats, target_matcher)
        twist, bfgs, last = self._register(cost, x0)
        M = ExpRtToMatrix.apply(twist).detach().cpu()
        transform = torch.eye(4, dtype=M.dtype)
        transform[:3, :4] = M[:3, :4]
        info = None
        if bfgs is not None:
            info = torch.from_numpy(np.linalg.inv(bfgs.hess_inv)).float()
        residual = float(last.detach()) if torch.is_tensor(last) else last
        return RegistrationResult(transform, info, residual, 1.0)

    def estimate(self, kcam, source_points, source_normals, source_mask, target_points=None,
                 target_mask=None, target_normals=None, target_feats=None, source_feats=None,
                 transform=None):
        """Registration of the masked source points against a target frame
        (``autogradicp.py:241-295``)."""
        keep = source_mask.reshape(-1).to(torch.bool)
        points = source_points.reshape(-1, 3)[keep]
        normals = source_normals.reshape(-1, 3)[keep]
        feats = None
        if source_feats is not None:
            feats = source_feats.reshape(source_feats.size(0), -1)[:, keep]
        if target_feats is None:
            target_feats = torch.zeros(0, *target_mask.shape, device=target_points.device)
        matcher = FramePointCloudMatcher(target_points, target_normals, target_mask,
                                         target_feats, kcam, self.distance_threshold,
                                         self.normals_angle_thresh)
        return self._estimate(points, normals, feats, matcher, transform)

    def estimate_pcl(self, source_pcl, target_pcl, transform=None, source_feats=None,
                     target_feats=None):
        raise NotImplementedError(
            "AutogradICP.estimate_pcl uses the reference's k-d tree point-cloud matcher, "
            "which slamtb_gb300 does not provide")

    def estimate_frame(self, source_frame, target_frame, source_feats=None, target_feats=None,
                       transform=None, device=None):
        """Registration between two frames (``autogradicp.py:335-374``)."""
        from ..frame import Frame, FramePointCloud, resolve_device
        device = resolve_device(device)
        frames = []
        for f in (source_frame, target_frame):
            frames.append(FramePointCloud.from_frame(f, device) if isinstance(f, Frame) else f)
        src, tgt = frames
        return self.estimate(src.kcam, src.points, src.normals, src.mask,
                             target_points=tgt.points, target_mask=tgt.mask,
                             target_normals=tgt.normals, target_feats=target_feats,
                             source_feats=source_feats, transform=transform)
