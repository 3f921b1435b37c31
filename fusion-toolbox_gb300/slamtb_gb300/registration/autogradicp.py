"""Pose estimation by autograd and BFGS (``slamtb/registration/autogradicp.py:1-374``).

The reference's algorithm as written: the pose is a twist ``[t; w]``; a
closure maps it to a matrix (``ExpRtToMatrix``), transforms the source
points, matches them against the target frame (``FramePointCloudMatcher``)
and evaluates the mean squared point-to-plane residual plus the Huber
feature residual.  scipy's BFGS minimises it (``num_iters`` iterations),
then ``gradient_descent_iters`` SGD steps keep the best twist.  The twist,
the transform and the matcher's work stay on the GPU; every kernel is one
of ``libslamtb_gb300`` (the twist map, the correspondence map, the matcher
and its backward) or a torch elementwise operation of the loss.

Differences: CUDA tensors only (the reference converts the twist on the
CPU); a registration without target features runs the geometric term
alone (the reference's matcher needs a feature map); ``estimate_pcl`` needs
the reference's k-d tree matcher, which is not part of this package, and
raises ``NotImplementedError``.
"""
import math

import numpy as np
import scipy.optimize
import torch

from ..camera import RigidTransform
from ..spatial.matching import FramePointCloudMatcher
from .result import RegistrationResult
from .se3 import ExpRtToMatrix, MatrixToExpRt


def _to_4x4(mtx):
    if mtx.size(0) == 4 and mtx.size(1) == 4:
        return mtx
    ret = torch.eye(4, device=mtx.device, dtype=mtx.dtype)
    ret[:3, :4] = mtx[:3, :4]
    return ret


class _ClosureBox:
    """scipy's view of the closure: value and 6-D gradient at x."""

    def __init__(self, closure, x):
        self.closure = closure
        self.x = x

    def func(self, x):
        with torch.no_grad():
            self.x.copy_(torch.from_numpy(np.asarray(x, dtype=np.float64)))
        loss = self.closure()
        if not torch.is_tensor(loss):
            return 0.0, np.zeros(6)
        value = loss.detach().cpu().item()
        loss.backward()
        return value, self.x.grad.cpu().numpy().astype(np.float64)


class _HuberLoss(torch.nn.Module):
    """The reference's feature loss (``autogradicp.py:60-90``): mean of the
    residuals below alpha plus mean of alpha |r| - alpha above it."""

    def __init__(self, alpha):
        super().__init__()
        self.alpha = alpha

    def forward(self, residual):
        loss1 = residual[residual < self.alpha]
        loss2 = residual[residual >= self.alpha]
        loss2 = self.alpha * torch.abs(loss2) - self.alpha
        loss = 0
        if loss1.numel() > 0:
            loss = loss1.mean()
        if loss2.numel() > 0:
            loss = loss + loss2.mean()
        return loss


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

    def _estimate(self, source_points, source_normals, source_feats, target_matcher,
                  transform=None):
        device = source_points.device
        dtype = source_points.dtype
        if transform is None:
            exp_rt = torch.zeros(6, device=device, dtype=dtype, requires_grad=True)
        else:
            init = torch.as_tensor(transform).to(device=device, dtype=dtype)
            exp_rt = MatrixToExpRt.apply(init[:3, :4]).detach().requires_grad_(True)
        loss = math.inf
        has_geom = self.geom_weight > 0
        has_feat = self.feat_weight > 0 and source_feats is not None
        huber_loss = _HuberLoss(self.huber_loss_alpha)

        def _closure():
            nonlocal loss
            if exp_rt.grad is not None:
                exp_rt.grad.zero_()
            geom_loss = 0
            feat_loss = 0
            rigid = RigidTransform(ExpRtToMatrix.apply(exp_rt))
            tsp = rigid @ source_points
            tpoints, tnormals, tfeatures, smask = target_matcher.find_correspondences(
                tsp, rigid.transform_normals(source_normals))
            if has_geom:
                diff = tpoints - tsp[smask]
                cost = torch.bmm(tnormals.view(-1, 1, 3), diff.view(-1, 3, 1)).squeeze()
                geom_loss = torch.pow(cost, 2).mean()
            if has_feat:
                feat_diff = torch.norm(tfeatures - source_feats[:, smask], 2, dim=0)
                if self.feat_residual_thresh > 0:
                    feat_diff = feat_diff[feat_diff.pow(2) < self.feat_residual_thresh
                                          * self.feat_residual_thresh]
                if self.huber_loss_alpha > 0:
                    feat_loss = huber_loss(feat_diff)
                else:
                    feat_loss = feat_diff.mean()
            loss = geom_loss * self.geom_weight + feat_loss * self.feat_weight
            if torch.is_tensor(loss) and torch.isnan(loss):
                return loss
            return loss * self.learning_rate

        box = _ClosureBox(_closure, exp_rt)
        opt_res = scipy.optimize.minimize(box.func, exp_rt.detach().cpu().numpy(),
                                          method="BFGS", jac=True, tol=1e-9,
                                          options=dict(disp=False, maxiter=self.num_iters))
        best_exp_rt = exp_rt.detach().clone()
        best_residual = 5555
        if self.gradient_descent_iters is not None:
            opt = torch.optim.SGD([exp_rt], 0.1)
            opt_res = None
            for _ in range(self.gradient_descent_iters):
                opt.zero_grad()
                _closure()
                if not torch.is_tensor(loss):
                    break
                loss.backward()
                tmp = loss.detach().cpu().item()
                if tmp < best_residual:
                    best_residual = tmp
                    best_exp_rt = exp_rt.detach().clone()
                opt.step()
        transform = _to_4x4(ExpRtToMatrix.apply(best_exp_rt).cpu())
        info = None
        if opt_res is not None:
            info = torch.from_numpy(np.linalg.inv(opt_res.hess_inv)).float()
        residual = float(loss.detach()) if torch.is_tensor(loss) else loss
        return RegistrationResult(transform, info, residual, 1.0)

    def estimate(self, kcam, source_points, source_normals, source_mask, target_points=None,
                 target_mask=None, target_normals=None, target_feats=None, source_feats=None,
                 transform=None):
        """Registration of masked source points against a target frame
        (``autogradicp.py:241-295``)."""
        source_points = source_points[source_mask].view(-1, 3)
        source_normals = source_normals[source_mask].view(-1, 3)
        if source_feats is not None:
            source_feats = source_feats[:, source_mask].view(source_feats.size(0), -1)
        if target_feats is None:
            target_feats = torch.zeros(0, *target_mask.shape, device=target_points.device)
        matcher = FramePointCloudMatcher(target_points, target_normals, target_mask,
                                         target_feats, kcam, self.distance_threshold,
                                         self.normals_angle_thresh)
        return self._estimate(source_points, source_normals, source_feats, matcher, transform)

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
        if isinstance(source_frame, Frame):
            source_frame = FramePointCloud.from_frame(source_frame, device)
        if isinstance(target_frame, Frame):
            target_frame = FramePointCloud.from_frame(target_frame, device)
        return self.estimate(source_frame.kcam, source_frame.points.view(-1, 3),
                             source_frame.normals.view(-1, 3), source_frame.mask.view(-1),
                             source_feats=None if source_feats is None
                             else source_feats.reshape(source_feats.size(0), -1),
                             target_points=target_frame.points,
                             target_mask=target_frame.mask,
                             target_normals=target_frame.normals,
                             target_feats=target_feats, transform=transform)
