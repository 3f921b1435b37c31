"""Differentiable point-to-plane loss with a hand-written adjoint.

``PointToPlaneLoss`` is a ``torch.autograd.Function`` over a batch of frame
pairs: forward = the ICP association at ``exp(twist) @ pose`` and
``L_p = sum r^2`` (``stb_icp_loss_forward``); backward = the adjoint kernel
(``stb_icp_loss_backward``) giving dL/dtwist (left perturbation, twist
ordered [translation; rotation]) and dL/d(source depth) per pixel, with the
correspondences of the forward pass held fixed.  Source normals only gate
the association and get no gradient.

The reference differentiates its registration through PyTorch ops and a
custom matcher (``slamtb/registration/autogradicp.py:145-239``,
``src/fpcl_matcher.cu:197-229``); here the whole loss and its adjoint are
two kernels per direction for the batch.

The kernels differentiate with respect to the left perturbation
``exp(e) @ exp(twist) @ pose`` at e = 0; ``stb_se3_twist_grad`` maps that
to the gradient with respect to ``twist`` itself through the SE(3) left
Jacobian (the identity at twist = 0).
"""
import ctypes

import torch

from .. import _native as N
from .. import processing


def se3_exp_compose(twist, base):
    """exp(twist) @ base for (B, 6) float64 twists and (B, 4, 4) poses, on
    the device in FP64."""
    twist = twist.detach().to(torch.float64).contiguous()
    base = base.detach().to(device=twist.device, dtype=torch.float64).contiguous()
    out = torch.empty(twist.size(0), 4, 4, dtype=torch.float64, device=twist.device)
    with torch.cuda.device(twist.device):
        N.check(N.lib().stb_se3_exp_compose(N.ptr(twist), N.ptr(base), N.ptr(out),
                                            twist.size(0), N.stream_of(twist.device)))
    return out


class _State:
    def __init__(self):
        self.ws = None


def _levels(points, normals, smask, tpoints, tnormals, tmask, kcam):
    B, H, W = tmask.shape
    fx, fy, cx, cy = kcam
    arr = (N.StbLevel * B)()
    for p in range(B):
        arr[p] = N.StbLevel(points[p].data_ptr(), normals[p].data_ptr(), smask[p].data_ptr(),
                            H * W, None, tpoints[p].data_ptr(), tnormals[p].data_ptr(),
                            tmask[p].data_ptr(), H, W, None, fx, fy, cx, cy)
    return torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(tmask.device)


class PointToPlaneLoss(torch.autograd.Function):
    """loss (B,) float64 = PointToPlaneLoss.apply(twist, source_depth,
    source_normals, source_mask, target_points, target_normals, target_mask,
    kcam, poses, distance_threshold, normals_angle_thresh)

    twist: (B, 6) float64; source_depth: (B, H, W) float32 (metres);
    source_normals / target_points / target_normals: (B, H, W, 3) float32;
    masks: (B, H, W) bool; kcam: (fx, fy, cx, cy) shared by source and
    target; poses: (B, 4, 4) float64, the loss is evaluated at
    exp(twist) @ poses."""

    @staticmethod
    def forward(ctx, twist, source_depth, source_normals, source_mask, target_points,
                target_normals, target_mask, kcam, poses, distance_threshold,
                normals_angle_thresh):
        dev = source_depth.device
        B, H, W = source_depth.shape
        T = se3_exp_compose(twist, poses)
        kmat = torch.tensor([[kcam[0], 0, kcam[2]], [0, kcam[1], kcam[3]], [0, 0, 1]],
                            dtype=torch.float32)
        pts = torch.stack([processing.depth_to_points(source_depth[p].detach(), kmat)[0]
                           for p in range(B)]).contiguous()
        keep = [pts, source_normals.contiguous(), source_mask.to(torch.bool).contiguous(),
                target_points.contiguous(), target_normals.contiguous(),
                target_mask.to(torch.bool).contiguous()]
        levels = _levels(*keep, kcam)
        need = int(N.lib().stb_icp_loss_workspace_bytes(B, H * W))
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        loss = torch.empty(B, dtype=torch.float64, device=dev)
        with torch.cuda.device(dev):
            N.check(N.lib().stb_icp_loss_forward(
                N.ptr(levels), B, N.ptr(T), float(distance_threshold),
                float(normals_angle_thresh), H * W, N.ptr(ws), need, N.ptr(loss),
                N.stream_of(dev)))
        ctx.keep = keep + [levels, ws, T, twist.detach().to(torch.float64).contiguous()]
        ctx.shape = (B, H, W)
        return loss

    @staticmethod
    def backward(ctx, grad_loss):
        B, H, W = ctx.shape
        levels, ws, T, twist = ctx.keep[-4:]
        dev = ws.device
        g = grad_loss.detach().to(device=dev, dtype=torch.float64).contiguous()
        grad_tangent = torch.empty(B, 6, dtype=torch.float64, device=dev)
        grad_twist = torch.empty(B, 6, dtype=torch.float64, device=dev)
        grad_depth = torch.empty(B, H, W, dtype=torch.float32, device=dev)
        ptrs = torch.tensor([grad_depth[p].data_ptr() for p in range(B)], dtype=torch.int64,
                            device=dev)
        with torch.cuda.device(dev):
            N.check(N.lib().stb_icp_loss_backward(
                N.ptr(levels), B, N.ptr(T), N.ptr(g), H * W, N.ptr(ws), ws.numel(),
                N.ptr(grad_tangent), N.ptr(ptrs), N.stream_of(dev)))
            N.check(N.lib().stb_se3_twist_grad(N.ptr(twist), N.ptr(grad_tangent),
                                               N.ptr(grad_twist), B, N.stream_of(dev)))
        return (grad_twist, grad_depth) + (None,) * 9


def point_to_plane_loss(twist, source_depth, source_normals, source_mask, target_points,
                        target_normals, target_mask, kcam, poses, distance_threshold=0.1,
                        normals_angle_thresh=0.349):
    """Functional form of ``PointToPlaneLoss``."""
    return PointToPlaneLoss.apply(twist, source_depth, source_normals, source_mask,
                                  target_points, target_normals, target_mask, kcam, poses,
                                  distance_threshold, normals_angle_thresh)
