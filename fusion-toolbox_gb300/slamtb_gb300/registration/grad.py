"""Differentiable point-to-plane loss with a hand-written adjoint.

``PointToPlaneLoss`` is a ``torch.autograd.Function`` over a batch of frame
pairs: forward = the ICP association at ``exp(twist) @ pose`` and
``L_p = sum r^2``; when the twist or the depth needs a gradient, the same
pass also evaluates the hand-written adjoint at a unit output gradient
(``stb_icp_loss_forward_adjoint``: dL_p/d(source depth) per pixel and the
gradient with respect to the left perturbation of the pose), so backward
only scales it by grad_loss (``stb_icp_loss_scale_adjoint``) and
``stb_se3_twist_grad`` maps the pose part through the SE(3) left Jacobian to
dL/dtwist (twist ordered [translation; rotation]).  Without gradients the
forward is ``stb_icp_loss_forward`` alone; ``stb_icp_loss_backward`` is the
same adjoint as a separate pass for callers of the C ABI.  The
correspondences of the forward pass are held fixed; source normals only
gate the association and get no gradient.

The reference differentiates its registration through PyTorch ops and a
custom matcher (``slamtb/registration/autogradicp.py:145-239``,
``src/fpcl_matcher.cu:197-229``); here the loss and its adjoint are two kernels
for the batch, reading dense (B, H, W) arrays, and the backward one
elementwise kernel.
"""
import contextlib

import torch

from .. import _native as N


def _on(dev):
    """The device context for the library's calls, entered only when dev is
    not already current (entering and leaving costs host time every step)."""
    return (contextlib.nullcontext() if dev.index == torch.cuda.current_device()
            else torch.cuda.device(dev))


def _exp_compose(twist, base, stream):
    """exp(twist) @ base into a new (B, 4, 4) tensor; twist float64
    contiguous on the device, stream the caller's."""
    base = base.detach().to(device=twist.device, dtype=torch.float64).contiguous()
    out = torch.empty(twist.size(0), 4, 4, dtype=torch.float64, device=twist.device)
    N.check(N.lib().stb_se3_exp_compose(N.ptr(twist), N.ptr(base), N.ptr(out), twist.size(0),
                                        stream))
    return out


def se3_exp_compose(twist, base):
    """exp(twist) @ base for (B, 6) float64 twists and (B, 4, 4) poses, on
    the device in FP64."""
    twist = twist.detach().to(torch.float64).contiguous()
    with _on(twist.device):
        return _exp_compose(twist, base, N.stream_of(twist.device))


_WS_BYTES = {}


def _workspace_bytes(B, H, W):
    key = (B, H, W)
    n = _WS_BYTES.get(key)
    if n is None:
        n = _WS_BYTES[key] = int(N.lib().stb_icp_loss_workspace_bytes(B, H, W))
    return n


def _f32(name, t, shape):
    if t.dtype != torch.float32 or t.device.type != "cuda" or tuple(t.shape) != shape:
        raise RuntimeError(f"Check failed: {name} must be a float32 CUDA tensor of shape {shape}")
    return t.contiguous()


def _mask(name, t, shape):
    if t.device.type != "cuda" or tuple(t.shape) != shape:
        raise RuntimeError(f"Check failed: {name} must be a CUDA tensor of shape {shape}")
    return t.to(torch.bool).contiguous()


class PointToPlaneLoss(torch.autograd.Function):
    """loss (B,) float64 = PointToPlaneLoss.apply(twist, source_depth,
    source_normals, source_mask, target_points, target_normals, target_mask,
    kcam, poses, distance_threshold, normals_angle_thresh)

    twist: (B, 6) float64; source_depth: (B, H, W) float32 (metres);
    source_normals / target_points / target_normals: (B, H, W, 3) float32;
    masks: (B, H, W) bool; kcam: (fx, fy, cx, cy) shared by every frame;
    poses: (B, 4, 4) float64, the loss is evaluated at exp(twist) @ poses."""

    @staticmethod
    def forward(ctx, twist, source_depth, source_normals, source_mask, target_points,
                target_normals, target_mask, kcam, poses, distance_threshold,
                normals_angle_thresh):
        B, H, W = source_depth.shape
        dev = source_depth.device
        ins = [_f32("source_depth", source_depth.detach(), (B, H, W)),
               _f32("source_normals", source_normals, (B, H, W, 3)),
               _mask("source_mask", source_mask, (B, H, W)),
               _f32("target_points", target_points, (B, H, W, 3)),
               _f32("target_normals", target_normals, (B, H, W, 3)),
               _mask("target_mask", target_mask, (B, H, W))]
        tw = twist.detach().to(device=dev, dtype=torch.float64).contiguous()
        need = _workspace_bytes(B, H, W)
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        loss = torch.empty(B, dtype=torch.float64, device=dev)
        k = tuple(float(x) for x in kcam)
        want_twist, want_depth = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        with _on(dev):
            st = N.stream_of(dev)
            T = _exp_compose(tw, poses, st)
            if not (want_twist or want_depth):
                N.check(N.lib().stb_icp_loss_forward(
                    *[N.ptr(t) for t in ins], B, H, W, *k, N.ptr(T),
                    float(distance_threshold), float(normals_angle_thresh), N.ptr(ws), need,
                    N.ptr(loss), st))
                return loss
            # the adjoint at a unit output gradient in the same pass: the
            # backward only scales it by grad_loss
            tangent = torch.empty(B, 6, dtype=torch.float64, device=dev)
            dadj = (torch.empty(B, H, W, dtype=torch.float32, device=dev)
                    if want_depth else None)
            N.check(N.lib().stb_icp_loss_forward_adjoint(
                *[N.ptr(t) for t in ins], B, H, W, *k, N.ptr(T), float(distance_threshold),
                float(normals_angle_thresh), N.ptr(ws), need, N.ptr(loss), N.ptr(tangent),
                N.ptr(dadj), st))
        ctx.keep = (tw, tangent, dadj, B, H, W)
        return loss

    @staticmethod
    def backward(ctx, grad_loss):
        tw, tangent, dadj, B, H, W = ctx.keep
        dev = tangent.device
        g = grad_loss.detach().to(device=dev, dtype=torch.float64).contiguous()
        grad_tangent = torch.empty(B, 6, dtype=torch.float64, device=dev)
        grad_twist = torch.empty(B, 6, dtype=torch.float64, device=dev)
        grad_depth = (torch.empty(B, H, W, dtype=torch.float32, device=dev)
                      if dadj is not None else None)
        with _on(dev):
            st = N.stream_of(dev)
            N.check(N.lib().stb_icp_loss_scale_adjoint(
                N.ptr(g), N.ptr(tangent), N.ptr(dadj), B, H, W, N.ptr(grad_tangent),
                N.ptr(grad_depth), st))
            N.check(N.lib().stb_se3_twist_grad(N.ptr(tw), N.ptr(grad_tangent),
                                               N.ptr(grad_twist), B, st))
        return (grad_twist, grad_depth) + (None,) * 9


def point_to_plane_loss(twist, source_depth, source_normals, source_mask, target_points,
                        target_normals, target_mask, kcam, poses, distance_threshold=0.1,
                        normals_angle_thresh=0.349):
    """Functional form of ``PointToPlaneLoss``."""
    return PointToPlaneLoss.apply(twist, source_depth, source_normals, source_mask,
                                  target_points, target_normals, target_mask, kcam, poses,
                                  distance_threshold, normals_angle_thresh)
