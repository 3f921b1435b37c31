"""Differentiable twist <-> rigid matrix layers (``slamtb/registration/se3.py:13-134``).

A twist is ``[t; w]``: the translation and the rotation axis times its
angle.  ``ExpRtToMatrix`` maps it to the 3x4 matrix ``[R(w) | t]`` (Rodrigues)
and back-propagates with the rotation derivative of Gallego and Yezzi;
``MatrixToExpRt`` is the inverse map (no backward, as the reference).  Both
run as CUDA kernels of ``libslamtb_gb300`` on float32 or float64 tensors.
"""
import torch

from .. import _native as N


def _code(t):
    if t.dtype == torch.float32:
        return N.STB_F32
    if t.dtype == torch.float64:
        return N.STB_F64
    raise RuntimeError(f"Check failed: expected float32 or float64, got {t.dtype}")


def _cuda(t, name):
    if not t.is_cuda:
        raise RuntimeError(f"Check failed: {name}: Expected a gpu tensor "
                           "(slamtb_gb300 runs on CUDA devices only)")
    return t


class ExpRtToMatrix(torch.autograd.Function):
    """[t; w] ([6] or [B, 6]) -> [R(w) | t] ([3, 4] or [B, 3, 4])."""

    @staticmethod
    def forward(ctx, exp_rt):
        x = _cuda(exp_rt, "exp_rt").detach().reshape(-1, 6).contiguous()
        m = torch.empty(x.size(0), 3, 4, dtype=x.dtype, device=x.device)
        with torch.cuda.device(x.device):
            N.check(N.lib().stb_exp_rt_to_matrix(N.ptr(x), N.ptr(m), x.size(0), _code(x),
                                                 N.stream_of(x.device)))
        ctx.save_for_backward(x, m)
        ctx.single = exp_rt.dim() == 1
        return m.squeeze(0) if ctx.single else m

    @staticmethod
    def backward(ctx, d_matrix):
        x, m = ctx.saved_tensors
        g = d_matrix.reshape(-1, 3, 4).to(dtype=x.dtype).contiguous()
        d = torch.empty(x.size(0), 6, dtype=x.dtype, device=x.device)
        with torch.cuda.device(x.device):
            N.check(N.lib().stb_exp_rt_to_matrix_backward(
                N.ptr(g), N.ptr(x), N.ptr(m), N.ptr(d), x.size(0), _code(x),
                N.stream_of(x.device)))
        return d.squeeze(0) if ctx.single else d


class MatrixToExpRt(torch.autograd.Function):
    """[R | t] ([3, 4] or [B, 3, 4]) -> [t; w] ([6] or [B, 6]).  The
    reference returns nothing for a batched input (``se3.py:111-116``);
    here both shapes return their twists."""

    @staticmethod
    def forward(ctx, matrix):
        m = _cuda(matrix, "matrix").detach()[..., :3, :4].reshape(-1, 3, 4).contiguous()
        x = torch.empty(m.size(0), 6, dtype=m.dtype, device=m.device)
        with torch.cuda.device(m.device):
            N.check(N.lib().stb_matrix_to_exp_rt(N.ptr(m), N.ptr(x), m.size(0), _code(m),
                                                 N.stream_of(m.device)))
        return x.squeeze(0) if matrix.dim() == 2 else x

    @staticmethod
    def backward(ctx, d_exp_rt_loss):
        raise NotImplementedError()
