"""ctypes binding of ``libslamtb_gb300.so`` (declared in
``include/slamtb_gb300.h``).

The library is the only compute path: when it is missing, every call
raises ``RuntimeError``; there is no CPU or PyTorch fallback.
"""
import ctypes
import re

import torch

from . import _build

STB_OK = 0
STB_EINVAL, STB_EDEVICE, STB_EDTYPE, STB_ECUDA, STB_ETIMEOUT = 1, 2, 3, 4, 5
STB_F32 = 0
STB_BF16 = 1
STB_F32_HWC = 2   # texel-major feature layout [count][channels]
STB_BF16_HWC = 3
STB_F64, STB_U8, STB_I16, STB_U16, STB_I32, STB_I64 = 4, 5, 6, 7, 8, 9

# result block layout (doubles), see the header
RES_TRANSFORM, RES_JTJ, RES_INFO = 0, 16, 52
RES_RESIDUAL, RES_MATCHES, RES_ITERS, RES_STATUS, RES_SIZE = 88, 89, 90, 91, 96
HIST_TRANSFORM, HIST_JTJ, HIST_JR, HIST_R2 = 0, 16, 52, 58
HIST_GEOM_COUNT, HIST_FEAT_COUNT, HIST_OK, HIST_SIZE = 59, 60, 61, 64
ST_NOT_PD, ST_NO_MATCHES, ST_NAN = 1, 2, 4
# option bits or-ed into the channel_mode argument of the registration calls
OPT_DW_SOLVE = 0x100
OPT_MULTI_LAUNCH = 0x200
OPT_GROUPS = 0x400

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32
_f32 = ctypes.c_float
_f64 = ctypes.c_double
_sz = ctypes.c_size_t

_SIGNATURES = {
    "stb_last_error": (ctypes.c_char_p, []),
    "stb_version": (ctypes.c_char_p, []),
    "stb_correspondence_map": (ctypes.c_int, [
        _vp, _vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _i32, _i32, _vp, _vp,
        _f64, _f64, _vp]),
    "stb_icp_jacobian_geometric": (ctypes.c_int, [
        _vp, _vp, _i64, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp,
        _vp, _vp]),
    "stb_icp_jacobian_feature": (ctypes.c_int, [
        _vp, _vp, _vp, _i64, _vp, _vp, _i32, _i32, _i32, _i32, _vp, _vp, _f32,
        _vp, _vp, _vp, _vp, _vp]),
    "stb_icp_jacobian_feature_so3": (ctypes.c_int, [
        _vp, _vp, _vp, _i64, _vp, _vp, _i32, _i32, _i32, _i32, _vp, _vp, _f32,
        _vp, _vp, _vp, _vp, _vp]),
    "stb_icp_information_partials": (ctypes.c_int, [
        _vp, _vp, _i64, _vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp]),
    "stb_icp_workspace_bytes": (_sz, [_i64, _i32, _i32]),
    "stb_icp_correspondences": (ctypes.c_int, [_vp, _i32, _i32, _i32, _vp, _vp]),
    "stb_icp_batch_correspondences": (ctypes.c_int, [_vp, _i32, _i64, _i32, _i32, _i32, _i32,
                                                     _vp, _vp]),
    "stb_icp_loss_correspondences": (ctypes.c_int, [_vp, _i32, _i32, _i32, _vp, _vp]),
    "stb_icp_batch_workspace_bytes": (_sz, [_i32, _i64]),
    "stb_icp_estimate_batch": (ctypes.c_int, [
        _vp, _i32, _i32, _vp, _i32, _i32, _i32, _vp, _i64, _vp, _sz, _vp, _vp, _i32, _vp]),
    "stb_feature_interleave": (ctypes.c_int, [_vp, _vp, _i32, _i64, _i32, _vp]),
    "stb_bilateral_depth_filter": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _f32,
                                                  _f32, _f32, _vp]),
    "stb_exp_rt_to_matrix": (ctypes.c_int, [_vp, _vp, _i64, _i32, _vp]),
    "stb_exp_rt_to_matrix_backward": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "stb_matrix_to_exp_rt": (ctypes.c_int, [_vp, _vp, _i64, _i32, _vp]),
    "stb_fpcl_match_forward": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _i64, _vp,
                                              _vp, _vp, _vp, _vp, _vp, _i32, _vp]),
    "stb_fpcl_match_backward": (ctypes.c_int, [_vp, _i32, _i32, _i32, _vp, _i64, _vp, _vp, _vp,
                                               _f64, _vp, _i32, _vp]),
    "stb_se3_exp_compose": (ctypes.c_int, [_vp, _vp, _vp, _i32, _vp]),
    "stb_se3_twist_grad": (ctypes.c_int, [_vp, _vp, _vp, _i32, _vp]),
    "stb_icp_loss_workspace_bytes": (_sz, [_i32, _i32, _i32]),
    "stb_icp_loss_forward": (ctypes.c_int, [_vp] * 6 + [_i32] * 3 + [_f32] * 4 + [
        _vp, _f64, _f64, _vp, _sz, _vp, _vp]),
    "stb_icp_loss_backward": (ctypes.c_int, [_vp] * 6 + [_i32] * 3 + [_f32] * 4 + [
        _vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    "stb_icp_loss_forward_adjoint": (ctypes.c_int, [_vp] * 6 + [_i32] * 3 + [_f32] * 4 + [
        _vp, _f64, _f64, _vp, _sz, _vp, _vp, _vp, _vp]),
    "stb_icp_loss_scale_adjoint": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp,
                                                  _vp]),
    "stb_icp_estimate_static": (ctypes.c_int, [
        _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _i32, _i32, _vp, _i32,
        _i32, _vp, _i32, _f64, _f64, _f64, _f64, _f64, _i32, _vp, _vp, _vp]),
    "stb_profile_enable": (ctypes.c_int, [_i32]),
    "stb_set_wait_test_limits": (ctypes.c_int, [ctypes.c_uint32, _i32]),
    "stb_verify_registrations": (ctypes.c_int, [_vp, _vp, _i32, _f64, _f64, _f64, _vp, _vp]),
    "stb_profile_read": (ctypes.c_int, [ctypes.POINTER(_f64), ctypes.POINTER(_i64), _i32]),
    "stb_depth_to_points": (ctypes.c_int, [_vp, _f32, _f32, _vp, _vp, _vp, _i32, _i32, _vp]),
    "stb_erode_mask": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp]),
    "stb_estimate_normals": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _vp]),
    "stb_downsample_xyz": (ctypes.c_int, [_vp, _vp, _i32, _i32, _f32, _vp, _i32, _i32, _vp]),
    "stb_downsample_mask": (ctypes.c_int, [_vp, _i32, _i32, _f32, _vp, _i32, _i32, _vp]),
    "stb_downsample_features": (ctypes.c_int, [_vp, _i32, _i32, _i32, _i32, _f32, _vp, _i32,
                                               _i32, _vp]),
    "stb_gaussian_blur3": (ctypes.c_int, [_vp, _i32, _i32, _i32, _i32, _f64, _vp, _vp]),
    "stb_icp_estimate": (ctypes.c_int, [
        _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _i32, _i32, _vp, _i32,
        _i32, _vp, _i32, _f64, _f64, _f64, _f64, _f64, _i32, _vp, _sz, _vp,
        _vp, _i32, _vp]),
}


class StbLevel(ctypes.Structure):
    """``stb_level`` of the header: one pyramid level of one frame pair."""
    _fields_ = [("src_points", _vp), ("src_normals", _vp), ("src_mask", _vp),
                ("num_source", _i64), ("src_feats", _vp), ("tgt_points", _vp),
                ("tgt_normals", _vp), ("tgt_mask", _vp), ("height", _i32), ("width", _i32),
                ("tgt_feats", _vp), ("fx", _f32), ("fy", _f32), ("cx", _f32), ("cy", _f32)]


class StbLevelParams(ctypes.Structure):
    """``stb_level_params`` of the header."""
    _fields_ = [("num_iters", _i32), ("geom_weight", _f64), ("feat_weight", _f64),
                ("distance_thresh", _f64), ("normal_angle_thresh", _f64),
                ("feat_residual_thresh", _f64)]


ST_TIMEOUT, ST_CAPACITY = 8, 16

_LIB = None


def header_symbols(header_text):
    """Names of the functions a header declares with STB_API."""
    return re.findall(r"STB_API\s+[\w\s\*]+?\b(stb_\w+)\s*\(", header_text)


def lib():
    """The loaded library (``RuntimeError`` if it was not built)."""
    global _LIB
    if _LIB is None:
        path = _build.library_path()
        if not path.exists():
            raise RuntimeError(
                f"slamtb_gb300 native library not built ({path}); build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        handle = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = handle
    return _LIB


def check(rc):
    if rc != STB_OK:
        raise RuntimeError(lib().stb_last_error().decode(errors="replace"))


def ptr(t):
    """Device address of a tensor (None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_of(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


PROFILE_KINDS = ("association", "reduction+solve", "information", "setup", "registration")


def profile_enable(on):
    check(lib().stb_profile_enable(1 if on else 0))


def profile_read():
    """{kind: (ms, launches)} of the most recent profiled estimate call
    (call after the stream has completed)."""
    n = len(PROFILE_KINDS)
    ms = (_f64 * n)()
    cnt = (_i64 * n)()
    check(lib().stb_profile_read(ms, cnt, n))
    return {k: (ms[i], cnt[i]) for i, k in enumerate(PROFILE_KINDS)}


def feat_dtype_code(t):
    if t.dtype == torch.float32:
        return STB_F32
    if t.dtype == torch.bfloat16:
        return STB_BF16
    raise RuntimeError(f"Check failed: feature maps must be float32 or bfloat16, got {t.dtype}")
