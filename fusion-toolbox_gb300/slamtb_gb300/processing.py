"""Frame preparation on the device (``slamtb/processing.py`` subset used by
the ICP path), backed by the ``stb_*`` prep kernels of libslamtb_gb300."""
import torch

from . import _native as N


def _dev(t):
    if not t.is_cuda:
        raise RuntimeError("Check failed: Expected a gpu tensor "
                           "(slamtb_gb300 runs on CUDA devices only)")
    return t.device


def _run(dev, fn, *args):
    with torch.cuda.device(dev):
        N.check(fn(*args, N.stream_of(dev)))


def depth_to_points(depth, kcam, depth_scale=1.0, depth_bias=0.0):
    """(H, W) depth -> ((H, W, 3) float32 points, (H, W) bool depth > 0)."""
    dev = _dev(depth)
    depth = depth.to(torch.float32).contiguous()
    k = kcam.to(device=dev, dtype=torch.float32).contiguous()
    h, w = depth.shape
    pts = torch.empty(h, w, 3, dtype=torch.float32, device=dev)
    mask = torch.empty(h, w, dtype=torch.bool, device=dev)
    _run(dev, N.lib().stb_depth_to_points, N.ptr(depth), float(depth_scale),
         float(depth_bias), N.ptr(k), N.ptr(pts), N.ptr(mask), h, w)
    return pts, mask


def erode_mask(mask):
    dev = _dev(mask)
    m = mask.to(torch.bool).contiguous()
    out = torch.empty_like(m)
    _run(dev, N.lib().stb_erode_mask, N.ptr(m), N.ptr(out), m.size(0), m.size(1))
    return out


def estimate_normals(points, mask):
    dev = _dev(points)
    p = points.to(torch.float32).contiguous()
    m = mask.to(torch.bool).contiguous()
    out = torch.empty_like(p)
    _run(dev, N.lib().stb_estimate_normals, N.ptr(p), N.ptr(m), N.ptr(out), p.size(0),
         p.size(1))
    return out


def downsample_xyz(xyz, mask, scale):
    dev = _dev(xyz)
    x = xyz.to(torch.float32).contiguous()
    m = mask.to(torch.bool).contiguous()
    h, w = m.shape
    dh, dw = int(h * scale), int(w * scale)
    out = torch.empty(dh, dw, 3, dtype=torch.float32, device=dev)
    _run(dev, N.lib().stb_downsample_xyz, N.ptr(x), N.ptr(m), h, w, float(scale), N.ptr(out),
         dh, dw)
    return out


def downsample_mask(mask, scale):
    dev = _dev(mask)
    m = mask.to(torch.bool).contiguous()
    h, w = m.shape
    dh, dw = int(h * scale), int(w * scale)
    out = torch.empty(dh, dw, dtype=torch.bool, device=dev)
    _run(dev, N.lib().stb_downsample_mask, N.ptr(m), h, w, float(scale), N.ptr(out), dh, dw)
    return out


def downsample_features(feats, scale):
    dev = _dev(feats)
    f = feats.contiguous()
    c, h, w = f.shape
    dh, dw = int(h * scale), int(w * scale)
    out = torch.empty(c, dh, dw, dtype=f.dtype, device=dev)
    _run(dev, N.lib().stb_downsample_features, N.ptr(f), c, h, w, N.feat_dtype_code(f),
         float(scale), N.ptr(out), dh, dw)
    return out


def gaussian_blur3(feats, sigma=0.849):
    dev = _dev(feats)
    f = feats.contiguous()
    c, h, w = f.shape
    out = torch.empty_like(f)
    _run(dev, N.lib().stb_gaussian_blur3, N.ptr(f), c, h, w, N.feat_dtype_code(f),
         float(sigma), N.ptr(out))
    return out


def feature_pyramid(feature_map, scales):
    """Blur + 2x2 mean for every scale below 1, coarsest first
    (``slamtb/processing.py:141-159``)."""
    pyr = []
    f = feature_map
    for s in scales:
        if s < 1.0:
            f = downsample_features(gaussian_blur3(f), s)
        pyr.append(f)
    pyr.reverse()
    return pyr


def interleave_features(feats):
    """(C, ...) feature maps -> (count, C): the texel-major layout the
    registration kernels sample with all channels of a pixel adjacent
    (``stb_feature_interleave``)."""
    dev = _dev(feats)
    f = feats.reshape(feats.size(0), -1).contiguous()
    c, n = f.shape
    out = torch.empty(n, c, dtype=f.dtype, device=dev)
    _run(dev, N.lib().stb_feature_interleave, N.ptr(f), N.ptr(out), c, n, N.feat_dtype_code(f))
    return out


_DEPTH_DTYPES = {torch.float32: N.STB_F32, torch.float64: N.STB_F64, torch.uint8: N.STB_U8,
                 torch.int16: N.STB_I16, torch.int32: N.STB_I32, torch.int64: N.STB_I64}
if hasattr(torch, "uint16"):
    _DEPTH_DTYPES[torch.uint16] = N.STB_U16


def bilateral_depth_filter(depth, mask=None, out_tensor=None, filter_width=6,
                           sigma_color=29.9999880000072, sigma_space=4.50000000225,
                           depth_scale=1.0):
    """Bilateral filter of a depth image (``slamtb/processing.py:17-55``,
    ``src/bilateral_depth_filter.cu``; defaults are ElasticFusion's).

    Args:
        depth: (H, W) depth image on a CUDA device, float32 / float64 or an
            integer type (the result has the same dtype; integers truncate).
        mask: (H, W) validity, default ``depth > 0``.
        out_tensor: optional output, reused when its size matches.
        filter_width (int): window size (at most 31).
        sigma_color, sigma_space (float): range and spatial sigmas.
        depth_scale (float): factor applied to the depth before filtering.
    """
    dev = _dev(depth)
    d = depth.contiguous()
    if d.dtype not in _DEPTH_DTYPES:
        raise RuntimeError(f"Check failed: unsupported depth dtype {d.dtype}")
    if mask is None:  # depth > 0 (unsigned 16-bit tensors compare through int16 bits)
        m = (d.view(torch.int16) != 0) if d.dtype == getattr(torch, "uint16", None) else d > 0
    else:
        m = mask
    m = m.to(device=dev, dtype=torch.bool).contiguous()
    h, w = d.shape
    if out_tensor is None or tuple(out_tensor.shape) != (h, w) or out_tensor.dtype != d.dtype \
            or out_tensor.device != dev:
        out_tensor = torch.empty(h, w, dtype=d.dtype, device=dev)
    _run(dev, N.lib().stb_bilateral_depth_filter, N.ptr(d), N.ptr(m), N.ptr(out_tensor), h, w,
         _DEPTH_DTYPES[d.dtype], int(filter_width), float(sigma_color), float(sigma_space),
         float(depth_scale))
    return out_tensor


class BilateralDepthFilter:
    """``slamtb/processing.py:58-76``: the filter with fixed parameters and
    a reused output tensor."""

    def __init__(self, filter_width=6, sigma_color=29.9999880000072,
                 sigma_space=4.50000000225, depth_scale=1.0):
        self.filter_width = filter_width
        self.sigma_color = sigma_color
        self.sigma_space = sigma_space
        self.depth_scale = depth_scale
        self._out_tensor = None

    def __call__(self, depth, mask=None):
        self._out_tensor = bilateral_depth_filter(
            depth, mask, self._out_tensor, self.filter_width, self.sigma_color,
            self.sigma_space, self.depth_scale)
        return self._out_tensor
