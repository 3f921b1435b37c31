"""numpy restatement of the frame preparation that feeds the ICP path.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Every function follows one reference routine and keeps its float32
operation order, so that the CUDA restatements can be compared bit for bit
(except the Gaussian blur, whose reference is kornia's conv2d: that one is
evaluated in float64 here and compared within a tolerance).
"""
import numpy as np

F32 = np.float32


def erode_mask(mask):
    """Mask erosion, ``src/erode_mask.cu:18-39``.

    Reference quirk kept: the neighbourhood table lists ``{0, 1}`` twice and
    never ``{1, 0}``, so a pixel is cleared when the pixel above, to the
    right or to the left is invalid; the pixel below is never checked.
    """
    m = np.asarray(mask, dtype=bool)
    h, w = m.shape
    up = np.ones_like(m)
    up[1:, :] = m[:-1, :]
    right = np.ones_like(m)
    right[:, :-1] = m[:, 1:]
    left = np.ones_like(m)
    left[:, 1:] = m[:, :-1]
    return m & up & right & left


def depth_to_points(depth, kcam):
    """Back-projection of a metric depth image, float32.

    ``slamtb/_utils.py:11-37`` (u, v, z grid) followed by
    ``slamtb/camera.py:127-149``: ``x = (u - cx) * z / fx``.
    """
    depth = np.asarray(depth, dtype=F32)
    k = np.asarray(kcam, dtype=F32)
    h, w = depth.shape
    xs = np.broadcast_to(np.arange(w, dtype=F32)[None, :], (h, w))
    ys = np.broadcast_to(np.arange(h, dtype=F32)[:, None], (h, w))
    fx, fy, cx, cy = k[0, 0], k[1, 1], k[0, 2], k[1, 2]
    out = np.empty((h, w, 3), dtype=F32)
    out[..., 0] = ((xs - cx) * depth) / fx
    out[..., 1] = ((ys - cy) * depth) / fy
    out[..., 2] = depth
    return out


def _sqnorm(a):
    """Eigen's ``squaredNorm`` of 3-vectors: ``a0^2 + (a1^2 + a2^2)`` (the
    unrolled redux of Eigen/src/Core/Redux.h splits three terms at one)."""
    return a[..., 0] * a[..., 0] + (a[..., 1] * a[..., 1] + a[..., 2] * a[..., 2])


def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def estimate_normals(xyz, mask):
    """Central-difference normals, ``src/normals.cu:27-100``, float32.

    Neighbours that are outside the image or masked out are taken as the
    zero vector; the ratio test uses 2.0 (squared: 4.0); a normal whose
    length is not above 1e-6 becomes (0, 0, -1); masked-out pixels get 0.
    """
    xyz = np.asarray(xyz, dtype=F32)
    m = np.asarray(mask, dtype=bool)
    h, w, _ = xyz.shape
    zero = np.zeros((h, w, 3), dtype=F32)

    def neighbour(dr, dc):
        # value at (r + dr, c + dc) when inside the image and valid, else 0
        out = zero.copy()
        valid = np.zeros((h, w), dtype=bool)
        r0, r1 = max(0, -dr), h - max(0, dr)
        c0, c1 = max(0, -dc), w - max(0, dc)
        valid[r0:r1, c0:c1] = m[r0 + dr:r1 + dr, c0 + dc:c1 + dc]
        out[r0:r1, c0:c1] = xyz[r0 + dr:r1 + dr, c0 + dc:c1 + dc]
        out[~valid] = 0
        return out

    center = xyz
    left = neighbour(0, -1)
    right = neighbour(0, 1)
    top = neighbour(-1, 0)
    bottom = neighbour(1, 0)
    thr2 = F32(4.0)
    inv_thr2 = F32(1.0) / thr2

    with np.errstate(divide="ignore", invalid="ignore"):
        lds = _sqnorm(left - center)
        rds = _sqnorm(right - center)
        lr_ratio = lds / rds
        lr_mid = (lr_ratio < thr2) & (lr_ratio > inv_thr2)
        lr_left = ~lr_mid & (lds < rds)
        l2r = np.where(lr_mid[..., None], right - left,
                       np.where(lr_left[..., None], center - left, right - center))

        bds = _sqnorm(bottom - center)
        tds = _sqnorm(top - center)
        bt_ratio = bds / tds
        bt_mid = (bt_ratio < thr2) & (bt_ratio > inv_thr2)
        bt_bottom = ~bt_mid & (bds < tds)
        b2t = np.where(bt_mid[..., None], top - bottom,
                       np.where(bt_bottom[..., None], center - bottom, top - center))

        normal = _cross(l2r, b2t)
        length = np.sqrt(_sqnorm(normal))
        ok = length > F32(1e-6)
        unit = normal / np.where(ok, length, F32(1))[..., None]
    fallback = np.broadcast_to(np.array([0, 0, -1], dtype=F32), (h, w, 3))
    out = np.where(ok[..., None], unit, fallback).astype(F32)
    out[~m] = 0
    return out


def downsample_xyz_nearest(xyz, mask, scale):
    """Nearest-to-mean XYZ downsample, ``src/downsample.cu:25-72``.

    For each destination pixel the 2x2 source block at ``int(row / scale)``
    is scanned, the mean of its valid points is taken, and the valid point
    nearest to that mean (first one on ties) is kept; a block without valid
    points gives (0, 0, 0).  Source rows past the image (only reachable with
    a destination taller than ``int(h * scale)``) count as invalid; the
    reference checks only columns and would read past the end.
    """
    xyz = np.asarray(xyz, dtype=F32)
    m = np.asarray(mask, dtype=bool)
    h, w, _ = xyz.shape
    dh, dw = int(h * scale), int(w * scale)
    inv = F32(1) / F32(scale)
    rows = (np.arange(dh, dtype=F32) * inv).astype(np.int64)
    cols = (np.arange(dw, dtype=F32) * inv).astype(np.int64)
    taps = [(0, 0), (0, 1), (1, 0), (1, 1)]
    pts, oks = [], []
    for dr, dc in taps:
        r = rows[:, None] + dr
        c = cols[None, :] + dc
        cin = (c < w) & (r < h)
        rr = np.broadcast_to(np.minimum(r, h - 1), (dh, dw))
        cc = np.broadcast_to(np.minimum(c, w - 1), (dh, dw))
        ok = np.broadcast_to(cin, (dh, dw)) & m[rr, cc]
        pts.append(xyz[rr, cc])
        oks.append(ok)
    acc = np.zeros((dh, dw, 3), dtype=F32)
    count = np.zeros((dh, dw), dtype=np.int64)
    for p, ok in zip(pts, oks):
        acc = np.where(ok[..., None], acc + p, acc)
        count += ok
    with np.errstate(divide="ignore", invalid="ignore"):
        mean = acc / count.astype(F32)[..., None]
    best = np.full((dh, dw), np.inf, dtype=F32)
    out = np.zeros((dh, dw, 3), dtype=F32)
    for p, ok in zip(pts, oks):
        with np.errstate(invalid="ignore"):
            d = _sqnorm(p - mean)
            take = ok & (d < best)
        best = np.where(take, d, best)
        out = np.where(take[..., None], p, out)
    return out


def downsample_mask(mask, scale):
    """Nearest mask downsample, ``src/downsample.cu:112-116``."""
    m = np.asarray(mask, dtype=bool)
    h, w = m.shape
    dh, dw = int(h * scale), int(w * scale)
    inv = F32(1.0) / F32(scale)
    rows = (np.arange(dh, dtype=F32) * inv).astype(np.int64)
    cols = (np.arange(dw, dtype=F32) * inv).astype(np.int64)
    return m[rows[:, None], cols[None, :]]


def scale_kcam(kcam, scale):
    """``KCamera.scaled`` (``slamtb/camera.py:172-198``), float32."""
    k = np.asarray(kcam, dtype=F32)
    s = F32(scale)
    out = np.eye(3, dtype=F32)
    out[0, 0] = k[0, 0] * s
    out[1, 1] = k[1, 1] * s
    out[0, 2] = k[0, 2] * s
    out[1, 2] = k[1, 2] * s
    return out


def gaussian_kernel1d(size=3, sigma=0.849):
    """kornia ``get_gaussian_kernel1d`` (restated): normalised exp(-x^2/2s^2)."""
    x = np.arange(size, dtype=np.float64) - size // 2
    g = np.exp(-(x ** 2) / (2.0 * sigma ** 2))
    return g / g.sum()


def gaussian_blur3(feats, sigma=0.849):
    """3x3 Gaussian blur with reflect borders, as kornia's
    ``GaussianBlur2d((3, 3), (0.849, 0.849))`` used by
    ``slamtb/processing.py:141-159``.  Evaluated in float64, returned as
    float32 (kornia is absent; parity with it is unpinned)."""
    f = np.asarray(feats, dtype=np.float64)
    g = gaussian_kernel1d(3, sigma)
    k2 = np.outer(g, g)
    pad = np.pad(f, ((0, 0), (1, 1), (1, 1)), mode="reflect")
    c, h, w = f.shape
    out = np.zeros_like(f)
    for dy in range(3):
        for dx in range(3):
            out += k2[dy, dx] * pad[:, dy:dy + h, dx:dx + w]
    return out.astype(F32)


def downsample_features(feats, scale):
    """2x2 mean feature downsample, ``src/downsample.cu:145-168``, float32
    (sum in tap order, then divide by the tap count; taps past the image
    are skipped -- the reference checks only columns)."""
    f = np.asarray(feats, dtype=F32)
    c, h, w = f.shape
    dh, dw = int(h * scale), int(w * scale)
    inv = F32(1) / F32(scale)
    rows = (np.arange(dh, dtype=F32) * inv).astype(np.int64)
    cols = (np.arange(dw, dtype=F32) * inv).astype(np.int64)
    acc = np.zeros((c, dh, dw), dtype=F32)
    count = np.zeros((dh, dw), dtype=np.int64)
    for dr, dc in [(0, 0), (0, 1), (1, 0), (1, 1)]:
        r_raw = rows[:, None] + dr
        r = np.minimum(r_raw, h - 1)
        cc = cols[None, :] + dc
        ok = np.broadcast_to((cc < w) & (r_raw < h), (dh, dw))
        ccl = np.minimum(cc, w - 1)
        val = f[:, np.broadcast_to(r, (dh, dw)), np.broadcast_to(ccl, (dh, dw))]
        acc = np.where(ok[None], acc + val, acc)
        count += ok
    return (acc / count.astype(F32)[None]).astype(F32)


def feature_pyramid(feats, scales):
    """``slamtb/processing.py:141-159``: blur + 2x2 mean for each scale
    below 1, returned coarsest first."""
    pyr = []
    f = np.asarray(feats, dtype=F32)
    for s in scales:
        if s < 1.0:
            f = downsample_features(gaussian_blur3(f), s)
        pyr.append(f)
    pyr.reverse()
    return pyr


class FramePointCloud:
    """The tensors ``FramePointCloud`` hands to the ICP path
    (``slamtb/frame.py:256-453``): points and normals (H, W, 3) float32,
    mask (H, W) bool and the 3x3 intrinsics."""

    def __init__(self, points, mask, kcam, normals=None):
        self.points = np.asarray(points, dtype=F32)
        self.mask = np.asarray(mask, dtype=bool)
        self.kcam = np.asarray(kcam, dtype=F32)
        self._normals = normals

    @classmethod
    def from_depth(cls, depth, kcam):
        """``FramePointCloud.from_frame`` (``slamtb/frame.py:272-306``) for
        a metric depth image: mask = erode(depth > 0)."""
        depth = np.asarray(depth, dtype=F32)
        mask = erode_mask(depth > 0)
        return cls(depth_to_points(depth, kcam), mask, kcam)

    @property
    def normals(self):
        if self._normals is None:
            self._normals = estimate_normals(self.points, self.mask)
        return self._normals

    def downsample(self, scale):
        """``FramePointCloud.downsample`` (``slamtb/frame.py:388-422``);
        normals are not carried over unless already computed."""
        pts = downsample_xyz_nearest(self.points, self.mask, scale)
        normals = None
        if self._normals is not None:
            normals = downsample_xyz_nearest(self._normals, self.mask, scale)
        return FramePointCloud(pts, downsample_mask(self.mask, scale),
                               scale_kcam(self.kcam, scale), normals)

    def pyramid(self, scales):
        """``FramePointCloud.pyramid`` (``slamtb/frame.py:424-453``),
        returned coarsest first."""
        out = []
        cur = self
        for s in scales:
            if s < 1.0:
                cur = cur.downsample(s)
            out.append(cur)
        out.reverse()
        return out


def bilateral_depth_filter(depth, mask=None, filter_width=6, sigma_color=29.9999880000072,
                           sigma_space=4.50000000225, depth_scale=1.0):
    """``BilateralDepthFilterKernel`` (src/bilateral_depth_filter.cu:15-72) in
    float32, operation by operation, for a depth image of any dtype:

    * depth z = input * depth_scale (an integer input is converted to
      float32 first; a float64 input is multiplied in float64 and rounded);
    * for every neighbour (row offsets outer, column offsets inner, both
      from -filter_width // 2) inside the image and the mask:
      w = exp(-0.5 (space^2 / sigma_space^2 + dz^2 / sigma_color^2)),
      sums of z w and w in that order;
    * result = (sum z w / sum w) / depth_scale, converted to the input
      dtype (integers truncate); 0 where the mask is 0.

    ``exp`` is numpy's float32 exponential, which may differ from the
    device's by an ulp: results agree within a few ulps, integer results
    within 1 (the tolerance of the reference's own CPU-vs-GPU test,
    slamtb/_test/test_processing.py:24-43)."""
    depth = np.asarray(depth)
    if mask is None:
        mask = depth > 0
    mask = np.asarray(mask, dtype=bool)
    hw = int(filter_width) // 2
    scale = F32(depth_scale)
    sc, ss = F32(sigma_color), F32(sigma_space)
    inv_sc = F32(1.0 / float(F32(sc * sc)))
    inv_ss = F32(1.0 / float(F32(ss * ss)))
    inv_scale = F32(1.0 / float(scale))
    if depth.dtype == np.float64:
        z = (depth * np.float64(scale)).astype(F32)
    else:
        z = (depth.astype(F32) * scale).astype(F32)
    h, w = z.shape
    zp = np.zeros((h + 2 * hw, w + 2 * hw), dtype=F32)
    mp = np.zeros((h + 2 * hw, w + 2 * hw), dtype=bool)
    zp[hw:hw + h, hw:hw + w] = z
    mp[hw:hw + h, hw:hw + w] = mask
    color_sum = np.zeros((h, w), dtype=F32)
    weight_sum = np.zeros((h, w), dtype=F32)
    half = F32(-0.5)
    with np.errstate(over="ignore", invalid="ignore"):
        for y in range(-hw, hw + 1):
            for x in range(-hw, hw + 1):
                cz = zp[hw + y:hw + y + h, hw + x:hw + x + w]
                cm = mp[hw + y:hw + y + h, hw + x:hw + x + w]
                dx, dy = F32(-x), F32(-y)
                space_sqr = F32(dx * dx) + F32(dy * dy)
                dcolor = (z - cz).astype(F32)
                color_sqr = (dcolor * dcolor).astype(F32)
                arg = (half * ((space_sqr * inv_ss).astype(F32)
                               + (color_sqr * inv_sc).astype(F32))).astype(F32)
                wt = np.exp(arg).astype(F32)
                color_sum = np.where(cm, (color_sum + (cz * wt).astype(F32)).astype(F32),
                                     color_sum)
                weight_sum = np.where(cm, (weight_sum + wt).astype(F32), weight_sum)
        r = (((color_sum / weight_sum).astype(F32)) * inv_scale).astype(F32)
    ok = mask & (weight_sum > 0)
    r = np.where(ok, r, F32(0))
    if np.issubdtype(depth.dtype, np.integer):
        return np.trunc(r).astype(depth.dtype)
    return r.astype(depth.dtype)
