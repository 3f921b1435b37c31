"""Frames and frame point clouds on the device.

The subset of ``slamtb/frame.py`` and ``slamtb/camera.py`` that the ICP
path consumes: a depth frame becomes an (H, W, 3) point grid, an eroded
validity mask and lazily computed central-difference normals, and can be
turned into a coarse-to-fine pyramid.  Every step runs as a CUDA kernel of
``libslamtb_gb300`` (see ``processing``).
"""
import torch

from . import processing


def resolve_device(device):
    """CUDA device for ``device`` (None -> current).  A CPU device is
    refused: this package has no CPU path."""
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    device = torch.device(device)
    if device.type != "cuda":
        raise RuntimeError("Check failed: device: Expected a gpu tensor "
                           "(slamtb_gb300 runs on CUDA devices only)")
    return device


class KCamera:
    """Intrinsics (``slamtb/camera.py:19-198``): a (3, 3) float32 matrix."""

    def __init__(self, matrix, undist_coeff=None, image_size=None):
        self.matrix = torch.as_tensor(matrix, dtype=torch.float32)
        self.undist_coeff = undist_coeff
        self.image_size = image_size

    @classmethod
    def from_params(cls, flen_x, flen_y, center_point, undist_coeff=None, image_size=None):
        cx, cy = center_point
        m = torch.tensor([[flen_x, 0.0, cx], [0.0, flen_y, cy], [0.0, 0.0, 1.0]],
                         dtype=torch.float32)
        return cls(m, undist_coeff, image_size)

    def scaled(self, xscale, yscale=None):
        """Intrinsics for an image scaled by (xscale, yscale)
        (``camera.py:172-198``; products in float32)."""
        if yscale is None:
            yscale = xscale
        m = self.matrix
        image_size = None
        if self.image_size is not None:
            image_size = (int(self.image_size[0] * xscale), int(self.image_size[1] * yscale))
        out = torch.eye(3, dtype=torch.float32, device=m.device)
        out[0, 0] = m[0, 0] * xscale
        out[1, 1] = m[1, 1] * yscale
        out[0, 2] = m[0, 2] * xscale
        out[1, 2] = m[1, 2] * yscale
        return KCamera(out, self.undist_coeff, image_size)

    def to(self, device):
        """Intrinsics are kept on the host (kernels take them by value or
        copy them per call); returns self."""
        return self

    def params(self):
        """(fx, fy, cx, cy) as Python floats."""
        m = self.matrix.detach().cpu()
        return float(m[0, 0]), float(m[1, 1]), float(m[0, 2]), float(m[1, 2])


class FrameInfo:
    """Per-frame metadata used by the path (``slamtb/frame.py:19-111``)."""

    def __init__(self, kcam=None, depth_scale=1.0, depth_bias=0.0, depth_max=4500.0,
                 rt_cam=None, timestamp=None):
        self.kcam = kcam
        self.depth_scale = depth_scale
        self.depth_bias = depth_bias
        self.depth_max = depth_max
        self.rt_cam = rt_cam
        self.timestamp = timestamp


class Frame:
    """A depth frame (``slamtb/frame.py:114-253``): ``depth_image`` (H, W)
    of any numeric type, scaled by ``info.depth_scale`` and offset by
    ``info.depth_bias`` into metres."""

    def __init__(self, info, depth_image, rgb_image=None, seg_image=None, normal_image=None):
        self.info = info
        self.depth_image = depth_image
        self.rgb_image = rgb_image
        self.seg_image = seg_image
        self.normal_image = normal_image


class FramePointCloud:
    """Point grid of a frame (``slamtb/frame.py:256-486``).

    Args:
        image_points: (H, W, 3) u, v, z grid or None when ``points`` given.
        mask: (H, W) bool validity.
        kcam: ``KCamera``.
        points / normals: (H, W, 3) float32, optional (normals are computed
            on first access by central differences).
    """

    def __init__(self, image_points, mask, kcam, rt_cam=None, points=None, normals=None,
                 colors=None):
        self.image_points = image_points
        self.mask = mask
        self.kcam = kcam
        self.rt_cam = rt_cam
        self._points = points
        self._normals = normals
        self.colors = colors

    @classmethod
    def from_frame(cls, frame, device=None):
        """``FramePointCloud.from_frame`` (``slamtb/frame.py:272-306``):
        back-projection and mask erosion on the device."""
        device = resolve_device(device)
        depth = torch.as_tensor(frame.depth_image).to(device=device, dtype=torch.float32)
        kcam = frame.info.kcam
        if not isinstance(kcam, KCamera):
            kcam = KCamera(kcam)
        points, raw_mask = processing.depth_to_points(
            depth, kcam.matrix.to(device), frame.info.depth_scale, frame.info.depth_bias)
        mask = processing.erode_mask(raw_mask)
        normals = None
        if frame.normal_image is not None:
            normals = torch.as_tensor(frame.normal_image).to(device=device, dtype=torch.float32)
        return cls(None, mask, kcam, frame.info.rt_cam, points=points, normals=normals)

    @property
    def device(self):
        return self.mask.device

    @property
    def points(self):
        if self._points is None:
            if self.image_points is None or self.kcam is None:
                raise RuntimeError("Frame point cloud has neither points nor image points")
            z = self.image_points[..., 2].to(torch.float32).contiguous()
            self._points, _ = processing.depth_to_points(
                z, self.kcam.matrix.to(z.device), 1.0, 0.0)
        return self._points

    @property
    def normals(self):
        if self._normals is None:
            self._normals = processing.estimate_normals(self.points, self.mask)
        return self._normals

    @normals.setter
    def normals(self, normals):
        self._normals = normals

    def downsample(self, scale, downsample_xyz_method=None, colored=False):
        """``FramePointCloud.downsample`` (``slamtb/frame.py:388-422``):
        nearest-to-mean XYZ, nearest mask, scaled intrinsics; normals are
        carried over only when already computed."""
        points = processing.downsample_xyz(self.points, self.mask, scale)
        normals = None
        if self._normals is not None:
            normals = processing.downsample_xyz(self._normals, self.mask, scale)
        mask = processing.downsample_mask(self.mask, scale)
        return FramePointCloud(None, mask, self.kcam.scaled(scale), rt_cam=self.rt_cam,
                               points=points, normals=normals)

    def pyramid(self, scales, downsample_xyz_method=None, colored=False):
        """Levels for decreasing ``scales`` (scales below 1 compound),
        returned coarsest first (``slamtb/frame.py:424-453``)."""
        out = []
        cur = self
        for s in scales:
            if s < 1.0:
                cur = cur.downsample(s)
            out.append(cur)
        out.reverse()
        return out

    def to(self, dst):
        dst = resolve_device(dst)
        conv = (lambda t: None if t is None else t.to(dst))
        return FramePointCloud(conv(self.image_points), conv(self.mask), self.kcam.to(dst),
                               self.rt_cam, conv(self._points), conv(self._normals),
                               conv(self.colors))
