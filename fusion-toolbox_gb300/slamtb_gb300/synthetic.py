"""Seeded synthetic RGB-D frame pairs for tests and benchmarks.

A scene is 8 random planes and 4 random spheres, ray-cast analytically with
a pinhole camera.  The target camera is the world frame; the source camera
sits at a random rigid offset (rotation axis uniform on the sphere, angle
uniform up to ``max_rot_deg``; translation direction uniform, length
uniform up to ``max_trans``).  The ground-truth ICP answer, the transform
taking source-camera points to target-camera points, is that offset.

Depth is the camera-frame z of the first hit, with Gaussian noise of
standard deviation 0.0012 z^2 m; hits outside [0.5, 4] m and a seeded 5 %
of pixels are set to 0 (invalid).  Feature maps are procedural textures
evaluated at the world hit point (so source and target agree on the
surface): a greyscale gradient-noise texture in [0, 1] (two octaves, 1.5
and 3.5 cycles per metre: smooth enough that the reference's weighting of
the feature term, J^T r by w but J^T J by w^2, stays stable at w = 0.1), or
``C`` smooth random channels normalised per pixel.

All parameters come from ``numpy.random.default_rng(seed)``; the
ray-casting runs in float64 with torch on any device.
"""
import math

import numpy as np
import torch

DEPTH_MIN, DEPTH_MAX = 0.5, 4.0


def default_kcam(width=640, height=480):
    """fx = fy = 525 at 480 rows (scaled with the height), principal point
    at the image centre: (319.5, 239.5) for 640x480."""
    f = 525.0 * height / 480.0
    return np.array([[f, 0.0, (width - 1) / 2.0],
                     [0.0, f, (height - 1) / 2.0],
                     [0.0, 0.0, 1.0]], dtype=np.float32)


def random_rigid(rng, max_rot_deg, max_trans):
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    angle = math.radians(rng.uniform(0.0, max_rot_deg))
    k = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + math.sin(angle) * k + (1 - math.cos(angle)) * (k @ k)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = d * rng.uniform(0.0, max_trans)
    return T


class Scene:
    """Primitive parameters (world = target camera frame).

    Plane 0 is an unbounded back wall 3.2-3.9 m away, tilted up to ~20
    degrees; planes 1-7 are rectangles 0.3-1.0 m in half-size at 1.0-3.5 m,
    tilted up to ~50 degrees; spheres have radius 0.15-0.45 m at 1.0-3.0 m.
    The bounded planes give the scene surfaces of many orientations, so all
    six degrees of freedom are observable."""

    def __init__(self, rng, kcam, width, height):
        fx, fy = float(kcam[0, 0]), float(kcam[1, 1])
        hx = 0.5 * width / fx
        hy = 0.5 * height / fy
        planes = []
        for k in range(8):
            if k == 0:
                z = rng.uniform(3.2, 3.9)
                c = np.array([0.0, 0.0, z])
                n = np.array([rng.uniform(-0.35, 0.35), rng.uniform(-0.35, 0.35), -1.0])
                half = (math.inf, math.inf)
            else:
                z = rng.uniform(1.0, 3.5)
                c = np.array([rng.uniform(-1, 1) * hx * z, rng.uniform(-1, 1) * hy * z, z])
                n = np.array([rng.uniform(-1.2, 1.2), rng.uniform(-1.2, 1.2), -1.0])
                half = (rng.uniform(0.3, 1.0), rng.uniform(0.3, 1.0))
            n = n / np.linalg.norm(n)
            e1 = np.cross(n, rng.normal(size=3))
            e1 /= np.linalg.norm(e1)
            e2 = np.cross(n, e1)
            planes.append((c, n, e1, e2, half))
        spheres = []
        for _ in range(4):
            z = rng.uniform(1.0, 3.0)
            c = np.array([rng.uniform(-0.7, 0.7) * hx * z, rng.uniform(-0.7, 0.7) * hy * z, z])
            spheres.append((c, rng.uniform(0.15, 0.45)))
        self.planes = planes
        self.spheres = spheres
        self.perm = rng.permutation(256)


_GRADS = np.array([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0],
                   [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
                   [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], dtype=np.float64)


def gradient_noise(p, perm):
    """3-D gradient noise (Perlin's improved noise, 2002) at points p
    (..., 3); perm is a 256-entry permutation.  Roughly in [-1, 1]."""
    dev = p.device
    P = torch.as_tensor(np.concatenate([perm, perm]), device=dev, dtype=torch.long)
    G = torch.as_tensor(_GRADS, device=dev)
    pi = torch.floor(p)
    f = p - pi
    i = pi.long() & 255
    u = f * f * f * (f * (f * 6 - 15) + 10)
    out = 0
    for corner in range(8):
        dx, dy, dz = corner & 1, (corner >> 1) & 1, (corner >> 2) & 1
        h = P[P[P[(i[..., 0] + dx) & 255] + ((i[..., 1] + dy) & 255)] + ((i[..., 2] + dz) & 255)]
        g = G[h % 12]
        d = f - torch.tensor([dx, dy, dz], device=dev, dtype=p.dtype)
        w = ((u[..., 0] if dx else 1 - u[..., 0]) * (u[..., 1] if dy else 1 - u[..., 1])
             * (u[..., 2] if dz else 1 - u[..., 2]))
        out = out + w * (g * d).sum(-1)
    return out


def _texture(points, perm, channels, offset):
    """Greyscale (channels == 0) or ``channels`` normalised fields."""
    if channels == 0:
        n = (gradient_noise(points * 1.5, perm) * 0.7
             + gradient_noise(points * 3.5 + 11.3, perm) * 0.3)
        return (0.5 + 0.5 * n).clamp(0.0, 1.0)[None]
    chans = []
    for c in range(channels):
        shift = 13.7 * (c + 1) + offset
        chans.append(gradient_noise(points * 2.5 + shift, perm) * 0.7
                     + gradient_noise(points * 6.0 - shift, perm) * 0.3)
    f = torch.stack(chans, 0)
    return f / f.norm(dim=0, keepdim=True).clamp_min(1e-6)


def render(scene, kcam, width, height, cam_to_world, device="cpu"):
    """Ray-cast the scene; returns (depth (H, W) float64 without noise,
    world hit points (H, W, 3), hit mask)."""
    dt = torch.float64
    k = torch.as_tensor(kcam, dtype=dt, device=device)
    T = torch.as_tensor(cam_to_world, dtype=dt, device=device)
    v, u = torch.meshgrid(torch.arange(height, dtype=dt, device=device),
                          torch.arange(width, dtype=dt, device=device), indexing="ij")
    dcam = torch.stack([(u - k[0, 2]) / k[0, 0], (v - k[1, 2]) / k[1, 1], torch.ones_like(u)], -1)
    d = dcam @ T[:3, :3].T
    o = T[:3, 3]
    best = torch.full((height, width), math.inf, dtype=dt, device=device)
    for c, n, e1, e2, half in scene.planes:
        c, n, e1, e2 = (torch.as_tensor(x, dtype=dt, device=device) for x in (c, n, e1, e2))
        den = d @ n
        t = torch.dot(n, c - o) / den
        ok = (den.abs() > 1e-12) & (t > 1e-6)
        if math.isfinite(half[0]):
            rel = o + d * t[..., None] - c
            ok &= ((rel @ e1).abs() <= half[0]) & ((rel @ e2).abs() <= half[1])
        t = torch.where(ok, t, torch.full_like(t, math.inf))
        best = torch.minimum(best, t)
    for c, r in scene.spheres:
        c = torch.as_tensor(c, dtype=dt, device=device)
        oc = o - c
        a = (d * d).sum(-1)
        b = d @ oc
        cc = torch.dot(oc, oc) - r * r
        disc = b * b - a * cc
        t = (-b - torch.sqrt(disc.clamp_min(0.0))) / a
        t = torch.where((disc >= 0) & (t > 1e-6), t, torch.full_like(t, math.inf))
        best = torch.minimum(best, t)
    hit = torch.isfinite(best)
    depth = torch.where(hit, best, torch.zeros_like(best))
    pts = o + d * torch.where(hit, best, torch.zeros_like(best))[..., None]
    return depth, pts, hit


def make_pair(seed, width=640, height=480, max_rot_deg=5.0, max_trans=0.05,
              feature_channels=None, noise=True, dropout=0.05, device="cpu"):
    """One seeded frame pair.

    Returns a dict with ``target_depth`` / ``source_depth`` (H, W) float32
    numpy arrays (0 = invalid), ``kcam`` (3, 3) float32, ``gt`` (4, 4)
    float64 (source camera -> target camera), and, when
    ``feature_channels`` is not None, ``target_feats`` / ``source_feats``
    (C, H, W) float32 (``feature_channels == 0`` gives one greyscale
    channel)."""
    rng = np.random.default_rng(seed)
    kcam = default_kcam(width, height)
    scene = Scene(rng, kcam, width, height)
    gt = random_rigid(rng, max_rot_deg, max_trans)
    out = dict(kcam=kcam, gt=gt)
    for name, pose in (("target", np.eye(4)), ("source", gt)):
        z, pts, hit = render(scene, kcam, width, height, pose, device)
        z = z.cpu().numpy()
        if noise:
            z = z + rng.standard_normal(z.shape) * (0.0012 * z * z)
        z = np.where((z >= DEPTH_MIN) & (z <= DEPTH_MAX) & hit.cpu().numpy(), z, 0.0)
        if dropout > 0:
            z = np.where(rng.random(z.shape) < dropout, 0.0, z)
        out[f"{name}_depth"] = z.astype(np.float32)
        if feature_channels is not None:
            f = _texture(pts, scene.perm, feature_channels, 0.0)
            out[f"{name}_feats"] = f.to(torch.float32).cpu().numpy()
    return out
