"""Extract the known-answer fixtures from the reference's own test data.

Run where a copy of the reference tree is available, with its root as the
only argument (it is read here, never at test time):

    python tests/golden/make_golden.py <reference root>

It decodes the 16-bit depth PNGs of ``test-data/rgbd/sample2`` frames used
by the reference's tests (frames 0 and 3: the synthetic pair of
``slamtb/registration/_test/test_icp.py:19-27``; frame 13: the pair of
``slamtb/registration/_test/test_correspondence_map.py:16-19``) and stores
them, with their intrinsics, depth scale and ground-truth camera-to-world
poses from ``frames.json``, as ``sample2.npz`` (depth stored as row-wise
first differences; ``load_sample2`` undoes that).

It also stores ``slamtb/_test/assets/frame_depth.png``, the depth frame of
the reference's bilateral-filter and erosion tests
(``slamtb/_test/test_processing.py:24-60``), as ``frame_depth.npz`` (same
encoding; ``load_frame_depth``).
"""
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle.png16 import read_png  # noqa: E402

FRAMES = (0, 3, 13)


def load_sample2(path=HERE / "sample2.npz"):
    """Return {frame: dict(depth uint16 (480, 640), rt_cam f64 (4, 4),
    kcam f32 (3, 3), depth_scale, depth_bias)}."""
    z = np.load(path)
    out = {}
    for i in FRAMES:
        depth = np.cumsum(z[f"depth_dx_{i}"].astype(np.int32), axis=1)
        out[i] = dict(depth=depth.astype(np.uint16), rt_cam=z[f"rt_cam_{i}"],
                      kcam=z[f"kcam_{i}"], depth_scale=z[f"depth_scale_{i}"],
                      depth_bias=z[f"depth_bias_{i}"])
    return out


def load_frame_depth(path=HERE / "frame_depth.npz"):
    """The uint16 (480, 640) depth frame of the reference's processing tests."""
    z = np.load(path)
    return np.cumsum(z["depth_dx"].astype(np.int32), axis=1).astype(np.uint16)


def _row_differences(depth):
    """int16 row-wise first differences of a uint16 image; the loaders undo
    them with a cumulative sum, so every difference must fit in int16."""
    dx = np.diff(depth.astype(np.int32), axis=1, prepend=0)
    assert np.abs(dx).max() <= np.iinfo(np.int16).max, "depth step does not fit int16"
    return dx.astype(np.int16)


def main(reference_root):
    root = pathlib.Path(reference_root) / "test-data" / "rgbd" / "sample2"
    meta = json.load(open(root / "frames.json"))["root"]
    out = {}
    for i in FRAMES:
        entry = meta[i]
        depth = read_png(root / entry["depth_image"])
        assert depth.dtype == np.uint16 and depth.shape == (480, 640)
        info = entry["info"]
        # row-wise first differences compress ~2.3x better than raw depth
        out[f"depth_dx_{i}"] = _row_differences(depth)
        out[f"rt_cam_{i}"] = np.array(info["rt_cam"]["matrix"], dtype=np.float64)
        out[f"kcam_{i}"] = np.array(info["kcam"]["matrix"], dtype=np.float32)
        out[f"depth_scale_{i}"] = np.float32(info["depth_scale"])
        out[f"depth_bias_{i}"] = np.float32(info["depth_bias"])
    np.savez_compressed(HERE / "sample2.npz", **out)
    print("wrote", HERE / "sample2.npz")
    depth = read_png(pathlib.Path(reference_root) / "slamtb" / "_test" / "assets" /
                     "frame_depth.png")
    assert depth.dtype == np.uint16
    np.savez_compressed(HERE / "frame_depth.npz", depth_dx=_row_differences(depth))
    print("wrote", HERE / "frame_depth.npz")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference root>")
    main(sys.argv[1])
