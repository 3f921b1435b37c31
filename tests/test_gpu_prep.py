"""Frame preparation kernels against the oracle's restatement: bit-exact
(the blur, restating kornia, within 1e-6)."""
import numpy as np
import pytest
import torch

from oracle import frame_prep as fp
from _helpers import sample2_pair
from slamtb_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def depth_pair():
    p = synthetic.make_pair(4, feature_channels=0)
    return p


def _eq(a, b):
    np.testing.assert_array_equal(a.cpu().numpy() if torch.is_tensor(a) else a, b)


def test_from_frame_and_normals(cuda, depth_pair):
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    depth = depth_pair["target_depth"]
    k = depth_pair["kcam"]
    fpc = FramePointCloud.from_frame(Frame(FrameInfo(KCamera(k)), depth), cuda)
    ref = fp.FramePointCloud.from_depth(depth, k)
    _eq(fpc.points, ref.points)
    _eq(fpc.mask, ref.mask)
    _eq(fpc.normals, ref.normals)


def test_scaled_depth_frame(cuda):
    """sample2 stores depth as uint16 with depth_scale 0.0002."""
    from make_golden import load_sample2
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    d = load_sample2()[0]
    info = FrameInfo(KCamera(d["kcam"]), depth_scale=float(d["depth_scale"]),
                     depth_bias=float(d["depth_bias"]))
    fpc = FramePointCloud.from_frame(Frame(info, d["depth"].astype(np.int32)), cuda)
    ref = sample2_pair(0, 3)["tgt_fpcl"]
    _eq(fpc.points, ref.points)
    _eq(fpc.mask, ref.mask)
    _eq(fpc.normals, ref.normals)


def test_pyramid_levels(cuda, depth_pair):
    from slamtb_gb300.frame import FramePointCloud, KCamera
    depth = depth_pair["source_depth"]
    k = depth_pair["kcam"]
    ref = fp.FramePointCloud.from_depth(depth, k)
    pts = torch.from_numpy(ref.points).to(cuda)
    mask = torch.from_numpy(ref.mask).to(cuda)
    fpc = FramePointCloud(None, mask, KCamera(k).to(cuda), points=pts)
    scales = [1.0, 0.5, 0.5]
    gpu = fpc.pyramid(scales)
    cpu = ref.pyramid(scales)
    assert [g.mask.shape for g in gpu] == [(120, 160), (240, 320), (480, 640)]
    for g, c in zip(gpu, cpu):
        _eq(g.points, c.points)
        _eq(g.mask, c.mask)
        _eq(g.normals, c.normals)
        _eq(g.kcam.matrix, c.kcam)


def test_odd_sizes(cuda):
    from slamtb_gb300 import processing as P
    rng = np.random.default_rng(0)
    xyz = rng.normal(size=(37, 53, 3)).astype(np.float32)
    mask = rng.random((37, 53)) > 0.3
    _eq(P.downsample_xyz(torch.from_numpy(xyz).to(cuda), torch.from_numpy(mask).to(cuda), 0.5),
        fp.downsample_xyz_nearest(xyz, mask, 0.5))
    _eq(P.downsample_mask(torch.from_numpy(mask).to(cuda), 0.5), fp.downsample_mask(mask, 0.5))
    _eq(P.erode_mask(torch.from_numpy(mask).to(cuda)), fp.erode_mask(mask))
    _eq(P.estimate_normals(torch.from_numpy(xyz).to(cuda), torch.from_numpy(mask).to(cuda)),
        fp.estimate_normals(xyz, mask))


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_feature_pyramid(cuda, dtype):
    from slamtb_gb300 import processing as P
    rng = np.random.default_rng(1)
    f = rng.random((3, 48, 64)).astype(np.float32)
    ft = torch.from_numpy(f).to(cuda).to(dtype)
    f32 = ft.float().cpu().numpy()
    blur = P.gaussian_blur3(ft).float().cpu().numpy()
    ref = fp.gaussian_blur3(f32)
    tol = 1e-6 if dtype == torch.float32 else 8e-3
    np.testing.assert_allclose(blur, ref, rtol=0, atol=tol)
    down = P.downsample_features(ft, 0.5).float().cpu().numpy()
    if dtype == torch.float32:
        _eq(down, fp.downsample_features(f32, 0.5))
    else:
        np.testing.assert_allclose(down, fp.downsample_features(f32, 0.5), atol=8e-3)
    pyr = P.feature_pyramid(ft, [1.0, 0.5, 0.5])
    assert [tuple(p.shape) for p in pyr] == [(3, 12, 16), (3, 24, 32), (3, 48, 64)]


def _frame_depth():
    import pathlib
    import sys
    sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent / "golden"))
    from make_golden import load_frame_depth
    return load_frame_depth()


def test_bilateral_reference_test_call(cuda):
    """The reference's own bilateral test (slamtb/_test/test_processing.py:24-43):
    its depth frame as int32, its positional arguments (filter width 13,
    sigma_color 4.5, sigma_space 29.99), against the float32 restatement:
    within 1 depth unit everywhere (that test's tolerance: expf may differ
    by an ulp between implementations), equal almost everywhere."""
    from slamtb_gb300.processing import bilateral_depth_filter
    depth = _frame_depth().astype(np.int32)
    mask = depth > 0
    ref = fp.bilateral_depth_filter(depth, mask, 13, 4.50000000225, 29.9999880000072)
    out = bilateral_depth_filter(torch.from_numpy(depth).to(cuda),
                                 torch.from_numpy(mask).to(cuda), None, 13, 4.50000000225,
                                 29.9999880000072).cpu().numpy()
    assert out.dtype == np.int32
    diff = np.abs(out.astype(np.int64) - ref)
    assert diff.max() <= 1
    assert (diff == 0).mean() > 0.999
    assert np.all(out[~mask] == 0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int16, np.uint16, np.int64])
def test_bilateral_dtypes_and_scale(cuda, dtype):
    from slamtb_gb300.processing import bilateral_depth_filter
    depth = _frame_depth()[100:260, 200:420]
    if dtype in (np.float32, np.float64):
        d, scale = (depth.astype(np.float64) * 0.001).astype(dtype), 1000.0
    else:
        d, scale = depth.astype(dtype), 0.001
    ref = fp.bilateral_depth_filter(d, d > 0, 6, depth_scale=scale)
    td = torch.from_numpy(d.astype(np.int32)).to(cuda).to(torch.uint16) \
        if dtype == np.uint16 else torch.from_numpy(d).to(cuda)
    out = bilateral_depth_filter(td, None, depth_scale=scale)
    if dtype == np.uint16:
        out = out.to(torch.int32)
    out = out.cpu().numpy()
    if np.issubdtype(dtype, np.integer):
        assert np.abs(out.astype(np.int64) - ref.astype(np.int64)).max() <= 1
    else:
        np.testing.assert_allclose(out, ref, rtol=2e-6, atol=0)


def test_bilateral_filter_class_reuses_output(cuda):
    from slamtb_gb300.processing import BilateralDepthFilter
    depth = torch.from_numpy(_frame_depth().astype(np.float32) * 0.001).to(cuda)
    f = BilateralDepthFilter(filter_width=6, depth_scale=1000.0)
    a = f(depth, depth > 0)
    ptr = a.data_ptr()
    b = f(depth * 1.0, depth > 0)
    assert b.data_ptr() == ptr
    ref = fp.bilateral_depth_filter(depth.cpu().numpy(), depth.cpu().numpy() > 0, 6,
                                    depth_scale=1000.0)
    np.testing.assert_allclose(b.cpu().numpy(), ref, rtol=2e-6, atol=0)
