"""Drop-in for the hot-path classes of the reference's native module
``slamtb._cslamtb`` (pybind registrations in ``src/_cslamtb.cpp:22-53``,
``src/matching.cpp:12-16``, ``src/icp_jacobian.cpp:7-13``).

Same class names, static-method names, argument order and meaning, and
in-place outputs.  Differences, all deliberate:

* CUDA tensors only.  A CPU tensor raises ``RuntimeError("Check failed:
  ...: Expected a gpu tensor")`` -- the reference's message for a device
  mismatch -- instead of running the reference's OpenMP CPU kernel.
* float32 points, normals, poses and intrinsics (the reference also
  dispatches float64); feature maps may be float32 or bfloat16.
* Ties in the correspondence z-buffer go to the smaller source index (the
  reference keeps whichever thread won the race).
* Calls are asynchronous on the current stream; only the entry points that
  return a match count wait for it, as the reference does.
"""
import torch

from . import _native as N


def _need_cuda(ref, *named):
    if not ref.is_cuda:
        raise RuntimeError("Check failed: source points: Expected a gpu tensor "
                           "(slamtb_gb300 runs on CUDA devices only)")
    dev = ref.device
    for name, t in named:
        if t is None:
            continue
        if not t.is_cuda or t.device != dev:
            raise RuntimeError(f"Check failed: {name}: Expected a gpu tensor on {dev}, "
                               f"got {t.device}")
    return dev


def _f32(name, t):
    if t.dtype != torch.float32:
        raise RuntimeError(f"Check failed: {name}: expected float32, got {t.dtype}")
    return t.contiguous()


def _mask(t):
    if t.dtype != torch.bool:
        t = t.to(torch.bool)
    return t.contiguous()


def _out(name, t, dtype=torch.float32):
    if t.dtype != dtype or not t.is_contiguous():
        raise RuntimeError(f"Check failed: {name}: expected a contiguous {dtype} tensor")
    return t


def _rt(rt_cam):
    rt = _f32("rt_cam", rt_cam)
    if rt.dim() != 2 or rt.size(1) != 4 or rt.size(0) < 3:
        raise RuntimeError("Check failed: rt_cam: expected a 3x4 or 4x4 matrix")
    return rt


def _kcam(kcam):
    k = _f32("kcam", kcam)
    if k.dim() != 2 or k.size(1) != 3 or k.size(0) < 2:
        raise RuntimeError("Check failed: kcam: expected a 3x3 (or 2x3) matrix")
    return k


class CorrespondenceMap:
    """``CorrespondenceMap::ComputeCorrespondenceMap``
    (src/correspondence_map.cu:64-102)."""

    @staticmethod
    def compute_correspondence_map(source_points, source_normals, source_mask,
                                   rt_cam, target_points, target_normals,
                                   target_mask, kcam, merge_map,
                                   distance_thresh, normal_angle_thresh):
        dev = _need_cuda(source_points, ("source_normals", source_normals),
                         ("source_mask", source_mask), ("rt_cam", rt_cam),
                         ("target_points", target_points),
                         ("target_normals", target_normals),
                         ("target_mask", target_mask), ("kcam", kcam),
                         ("merge_map", merge_map))
        sp = _f32("source_points", source_points).view(-1, 3)
        sn = _f32("source_normals", source_normals).view(-1, 3)
        sm = _mask(source_mask).view(-1)
        tp = _f32("target_points", target_points)
        tn = _f32("target_normals", target_normals)
        tm = _mask(target_mask)
        _out("merge_map", merge_map, torch.int64)
        h, w = tm.shape
        rt, k = _rt(rt_cam), _kcam(kcam)
        with torch.cuda.device(dev):
            N.check(N.lib().stb_correspondence_map(
                N.ptr(sp), N.ptr(sn), N.ptr(sm), sp.size(0), sm.numel(), N.ptr(rt),
                N.ptr(tp), N.ptr(tn), N.ptr(tm), h, w, N.ptr(k), N.ptr(merge_map),
                float(distance_thresh), float(normal_angle_thresh), N.stream_of(dev)))


def _count_buffer(dev):
    return torch.zeros(1, dtype=torch.int32, device=dev)


class ICPJacobian:
    """``ICPJacobian`` static methods (include/slamtb/icp_jacobian.hpp)."""

    @staticmethod
    def estimate_geometric(src_points, src_mask, rt_cam, tgt_points, tgt_normals,
                           kcam, merge_map, JtJ_partial, Jr_partial,
                           squared_residual):
        """``ICPJacobian::EstimateGeometric``
        (src/icp_jacobian_geometric.cu:163-214); returns the match count."""
        dev = _need_cuda(src_points, ("src_mask", src_mask), ("rt_cam", rt_cam),
                         ("tgt_points", tgt_points), ("tgt_normals", tgt_normals),
                         ("kcam", kcam), ("merge_map", merge_map),
                         ("JtJ_partial", JtJ_partial), ("Jr_partial", Jr_partial),
                         ("squared_residual", squared_residual))
        sp = _f32("src_points", src_points).view(-1, 3)
        sm = _mask(src_mask).view(-1)
        tp = _f32("tgt_points", tgt_points)
        tn = _f32("tgt_normals", tgt_normals)
        h, w = tp.shape[:2]
        cnt = _count_buffer(dev)
        with torch.cuda.device(dev):
            N.check(N.lib().stb_icp_jacobian_geometric(
                N.ptr(sp), N.ptr(sm), sp.size(0), N.ptr(_rt(rt_cam)), N.ptr(tp),
                N.ptr(tn), h, w, N.ptr(_kcam(kcam)),
                N.ptr(_out("merge_map", merge_map, torch.int64)),
                N.ptr(_out("JtJ_partial", JtJ_partial)), N.ptr(_out("Jr_partial", Jr_partial)),
                N.ptr(_out("squared_residual", squared_residual)), N.ptr(cnt),
                N.stream_of(dev)))
        return int(cnt.item())

    @staticmethod
    def _feature(fn, src_points, src_feats, src_mask, rt_cam, tgt_feats, kcam,
                 merge_map, residual_thresh, JtJ_partial, Jr_partial,
                 squared_residuals):
        dev = _need_cuda(src_points, ("src_feats", src_feats), ("src_mask", src_mask),
                         ("rt_cam", rt_cam), ("tgt_feats", tgt_feats), ("kcam", kcam),
                         ("merge_map", merge_map), ("JtJ_partial", JtJ_partial),
                         ("Jr_partial", Jr_partial),
                         ("squared_residuals", squared_residuals))
        sp = _f32("src_points", src_points).view(-1, 3)
        sm = _mask(src_mask).view(-1)
        tf = tgt_feats.contiguous()
        sf = src_feats.contiguous()
        code = N.feat_dtype_code(tf)
        if sf.dtype != tf.dtype:
            raise RuntimeError("Check failed: src_feats and tgt_feats must share a dtype")
        c, h, w = tf.shape
        cnt = _count_buffer(dev)
        with torch.cuda.device(dev):
            N.check(fn(
                N.ptr(sp), N.ptr(sf), N.ptr(sm), sp.size(0), N.ptr(_rt(rt_cam)),
                N.ptr(tf), c, h, w, code, N.ptr(_kcam(kcam)),
                N.ptr(_out("merge_map", merge_map, torch.int64)), float(residual_thresh),
                N.ptr(_out("JtJ_partial", JtJ_partial)), N.ptr(_out("Jr_partial", Jr_partial)),
                N.ptr(_out("squared_residuals", squared_residuals)), N.ptr(cnt),
                N.stream_of(dev)))
        return int(cnt.item())

    @staticmethod
    def estimate_feature(src_points, src_feats, src_mask, rt_cam, tgt_feats, kcam,
                         merge_map, residual_thresh, JtJ_partial, Jr_partial,
                         squared_residuals):
        """``ICPJacobian::EstimateFeature``
        (src/icp_jacobian_feature.cu:113-169); returns the match count."""
        return ICPJacobian._feature(N.lib().stb_icp_jacobian_feature, src_points,
                                    src_feats, src_mask, rt_cam, tgt_feats, kcam,
                                    merge_map, residual_thresh, JtJ_partial,
                                    Jr_partial, squared_residuals)

    @staticmethod
    def estimate_feature_so3(src_points, src_feats, src_mask, rt_cam, tgt_feats,
                             kcam, merge_map, residual_thresh, JtJ_partial,
                             Jr_partial, squared_residuals):
        """``ICPJacobian::EstimateFeatureSO3``
        (src/icp_jacobian_feature.cu:171-228); returns the match count."""
        return ICPJacobian._feature(N.lib().stb_icp_jacobian_feature_so3, src_points,
                                    src_feats, src_mask, rt_cam, tgt_feats, kcam,
                                    merge_map, residual_thresh, JtJ_partial,
                                    Jr_partial, squared_residuals)

    @staticmethod
    def get_information_matrix(src_points, src_mask, rt_cam, tgt_points, kcam,
                               merge_map, GtG_partial):
        """``ICPJacobian::GetInformationMatrix``
        (src/icp_jacobian_geometric.cu:216-249)."""
        dev = _need_cuda(src_points, ("src_mask", src_mask), ("rt_cam", rt_cam),
                         ("tgt_points", tgt_points), ("kcam", kcam),
                         ("merge_map", merge_map), ("GtG_partial", GtG_partial))
        sp = _f32("src_points", src_points).view(-1, 3)
        sm = _mask(src_mask).view(-1)
        tp = _f32("tgt_points", tgt_points)
        h, w = tp.shape[:2]
        with torch.cuda.device(dev):
            N.check(N.lib().stb_icp_information_partials(
                N.ptr(sp), N.ptr(sm), sp.size(0), N.ptr(_rt(rt_cam)), N.ptr(tp), h, w,
                N.ptr(_kcam(kcam)), N.ptr(_out("merge_map", merge_map, torch.int64)),
                N.ptr(_out("GtG_partial", GtG_partial)), N.stream_of(dev)))
