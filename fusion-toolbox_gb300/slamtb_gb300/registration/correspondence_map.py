"""``slamtb/registration/correspondence_map.py:8-79`` on the GB300 path."""
import torch

from .._cslamtb import CorrespondenceMap as _CorrespondenceMap

_CORRESP_INF = 0x0FFFFFFF7F800000


class CorrespondenceMap:
    """Projective association of source points onto a target point grid.

    Calling it returns an int64 (H, W) map: the high 32 bits hold the index
    of the winning source point (0x0fffffff when none), the low 32 bits the
    float32 distance of the pair.
    """

    def __init__(self, distance_threshold, normals_angle_thresh):
        self.distance_threshold = distance_threshold
        self.normals_angle_thresh = normals_angle_thresh

    def __call__(self, source_points, source_normals, source_mask, transform,
                 target_points, target_normals, target_mask, kcam):
        corresp_map = torch.full((target_points.size(0), target_points.size(1)),
                                 _CORRESP_INF, dtype=torch.int64, device=source_points.device)
        _CorrespondenceMap.compute_correspondence_map(
            source_points.view(-1, 3), source_normals.view(-1, 3), source_mask.view(-1),
            transform, target_points, target_normals, target_mask, kcam, corresp_map,
            float(self.distance_threshold), float(self.normals_angle_thresh))
        return corresp_map
