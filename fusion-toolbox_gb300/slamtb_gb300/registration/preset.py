"""Factory presets (``slamtb/registration/preset.py:10-49``)."""
import math

from .icp import ICPOdometry
from .multiscale import MultiscaleRegistration


def create_multiscale_odometry(geom_weight=10.0, feat_weight=1.0):
    """Three-level odometry with the reference's parameters."""
    params1 = dict(geom_weight=geom_weight, feat_weight=feat_weight, distance_threshold=1.5,
                   normals_angle_thresh=math.pi, feat_residual_thresh=5)
    params2 = dict(geom_weight=geom_weight, feat_weight=feat_weight, distance_threshold=1,
                   normals_angle_thresh=math.pi / 2, feat_residual_thresh=2)
    params3 = dict(geom_weight=geom_weight, feat_weight=feat_weight, distance_threshold=1,
                   normals_angle_thresh=math.pi / 4, feat_residual_thresh=2)
    return MultiscaleRegistration([
        (1.0, ICPOdometry(5, **params1)),
        (0.5, ICPOdometry(10, **params2)),
        (0.5, ICPOdometry(20, **params3))])
