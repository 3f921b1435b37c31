"""Registration algorithms (``slamtb.registration`` drop-in)."""
from .icp import ICPOdometry
from .multiscale import MultiscaleRegistration, MultiscaleICPOdometry
from .result import RegistrationResult, RegistrationVerifier
from .correspondence_map import CorrespondenceMap
from .preset import create_multiscale_odometry
from .batch import BatchRegistration
from .grad import PointToPlaneLoss, point_to_plane_loss, se3_exp_compose
from .se3 import ExpRtToMatrix, MatrixToExpRt
from .autogradicp import AutogradICP

__all__ = ["ICPOdometry", "MultiscaleRegistration", "MultiscaleICPOdometry",
           "RegistrationResult", "RegistrationVerifier", "CorrespondenceMap",
           "create_multiscale_odometry", "BatchRegistration", "PointToPlaneLoss",
           "point_to_plane_loss", "se3_exp_compose", "ExpRtToMatrix", "MatrixToExpRt",
           "AutogradICP"]
