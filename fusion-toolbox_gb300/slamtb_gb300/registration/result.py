"""Registration result structures, as ``slamtb/registration/result.py:9-95``."""
import math

import torch


class RegistrationResult:
    """Result of a registration.

    Attributes:
        transform (torch.Tensor): (4, 4) float64 CPU matrix taking source
            points to the target frame, or None when the first Gauss-Newton
            iteration already failed.
        information (torch.Tensor): (6, 6) information matrix at the final
            pose (the source points' dtype, as the reference's
            ``GtG.sum(0).cpu()``).
        residual (float): weighted squared residual over the match count of
            the last successful iteration.
        match_ratio (float): matched / source points of that iteration.
    """

    def __init__(self, transform=None, information=None, residual=math.inf,
                 match_ratio=0, source_size=None, target_size=None):
        self.transform = transform
        self.information = information
        self.residual = residual
        self.match_ratio = match_ratio
        self.source_size = source_size
        self.target_size = target_size

    def __str__(self):
        return (f"RegistrationResult with: transform = {self.transform} "
                f"information = {self.information} residual = {self.residual} "
                f"match_ratio = {self.match_ratio}")

    def __repr__(self):
        return str(self)


class RegistrationVerifier:
    """Heuristic check of a registration (``result.py:49-95``).  The
    covariance test uses ``torch.linalg.eigvals`` (the reference's
    ``torch.eig`` no longer exists)."""

    def __init__(self, match_ratio_threshold=6e-1, covariance_max_threshold=1e-04,
                 residual_threshhold=1e-4):
        self.match_ratio_threshold = match_ratio_threshold
        self.covariance_max_threshold = covariance_max_threshold
        self.residual_threshhold = residual_threshhold

    def __call__(self, result):
        if result.residual > self.residual_threshhold:
            return False
        if result.information is not None:
            eigvals = torch.linalg.eigvals(result.information.double().inverse())
            if torch.any(eigvals.real > self.covariance_max_threshold):
                return False
        if result.match_ratio < self.match_ratio_threshold:
            return False
        return True

    def __str__(self):
        return (f"RegistrationVerifier with: match_ratio_threshold = "
                f"{self.match_ratio_threshold} covariance_max_threshold = "
                f"{self.covariance_max_threshold}")

    def __repr__(self):
        return str(self)
