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

    def verify_batch(self, results, num_source):
        """Verdicts for many registrations without leaving the device:
        ``results`` a (B, 96) float64 CUDA tensor of result blocks (what
        ``BatchRegistration.run`` or ``ICPOdometry.launch`` return),
        ``num_source`` the B source point counts (a sequence or an int64
        tensor).  Returns a (B,) bool CUDA tensor (``stb_verify_registrations``:
        the tests of ``__call__`` on the blocks, the covariance test as an
        FP64 positive-definiteness test of information - I / threshold)."""
        from .. import _native as N
        if results.device.type != "cuda" or results.dtype != torch.float64:
            raise RuntimeError("Check failed: results must be a float64 CUDA tensor")
        res = results.reshape(-1, N.RES_SIZE).contiguous()
        dev = res.device
        n = torch.as_tensor(num_source, dtype=torch.int64).to(dev).reshape(-1).contiguous()
        if n.numel() != res.size(0):
            raise RuntimeError("Check failed: one source count per result block")
        out = torch.empty(res.size(0), dtype=torch.int32, device=dev)
        with torch.cuda.device(dev):
            N.check(N.lib().stb_verify_registrations(
                N.ptr(res), N.ptr(n), res.size(0), float(self.match_ratio_threshold),
                float(self.covariance_max_threshold), float(self.residual_threshhold),
                N.ptr(out), N.stream_of(dev)))
        return out.bool()

    def __str__(self):
        return (f"RegistrationVerifier with: match_ratio_threshold = "
                f"{self.match_ratio_threshold} covariance_max_threshold = "
                f"{self.covariance_max_threshold}")

    def __repr__(self):
        return str(self)
