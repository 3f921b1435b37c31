"""Coarse-to-fine registration (``slamtb/registration/multiscale.py:10-67``)."""
from ..frame import Frame, FramePointCloud, resolve_device
from ..processing import feature_pyramid


class MultiscaleRegistration:
    """Runs one estimator per pyramid level, coarsest first.

    Args:
        estimators (list of (float, estimator)): scale and estimator per
            level, listed finest first as in the reference; scales below 1
            compound (``[(1.0, a), (0.5, b), (0.5, c)]`` runs ``c`` at 1/4,
            then ``b`` at 1/2, then ``a`` at full resolution).
        downsample_xyz_method: accepted for interface compatibility; the
            nearest-to-mean method is the only one.
    """

    def __init__(self, estimators, downsample_xyz_method=None):
        self.estimators = estimators
        self.downsample_xyz_method = downsample_xyz_method

    def estimate_frame(self, source_frame, target_frame, source_feats=None,
                       target_feats=None, transform=None, device=None):
        """Reference quirk kept: a level's result is always truthy, so a
        level whose first iteration fails passes ``transform=None``
        (identity) to the next level (multiscale.py:64-65)."""
        device = resolve_device(device)
        if isinstance(source_frame, Frame):
            source_frame = FramePointCloud.from_frame(source_frame, device)
        if isinstance(target_frame, Frame):
            target_frame = FramePointCloud.from_frame(target_frame, device)
        scales = [scale for scale, _ in self.estimators]
        source_pyr = source_frame.pyramid(scales)
        target_pyr = target_frame.pyramid(scales)
        src_feat_pyr = tgt_feat_pyr = [None] * len(scales)
        if source_feats is not None:
            src_feat_pyr = feature_pyramid(source_feats.to(device), scales)
        if target_feats is not None:
            tgt_feat_pyr = feature_pyramid(target_feats.to(device), scales)
        return self.estimate_pyramid(source_pyr, target_pyr, src_feat_pyr, tgt_feat_pyr,
                                     transform, device)

    def estimate_pyramid(self, source_pyr, target_pyr, src_feat_pyr=None, tgt_feat_pyr=None,
                         transform=None, device=None):
        """The level loop of ``estimate_frame`` on prepared pyramids
        (``FramePointCloud`` levels and feature maps, coarsest first)."""
        n = len(self.estimators)
        src_feat_pyr = src_feat_pyr or [None] * n
        tgt_feat_pyr = tgt_feat_pyr or [None] * n
        curr_result = None
        for ((_, estimator), source, src_feats, target, tgt_feats) in zip(
                self.estimators[::-1], source_pyr, src_feat_pyr, target_pyr, tgt_feat_pyr):
            curr_result = estimator.estimate_frame(
                source, target, source_feats=src_feats, target_feats=tgt_feats,
                transform=transform, device=device)
            transform = curr_result.transform
        return curr_result


# The other name of the multiscale ICP wrapper (MultiscaleICPOdometry).
MultiscaleICPOdometry = MultiscaleRegistration
