"""Matching layers (``slamtb/spatial``): the frame point-cloud matcher."""
from .matching import FPCLMatcherOp, FramePointCloudMatcher

__all__ = ["FPCLMatcherOp", "FramePointCloudMatcher"]
