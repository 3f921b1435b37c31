"""Camera helpers (``slamtb/camera.py``): the intrinsics class and the
differentiable rigid transform of (N, 3) point arrays."""
import torch

from .frame import KCamera

__all__ = ["KCamera", "RigidTransform", "normal_transform_matrix"]


def normal_transform_matrix(matrix):
    """Transpose of the inverse of the 3x3 block (``camera.py:409-420``)."""
    return torch.inverse(matrix[:3, :3]).transpose(1, 0)


class RigidTransform:
    """``R p + t`` for (N, 3) points and ``(R^-1)^T n`` for normals
    (``camera.py:310-408``); plain torch operations, so gradients reach the
    matrix."""

    def __init__(self, matrix):
        self.matrix = matrix
        self._normal_matrix = None

    def __matmul__(self, points):
        points = self.matrix[:3, :3].matmul(points.view(-1, 3, 1))
        points = points + self.matrix[:3, 3].view(3, 1)
        return points.squeeze()

    def transform_normals(self, normals):
        return (self.normal_matrix @ normals.view(-1, 3, 1)).view(-1, 3)

    @property
    def normal_matrix(self):
        if self._normal_matrix is None:
            self._normal_matrix = normal_transform_matrix(self.matrix)
        return self._normal_matrix
