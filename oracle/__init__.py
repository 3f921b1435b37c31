"""CPU oracle for the ICP registration hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory: only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``
use it, and only as the checker: the ``cpu_baseline`` / ``--impl
reference`` legs time the C restatement of the reference's CPU path, and
the accuracy report of the secondary workloads compares the GPU results,
after their timed runs, with free-running FP64 oracle registrations.

Contents
--------
``icp_oracle``   numpy restatement of fusion-toolbox's ICP path:
                 projective association (FP32, op-by-op, bit-exact gate),
                 per-point partials (FP32, op-by-op), and FP64 sums, 6x6
                 Cholesky and SE(3) exponential (the 1e-5 error reference).
``frame_prep``   numpy restatement of the frame preparation that feeds the
                 path (mask erosion, back-projection, central-difference
                 normals, XYZ / mask / feature pyramids).
``autograd_oracle``  restatement of the differentiable registration layer
                 (twist <-> matrix maps and their backward in FP64; the
                 frame point-cloud matcher, FP32 op by op).
``png16``        a small PNG reader for the reference's 16-bit depth test
                 frames (the image has neither cv2 nor PIL).
``icp_port.c``   C/OpenMP restatement of the reference's CPU ICP path,
                 timed as the CPU baseline (``kind: "port"``).
``build_ref``    builds the reference's own registration and frame-
                 preparation sources (with ``ref_shim``, the project's
                 Eigen subset, and ``ref_binding.cpp``) into ``_ref/`` where
                 the reference tree is available.

Parity status
-------------
The oracle is pinned to the reference's own code: ``tests/test_oracle_ref.py``
runs the ``build_ref`` module (the reference's CPU path) on the oracle's
inputs and requires equal bits for correspondence maps, per-point partials,
match counts and the frame preparation; digests of the reference's outputs
on its sample2 frames (``tests/golden/ref_vectors.npz``) pin the oracle and
the GPU kernels where the reference tree is absent.  Not built: the
reference's Python loop (weighting, solve, tenviz SE(3) exponential) and
kornia's blur, which stay restatements.
"""
