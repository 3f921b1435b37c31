"""CPU oracle for the ICP registration hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only
as the checker (or as the timed CPU restatement of the reference's CPU path).

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

Parity status
-------------
The reference cannot be built or imported here (its native module needs
Eigen, which is absent, and its Python side needs tenviz/cv2/kornia), so
no reference-generated vectors exist.  The reference's own tests hold no
golden vectors for ICP.  The oracle is pinned by the known answers that
the reference's fixtures do hold: the ground-truth relative poses of the
``test-data/rgbd/sample2`` frame pairs used by its ICP tests
(``slamtb/registration/_test/test_icp.py:19-27``), checked in
``tests/test_oracle_pins.py`` from fixtures extracted by
``tests/golden/make_golden.py``.  Bit-level parity with the reference's own
binaries is therefore unpinned; the pins are known-answer pins.
"""
