"""RegistrationVerifier on the device (stb_verify_registrations) against the
host verifier (slamtb/registration/result.py:49-95 with
torch.linalg.eigvals) on crafted result blocks: information matrices with
chosen eigenvalues on both sides of 1 / covariance threshold (none at it),
residuals and match ratios on both sides of theirs, and NaN residuals; then
on the result blocks of a real batch."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _blocks(rng, n, thr_cov):
    from slamtb_gb300 import _native as N
    R = np.zeros((n, N.RES_SIZE))
    num = rng.integers(1000, 5000, size=n)
    for p in range(n):
        Q, _ = np.linalg.qr(rng.normal(size=(6, 6)))
        lam = rng.uniform(1.5, 50.0, size=6) / thr_cov
        if p % 3 == 1:
            lam[rng.integers(6)] = rng.uniform(0.05, 0.7) / thr_cov  # covariance too large
        A = (Q * lam) @ Q.T
        R[p, N.RES_INFO:N.RES_INFO + 36] = ((A + A.T) / 2).reshape(-1)
        R[p, N.RES_RESIDUAL] = rng.choice([1e-6, 5e-5, 3e-4, np.inf, np.nan])
        R[p, N.RES_MATCHES] = float(int(num[p] * rng.uniform(0.3, 1.0)))
    return R, num


def test_device_verifier_equals_host_verifier(cuda):
    from slamtb_gb300 import _native as N
    from slamtb_gb300.registration import RegistrationResult, RegistrationVerifier
    rng = np.random.default_rng(7)
    for thr_cov in (1e-4, 1e-2):
        R, num = _blocks(rng, 300, thr_cov)
        ver = RegistrationVerifier(covariance_max_threshold=thr_cov)
        dev = ver.verify_batch(torch.from_numpy(R).to(cuda), num).cpu().numpy()
        host = []
        for p in range(R.shape[0]):
            res = RegistrationResult(
                torch.eye(4, dtype=torch.float64),
                torch.from_numpy(R[p, N.RES_INFO:N.RES_INFO + 36].reshape(6, 6).copy()),
                float(R[p, N.RES_RESIDUAL]), float(R[p, N.RES_MATCHES] / num[p]))
            host.append(ver(res))
        np.testing.assert_array_equal(dev, np.array(host))
        assert 0 < dev.sum() < dev.size  # both verdicts occur


def test_device_verifier_on_batch_results(cuda):
    """A real batch: the device verdicts equal the host verifier's on the
    RegistrationResults (information cast to float64)."""
    from slamtb_gb300.frame import Frame, FrameInfo, FramePointCloud, KCamera
    from slamtb_gb300 import synthetic
    from slamtb_gb300.registration import (BatchRegistration, ICPOdometry,
                                           RegistrationResult, RegistrationVerifier)
    srcs, tgts = [], []
    for seed in range(4):
        p = synthetic.make_pair(90 + seed, width=320, height=240)
        k = KCamera(p["kcam"])
        srcs.append([FramePointCloud.from_frame(Frame(FrameInfo(k), p["source_depth"]), cuda)])
        tgts.append([FramePointCloud.from_frame(Frame(FrameInfo(k), p["target_depth"]), cuda)])
    br = BatchRegistration([(1.0, ICPOdometry(10, geom_weight=1.0, feat_weight=0.0,
                                              distance_threshold=0.1,
                                              normals_angle_thresh=math.radians(20)))])
    results, _, plan = br.launch(srcs, tgts)
    res = br.results(plan)
    for ver in (RegistrationVerifier(), RegistrationVerifier(residual_threshhold=1.0,
                                                             match_ratio_threshold=0.1,
                                                             covariance_max_threshold=1.0)):
        dev = ver.verify_batch(results, plan.num_source).cpu().numpy()
        host = [ver(RegistrationResult(r.transform, r.information.double(), r.residual,
                                       r.match_ratio)) for r in res]
        np.testing.assert_array_equal(dev, np.array(host))
