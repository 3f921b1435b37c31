"""slamtb_gb300: fusion-toolbox's ICP registration path on GB300 (sm_103a).

Public modules mirror the reference package ``slamtb``:
``slamtb_gb300.registration`` (ICPOdometry, MultiscaleRegistration,
RegistrationResult, ...), ``slamtb_gb300._cslamtb`` (CorrespondenceMap and
ICPJacobian with the native module's signatures), ``slamtb_gb300.frame``
and ``slamtb_gb300.processing`` (device-side frame preparation).  All
compute runs in ``libslamtb_gb300.so`` (C ABI in ``include/slamtb_gb300.h``).
"""
__version__ = "0.1.0"
