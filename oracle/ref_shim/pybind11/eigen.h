// Test infrastructure (oracle/build_ref.py).  The reference's
// src/icp_jacobian_feature.cu includes <pybind11/eigen.h> and
// <torch/csrc/utils/pybind.h> but defines no binding: its CUDA compile gets
// this empty header instead (the Eigen subset of oracle/ref_shim lacks what
// pybind11's Eigen casters need).  Other translation units get the real one.
#pragma once
#ifndef __CUDACC__
#include_next <pybind11/eigen.h>
#endif
