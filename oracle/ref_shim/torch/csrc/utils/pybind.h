// Test infrastructure (oracle/build_ref.py).  The reference's
// src/icp_jacobian_feature.cu includes this header after
// include/slamtb/icp_jacobian.hpp, whose forward declaration of
// `pybind11::module` as a class conflicts with the alias of current
// pybind11; that file defines no binding, so its CUDA compile gets this
// empty header.  Other translation units (the module's own binding) get the
// real one.
#pragma once
#ifndef __CUDACC__
#include_next <torch/csrc/utils/pybind.h>
#endif
