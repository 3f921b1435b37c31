// Test infrastructure: a Python module over the reference's own hot-path
// entry points, compiled from the reference's sources by oracle/build_ref.py
// into oracle/_ref/.  Nothing in the product imports it; the CPU tests use
// it to pin the oracle (tests/test_oracle_ref.py).
//
// The reference binds these functions in src/matching.cpp:12-16 and
// src/icp_jacobian.cpp:7-13 together with the rest of its module; this file
// binds only the functions of the registration path, under the names of
// those bindings.  The reference's headers forward-declare
// `pybind11::module` as a class, which the pybind11 of current torch defines
// as an alias, so this file declares the bound functions itself, with the
// signatures of include/slamtb/matching.hpp:12-18,
// include/slamtb/icp_jacobian.hpp:72-85,140-146,201-207 and
// include/slamtb/processing.hpp:11-38.
#include <torch/extension.h>

namespace slamtb {
struct CorrespondenceMap {
  static void ComputeCorrespondenceMap(
      const torch::Tensor &source_points, const torch::Tensor &source_normals,
      const torch::Tensor &source_mask, const torch::Tensor &rt_cam,
      const torch::Tensor &target_points, const torch::Tensor &target_normals,
      const torch::Tensor &target_mask, const torch::Tensor &kcam, torch::Tensor merge_map,
      double distance_thresh, double normal_angle_thesh);
};

struct ICPJacobian {
  static int EstimateGeometric(const torch::Tensor &src_points, const torch::Tensor &src_mask,
                               const torch::Tensor &rt_cam, const torch::Tensor &tgt_points,
                               const torch::Tensor &tgt_normals, const torch::Tensor &kcam,
                               const torch::Tensor &merge_map, torch::Tensor JtJ_partial,
                               torch::Tensor Jr_partial, torch::Tensor squared_residual);
  static void GetInformationMatrix(const torch::Tensor &src_points,
                                   const torch::Tensor &src_mask, const torch::Tensor &rt_cam,
                                   const torch::Tensor &tgt_points, const torch::Tensor &kcam,
                                   const torch::Tensor &merge_map, torch::Tensor GtG_partial);
  static int EstimateFeature(const torch::Tensor &src_points, const torch::Tensor &src_feats,
                             const torch::Tensor &src_mask, const torch::Tensor &rt_cam,
                             const torch::Tensor &tgt_feats, const torch::Tensor &kcam,
                             const torch::Tensor merge_map, float residual_thresh,
                             torch::Tensor JtJ_partial, torch::Tensor Jr_partial,
                             torch::Tensor squared_residuals);
  static int EstimateFeatureSO3(const torch::Tensor &src_points, const torch::Tensor &src_feats,
                                const torch::Tensor &src_mask, const torch::Tensor &rt_cam,
                                const torch::Tensor &tgt_feats, const torch::Tensor &kcam,
                                const torch::Tensor merge_map, float residual_thresh,
                                torch::Tensor JtJ_partial, torch::Tensor Jr_partial,
                                torch::Tensor squared_residuals);
};

// include/slamtb/processing.hpp:11-38
enum EstimateNormalsMethod { kCentralDifferences, kAverage8 };
enum DownsampleXYZMethod { kNearest };

struct Processing {
  static torch::Tensor BilateralDepthFilter(const torch::Tensor &input,
                                            const torch::Tensor &mask, torch::Tensor result,
                                            int filter_width, float sigma_color,
                                            float sigma_space, float depth_scale);
  static void EstimateNormals(const torch::Tensor xyz_image, const torch::Tensor mask_image,
                              torch::Tensor out_normals, EstimateNormalsMethod method);
  static void DownsampleXYZ(const torch::Tensor &src, const torch::Tensor &mask, float scale,
                            torch::Tensor dst, bool normalize, DownsampleXYZMethod method);
  static void DownsampleMask(const torch::Tensor &mask, float scale, torch::Tensor dst);
  static void DownsampleFeatures(const torch::Tensor &feature_image, float scale,
                                 torch::Tensor dst);
  static void ErodeMask(const torch::Tensor &in_mask, torch::Tensor out_mask);
};
}  // namespace slamtb

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
  m.def("compute_correspondence_map", &slamtb::CorrespondenceMap::ComputeCorrespondenceMap);
  m.def("estimate_geometric", &slamtb::ICPJacobian::EstimateGeometric);
  m.def("get_information_matrix", &slamtb::ICPJacobian::GetInformationMatrix);
  m.def("estimate_feature", &slamtb::ICPJacobian::EstimateFeature);
  m.def("estimate_feature_so3", &slamtb::ICPJacobian::EstimateFeatureSO3);
  // frame preparation (src/processing.cpp binds these with default
  // arguments; here they are explicit)
  m.def("bilateral_depth_filter",
        [](const torch::Tensor &input, const torch::Tensor &mask, torch::Tensor result,
           int filter_width, float sigma_color, float sigma_space, float depth_scale) {
          return slamtb::Processing::BilateralDepthFilter(input, mask, result, filter_width,
                                                          sigma_color, sigma_space, depth_scale);
        });
  m.def("estimate_normals_central_differences",
        [](const torch::Tensor &xyz, const torch::Tensor &mask, torch::Tensor out) {
          slamtb::Processing::EstimateNormals(xyz, mask, out, slamtb::kCentralDifferences);
        });
  m.def("downsample_xyz_nearest",
        [](const torch::Tensor &src, const torch::Tensor &mask, float scale, torch::Tensor dst,
           bool normalize) {
          slamtb::Processing::DownsampleXYZ(src, mask, scale, dst, normalize, slamtb::kNearest);
        });
  m.def("downsample_mask", &slamtb::Processing::DownsampleMask);
  m.def("downsample_features", &slamtb::Processing::DownsampleFeatures);
  m.def("erode_mask", &slamtb::Processing::ErodeMask);
}
