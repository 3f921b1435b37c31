/*
 * slamtb_gb300 -- C ABI of the GB300 (sm_103a) ICP registration path.
 *
 * Conventions shared by every entry point:
 *   - All array arguments are DEVICE pointers to contiguous row-major data
 *     on the calling thread's current CUDA device, unless stated otherwise.
 *   - Masks are one byte per element (0 = invalid), like torch.bool.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Every
 *     entry point is asynchronous on that stream; none synchronises.
 *   - The library never allocates or frees memory the caller sees: outputs
 *     and scratch ("workspace") are caller-provided.
 *   - Return value: STB_OK (0) or one of the STB_E* codes below;
 *     stb_last_error() returns a message for the calling thread.
 *
 * Reference interfaces replaced (fusion-toolbox, paths in that project):
 *   _cslamtb.CorrespondenceMap.compute_correspondence_map
 *        include/slamtb/matching.hpp:12-18, src/correspondence_map.cu:64-102
 *   _cslamtb.ICPJacobian.estimate_geometric
 *        include/slamtb/icp_jacobian.hpp:72-77, src/icp_jacobian_geometric.cu:163-214
 *   _cslamtb.ICPJacobian.estimate_feature
 *        include/slamtb/icp_jacobian.hpp:140-146, src/icp_jacobian_feature.cu:113-169
 *   _cslamtb.ICPJacobian.estimate_feature_so3
 *        include/slamtb/icp_jacobian.hpp:201-207, src/icp_jacobian_feature.cu:171-228
 *   _cslamtb.ICPJacobian.get_information_matrix
 *        include/slamtb/icp_jacobian.hpp:79-85, src/icp_jacobian_geometric.cu:216-249
 *   slamtb.registration.icp.ICPOdometry.estimate (the whole Gauss-Newton
 *        loop, with the sums of icp.py:78-80, the CPU Cholesky solve and
 *        SE3.exp update of icp.py:236-256 and the information matrix of
 *        icp.py:258-261 moved onto the device)
 *        slamtb/registration/icp.py:152-262
 */
#ifndef SLAMTB_GB300_H_
#define SLAMTB_GB300_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define STB_API __attribute__((visibility("default")))
#else
#define STB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define STB_OK 0
#define STB_EINVAL 1   /* bad size, shape or argument value          */
#define STB_EDEVICE 2  /* pointer is not device memory of this device */
#define STB_EDTYPE 3   /* unsupported element type                    */
#define STB_ECUDA 4    /* CUDA runtime error                          */
#define STB_ETIMEOUT 5 /* a bounded device-side wait gave up          */

/* ---- element types for feature maps ----------------------------------- */
#define STB_F32 0
#define STB_BF16 1
/* Texel-major feature layout ([count][channels]: all channels of a pixel
 * adjacent) of the same element types, accepted by stb_icp_estimate and
 * stb_icp_estimate_batch; produce it with stb_feature_interleave.  The
 * reference's layout ([channels][count]) is STB_F32 / STB_BF16. */
#define STB_F32_HWC 2
#define STB_BF16_HWC 3
/* Further element types of depth images (stb_bilateral_depth_filter). */
#define STB_F64 4
#define STB_U8 5
#define STB_I16 6
#define STB_U16 7
#define STB_I32 8
#define STB_I64 9

/* ---- option bits, or-ed into the channel_mode argument of the
 * registration entry points (the low byte is the channel mode) ---------- */
/* Gauss-Newton step in double-word float32 arithmetic (~48 significant
 * bits, FP32 pipes only) instead of the default FP64 solve, exponential
 * and pose composition.  No counterpart in the reference (its solve is
 * FP64 on the host, slamtb/registration/icp.py:236-251). */
#define STB_OPT_DW_SOLVE 0x100
/* stb_icp_estimate(_static): the kernel sequence of two launches per
 * iteration (association, then reduction with the solve in its last block),
 * replayable as a CUDA graph, instead of the default single cooperative
 * launch that runs the whole registration with grid barriers. */
#define STB_OPT_MULTI_LAUNCH 0x200
/* stb_icp_estimate_batch: the grouped schedule instead of the lock-step
 * one.  The grid is split into tile_config groups (1 .. 96) of equal size;
 * each group registers whole pairs (all levels and iterations, then the
 * information matrix), one after the other, largest pairs first, with
 * barriers of its own, so a pair's frames stay in L2 across its iterations
 * and the groups' serial steps overlap.  Results are those of the
 * lock-step schedule up to the order of float32 sums. */
#define STB_OPT_GROUPS 0x400

/* ---- per-registration status bits (result block, STB_RES_STATUS) ------- */
#define STB_ST_NOT_PD 1u     /* 6x6 J^T J was not positive definite: stopped */
#define STB_ST_NO_MATCHES 2u /* an iteration found no correspondence        */
#define STB_ST_NAN 4u        /* a non-finite update was produced            */
#define STB_ST_TIMEOUT 8u    /* a bounded grid barrier gave up (batch path) */
#define STB_ST_CAPACITY 16u  /* workspace sized for fewer pixels (batch path) */

/* ---- layout of the device result block (doubles) ----------------------- */
#define STB_RES_TRANSFORM 0   /* 16: final 4x4 pose, row-major             */
#define STB_RES_JTJ 16        /* 36: combined J^T J of the last good step  */
#define STB_RES_INFO 52       /* 36: information matrix at the final pose  */
#define STB_RES_RESIDUAL 88   /* residual / match count of last good step  */
#define STB_RES_MATCHES 89    /* match count of the last good step         */
#define STB_RES_ITERS 90      /* number of successful iterations           */
#define STB_RES_STATUS 91     /* STB_ST_* bits                             */
#define STB_RES_SIZE 96

/* ---- layout of one per-iteration history record (doubles) ------------- */
#define STB_HIST_TRANSFORM 0 /* 16: pose after this iteration's update     */
#define STB_HIST_JTJ 16      /* 36: combined J^T J                          */
#define STB_HIST_JR 52       /*  6: combined J^T r                          */
#define STB_HIST_R2 58       /* weighted sum of squared residuals           */
#define STB_HIST_GEOM_COUNT 59
#define STB_HIST_FEAT_COUNT 60
#define STB_HIST_OK 61       /* 1 when the solve succeeded                 */
#define STB_HIST_SIZE 64

/* Message of the last failing call on this thread ("" if none). */
STB_API const char *stb_last_error(void);

/* Library version string. */
STB_API const char *stb_version(void);

/* ======================================================================= *
 * _cslamtb-compatible entry points (per-point partial outputs)
 * ======================================================================= */

/*
 * Projective data association into a reference-layout correspondence map.
 * Replaces CorrespondenceMap::ComputeCorrespondenceMap
 * (src/correspondence_map.cu:64-102; pybind at src/matching.cpp:12-16).
 *
 * source_points/normals: float32 [num_source, 3]; source_mask: bool
 * [source_mask_len] (the mask is ignored unless source_mask_len ==
 * num_source, as the reference).  rt_cam: float32 row-major 3x4 or 4x4
 * (first three rows used).  target_points/normals: float32 [height, width,
 * 3]; target_mask: bool [height, width].  kcam: float32 row-major 3x3.
 * merge_map: int64 [height, width], in/out, normally prefilled with
 * 0x0fffffff7f800000; an entry is (source index << 32) | float bits of the
 * distance, and a candidate replaces it when its (distance, index) pair is
 * lexicographically smaller.
 */
STB_API int stb_correspondence_map(const float *source_points,
                           const float *source_normals,
                           const uint8_t *source_mask, int64_t num_source,
                           int64_t source_mask_len, const float *rt_cam,
                           const float *target_points,
                           const float *target_normals,
                           const uint8_t *target_mask, int32_t height,
                           int32_t width, const float *kcam, int64_t *merge_map,
                           double distance_thresh, double normal_angle_thresh,
                           void *stream);

/*
 * Point-to-plane partials.  Replaces ICPJacobian::EstimateGeometric
 * (src/icp_jacobian_geometric.cu:163-214).
 * Writes JtJ_partial float32 [num_source, 6, 6], Jr_partial [num_source, 6]
 * and squared_residual [num_source] for every source point (zeros where
 * unmatched) and adds the number of matches to *match_count (device int32;
 * the caller zeroes it).
 */
STB_API int stb_icp_jacobian_geometric(const float *src_points, const uint8_t *src_mask,
                               int64_t num_source, const float *rt_cam,
                               const float *tgt_points,
                               const float *tgt_normals, int32_t height,
                               int32_t width, const float *kcam,
                               const int64_t *merge_map, float *JtJ_partial,
                               float *Jr_partial, float *squared_residual,
                               int32_t *match_count, void *stream);

/*
 * Feature-residual partials.  Replaces ICPJacobian::EstimateFeature
 * (src/icp_jacobian_feature.cu:113-169).  src_feats: [channels, num_source],
 * tgt_feats: [channels, height, width], both of element type feat_dtype
 * (STB_F32 or STB_BF16).  Reproduces the reference's partials exactly,
 * including that with several channels only the last channel's J and J*r
 * survive (the squared residual sums all channels).
 */
STB_API int stb_icp_jacobian_feature(const float *src_points, const void *src_feats,
                             const uint8_t *src_mask, int64_t num_source,
                             const float *rt_cam, const void *tgt_feats,
                             int32_t channels, int32_t height, int32_t width,
                             int32_t feat_dtype, const float *kcam,
                             const int64_t *merge_map, float residual_thresh,
                             float *JtJ_partial, float *Jr_partial,
                             float *squared_residuals, int32_t *match_count,
                             void *stream);

/*
 * Rotation-only feature partials (3x3 block of the 6x6 buffers, the rest
 * zero).  Replaces ICPJacobian::EstimateFeatureSO3
 * (src/icp_jacobian_feature.cu:171-228, SO3ICPJacobian at
 * src/icp_jacobian_common.hpp:64-113).  Same arguments as
 * stb_icp_jacobian_feature.
 */
STB_API int stb_icp_jacobian_feature_so3(const float *src_points, const void *src_feats,
                                 const uint8_t *src_mask, int64_t num_source,
                                 const float *rt_cam, const void *tgt_feats,
                                 int32_t channels, int32_t height,
                                 int32_t width, int32_t feat_dtype,
                                 const float *kcam, const int64_t *merge_map,
                                 float residual_thresh, float *JtJ_partial,
                                 float *Jr_partial, float *squared_residuals,
                                 int32_t *match_count, void *stream);

/*
 * Information-matrix partials G^T G.  Replaces
 * ICPJacobian::GetInformationMatrix (src/icp_jacobian_geometric.cu:216-249).
 * GtG_partial: float32 [num_source, 6, 6].
 */
STB_API int stb_icp_information_partials(const float *src_points,
                                 const uint8_t *src_mask, int64_t num_source,
                                 const float *rt_cam, const float *tgt_points,
                                 int32_t height, int32_t width,
                                 const float *kcam, const int64_t *merge_map,
                                 float *GtG_partial, void *stream);

/* ======================================================================= *
 * Fused Gauss-Newton registration (the ICPOdometry.estimate hot loop)
 * ======================================================================= */

/* Scratch bytes stb_icp_estimate needs for these sizes (256-byte aligned
 * base required). */
STB_API size_t stb_icp_workspace_bytes(int64_t num_source, int32_t height,
                               int32_t width);

/*
 * The whole ICPOdometry.estimate loop (slamtb/registration/icp.py:152-262)
 * on the device, without host synchronisation:
 *   per iteration: association (shared by both terms), fused residual /
 *   Jacobian / normal-equation reduction (compensated float32), 6x6 LDL^T
 *   solve, SE(3) exponential and left pose update in FP64 (double-word
 *   float32 with STB_OPT_DW_SOLVE); then the information matrix at the
 *   final pose.  By default one cooperative launch runs it all, its phases
 *   separated by bounded grid barriers (a wait that runs out sets
 *   STB_ST_TIMEOUT); STB_OPT_MULTI_LAUNCH selects two launches per
 *   iteration instead.
 * Weighting follows the reference: J^T J = sum w_t^2 J_t^T J_t,
 * J^T r = w_g J_g^T r_g - w_f J_f^T r_f, residual = sum w_t r_t^2 divided by
 * the larger match count.  A non-positive-definite J^T J stops the loop
 * (STB_ST_NOT_PD) and keeps the last good step, as the reference's
 * `except: break`.
 *
 * kcam: float32 3x3.  src_*: as stb_correspondence_map (source_mask must
 * have num_source entries).  src_feats / tgt_feats: NULL for geometric-only
 * or [channels, num_source] / [channels, height, width] of feat_dtype.
 * init_transform: float64 4x4 or NULL (identity).  kcam and init_transform
 * may be device or host pointers: host values are read during the call and
 * carried in the launch parameters (no copy, no synchronisation), so the
 * host buffers can be reused as soon as the call returns.
 * channel_mode: 0 = reference behaviour (last channel's J), 1 = sum over
 * channels; or-ed with STB_OPT_* bits.  result: float64 [STB_RES_SIZE] device block.  history: NULL or
 * float64 [num_iters, STB_HIST_SIZE] per-iteration records.
 * num_iters <= 254.  workspace: stb_icp_workspace_bytes() bytes.
 * use_graph != 0 (with STB_OPT_MULTI_LAUNCH) captures the launch sequence
 * in a CUDA graph on first use for this (workspace, sizes, options) and
 * replays it afterwards; the single launch needs no graph.
 */
STB_API int stb_icp_estimate(const float *kcam, const float *src_points,
                     const float *src_normals, const uint8_t *src_mask,
                     int64_t num_source, const void *src_feats,
                     const float *tgt_points, const float *tgt_normals,
                     const uint8_t *tgt_mask, int32_t height, int32_t width,
                     const void *tgt_feats, int32_t channels,
                     int32_t feat_dtype, const double *init_transform,
                     int32_t num_iters, double geom_weight, double feat_weight,
                     double distance_thresh, double normal_angle_thresh,
                     double feat_residual_thresh, int32_t channel_mode,
                     void *workspace, size_t workspace_bytes, double *result,
                     double *history, int32_t use_graph, void *stream);

/*
 * The correspondences of the association at the final pose of the last
 * stb_icp_estimate call on this workspace (the pass that feeds the
 * information matrix, icp.py:258-261), in the reference's correspondence-map
 * layout: merge_map int64 [height, width] = (source index << 32) | float32
 * bits of the distance, 0x0fffffff7f800000 where no source point matched
 * (slamtb/registration/correspondence_map.py:5, src/merge_map.hpp:54-98).
 * height, width and num_iters are those of that call; run it first on the
 * same stream (or synchronise).  The fused kernels keep an epoch-tagged key
 * map that no reference function exposes; this entry point decodes it, so
 * callers that consume the reference's map (FPCLMatcherOp, the partial
 * entry points above) can reuse the registration's last association.
 */
STB_API int stb_icp_correspondences(const void *workspace, int32_t height, int32_t width,
                                    int32_t num_iters, int64_t *merge_map, void *stream);

/* ======================================================================= *
 * Batched, multiscale registration in one persistent launch
 * ======================================================================= */

/* One pyramid level of one frame pair (device pointers; layouts as
 * stb_icp_estimate).  src_feats / tgt_feats may be NULL. */
typedef struct {
  const float *src_points;
  const float *src_normals;
  const uint8_t *src_mask;
  int64_t num_source;
  const void *src_feats;
  const float *tgt_points;
  const float *tgt_normals;
  const uint8_t *tgt_mask;
  int32_t height;
  int32_t width;
  const void *tgt_feats;
  float fx, fy, cx, cy; /* this level's intrinsics */
} stb_level;

/* Estimator parameters of one level, shared by all pairs: the
 * ICPOdometry(num_iters, geom_weight, feat_weight, distance_threshold,
 * normals_angle_thresh, feat_residual_thresh) of that level. */
typedef struct {
  int32_t num_iters;
  double geom_weight;
  double feat_weight;
  double distance_thresh;
  double normal_angle_thresh;
  double feat_residual_thresh;
} stb_level_params;

/* Workspace bytes for num_pairs pairs whose largest levels hold
 * total_target_pixels target pixels together. */
STB_API size_t stb_icp_batch_workspace_bytes(int32_t num_pairs,
                                             int64_t total_target_pixels);

/*
 * MultiscaleRegistration.estimate_frame (slamtb/registration/multiscale.py:
 * 30-67) for many frame pairs at once: every pair runs the levels coarsest
 * first, each level the Gauss-Newton loop of ICPOdometry.estimate
 * (icp.py:152-262) with that level's parameters, the next level starting
 * from the previous level's pose (identity when that level's first
 * iteration failed, as the reference), then the information matrix at the
 * final pose.  One cooperative persistent kernel covers all pairs, levels
 * and iterations: phases (association, reduction + per-pair FP64 solve) are
 * separated by grid barriers whose waits are bounded (a barrier that waits
 * too long sets STB_ST_TIMEOUT in every pair's status and the kernel
 * returns).
 *
 * levels: device array [num_pairs][num_levels], coarsest level first;
 * finest level last.  params: host array [num_levels].  All levels share
 * channels / feat_dtype.  init_transforms: device float64 [num_pairs][16]
 * or NULL.  total_target_pixels: sum over pairs of the largest level's
 * height * width.  results: device float64
 * [num_pairs][STB_RES_SIZE] (the last level's RegistrationResult).
 * history: NULL or device float64 [num_pairs][sum of num_iters][STB_HIST_SIZE].
 * tile_config: largest pixels per work item, 0 = 8192, 1..5 = 512 <<
 * (tile_config - 1); every level uses the largest power of two up to it that
 * still gives half of the blocks a work item per phase.  With
 * STB_OPT_GROUPS in channel_mode, tile_config is the number of groups of
 * the grouped schedule (1 .. 96).
 */
STB_API int stb_icp_estimate_batch(
    const stb_level *levels, int32_t num_pairs, int32_t num_levels,
    const stb_level_params *params, int32_t channels, int32_t feat_dtype,
    int32_t channel_mode, const double *init_transforms,
    int64_t total_target_pixels, void *workspace, size_t workspace_bytes,
    double *results, double *history, int32_t tile_config, void *stream);

/*
 * Pair `pair`'s correspondences at its final pose after the last
 * stb_icp_estimate_batch call on this workspace (the association of the
 * information pass on the finest level), in the layout of
 * stb_icp_correspondences.  num_pairs and total_target_pixels are those of
 * that call; height x width is the pair's finest level; total_iters is the
 * sum of num_iters over the levels of that call.
 */
STB_API int stb_icp_batch_correspondences(const void *workspace, int32_t num_pairs,
                                          int64_t total_target_pixels, int32_t pair,
                                          int32_t height, int32_t width, int32_t total_iters,
                                          int64_t *merge_map, void *stream);

/*
 * RegistrationVerifier.__call__ (slamtb/registration/result.py:49-95) for
 * num_results result blocks on the device: verdict[p] = 1 when
 * residual <= residual_thresh, every eigenvalue of the inverse of the
 * information matrix is <= covariance_max_thresh and matches /
 * num_source[p] >= match_ratio_thresh, else 0.  results: float64
 * [num_results][STB_RES_SIZE] (stb_icp_estimate / stb_icp_estimate_batch
 * blocks); num_source: int64 [num_results]; verdict: int32 [num_results];
 * all device arrays.  The covariance test is an FP64 LDL^T of
 * information - I / covariance_max_thresh (positive definite exactly when
 * every eigenvalue of the information matrix exceeds 1 / threshold); it
 * assumes a positive semi-definite information matrix, which G^T G sums
 * are, and rejects an eigenvalue exactly at the threshold.
 */
STB_API int stb_verify_registrations(const double *results, const int64_t *num_source,
                                     int32_t num_results, double match_ratio_thresh,
                                     double covariance_max_thresh, double residual_thresh,
                                     int32_t *verdict, void *stream);

/*
 * Processing::BilateralDepthFilter (src/bilateral_depth_filter.cu:15-110):
 * out[r][c] = 0 where mask[r][c] is 0, else the average of the masked
 * neighbours' depth within filter_width / 2 pixels, weighted by
 * exp(-0.5 (d_space^2 / sigma_space^2 + d_depth^2 / sigma_color^2)),
 * computed in float32 on depth * depth_scale and divided back.  depth and
 * out: [height][width] of element type dtype (STB_F32, STB_F64, STB_U8,
 * STB_I16, STB_U16, STB_I32 or STB_I64; integers truncate), mask:
 * uint8 [height][width].  filter_width <= 31.
 */
STB_API int stb_bilateral_depth_filter(const void *depth, const uint8_t *mask, void *out,
                                       int32_t height, int32_t width, int32_t dtype,
                                       int32_t filter_width, float sigma_color,
                                       float sigma_space, float depth_scale, void *stream);

/*
 * dst[k * channels + c] = src[c * count + k]: feature maps from the
 * reference's planar layout [channels][count] to the texel-major layout
 * [count][channels] (STB_F32_HWC / STB_BF16_HWC) that the registration
 * kernels sample with all channels of a texel in adjacent bytes.
 * feat_dtype: STB_F32 or STB_BF16 (the element type of both arrays).  No
 * counterpart in the reference.
 */
STB_API int stb_feature_interleave(const void *src, void *dst, int32_t channels,
                                   int64_t count, int32_t feat_dtype, void *stream);

/* ======================================================================= *
 * Differentiable point-to-plane loss (hand-written adjoint)
 * ======================================================================= */

/*
 * out[p] = exp(twist[p]) * base[p] for p < num_pairs: FP64 SE(3)
 * exponential of [translation; rotation] twists and left composition.
 * twist: device float64 [num_pairs][6]; base, out: [num_pairs][16].  No
 * counterpart in the reference (it uses tenviz SE3.exp on the CPU,
 * icp.py:245-247).
 */
STB_API int stb_se3_exp_compose(const double *twist, const double *base,
                                double *out, int32_t num_pairs, void *stream);

/*
 * grad_twist[p] = J_l(twist[p])^T grad_tangent[p]: turns the gradient of a
 * loss with respect to the left perturbation of exp(twist) * base (what
 * stb_icp_loss_backward returns) into its gradient with respect to twist.
 * J_l is the SE(3) left Jacobian of [translation; rotation] twists, summed
 * in FP64 from its power series.  All arrays device float64 [num_pairs][6].
 */
STB_API int stb_se3_twist_grad(const double *twist, const double *grad_tangent,
                               double *grad_twist, int32_t num_pairs, void *stream);

/* Workspace bytes of stb_icp_loss_forward / _backward for num_pairs pairs
 * of height x width frames. */
STB_API size_t stb_icp_loss_workspace_bytes(int32_t num_pairs, int32_t height,
                                            int32_t width);

/*
 * Point-to-plane loss L_p = sum over correspondences of ((q - T_p s).n)^2
 * for each pair p of a batch at pose T_p (device float64 [num_pairs][16]).
 * Inputs are dense device arrays over the batch, pair p at pixel offset
 * p * height * width: src_depth float32 [B][H][W] (metres), src_normals
 * float32 [B][H][W][3], src_mask uint8 [B][H][W], tgt_points / tgt_normals
 * float32 [B][H][W][3], tgt_mask uint8 [B][H][W]; fx, fy, cx, cy are the
 * intrinsics of every frame.  Source points are the back-projection of
 * stb_depth_to_points (scale 1, bias 0) computed in the kernels.  The
 * association of ICPOdometry (thresholds as stb_icp_estimate) runs at the
 * float32 cast of T_p, then the residuals of the geometric term
 * (icp_jacobian_geometric.cu:82) are summed in compensated float32 into
 * loss[p] (device float64 [num_pairs]).  The correspondences stay in the
 * workspace for stb_icp_loss_backward.  No counterpart in the reference
 * (its autograd ICP differentiates through PyTorch ops,
 * slamtb/registration/autogradicp.py:145-239).
 */
STB_API int stb_icp_loss_forward(const float *src_depth, const float *src_normals,
                                 const uint8_t *src_mask, const float *tgt_points,
                                 const float *tgt_normals, const uint8_t *tgt_mask,
                                 int32_t num_pairs, int32_t height, int32_t width,
                                 float fx, float fy, float cx, float cy,
                                 const double *poses, double distance_thresh,
                                 double normal_angle_thresh, void *workspace,
                                 size_t workspace_bytes, double *loss, void *stream);

/*
 * The correspondences that the last stb_icp_loss_forward call on this
 * workspace found, for every pair: merge_map int64 [num_pairs][height]
 * [width] in the layout of stb_icp_correspondences.
 */
STB_API int stb_icp_loss_correspondences(const void *workspace, int32_t num_pairs,
                                         int32_t height, int32_t width, int64_t *merge_map,
                                         void *stream);

/*
 * Adjoint of stb_icp_loss_forward at the correspondences it found (same
 * inputs, poses and workspace): with g = grad_loss[p],
 *   grad_tangent[p] = g * dL_p/de = -2 g sum r J,  J = [n; Tp x n], for the
 *     left perturbation T <- exp(e) T_p (device float64 [num_pairs][6]),
 *   grad_depth[p][i] = g * dL_p/dz_i = -2 g r_i (R^T n).((u_i - cx)/fx,
 *     (v_i - cy)/fy, 1) for source pixel i = v_i * width + u_i, 0 where
 *     source pixel i has no correspondence (device float32 [B][H][W]).
 * Either output may be NULL.  Source normals only gate the association and
 * get no gradient.
 */
STB_API int stb_icp_loss_backward(const float *src_depth, const float *src_normals,
                                  const uint8_t *src_mask, const float *tgt_points,
                                  const float *tgt_normals, const uint8_t *tgt_mask,
                                  int32_t num_pairs, int32_t height, int32_t width,
                                  float fx, float fy, float cx, float cy,
                                  const double *poses, const double *grad_loss,
                                  void *workspace, size_t workspace_bytes,
                                  double *grad_tangent, float *grad_depth, void *stream);

/*
 * stb_icp_loss_forward with the adjoint at a unit output gradient computed
 * in the same pass over the correspondences: loss[p] as stb_icp_loss_forward,
 * tangent[p] = dL_p/de (device float64 [num_pairs][6]) and depth_adjoint
 * [p][i] = dL_p/dz_i (device float32 [B][H][W], 0 where source pixel i has
 * no correspondence; may be NULL), i.e. stb_icp_loss_backward's outputs at
 * grad_loss = 1, bit for bit.  stb_icp_loss_scale_adjoint then gives the
 * gradients for any grad_loss without reading the frames again.  Same
 * counterpart as stb_icp_loss_forward (the reference's autograd ICP,
 * slamtb/registration/autogradicp.py:145-239, differentiates through
 * PyTorch ops).
 */
STB_API int stb_icp_loss_forward_adjoint(const float *src_depth, const float *src_normals,
                                         const uint8_t *src_mask, const float *tgt_points,
                                         const float *tgt_normals, const uint8_t *tgt_mask,
                                         int32_t num_pairs, int32_t height, int32_t width,
                                         float fx, float fy, float cx, float cy,
                                         const double *poses, double distance_thresh,
                                         double normal_angle_thresh, void *workspace,
                                         size_t workspace_bytes, double *loss,
                                         double *tangent, float *depth_adjoint,
                                         void *stream);

/*
 * The gradients of stb_icp_loss_backward from stb_icp_loss_forward_adjoint's
 * unit-gradient outputs: grad_tangent[p] = grad_loss[p] * tangent[p] (FP64)
 * and grad_depth[p][i] = (float)grad_loss[p] * depth_adjoint[p][i].  Either
 * output may be NULL (then its input may be NULL too).  Equal to
 * stb_icp_loss_backward at grad_loss = 1; otherwise within float32 rounding
 * of it (the product is rounded once more).
 */
STB_API int stb_icp_loss_scale_adjoint(const double *grad_loss, const double *tangent,
                                       const float *depth_adjoint, int32_t num_pairs,
                                       int32_t height, int32_t width, double *grad_tangent,
                                       float *grad_depth, void *stream);

/*
 * stb_icp_estimate without any allocation.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc while they track -- C or
 * FFI hosts with no CUDA allocator of their own, and applications that fix
 * their device-memory budget at start-up (cudaMalloc / cudaFree synchronise
 * the device and would stall a real-time loop).  The scratch is a fixed
 * device array inside the library, sized for at most 1,048,576 target
 * pixels (height * width; about 8.9 MB, held by every GPU that loads the
 * library until the process exits); larger frames are rejected with
 * STB_EINVAL.  The first call on a device looks up that array's address
 * (cudaGetSymbolAddress), so make it before any stream capture.  The
 * address is kept for the life of the process: after cudaDeviceReset on a
 * device, this entry point must not be called on that device again (the
 * library's module, and the array with it, may be reloaded elsewhere).
 * Every call uses the same array: calls whose work overlaps on the GPU race.
 * Same arguments and results as stb_icp_estimate, minus workspace and
 * graphs.
 */
STB_API int stb_icp_estimate_static(
    const float *kcam, const float *src_points, const float *src_normals,
    const uint8_t *src_mask, int64_t num_source, const void *src_feats,
    const float *tgt_points, const float *tgt_normals, const uint8_t *tgt_mask,
    int32_t height, int32_t width, const void *tgt_feats, int32_t channels,
    int32_t feat_dtype, const double *init_transform, int32_t num_iters,
    double geom_weight, double feat_weight, double distance_thresh,
    double normal_angle_thresh, double feat_residual_thresh, int32_t channel_mode,
    double *result, double *history, void *stream);

/*
 * Test hook of the bounded waits of the single-launch registration and of
 * stb_icp_estimate_batch (no counterpart in the reference): their grid
 * barriers give up after spin_limit polls (0 restores the defaults) and
 * expect phantom_arrivals more blocks than the grid has (0 restores the
 * default).
 * With phantom_arrivals > 0 no barrier can complete, so every wait runs out
 * and the registration returns with STB_ST_TIMEOUT in its status instead of
 * hanging: the way to test that failure path without a faulty GPU.
 * Process-wide; applies to calls made after it.
 */
STB_API int stb_set_wait_test_limits(uint32_t spin_limit, int32_t phantom_arrivals);

/*
 * Measurement hook (no counterpart in the reference, which has no device
 * timers).  stb_profile_enable(1) makes later stb_icp_estimate calls
 * bracket every kernel launch with CUDA events on the launching stream
 * (event nodes when the call replays a graph; graphs are cached separately
 * for profiled and plain calls).  After the stream has completed,
 * stb_profile_read() returns, for the most recent profiled call, the summed
 * event time (ms) and launch count per kernel kind:
 *   0 association, 1 reduction + solve, 2 information, 3 setup (the
 *   STB_OPT_MULTI_LAUNCH sequence), 4 the single-launch registration.
 * num_kinds >= 4; kinds at or past num_kinds are not reported.
 */
STB_API int stb_profile_enable(int32_t on);
STB_API int stb_profile_read(double *ms_by_kind, int64_t *launches_by_kind,
                             int32_t num_kinds);

/* ======================================================================= *
 * Frame preparation (inputs of every pyramid level)
 * ======================================================================= */

/*
 * Metric depth -> camera-space points and raw validity mask.  Replaces
 * depth_image_to_uvz (slamtb/_utils.py:11-37) + KCamera.backproject
 * (slamtb/camera.py:127-149): z = depth * depth_scale + depth_bias,
 * x = (u - cx) z / fx, y = (v - cy) z / fy; raw_mask = depth > 0
 * (slamtb/frame.py:290).  depth float32 [h, w]; points float32 [h, w, 3].
 */
STB_API int stb_depth_to_points(const float *depth, float depth_scale,
                                float depth_bias, const float *kcam,
                                float *points, uint8_t *raw_mask,
                                int32_t height, int32_t width, void *stream);

/* Mask erosion.  Replaces Processing::ErodeMask (src/erode_mask.cu:42-54),
 * including its neighbourhood (above, right, left; never below). */
STB_API int stb_erode_mask(const uint8_t *in_mask, uint8_t *out_mask,
                           int32_t height, int32_t width, void *stream);

/* Central-difference normals.  Replaces Processing::EstimateNormals with
 * kCentralDifferences (src/normals.cu:27-100,190-208). */
STB_API int stb_estimate_normals(const float *xyz, const uint8_t *mask,
                                 float *normals, int32_t height, int32_t width,
                                 void *stream);

/* Nearest-to-mean 2x2 XYZ downsample.  Replaces Processing::DownsampleXYZ
 * (src/downsample.cu:25-98); dst is int(size * scale). */
STB_API int stb_downsample_xyz(const float *xyz, const uint8_t *mask,
                               int32_t height, int32_t width, float scale,
                               float *dst, int32_t dst_height,
                               int32_t dst_width, void *stream);

/* Nearest mask downsample.  Replaces Processing::DownsampleMask
 * (src/downsample.cu:100-131). */
STB_API int stb_downsample_mask(const uint8_t *mask, int32_t height,
                                int32_t width, float scale, uint8_t *dst,
                                int32_t dst_height, int32_t dst_width,
                                void *stream);

/* 2x2 mean feature downsample.  Replaces Processing::DownsampleFeatures
 * (src/downsample.cu:133-191).  feats/dst: [channels, h, w] of feat_dtype. */
STB_API int stb_downsample_features(const void *feats, int32_t channels,
                                    int32_t height, int32_t width,
                                    int32_t feat_dtype, float scale, void *dst,
                                    int32_t dst_height, int32_t dst_width,
                                    void *stream);

/* 3x3 Gaussian blur with reflect borders: the kornia
 * GaussianBlur2d((3, 3), (sigma, sigma)) of feature_pyramid
 * (slamtb/processing.py:141-159). */
STB_API int stb_gaussian_blur3(const void *feats, int32_t channels,
                               int32_t height, int32_t width,
                               int32_t feat_dtype, double sigma, void *dst,
                               void *stream);

/* ---- differentiable registration layer (AutogradICP) ------------------ */

/*
 * ExpRtToMatrixOp::Forward (src/exp_rt_to_matrix.cu:41-53): count twists
 * exp_rt [count][6] = [t; w] (t the translation, w the rotation axis times
 * its angle) to matrix [count][3][4] = [R(w) | t], R by Rodrigues' formula.
 * dtype: STB_F32 or STB_F64 (both arrays).
 */
STB_API int stb_exp_rt_to_matrix(const void *exp_rt, void *matrix, int64_t count,
                                 int32_t dtype, void *stream);

/*
 * ExpRtToMatrixOp::Backward (src/exp_rt_to_matrix.cu:101-121): d_exp_rt
 * [count][6] from d_matrix [count][3][4], the forward's exp_rt and matrix,
 * with the rotation derivative of Gallego and Yezzi (src/exp_rt.hpp:90-138).
 */
STB_API int stb_exp_rt_to_matrix_backward(const void *d_matrix, const void *exp_rt,
                                          const void *matrix, void *d_exp_rt, int64_t count,
                                          int32_t dtype, void *stream);

/*
 * MatrixToExpRtOp::Forward (src/matrix_to_exp_rt.cu:35-48): matrix
 * [count][3][4] to exp_rt [count][6] (translation, axis x angle of R).
 */
STB_API int stb_matrix_to_exp_rt(const void *matrix, void *exp_rt, int64_t count,
                                 int32_t dtype, void *stream);

/*
 * FPCLMatcherOp::Forward (src/fpcl_matcher.cu:85-123).  src_points
 * [num_source][3] (already in the target camera frame) are projected with
 * kcam [3][3]; point i matches when its rounded projection lies in the
 * height x width image and the high 32 bits of merge_map [height][width]
 * (a stb_correspondence_map result) there equal i.  A match writes the
 * target point and normal at that pixel to out_points / out_normals
 * [num_source][3] and the bilinear sample of tgt_feats [channels][height]
 * [width] at the unrounded projection to out_feats [channels][num_source];
 * match_mask [num_source] gets 1.  Points that do not match get 0 and zero
 * outputs.  dtype: STB_F32 or STB_F64 (every float array and kcam).
 */
STB_API int stb_fpcl_match_forward(const void *tgt_points, const void *tgt_normals,
                                   const void *tgt_feats, int32_t channels, int32_t height,
                                   int32_t width, const void *src_points, int64_t num_source,
                                   const void *kcam, const int64_t *merge_map, void *out_points,
                                   void *out_normals, void *out_feats, uint8_t *match_mask,
                                   int32_t dtype, void *stream);

/*
 * FPCLMatcherOp::Backward (src/fpcl_matcher.cu:193-226): dx_points
 * [num_source][3] = d loss / d source point from dl_feats [channels]
 * [num_source] = d loss / d out_feats, by central differences of the
 * bilinear sample with step grad_precision (0 < grad_precision < 0.5)
 * through the projection's Jacobian; 0 where match_mask is 0.
 */
STB_API int stb_fpcl_match_backward(const void *tgt_feats, int32_t channels, int32_t height,
                                    int32_t width, const void *src_points, int64_t num_source,
                                    const uint8_t *match_mask, const void *dl_feats,
                                    const void *kcam, double grad_precision, void *dx_points,
                                    int32_t dtype, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SLAMTB_GB300_H_ */
