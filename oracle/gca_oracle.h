/*
 * gca_oracle.h -- CPU oracle for the RGB-D registration path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path is
 * compared against; only tests, the smoke entry and the CPU-baseline leg of the
 * bench load it. The product path never calls it.
 *
 * Two flavours of every step:
 *   *_ref32  FP32, same operation order as the reference implementation
 *            (XssZuiNB/CUDA_3D), compiled with -ffp-contract=off.  Where the
 *            reference sums in parallel, the oracle sums sequentially in
 *            ascending index / scan order (this is the documented order the
 *            bit-exact GPU outputs are defined against).
 *   *_f64    FP64 restatement of the same mathematics; the tolerance anchor for
 *            normals, colour gradients, fitness, inlier RMSE and the pose.
 *
 * Parity pin: the FP32 flavour is checked against the reference's own Thrust
 * code compiled as host C++ (oracle/_ref, serial backend) through the golden
 * fixtures in tests/golden.  The pixel-stage bilateral kernel of the reference
 * cannot be compiled as host code (it is a CUDA kernel launch), so that stage is
 * pinned by restatement only.
 */
#ifndef GCA_ORACLE_H
#define GCA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float fx, fy, cx, cy; } orc_intrinsics;
/* rotation is column-major, as camera/camera_param.hpp:13-17 and
 * cuda_point_cloud_factory.cu:160-170 use it */
typedef struct { float rotation[9]; float translation[3]; } orc_extrinsics;

enum { ORC_FILTER_NONE = 0, ORC_FILTER_ADAPTIVE = 1, ORC_FILTER_FIXED = 2 };
enum { ORC_TIE_SCAN_ORDER = 0, ORC_TIE_MIN_INDEX = 1 };
enum { ORC_UPDATE_EULER_ZYX = 0, ORC_UPDATE_SE3_EXP = 1 };

void orc_set_threads(int n);
int orc_get_threads(void);

/* the FP32 exp used by the depth filter (same operation sequence on the GPU) */
float orc_exp32(float x);

/* color3::to_intensity (geometry/type.hpp:45-51): FP64 weighted sum rounded to float */
float orc_intensity(float r, float g, float b);

/* cuda_compute_min_max_bound (geometry/geometry_util.cuh:88-105).  With
 * flt_min_bug = 1 the max starts at FLT_MIN as the reference does. */
void orc_aabb(const float *xyz, int64_t n, int flt_min_bug, float mn[3], float mx[3]);

/* depth filter + back-projection + compaction
 * (geometry/cuda_point_cloud_factory.cu:19-267, geometry_util.cuh:124-130).
 * Returns the number of valid points written to out_xyz/out_rgb (raster order).
 * out_depth (optional, w*h) receives the filtered depth in depth units. */
int64_t orc_make_point_cloud(const uint16_t *depth, const uint8_t *bgr, int w, int h,
                             const orc_intrinsics *depth_intrin,
                             const orc_intrinsics *color_intrin,
                             const orc_extrinsics *depth2color, float depth_scale,
                             float tmin, float tmax, int filter_mode, int fixed_radius,
                             float fixed_sigma_space, float fixed_sigma_depth,
                             float *out_xyz, float *out_rgb, float *out_depth);

/* cuda_voxel_grid_downsample (geometry/cuda_voxel_grid_down_sample.cu:123-161).
 * Returns M; writes M means, M counts and M int3 keys, ascending key order. */
int64_t orc_voxel_downsample(const float *xyz, const float *rgb, int64_t n, const float mn[3],
                             float voxel, float *out_xyz, float *out_rgb, int32_t *out_count,
                             int32_t *out_key);

/* nearest neighbour within radius (geometry/cuda_nn_search.cu:113-214,545-619).
 * grid_min is the grid origin; tie_mode selects the reference's scan order or
 * the (distance, index) minimum. */
void orc_nn_search(const float *q, int64_t nq, const float *r, int64_t nr, float radius,
                   const float grid_min[3], int tie_mode, int32_t *out_idx);

/* radius neighbour lists in scan order (geometry/cuda_nn_search.cu:216-414,622-723).
 * counts[nq]; starts[nq] (exclusive scan); list[cap].  Returns the total. */
int64_t orc_radius_search(const float *q, int64_t nq, const float *r, int64_t nr, float radius,
                          const float grid_min[3], int32_t *counts, int64_t *starts,
                          int32_t *list, int64_t list_cap);

/* normals, reference order (geometry/cuda_estimate_normals.cu:46-199 and
 * util/fast_eigen_val_vec.cuh:115-205) */
void orc_normals_ref32(const float *xyz, int64_t n, float radius, const float grid_min[3],
                       float *out_nrm);
/* normals, FP64: covariance about the neighbourhood mean, Jacobi eigenvectors.
 * max_nn > 0 keeps the max_nn nearest (distance, index) neighbours. */
void orc_normals_f64(const float *xyz, int64_t n, float radius, int max_nn, double *out_nrm);

/* radius outlier removal (geometry/point_cloud.cu:238-280, cuda_nn_search.cu:416-542,
 * 725-800): survivors (more than min_nn neighbours within radius, self included) in
 * input order; returns their count */
int64_t orc_radius_outlier_removal(const float *xyz, const float *rgb, int64_t n, float radius, int min_nn,
                                   float *out_xyz, float *out_rgb);

/* colour gradient (registration/cuda_compute_color_gradient.cu:13-127,
 * util/little_3x3_ldlt_solve.cuh) */
void orc_gradient_ref32(const float *xyz, const float *rgb, const float *nrm, int64_t n,
                        float radius, const float grid_min[3], float *out_grad);
void orc_gradient_f64(const float *xyz, const float *rgb, const double *nrm, int64_t n,
                      float radius, double *out_grad);

/* per-correspondence system (registration/cuda_color_icp_build_least_square.cu:134-254,
 * 431-474).  jtj row-major 6x6.  Source points are already transformed. */
void orc_build_gn_ref32(const float *src_xyz, const float *src_rgb, int64_t ns,
                        const float *tgt_xyz, const float *tgt_rgb, const float *tgt_nrm,
                        const float *tgt_grad, const int32_t *nn, float lambda, float jtj[36],
                        float jtr[6], float *r2);

/* per-point residual helpers (cuda_color_icp_build_least_square.cu:13-132) */
void orc_abs_residual_ref32(const float *src_xyz, const float *src_rgb, int64_t ns,
                            const float *tgt_xyz, const float *tgt_rgb, const float *tgt_nrm,
                            const float *tgt_grad, const int32_t *nn, float lambda,
                            float *out);

/* FP64 6x6 LDLT with symmetric pivoting; x = -JTJ^-1 JTr; pose map.
 * Returns 0 on success, 1 when a pivot vanished (that component is zeroed). */
int orc_solve6(const double jtj[36], const double jtr[6], double x[6]);
void orc_pose_from_x(const double x[6], int update_map, double T[16]);

typedef struct {
    int max_iter;
    float max_corr;
    float lambda;
    int update_map;
    double rot_eps;   /* converged when cos(step angle) >= 1 - rot_eps */
    double trans_eps; /* ... and |step t|^2 <= trans_eps */
    int search_f32;   /* 1: correspondences of the FP32 points the GPU kernels search
                       * (pose rounded to float, fused x' = fma(r0,x,fma(r1,y,fma(r2,z,t))),
                       * unfused FP32 d^2 < max_corr^2); residuals, Jacobians and sums
                       * stay FP64 on those points.  0: FP64 transform and search. */
} orc_icp_params;

typedef struct {
    double T[16];
    double rmse_ref;    /* sum r^2 of the last built system / N_src (color_icp.cu:231) */
    double fitness;     /* inliers / N_src, last built system */
    double inlier_rmse; /* sqrt(sum d^2 over inliers / inliers), last built system */
    int iterations;
    int converged;
    int status;
} orc_icp_result;

/* colored ICP in FP64 (color_icp.cu:151-234 with FP64 everywhere, pose applied on
 * the fly, (distance, index) NN tie-break).  tgt_nrm/tgt_grad are FP64.  With
 * p->search_f32 the correspondences are those of the FP32 points (above). */
void orc_color_icp_f64(const float *src_xyz, const float *src_rgb, int64_t ns,
                       const float *tgt_xyz, const float *tgt_rgb, const double *tgt_nrm,
                       const double *tgt_grad, int64_t nt, const orc_icp_params *p,
                       const double T_init[16], orc_icp_result *res);

/* colored ICP as the reference runs it (FP32 points transformed in place,
 * FP32 4x4 composition, FP64 solve, Euler ZYX map, reference bounds/scan order) */
void orc_color_icp_ref32(const float *src_xyz, const float *src_rgb, int64_t ns,
                         const float *tgt_xyz, const float *tgt_rgb, const float *tgt_nrm,
                         const float *tgt_grad, int64_t nt, int max_iter, float max_corr,
                         const float T_init[16], orc_icp_result *res);

/* ------------------------------------------------------------------
 * K unrolled Gauss-Newton steps of the colored-ICP objective and their
 * adjoint (no reference counterpart; FP64).  T_0 = Exp(xi0) (SE(3)
 * exponential, xi = (w, v)); step k solves the system built at T_k and
 * composes T_{k+1} = U(x_k) T_k with the chosen map; E = sum of the weighted
 * r_g^2 + r_c^2 at T_K.  Source points and colours are FP64 (finite differences
 * of the inputs stay exact); the source intensity is the exact FP64 weighted sum.
 * corr: (K + 1) x ns target indices (-1: none), one row per evaluation; when
 * given, the correspondences are frozen (the function is then smooth), else they
 * are searched ((distance, index) minimum within max_corr) and written to
 * corr_out when it is not NULL.
 * ------------------------------------------------------------------ */
typedef struct {
    int K;
    float max_corr;
    float lambda;
    int update_map;
} orc_unroll_params;

/* the GPU ICP kernels' FP32 pose application: fused multiply-adds in the order
 * fma(r0, x, fma(r1, y, fma(r2, z, t))), T rounded to float (row-major 4x4 in) */
void orc_apply_pose_f32(const double T[16], const float *xyz, int64_t n, float *out);

/* dU/dx_m as 3x4 row-major blocks for U = pose map(x) */
void orc_pose_jacobian(const double x[6], int update_map, double dU[6][12]);

/* returns E; T_out receives T_K */
double orc_icp_unrolled_f64(const double *sx, const double *srgb, int64_t ns, const float *tx,
                            const float *trgb, const double *tn, const double *tg, int64_t nt,
                            const orc_unroll_params *p, const double xi0[6], const int32_t *corr_in,
                            int32_t *corr_out, double T_out[16]);

/* gradient of L = <dT, T_K> (rows 0-2) + dE * E with respect to xi0, the source
 * points and the source colours, correspondences frozen to corr.  Returns nonzero
 * when a step's system was singular. */
int orc_icp_unrolled_vjp_f64(const double *sx, const double *srgb, int64_t ns, const float *tx,
                             const float *trgb, const double *tn, const double *tg, int64_t nt,
                             const orc_unroll_params *p, const double xi0[6], const int32_t *corr,
                             const double dT[16], double dE, double dxi0[6], double *dxyz,
                             double *drgb);

#ifdef __cplusplus
}
#endif
#endif
