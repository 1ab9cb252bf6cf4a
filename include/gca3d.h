/*
 * gca3d.h -- C ABI of the GB300-native RGB-D registration path.
 *
 * Replaces the GPU entry points of XssZuiNB/CUDA_3D's registration path (the
 * reference exposes them as C++ classes and free functions returning
 * cudaError_t; each declaration below names the reference interface it stands
 * in for).  Every call is stream-ordered on the context's stream and returns an
 * int status (GCA3D_OK = 0).  Clouds are opaque device-resident handles owned by
 * the caller; pointers marked "device" are device pointers, every other pointer
 * is host memory unless stated.  A context belongs to one host thread at a time.
 *
 * Layout of a cloud on the device (structure of arrays, 16-byte elements):
 *   pos  float4 {x, y, z, intensity}   intensity = 0.2126 r + 0.7152 g + 0.0722 b
 *   col  float4 {r, g, b, 0}           colours in [0, 1]
 *   nrm  float4 {nx, ny, nz, 0}        after gca3d_estimate_normals
 *   grd  float4 {gx, gy, gz, 0}        after gca3d_color_gradient
 * The point count lives on the device so that variable-size stages need no host
 * round trip; gca3d_cloud_size reads it back.
 */
#ifndef GCA3D_H
#define GCA3D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (reference: cudaError_t returns and false/nullptr results,
 *      e.g. src/registration/cuda_color_icp_build_least_square.cu:438-452) ---- */
#define GCA3D_OK 0
#define GCA3D_ERR_INVALID_VALUE 1
#define GCA3D_ERR_OUT_OF_MEMORY 2
#define GCA3D_ERR_NO_CORRESPONDENCES 3
#define GCA3D_ERR_SINGULAR 4
#define GCA3D_ERR_TIMEOUT 5
#define GCA3D_ERR_CUDA 6
#define GCA3D_ERR_CAPACITY 7
#define GCA3D_ERR_NOT_SUPPORTED 8

typedef struct gca3d_context gca3d_context;
typedef struct gca3d_cloud gca3d_cloud;
typedef struct gca3d_icp_plan gca3d_icp_plan;

/* camera model (reference: src/camera/camera_param.hpp:5-18) */
typedef struct {
    float fx, fy, cx, cy;
} gca3d_intrinsics;

/* rotation column-major, as the reference stores it */
typedef struct {
    float rotation[9];
    float translation[3];
} gca3d_extrinsics;

#define GCA3D_FILTER_NONE 0
#define GCA3D_FILTER_ADAPTIVE 1 /* the reference's adaptive bilateral filter */
#define GCA3D_FILTER_FIXED 2    /* fixed window: radius, sigma_space (px), sigma_depth (depth units) */

typedef struct {
    int mode;
    int radius;
    float sigma_space;
    float sigma_depth;
} gca3d_filter;

#define GCA3D_UPDATE_EULER_ZYX 0 /* R = Rz Ry Rx, t = x[3..5] (reference eigen_solver.hpp:30-40) */
#define GCA3D_UPDATE_SE3_EXP 1   /* SE(3) exponential */

#define GCA3D_MAX_SCALES 8

/* one level of the coarse-to-fine schedule.  voxel <= 0 uses the clouds as
 * given (the reference's single-level color_icp::align). */
typedef struct {
    float voxel;
    int max_iter;
    float max_corr;
    float normal_radius;
    float grad_radius;
    int max_nn; /* 0 = every neighbour inside normal_radius (reference) */
} gca3d_scale;

/* launch shape of the ICP iterations (0 = default).  Only the shape changes: results are
 * bit-identical for every setting.  gca3d_icp_autotune picks one for a workload. */
typedef struct {
    int nn_item_points;      /* source points per correspondence work item: 64, 128, 256 (default), 512 */
    int nn_blocks_per_sm;    /* correspondence grid = SMs x this (default 10), at most the items */
    int accum_blocks_per_sm; /* accumulate grid = SMs x this (default 6), at most the items */
    int voxel_resort;        /* 1: sort every scale's voxels anew; 0 (default): where the next
                                scales' voxel sizes halve exactly, one sort at the coarser scale
                                carries their sub-cell bits and each finer scale splits its runs */
    int fused_finalize;      /* 1: the last accumulate block of each pair runs the pair's solve and
                                pose update; 0 (default): they are a launch of their own */
    int serial_prep;         /* 1: every scale's clouds, grids and normals on the context stream,
                                before its iterations; 0 (default): on a branch of their own that
                                runs ahead, so finer scales are prepared while coarser ones iterate */
} gca3d_tuning;

typedef struct {
    int n_scales;
    gca3d_scale scales[GCA3D_MAX_SCALES];
    float lambda;      /* geometric weight, 0.968 in the reference (color_icp.hpp:46) */
    int update_map;    /* GCA3D_UPDATE_* */
    double rot_eps;    /* converged when cos(step angle) >= 1 - rot_eps ... */
    double trans_eps;  /* ... and |step translation|^2 <= trans_eps (color_icp.hpp:47-48) */
    int compensated;   /* 1: Kahan FP32 in each block, FP64 across blocks; 0: plain FP32 */
    int use_graph;     /* 1: replay the whole schedule as one CUDA graph */
    int keep_target_normals; /* 1 with voxel <= 0: use the normals already on the target */
    gca3d_tuning tuning;
} gca3d_icp_params;

typedef struct {
    double T[16];       /* row-major 4x4, maps source onto target */
    double rmse_ref;    /* sum of squared weighted residuals / N_src of the last built
                           system (reference color_icp::get_RSME, color_icp.cu:231) */
    double fitness;     /* correspondences / N_src, last built system */
    double inlier_rmse; /* sqrt(mean squared point distance over correspondences) */
    int iterations;     /* summed over scales */
    int converged;      /* the last scale met the convergence test */
    int status;         /* GCA3D_OK, NO_CORRESPONDENCES, SINGULAR, TIMEOUT */
    int n_src;          /* source points at the last scale */
    int n_tgt;          /* target points at the last scale */
    int scale_iterations[GCA3D_MAX_SCALES]; /* per scale */
    int scale_n_src[GCA3D_MAX_SCALES];
    int scale_n_tgt[GCA3D_MAX_SCALES];
} gca3d_icp_result;

/* ---------------------------------------------------------------------------
 * context and clouds
 * ------------------------------------------------------------------------- */

/* stream: a cudaStream_t, or NULL for a new non-blocking stream owned by the context */
int gca3d_create(int device, void *stream, gca3d_context **ctx);
int gca3d_destroy(gca3d_context *ctx);
int gca3d_synchronize(gca3d_context *ctx);
const char *gca3d_status_string(int status);
/* detail of the last failure on this context (static storage, overwritten) */
const char *gca3d_last_error(gca3d_context *ctx);
/* number of kernels this library launched on the context since creation */
int64_t gca3d_kernel_launches(gca3d_context *ctx);
/* kernel timing with CUDA events on the context stream: while a profile is open,
 * every launch of the named kernel ("icp_iter", "sort_pass", "normals", "voxel_reduce",
 * "grid_scatter", "frame") is bracketed by events; read sums their durations */
int gca3d_profile_begin(gca3d_context *ctx, const char *kernel);
int gca3d_profile_read(gca3d_context *ctx, double *total_ms, int64_t *launches);
/* the context's stream (cudaStream_t) */
void *gca3d_stream(gca3d_context *ctx);
/* plain device buffers for callers without their own allocator */
int gca3d_device_alloc(gca3d_context *ctx, int64_t bytes, void **ptr);
int gca3d_device_free(gca3d_context *ctx, void *ptr);
/* stream-ordered copy between any two pointers (host or device); synchronises */
int gca3d_copy(gca3d_context *ctx, void *dst, const void *src, int64_t bytes);

/* reference: gca::point_cloud(size_t) (src/geometry/point_cloud.hpp:26) */
int gca3d_cloud_create(gca3d_context *ctx, int64_t capacity, gca3d_cloud **cloud);
int gca3d_cloud_destroy(gca3d_cloud *cloud);
/* xyz, rgb: n x 3 floats, host or device memory.  rgb may be NULL (black).  Pinned
 * host memory (and memory of the context's device) is read in place by the packing
 * kernel on the context stream, so, as with cudaMemcpyAsync, it must not change
 * before the stream has passed the call; pageable or managed host memory and other
 * devices' memory go through a staging copy.
 * reference: point_cloud::create_from_pcl (src/geometry/point_cloud.cu:481-504) */
int gca3d_cloud_upload(gca3d_context *ctx, gca3d_cloud *cloud, const float *xyz,
                       const float *rgb, int64_t n);
/* count uploads in one call (no reference counterpart: the reference creates clouds
 * one at a time): cloud k gets xyz[k], rgb[k] (rgb or rgb[k] may be NULL), n[k]
 * points, as gca3d_cloud_upload.  The clouds whose buffers the device reads in place
 * (pinned host memory, memory of the context's device) are packed by one kernel
 * launch per 64; the others go through gca3d_cloud_upload's staging copy. */
int gca3d_cloud_upload_many(gca3d_context *ctx, int count, gca3d_cloud *const *clouds,
                            const float *const *xyz, const float *const *rgb, const int64_t *n);
/* how the context's uploads read pinned host memory (no reference counterpart).
 * GCA3D_UPLOAD_IN_PLACE (default): the packing kernel reads it over the host link
 * itself -- the fastest upload when nothing else runs.  GCA3D_UPLOAD_COPY_ENGINE: the
 * GPU's copy engines first copy it into the context's scratch, then the packing kernel
 * reads that -- the copies occupy no SMs, so the uploads of a context kept for them
 * overlap the registration running on another context's stream (double buffering).
 * Device sources are read in place and pageable ones staged in both modes. */
#define GCA3D_UPLOAD_IN_PLACE 0
#define GCA3D_UPLOAD_COPY_ENGINE 1
int gca3d_set_upload_mode(gca3d_context *ctx, int mode);
/* normals (n x 3) supplied by the caller; marks the cloud as having normals */
int gca3d_cloud_set_normals(gca3d_context *ctx, gca3d_cloud *cloud, const float *nrm, int64_t n);
/* colour gradients (n x 3) supplied by the caller; needs normals */
int gca3d_cloud_set_gradients(gca3d_context *ctx, gca3d_cloud *cloud, const float *grd, int64_t n);
int gca3d_cloud_capacity(const gca3d_cloud *cloud, int64_t *capacity);
/* reads the device-side count (synchronises) */
int gca3d_cloud_size(gca3d_context *ctx, gca3d_cloud *cloud, int64_t *n);
int gca3d_cloud_has_normals(const gca3d_cloud *cloud, int *has);
/* any output pointer may be NULL; each is n x 3 floats of host or device memory.
 * reference: point_cloud::download / download_normals (point_cloud.cu:75-91) */
int gca3d_cloud_download(gca3d_context *ctx, gca3d_cloud *cloud, float *xyz, float *rgb,
                         float *nrm, float *grd, int64_t cap, int64_t *n);
/* raw device views (float4 SoA) and the device count */
int gca3d_cloud_device_views(gca3d_cloud *cloud, void **pos, void **col, void **nrm,
                             void **grd, int32_t **d_count);
/* reference: point_cloud::operator= (point_cloud.cu:39-50) */
int gca3d_cloud_copy(gca3d_context *ctx, const gca3d_cloud *src, gca3d_cloud *dst);
/* reference: point_cloud::operator+= (point_cloud.cu:55-73) */
int gca3d_cloud_append(gca3d_context *ctx, gca3d_cloud *dst, const gca3d_cloud *src);

/* ---------------------------------------------------------------------------
 * path stages
 * ------------------------------------------------------------------------- */

/* AABB of the cloud (true max; the reference starts its max at FLT_MIN).
 * reference: cuda_compute_min_max_bound (src/geometry/geometry_util.cuh:88-105) */
int gca3d_bounds(gca3d_context *ctx, gca3d_cloud *cloud, float mn[3], float mx[3]);

/* p <- R p + t, n <- R n; T row-major 4x4.
 * reference: point_cloud::transform (src/geometry/point_cloud.cu:93-105) */
int gca3d_transform(gca3d_context *ctx, gca3d_cloud *cloud, const double T[16]);

/* depth (uint16, h x w) and BGR8 colour (h x w x 3) in device memory -> cloud of the
 * valid pixels in raster order.  reference: point_cloud::create_from_rgbd
 * (src/geometry/point_cloud.cu:455-479) / cuda_make_point_cloud
 * (src/geometry/cuda_point_cloud_factory.cu:269-313) */
int gca3d_frame_to_cloud(gca3d_context *ctx, const uint16_t *depth, const uint8_t *bgr, int w,
                         int h, const gca3d_intrinsics *depth_intrin,
                         const gca3d_intrinsics *color_intrin,
                         const gca3d_extrinsics *depth_to_color, float depth_scale, float tmin,
                         float tmax, const gca3d_filter *filter, gca3d_cloud *out);

/* reference: point_cloud::voxel_grid_down_sample (src/geometry/point_cloud.cu:198-229),
 * cuda_voxel_grid_downsample (src/geometry/cuda_voxel_grid_down_sample.cu:123-161) */
int gca3d_voxel_downsample(gca3d_context *ctx, gca3d_cloud *in, float voxel, gca3d_cloud *out);

/* reference: point_cloud::estimate_normals (src/geometry/point_cloud.cu:145-181),
 * cuda_estimate_normals (src/geometry/cuda_estimate_normals.cu:153-199).
 * max_nn > 0 keeps the max_nn nearest neighbours (distance, then index). */
int gca3d_estimate_normals(gca3d_context *ctx, gca3d_cloud *cloud, float radius, int max_nn);

/* reference: cuda_compute_color_gradient
 * (src/registration/cuda_compute_color_gradient.cu:92-127); needs normals */
int gca3d_color_gradient(gca3d_context *ctx, gca3d_cloud *cloud, float radius);

/* points with more than min_neighbors neighbours (the point itself included) within
 * radius, in input order, without normals.  out->capacity >= in->capacity.
 * reference: point_cloud::radius_outlier_removal (src/geometry/point_cloud.cu:238-280),
 * cuda_grid_radius_outliers_removal (src/geometry/cuda_nn_search.cu:416-542,725-800) */
int gca3d_radius_outlier_removal(gca3d_context *ctx, gca3d_cloud *in, float radius,
                                 int min_neighbors, gca3d_cloud *out);

/* out[k] = in[idx[k]] for k < n (points, colours and normals when present); idx is
 * host or device memory; an index outside the cloud gives GCA3D_ERR_INVALID_VALUE.
 * reference: point_cloud::create_new_by_index (src/geometry/point_cloud.cu:438-453) */
int gca3d_cloud_select(gca3d_context *ctx, gca3d_cloud *in, const int32_t *idx, int64_t n,
                       gca3d_cloud *out);

/* the cloud as the reference's 28-byte point_t records (geometry/type.hpp:65-70,
 * property = active) into device memory, and the normals as float3 (may be NULL).
 * Stream-ordered; no synchronisation. */
int gca3d_cloud_to_aos(gca3d_context *ctx, gca3d_cloud *cloud, void *d_points, float *d_normals);

/* nearest reference point within radius for every query point, -1 if none; ties on
 * distance go to the smaller index.  out_idx: device int32[n_query].
 * reference: point_cloud::nn_search (src/geometry/point_cloud.cu:506-557),
 * cuda_nn_search (src/geometry/cuda_nn_search.cu:545-619) */
int gca3d_nn_search(gca3d_context *ctx, gca3d_cloud *query, gca3d_cloud *ref, float radius,
                    int32_t *out_idx);

/* neighbour lists inside radius (self included), in the reference's scan order for
 * the given grid origin (NULL: the reference's normal-estimation bounds).
 * counts/starts: device int32[n_query]; list: device int32[list_cap]; *total is
 * written on the host (synchronises).  reference: cuda_search_radius_neighbors
 * (src/geometry/cuda_nn_search.cu:622-723) */
int gca3d_radius_search(gca3d_context *ctx, gca3d_cloud *query, gca3d_cloud *ref, float radius,
                        const float grid_min[3], int32_t *counts, int32_t *starts,
                        int32_t *list, int64_t list_cap, int64_t *total);

/* Gauss-Newton system of the colored-ICP objective for given correspondences
 * (device int32[n_src]); jtj row-major 6x6, all outputs host memory.
 * reference: cuda_build_gauss_newton_color_icp
 * (src/registration/cuda_color_icp_build_least_square.cu:431-474) */
int gca3d_build_gauss_newton(gca3d_context *ctx, gca3d_cloud *src, gca3d_cloud *tgt,
                             const int32_t *nn, float lambda, double jtj[36], double jtr[6],
                             double *r2);

/* The same system as gca3d_build_gauss_newton for callers that cannot allocate device
 * memory while they run (a real-time loop that must not stall on cudaMalloc's device
 * synchronisation, or a host whose memory manager already owns the GPU's memory).  No
 * counterpart in the reference.  It needs no context and allocates nothing: inputs and
 * outputs are the caller's device pointers, and the scratch (block partials, count,
 * ticket) is a fixed 512 KiB array inside the library that every GPU loading the
 * library holds until exit.
 *   stream   cudaStream_t (NULL: the legacy default stream)
 *   src_pos  device float4[n_src] {x, y, z, intensity} (the cloud layout above)
 *   tgt_pos, tgt_nrm, tgt_grd  device float4 arrays of the target (layout above)
 *   nn       device int32[n_src], target index or -1
 *   jtj, jtr, r2  device double[36], double[6], double[1] outputs
 * n_src above 8,388,608 returns GCA3D_ERR_CAPACITY.  The first call on each device
 * looks up the scratch array's device address (cudaGetSymbolAddress); make that first
 * call before any stream capture.  Every call uses the same array: calls that overlap
 * on the GPU (other streams, other threads) race and must be serialised by the caller. */
int gca3d_build_gauss_newton_static(void *stream, const void *src_pos, int32_t n_src,
                                    const void *tgt_pos, const void *tgt_nrm,
                                    const void *tgt_grd, const int32_t *nn, float lambda,
                                    double *jtj, double *jtr, double *r2);

/* |r_geometric| + |r_colour| per source point (device float[n_src]).
 * reference: cuda_compute_abs_residual_color_icp
 * (src/registration/cuda_color_icp_build_least_square.cu:310-350) */
int gca3d_abs_residual(gca3d_context *ctx, gca3d_cloud *src, gca3d_cloud *tgt, const int32_t *nn,
                       float lambda, float *out);

/* the colored ICP of one pair, optionally coarse to fine; T_init may be NULL.
 * The source cloud is not modified.  reference: color_icp::align
 * (src/registration/color_icp.cu:151-234) */
int gca3d_color_icp(gca3d_context *ctx, gca3d_cloud *src, gca3d_cloud *tgt,
                    const gca3d_icp_params *params, const double T_init[16],
                    gca3d_icp_result *result);

/* many pairs of uneven size in one batched schedule (every stage launched once
 * for all pairs).  T_init: n_pairs x 16 or NULL.  No reference counterpart (the
 * reference aligns one pair per call). */
int gca3d_color_icp_batched(gca3d_context *ctx, int n_pairs, gca3d_cloud *const *src,
                            gca3d_cloud *const *tgt, const gca3d_icp_params *params,
                            const double *T_init, gca3d_icp_result *results);

/* a reusable plan: workspace allocated and (with use_graph) the whole schedule
 * captured once; execute replays it on the clouds' current contents.  No
 * reference counterpart. */
int gca3d_icp_plan_create(gca3d_context *ctx, int n_pairs, gca3d_cloud *const *src,
                          gca3d_cloud *const *tgt, const gca3d_icp_params *params,
                          gca3d_icp_plan **plan);
/* T_init: n_pairs x 16 host doubles or NULL (identity); results may be NULL, in
 * which case execute does not synchronise */
int gca3d_icp_plan_execute(gca3d_icp_plan *plan, const double *T_init,
                           gca3d_icp_result *results);
/* the results of the plan's last execute: waits for that execute only (its copy of
 * the pair states, queued behind it), not for work queued after it.  With
 * execute(..., NULL) first, the host is free in between: it can enqueue the next
 * step's uploads on another context's stream and the next execute of another plan
 * (which then runs right behind this one) before reading these results. */
int gca3d_icp_plan_results(gca3d_icp_plan *plan, gca3d_icp_result *results);
/* bytes an execute copies back to the host (the pair states and the error word) */
int gca3d_icp_plan_readback_bytes(gca3d_icp_plan *plan, int64_t *bytes);
int gca3d_icp_plan_destroy(gca3d_icp_plan *plan);
/* kernels one execute launches (graph nodes, or the eager launches of the last run) */
int gca3d_icp_plan_kernels(gca3d_icp_plan *plan, int64_t *n);

/* time candidate launch shapes on this workload (plans built as params say, each executed
 * `reps` times after one warm-up, CUDA events on the context stream) by coordinate descent
 * from the defaults; writes the fastest to *best and its time per execute to *best_ms
 * (either may be NULL).  params->tuning is the starting point when set. */
int gca3d_icp_autotune(gca3d_context *ctx, int n_pairs, gca3d_cloud *const *src,
                       gca3d_cloud *const *tgt, const gca3d_icp_params *params, int reps,
                       gca3d_tuning *best, double *best_ms);

/* ---------------------------------------------------------------------------
 * PLY point files (host only; no context).  ascii or binary little-endian, a
 * vertex element with x, y, z and optional nx, ny, nz and red, green, blue (8-bit
 * colours are scaled by 1/255 as point_cloud::create_from_pcl does,
 * src/geometry/point_cloud.cu:481-504).  rgb / nrm may be NULL; arrays are n x 3.
 * ------------------------------------------------------------------------- */
int gca3d_ply_info(const char *path, int64_t *n_points, int *has_normals, int *has_colors);
int gca3d_ply_read(const char *path, float *xyz, float *rgb, float *nrm, int64_t cap, int64_t *n);
/* colours are written as 8-bit (round(c * 255)) */
int gca3d_ply_write(const char *path, const float *xyz, const float *rgb, const float *nrm, int64_t n,
                    int binary);

/* ---------------------------------------------------------------------------
 * frame-to-frame tracking of an RGB-D stream (the reference's demo loop,
 * app.cpp:316-350, without its model accumulation)
 * ------------------------------------------------------------------------- */
typedef struct gca3d_tracker gca3d_tracker;
typedef struct gca3d_tracker_params {
    int width, height;
    gca3d_intrinsics depth_intrin;
    gca3d_intrinsics color_intrin;
    gca3d_extrinsics depth_to_color;
    float depth_scale, tmin, tmax;
    gca3d_filter filter;
    gca3d_icp_params icp;  /* every scale needs voxel > 0; use_graph captures the whole
                              per-frame sequence as one CUDA graph */
    int constant_velocity; /* start each registration from the previous relative motion */
} gca3d_tracker_params;

int gca3d_tracker_create(gca3d_context *ctx, const gca3d_tracker_params *params,
                         gca3d_tracker **tracker);
int gca3d_tracker_destroy(gca3d_tracker *tracker);
/* the pinned host staging of the next frame (depth uint16[w*h], colour BGR
 * uint8[w*h*3]); a producer may write there and push with NULL frame pointers */
int gca3d_tracker_frame_buffers(gca3d_tracker *tracker, uint16_t **depth, uint8_t **bgr);
/* process one frame (host pointers, copied into the staging, or NULL).  For every
 * frame after the first, result (may be NULL) is the registration of the new frame
 * onto the previous one: T maps the new camera's coordinates into the previous
 * camera's.  pose (may be NULL): the camera pose relative to the first frame
 * (row-major 4x4).  The first frame's result has status GCA3D_ERR_NO_CORRESPONDENCES. */
int gca3d_tracker_push(gca3d_tracker *tracker, const uint16_t *depth, const uint8_t *bgr,
                       gca3d_icp_result *result, double pose[16]);
/* kernels the last push launched */
int gca3d_tracker_kernels(gca3d_tracker *tracker, int64_t *n);

/* ---------------------------------------------------------------------------
 * frame-to-model accumulation (the reference demo's reconstruction loop,
 * apps/app.cpp:111-128 and 315-349).  The model lives in the latest camera's
 * coordinates.  Reference settings: voxel 0.008, ror_radius 0.01,
 * ror_min_neighbors 4, normal_radius 0.04, max_iter 10, max_corr 0.05,
 * grad_radius 0.05, revoxel_every 5, filter mode GCA3D_FILTER_ADAPTIVE, t_min 0.2,
 * t_max 2.5.
 * ------------------------------------------------------------------------- */
typedef struct gca3d_model gca3d_model;
typedef struct gca3d_model_params {
    int width, height;
    gca3d_intrinsics depth_intrin;
    gca3d_intrinsics color_intrin;
    gca3d_extrinsics depth_to_color;
    float depth_scale, tmin, tmax;
    gca3d_filter filter;
    float voxel;            /* frame and model downsampling */
    float ror_radius;       /* radius outlier removal of each frame */
    int ror_min_neighbors;
    float normal_radius;
    int max_iter;           /* colored ICP of the model (or previous frame) onto the frame */
    float max_corr;
    float grad_radius;
    int revoxel_every;      /* re-voxelise the model after this many appends */
    int64_t model_capacity; /* points; at least width * height */
} gca3d_model_params;

int gca3d_model_create(gca3d_context *ctx, const gca3d_model_params *params, gca3d_model **model);
int gca3d_model_destroy(gca3d_model *model);
/* one frame (host or device pointers).  result (may be NULL): the registration onto this
 * frame (status GCA3D_ERR_NO_CORRESPONDENCES for the first frame); appended (may be
 * NULL): 1 when the frame was added to the model.  A model that outgrows its capacity
 * gives GCA3D_ERR_CAPACITY. */
int gca3d_model_push(gca3d_model *model, const uint16_t *depth, const uint8_t *bgr,
                     gca3d_icp_result *result, int *appended);
/* the model cloud (owned by the model object; valid until the next push) */
int gca3d_model_cloud(gca3d_model *model, gca3d_cloud **cloud);

/* ---------------------------------------------------------------------------
 * adjoint of K unrolled Gauss-Newton steps (no reference counterpart)
 * ------------------------------------------------------------------------- */
#define GCA3D_VJP_MAX_STEPS 64
typedef struct gca3d_vjp_params {
    int K;          /* Gauss-Newton steps, 1..GCA3D_VJP_MAX_STEPS */
    float max_corr; /* correspondence distance (m) */
    float lambda;   /* weight of the geometric term, [0, 1] */
    int update_map; /* GCA3D_UPDATE_* */
} gca3d_vjp_params;

/* K colored-ICP Gauss-Newton steps of one pair from T_0 = Exp(xi0) (SE(3)
 * exponential, xi = (w, v)), no convergence test, and -- when dT is not NULL -- the
 * gradient of L = <dT, T_K> (rows 0-2 of the row-major 4x4) + dE * E with respect
 * to xi0, the source points and the source colours, correspondences held fixed
 * (they are piecewise constant).  E is the sum of the weighted r_g^2 + r_c^2 at T_K.
 * The target needs normals and colour gradients (gca3d_estimate_normals,
 * gca3d_color_gradient).  T_out, E_out: may be NULL.  d_dxyz, d_drgb: device
 * float[n_src * 3].  d_corr (may be NULL): device int32[(K + 1) * n_src], the
 * target index of every source point at every evaluation (-1: none).
 * Returns GCA3D_ERR_SINGULAR (outputs written) when a step's system was singular. */
int gca3d_color_icp_vjp(gca3d_context *ctx, gca3d_cloud *src, gca3d_cloud *tgt,
                        const gca3d_vjp_params *params, const double xi0[6], const double dT[16],
                        double dE, double T_out[16], double *E_out, double dxi0[6], float *d_dxyz,
                        float *d_drgb, int32_t *d_corr);

/* ---------------------------------------------------------------------------
 * self-check of the short FP64 routines of the pose update (no reference
 * counterpart): over n sample points, out[0] = the largest error of the Newton
 * reciprocal against IEEE 1/d in units in the last place (d over 2^-60 .. 2^60),
 * out[1], out[2] = those of the small-angle sine and cosine against sincos
 * (|x| <= 0.25), out[3] = the largest relative difference of the series for the
 * exponential map's coefficients from their closed forms (rotation angle t in
 * 0.05 .. 0.25), in units of the closed forms' own rounding bound eps (4 + 8 / t^2)
 * (they cancel: 1 - cos t and t - sin t).
 * ------------------------------------------------------------------------- */
int gca3d_selfcheck_fp64(gca3d_context *ctx, int n, double out[4]);

/* ---------------------------------------------------------------------------
 * bounded cross-block waits (no reference counterpart: the reference's kernels
 * never wait on one another).  The look-backs of the radix sort, the scan and the
 * frame compaction poll their predecessors' states; after `polls` unanswered
 * polls (64 ns sleeps between them after the first 64) a wait gives up, the
 * state counts as the end of the look-back (offsets stay inside the outputs) and
 * the call returns GCA3D_ERR_TIMEOUT.  Default 4,194,304 polls (about 0.3 s).
 * The limit is read by the kernels when they run, so it also applies to graphs
 * captured before it was set.  polls >= 1.
 * ------------------------------------------------------------------------- */
int gca3d_set_wait_limit(gca3d_context *ctx, int polls);
int gca3d_get_wait_limit(gca3d_context *ctx, int *polls);

/* self-check of the bounded waits: a scan over `tiles` tiles (2..64) whose first
 * tile is never run, so its successor's look-back waits on a state that never
 * comes; the wait limit is `polls` for this call.  *wait_status receives the status
 * the scan's call reports (GCA3D_ERR_TIMEOUT when the wait gave up), *elapsed_ms its
 * duration on the context stream.  The context stays usable afterwards. */
int gca3d_selfcheck_wait(gca3d_context *ctx, int tiles, int polls, int *wait_status, double *elapsed_ms);

#ifdef __cplusplus
}
#endif
#endif
