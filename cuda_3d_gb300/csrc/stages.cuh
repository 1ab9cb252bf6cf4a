// stages.cuh -- batched stage interfaces shared by the translation units.
#pragma once

#include "internal.cuh"

#include <functional>

namespace gca3d
{

struct Pose34f
{
    float m[12]; // row-major 3x4
};
Pose34f pose_to_f32(const double T[16]);

// P point sets back to back in structure-of-arrays form
struct Batch
{
    float4 *pos = nullptr, *col = nullptr, *nrm = nullptr, *grd = nullptr;
    int32_t *seg_off = nullptr; // device [P + 1]
    int P = 0;
    int64_t cap = 0;         // total capacity
    int64_t max_seg_cap = 0; // largest segment capacity
};

// a source cloud of a batched stage, read through a device pointer table
struct SegSrc
{
    const float4 *pos;
    const float4 *col;
    const float4 *nrm;
    const int32_t *d_n;
};

enum GridOrigin : int
{
    kOriginPadF32 = 0, // aabb_min - 1.5f * cell            (color_icp.cu:55-66, point_cloud.cu:519-537)
    kOriginPadF64 = 1, // (float)((double)aabb_min - 1.5 * (double)cell)   (point_cloud.cu:153-159)
    kOriginGiven = 2,  // caller-supplied origin (single segment)
};

struct Grid
{
    GridDev dev;
    int64_t cap = 0;
    int P = 0;
    uint32_t hcap = 0;
};

int seg_bounds(gca3d_context *ctx, const float4 *pos, const int32_t *seg_off, int P, int64_t max_seg_cap,
               int *ord);
int single_seg_offsets(gca3d_context *ctx, const int32_t *d_n, int32_t *seg_off);

// a depth + colour frame: camera model, filter and limits of the frame kernel
constexpr int kMaxFilterRadius = 7;
constexpr int kMaxFrameWidth = 2048;
struct FrameParams
{
    int w, h;
    float fx, fy, cx, cy;     // depth intrinsics
    float cfx, cfy, ccx, ccy; // colour intrinsics
    float R[9], t[3];         // depth -> colour, column-major rotation
    float depth_scale, tmin, tmax;
    int mode, radius;
    float sigma_space, sigma_depth;
};
int frame_params(gca3d_context *ctx, int w, int h, const gca3d_intrinsics *di, const gca3d_intrinsics *ci,
                 const gca3d_extrinsics *d2c, float depth_scale, float tmin, float tmax, const gca3d_filter *filter,
                 FrameParams &P);
// filtered, back-projected and compacted frame into `out` (device count); scratch
// from the context arena; no host synchronisation (capture-safe)
int frame_to_cloud(gca3d_context *ctx, const uint16_t *depth, const uint8_t *bgr, const FrameParams &P,
                   gca3d_cloud *out);

// an ICP plan whose graph (or eager run) starts with `prologue`, enqueued on the
// context stream with the plan's arena active (the frame stage of a tracker)
using PlanPrologue = std::function<int(gca3d_context *)>;
// voxel batches supplied by the caller (one pair, every scale downsampled): per
// scale the source is downsampled into src[s] and tgt[s] is the target as it is
// (a tracker passes the previous frame's source batches, so every frame is
// downsampled once)
struct PlanVoxels
{
    Batch src[GCA3D_MAX_SCALES];
    Batch tgt[GCA3D_MAX_SCALES];
};
int icp_plan_create_internal(gca3d_context *ctx, int P, gca3d_cloud *const *src, gca3d_cloud *const *tgt,
                             const gca3d_icp_params *params, bool capture, PlanPrologue prologue,
                             gca3d_icp_plan **out, const PlanVoxels *voxels = nullptr);

// a single-segment batch view of a cloud (no copy; segment offsets from the arena)
int cloud_batch(gca3d_context *ctx, gca3d_cloud *c, Batch &b);

// allocate a batch from the context arena
int batch_alloc(gca3d_context *ctx, Batch &b, int P, int64_t cap, int64_t max_seg_cap, bool nrm, bool grd);

// stage 0 of a scale: voxel downsample (voxel > 0) or gather copy into a batch
// morton: output in Z-order of the voxels instead of the reference's (x, y, z) order
// (same voxels, same centroids)
// finer scales carried by a voxel stage: their voxel sizes, each half the previous one
// (exactly, in float), so their cells refine the stage's cells (see k_voxel_keys)
constexpr int kMaxSubLevels = 4;
struct SubLevels
{
    int n = 0;
    float voxel[kMaxSubLevels] = {0.0f, 0.0f, 0.0f, 0.0f};
};

// the sorted state of a voxel stage that finer scales refine instead of sorting again
struct VoxelChain
{
    SortBuffers sb;          // the sort arrays (shared by the scales) and the last scale's view
    const int32_t *in_off = nullptr;
    int32_t *starts = nullptr, *d_m = nullptr; // the last scale's voxel runs
    const KeyLayout *lay = nullptr;            // the last scale's key layout
    int levels = 0, used = 0;
    int P = 0;
    int64_t total_cap = 0, max_seg_cap = 0;
};

// voxel-grid downsampling of P segments; morton: Z-order keys; finer (with morton):
// carry the sub-cell bits of finer scales and record the sorted state in *chain, which
// voxel_refine then turns into each finer scale's downsampling, in order
int voxel_stage(gca3d_context *ctx, const SegSrc *d_src, int P, int64_t total_cap, int64_t max_seg_cap,
                float voxel, Batch &out, bool morton = false, const SubLevels *finer = nullptr,
                VoxelChain *chain = nullptr);
int voxel_refine(gca3d_context *ctx, const SegSrc *d_src, VoxelChain &chain, Batch &out);
int gather_stage(gca3d_context *ctx, const SegSrc *d_src, int P, int64_t max_seg_cap, Batch &out,
                 bool with_normals);

// uniform grid over a batch; cell edge `cell`
int grid_build(gca3d_context *ctx, const Batch &b, float cell, int origin_mode, const float *host_origin,
               Grid &g);

// fused normals + colour gradient over the grid's own points (targets).  Writes
// attr0 = {n, intensity} and attr1 = {gradient, 0} in grid order, and scatters
// normals / gradients back to the batch (original order) when nrm_out / grd_out
// are set.  in_nrm (original order) supplies normals when do_normals is false.
int normals_stage(gca3d_context *ctx, const Batch &b, const Grid &g, bool do_normals, float normal_radius,
                  int max_nn, bool do_grad, float grad_radius, const float4 *in_nrm, float4 *attr0,
                  float4 *attr1, float4 *nrm_out, float4 *grd_out);

// the target records of grid g gathered from original-order normals / gradients
int gather_attrs(gca3d_context *ctx, const Batch &b, const Grid &g, const float4 *nrm, const float4 *grd,
                 float4 *attr0, float4 *attr1);

// nearest neighbour / radius lists of query batch points against a single-segment grid
int nn_query(gca3d_context *ctx, const float4 *qpos, const int32_t *d_nq, int64_t qcap, const Grid &g,
             float radius, int32_t *out_idx);
int radius_query(gca3d_context *ctx, const float4 *qpos, const int32_t *d_nq, int64_t qcap, const Grid &g,
                 float radius, int32_t *counts, int32_t *starts, int32_t *list, int64_t list_cap,
                 int32_t *d_total);

} // namespace gca3d
