// tracker.cu -- frame-to-frame colored-ICP tracking of an RGB-D stream.
//
// reference: the demo loop of apps (app.cpp:316-350): per frame, create_from_rgbd
// (src/geometry/point_cloud.cu:455-479), voxel_grid_down_sample, estimate_normals
// and color_icp against the previous frame, composing the camera pose.  (The
// reference also accumulates a model cloud; that is not part of tracking.)
//
// A tracker owns pinned host staging for one depth + colour frame, device frame
// buffers and two raw-cloud slots used alternately.  Frame k (k >= 1) registers
// slot k % 2 (this frame, the source) onto slot 1 - k % 2 (the previous frame, the
// target) with an ICP plan whose prologue uploads the staged frame and runs the
// frame kernel into the source slot.  Every slot also owns one voxel batch per
// scale: a frame is downsampled once, as the source, and its batches are the
// target of the next frame.  With use_graph the whole per-frame sequence --
// upload, filter and back-projection, voxel downsampling, target normals and colour
// gradients, the coarse-to-fine iterations -- is one CUDA graph per slot parity,
// replayed every frame.  The only host work per frame is the copy into staging,
// the graph launch and the read-back of the pair state.
#include "icp.cuh"
#include "stages.cuh"

#include <cstring>

using namespace gca3d;

struct gca3d_tracker
{
    gca3d_context *ctx = nullptr;
    gca3d_tracker_params prm{};
    FrameParams fp{};
    size_t depth_bytes = 0, bgr_bytes = 0;
    uint16_t *d_depth = nullptr, *h_depth = nullptr;
    uint8_t *d_bgr = nullptr, *h_bgr = nullptr;
    gca3d_cloud *raw[2] = {nullptr, nullptr};
    gca3d_icp_plan *plan[2] = {nullptr, nullptr};
    PlanVoxels vox[2];              // per slot: .src = its voxel batches per scale
    SegSrc *d_seg[2] = {nullptr, nullptr}; // per slot: the raw cloud as a stage source
    int64_t frames = 0;
    double pose[16];
    double last[16];
};

namespace
{

void set_identity(double *T)
{
    for (int k = 0; k < 16; ++k)
        T[k] = (k % 5 == 0) ? 1.0 : 0.0;
}

void mat4_mul(const double *A, const double *B, double *C)
{
    double R[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
        {
            double s = 0.0;
            for (int k = 0; k < 4; ++k)
                s += A[4 * i + k] * B[4 * k + j];
            R[4 * i + j] = s;
        }
    memcpy(C, R, sizeof R);
}

// upload the staged frame and run the frame kernel into `out` (capture-safe)
int enqueue_frame(gca3d_tracker *t, gca3d_cloud *out)
{
    gca3d_context *ctx = t->ctx;
    GCA_CUDA(ctx, cudaMemcpyAsync(t->d_depth, t->h_depth, t->depth_bytes, cudaMemcpyHostToDevice, ctx->stream));
    GCA_CUDA(ctx, cudaMemcpyAsync(t->d_bgr, t->h_bgr, t->bgr_bytes, cudaMemcpyHostToDevice, ctx->stream));
    return frame_to_cloud(ctx, t->d_depth, t->d_bgr, t->fp, out);
}

} // namespace

extern "C" {

int gca3d_tracker_destroy(gca3d_tracker *t)
{
    if (!t)
        return GCA3D_ERR_INVALID_VALUE;
    if (t->ctx)
        cudaStreamSynchronize(t->ctx->stream);
    for (int k = 0; k < 2; ++k)
    {
        if (t->plan[k])
            gca3d_icp_plan_destroy(t->plan[k]);
        if (t->raw[k])
            gca3d_cloud_destroy(t->raw[k]);
        for (int s = 0; s < GCA3D_MAX_SCALES; ++s)
        {
            cudaFree(t->vox[k].src[s].pos);
            cudaFree(t->vox[k].src[s].col);
            cudaFree(t->vox[k].src[s].seg_off);
        }
        cudaFree(t->d_seg[k]);
    }
    cudaFree(t->d_depth);
    cudaFree(t->d_bgr);
    if (t->h_depth)
        cudaFreeHost(t->h_depth);
    if (t->h_bgr)
        cudaFreeHost(t->h_bgr);
    delete t;
    return GCA3D_OK;
}

int gca3d_tracker_create(gca3d_context *ctx, const gca3d_tracker_params *p, gca3d_tracker **out)
{
    if (!ctx || !p || !out)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "tracker: null argument");
    *out = nullptr;
    FrameParams fp;
    int st = frame_params(ctx, p->width, p->height, &p->depth_intrin, &p->color_intrin, &p->depth_to_color,
                          p->depth_scale, p->tmin, p->tmax, &p->filter, fp);
    if (st)
        return st;
    if (p->icp.n_scales < 1 || p->icp.n_scales > GCA3D_MAX_SCALES)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "tracker: n_scales must be in [1, 8]");
    for (int s = 0; s < p->icp.n_scales; ++s)
        if (!(p->icp.scales[s].voxel > 0.0f))
            return fail(ctx, GCA3D_ERR_INVALID_VALUE, "tracker: every scale needs a voxel size (frames are raw)");
    auto *t = new gca3d_tracker();
    t->ctx = ctx;
    t->prm = *p;
    t->fp = fp;
    const int64_t n = (int64_t)p->width * p->height;
    t->depth_bytes = sizeof(uint16_t) * (size_t)n;
    t->bgr_bytes = 3 * (size_t)n;
    if (cudaMalloc(&t->d_depth, t->depth_bytes) != cudaSuccess || cudaMalloc(&t->d_bgr, t->bgr_bytes) != cudaSuccess ||
        cudaMallocHost(&t->h_depth, t->depth_bytes) != cudaSuccess ||
        cudaMallocHost(&t->h_bgr, t->bgr_bytes) != cudaSuccess)
    {
        cudaGetLastError();
        gca3d_tracker_destroy(t);
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "tracker: frame buffers");
    }
    memset(t->h_depth, 0, t->depth_bytes);
    memset(t->h_bgr, 0, t->bgr_bytes);
    for (int k = 0; k < 2; ++k)
    {
        if ((st = gca3d_cloud_create(ctx, n, &t->raw[k])))
        {
            gca3d_tracker_destroy(t);
            return st;
        }
        const SegSrc seg{t->raw[k]->pos, t->raw[k]->col, nullptr, t->raw[k]->d_count};
        bool ok = cudaMalloc(&t->d_seg[k], sizeof(SegSrc)) == cudaSuccess &&
                  cudaMemcpy(t->d_seg[k], &seg, sizeof(SegSrc), cudaMemcpyHostToDevice) == cudaSuccess;
        for (int s = 0; ok && s < p->icp.n_scales; ++s)
        {
            Batch &b = t->vox[k].src[s];
            b.P = 1;
            b.cap = b.max_seg_cap = n;
            ok = cudaMalloc(&b.pos, sizeof(float4) * (size_t)n) == cudaSuccess &&
                 cudaMalloc(&b.col, sizeof(float4) * (size_t)n) == cudaSuccess &&
                 cudaMalloc(&b.seg_off, sizeof(int32_t) * 2) == cudaSuccess;
        }
        if (!ok)
        {
            cudaGetLastError();
            gca3d_tracker_destroy(t);
            return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "tracker: voxel batches");
        }
    }
    set_identity(t->pose);
    set_identity(t->last);
    *out = t;
    return GCA3D_OK;
}

int gca3d_tracker_frame_buffers(gca3d_tracker *t, uint16_t **depth, uint8_t **bgr)
{
    if (!t)
        return GCA3D_ERR_INVALID_VALUE;
    if (depth)
        *depth = t->h_depth;
    if (bgr)
        *bgr = t->h_bgr;
    return GCA3D_OK;
}

int gca3d_tracker_push(gca3d_tracker *t, const uint16_t *depth, const uint8_t *bgr, gca3d_icp_result *result,
                       double pose[16])
{
    if (!t)
        return GCA3D_ERR_INVALID_VALUE;
    gca3d_context *ctx = t->ctx;
    // the previous frame's graph may still read the staging buffers
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (depth)
        memcpy(t->h_depth, depth, t->depth_bytes);
    if (bgr)
        memcpy(t->h_bgr, bgr, t->bgr_bytes);
    gca3d_icp_result res;
    memset(&res, 0, sizeof res);
    set_identity(res.T);
    int st;
    if (t->frames == 0)
    {
        ctx->arena.reset();
        if ((st = enqueue_frame(t, t->raw[0])))
            return st;
        // the first frame is downsampled here: it is the target of the next
        for (int s = 0; s < t->prm.icp.n_scales; ++s)
            if ((st = voxel_stage(ctx, t->d_seg[0], 1, t->raw[0]->capacity, t->raw[0]->capacity,
                                  t->prm.icp.scales[s].voxel, t->vox[0].src[s], true)))
                return st;
        GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if ((st = consume_device_error(ctx, "tracker")))
            return st;
        res.status = GCA3D_ERR_NO_CORRESPONDENCES; // nothing to register against yet
    }
    else
    {
        const int cur = (int)(t->frames & 1);
        if (!t->plan[cur])
        {
            gca3d_cloud *s = t->raw[cur], *g = t->raw[1 - cur];
            gca3d_cloud *src_slot = t->raw[cur];
            PlanVoxels v;
            for (int s2 = 0; s2 < t->prm.icp.n_scales; ++s2)
            {
                v.src[s2] = t->vox[cur].src[s2];
                v.tgt[s2] = t->vox[1 - cur].src[s2];
            }
            st = icp_plan_create_internal(
                ctx, 1, &s, &g, &t->prm.icp, t->prm.icp.use_graph != 0,
                [t, src_slot](gca3d_context *) { return enqueue_frame(t, src_slot); }, &t->plan[cur], &v);
            if (st)
                return st;
        }
        double T_init[16];
        if (t->prm.constant_velocity)
            memcpy(T_init, t->last, sizeof T_init);
        else
            set_identity(T_init);
        if ((st = gca3d_icp_plan_execute(t->plan[cur], T_init, &res)))
            return st;
        if (res.status == GCA3D_OK)
        {
            memcpy(t->last, res.T, sizeof t->last);
            mat4_mul(t->pose, res.T, t->pose);
        }
        else
            set_identity(t->last);
    }
    t->frames += 1;
    if (result)
        *result = res;
    if (pose)
        memcpy(pose, t->pose, sizeof t->pose);
    return GCA3D_OK;
}

int gca3d_tracker_kernels(gca3d_tracker *t, int64_t *n)
{
    if (!t || !n)
        return GCA3D_ERR_INVALID_VALUE;
    const gca3d_icp_plan *pl = t->plan[(t->frames + 1) & 1];
    *n = 0;
    if (pl)
        return gca3d_icp_plan_kernels(const_cast<gca3d_icp_plan *>(pl), n);
    return GCA3D_OK;
}

} // extern "C"
