// model.cu -- the frame-to-model accumulation loop of the reference's demo.
//
// reference: apps/app.cpp:111-128 (per frame: create_from_rgbd with t_min / t_max,
// voxel_grid_down_sample(0.008), radius_outlier_removal(0.01, 4),
// estimate_normals(0.04)) and app.cpp:315-349 (the first frame starts the model;
// afterwards color_icp(10, 0.05, 0.05) registers the model -- or, while the
// counter is not zero, the previous frame -- onto the new frame; when the step is
// significant (cos theta <= 0.999999 or |t|^2 >= 1e-6, in FP32) the model is
// transformed into the new camera's coordinates and the frame is appended
// (point_cloud::operator+=, src/geometry/point_cloud.cu:55-73); every 5 appends the
// model is voxel-downsampled again).  The model therefore lives in the coordinates
// of the latest camera.
//
// Each step is one of the library's stage entry points on the context stream; the
// per-frame host work is the frame upload, the read-back of the registration and
// the counter logic above.
#include "internal.cuh"

#include <cstring>

using namespace gca3d;

struct gca3d_model
{
    gca3d_context *ctx = nullptr;
    gca3d_model_params prm{};
    uint16_t *d_depth = nullptr;
    uint8_t *d_bgr = nullptr;
    gca3d_cloud *raw = nullptr, *ds = nullptr;
    gca3d_cloud *frame[2] = {nullptr, nullptr}; // cleaned frames: this one and the previous one
    gca3d_cloud *model[2] = {nullptr, nullptr}; // the model and the target of its re-voxelisation
    int cur = 0, m = 0, counter = 0;
    int64_t frames = 0;
};

extern "C" {

int gca3d_model_destroy(gca3d_model *s)
{
    if (!s)
        return GCA3D_ERR_INVALID_VALUE;
    if (s->ctx)
        cudaStreamSynchronize(s->ctx->stream);
    gca3d_cloud *all[] = {s->raw, s->ds, s->frame[0], s->frame[1], s->model[0], s->model[1]};
    for (gca3d_cloud *c : all)
        if (c)
            gca3d_cloud_destroy(c);
    cudaFree(s->d_depth);
    cudaFree(s->d_bgr);
    delete s;
    return GCA3D_OK;
}

int gca3d_model_create(gca3d_context *ctx, const gca3d_model_params *p, gca3d_model **out)
{
    if (!ctx || !p || !out)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "model: null argument");
    *out = nullptr;
    if (p->width <= 0 || p->height <= 0 || !(p->voxel > 0.0f) || !(p->ror_radius > 0.0f) ||
        p->ror_min_neighbors < 0 || !(p->normal_radius > 0.0f) || p->max_iter < 1 || !(p->max_corr > 0.0f) ||
        !(p->grad_radius > 0.0f) || p->revoxel_every < 1 || p->model_capacity < (int64_t)p->width * p->height)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "model: bad parameters");
    auto *s = new gca3d_model();
    s->ctx = ctx;
    s->prm = *p;
    const int64_t n = (int64_t)p->width * p->height;
    int st = GCA3D_OK;
    if (cudaMalloc(&s->d_depth, sizeof(uint16_t) * (size_t)n) != cudaSuccess ||
        cudaMalloc(&s->d_bgr, 3 * (size_t)n) != cudaSuccess)
    {
        cudaGetLastError();
        st = fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "model: frame buffers");
    }
    gca3d_cloud **frame_sized[] = {&s->raw, &s->ds, &s->frame[0], &s->frame[1]};
    for (gca3d_cloud **c : frame_sized)
        if (!st)
            st = gca3d_cloud_create(ctx, n, c);
    for (int k = 0; k < 2 && !st; ++k)
        st = gca3d_cloud_create(ctx, p->model_capacity, &s->model[k]);
    if (st)
    {
        gca3d_model_destroy(s);
        return st;
    }
    *out = s;
    return GCA3D_OK;
}

int gca3d_model_push(gca3d_model *s, const uint16_t *depth, const uint8_t *bgr, gca3d_icp_result *result,
                     int *appended)
{
    if (!s || !depth || !bgr)
        return GCA3D_ERR_INVALID_VALUE;
    gca3d_context *ctx = s->ctx;
    const gca3d_model_params &p = s->prm;
    const int64_t npix = (int64_t)p.width * p.height;
    if (appended)
        *appended = 0;
    gca3d_icp_result res;
    memset(&res, 0, sizeof res);
    for (int k = 0; k < 16; ++k)
        res.T[k] = (k % 5 == 0) ? 1.0 : 0.0;
    res.status = GCA3D_ERR_NO_CORRESPONDENCES;
    // app.cpp:118-128: the frame, cleaned
    GCA_CUDA(ctx, cudaMemcpyAsync(s->d_depth, depth, sizeof(uint16_t) * (size_t)npix, cudaMemcpyDefault, ctx->stream));
    GCA_CUDA(ctx, cudaMemcpyAsync(s->d_bgr, bgr, 3 * (size_t)npix, cudaMemcpyDefault, ctx->stream));
    gca3d_cloud *cur = s->frame[s->cur], *prev = s->frame[s->cur ^ 1];
    int st = gca3d_frame_to_cloud(ctx, s->d_depth, s->d_bgr, p.width, p.height, &p.depth_intrin, &p.color_intrin,
                                  &p.depth_to_color, p.depth_scale, p.tmin, p.tmax, &p.filter, s->raw);
    if (!st)
        st = gca3d_voxel_downsample(ctx, s->raw, p.voxel, s->ds);
    if (!st)
        st = gca3d_radius_outlier_removal(ctx, s->ds, p.ror_radius, p.ror_min_neighbors, cur);
    if (!st)
        st = gca3d_estimate_normals(ctx, cur, p.normal_radius, 0);
    if (st)
        return st;
    if (s->frames == 0)
    {
        // app.cpp:315-321: the first frame starts the model
        if ((st = gca3d_cloud_copy(ctx, cur, s->model[s->m])))
            return st;
    }
    else
    {
        // app.cpp:322-327: the model (counter 0) or the previous frame onto this frame
        gca3d_icp_params ip;
        memset(&ip, 0, sizeof ip);
        ip.n_scales = 1;
        ip.scales[0].voxel = 0.0f;
        ip.scales[0].max_iter = p.max_iter;
        ip.scales[0].max_corr = p.max_corr;
        ip.scales[0].grad_radius = p.grad_radius;
        ip.lambda = 0.968f;
        ip.update_map = GCA3D_UPDATE_EULER_ZYX;
        ip.rot_eps = ip.trans_eps = (double)0.000001f; // color_icp.hpp:47-48
        ip.compensated = 1;
        ip.keep_target_normals = 1;
        gca3d_cloud *src = s->counter == 0 ? s->model[s->m] : prev;
        if ((st = gca3d_color_icp(ctx, src, cur, &ip, nullptr, &res)))
            return st;
        if (res.status == GCA3D_OK)
        {
            // app.cpp:328-340, in FP32 as the reference computes it
            float Tf[16];
            for (int k = 0; k < 16; ++k)
                Tf[k] = (float)res.T[k];
            const float cth = 0.5f * (Tf[0] + Tf[5] + Tf[10] - 1.0f);
            const float tsq = Tf[3] * Tf[3] + Tf[7] * Tf[7] + Tf[11] * Tf[11];
            if (cth <= 0.999999f || tsq >= 0.000001f)
            {
                double Td[16];
                for (int k = 0; k < 16; ++k)
                    Td[k] = (double)Tf[k];
                if ((st = gca3d_transform(ctx, s->model[s->m], Td)) ||
                    (st = gca3d_cloud_append(ctx, s->model[s->m], cur)))
                    return st;
                s->counter += 1;
                if (appended)
                    *appended = 1;
            }
            // app.cpp:342-347: re-voxelise every revoxel_every appends
            if (s->counter == p.revoxel_every)
            {
                if ((st = gca3d_voxel_downsample(ctx, s->model[s->m], p.voxel, s->model[s->m ^ 1])))
                    return st;
                s->m ^= 1;
                s->counter = 0;
            }
        }
    }
    s->cur ^= 1; // app.cpp:349: this frame is the next one's previous frame
    s->frames += 1;
    if (result)
        *result = res;
    return GCA3D_OK;
}

int gca3d_model_cloud(gca3d_model *s, gca3d_cloud **model)
{
    if (!s || !model)
        return GCA3D_ERR_INVALID_VALUE;
    *model = s->model[s->m];
    return GCA3D_OK;
}

} // extern "C"
