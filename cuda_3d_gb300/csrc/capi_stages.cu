// capi_stages.cu -- C ABI of the individual path stages (single cloud / pair).
#include "icp.cuh"
#include "stages.cuh"

#include <algorithm>
#include <cmath>

using namespace gca3d;

namespace
{

__global__ void k_set_count(const int32_t *src, int32_t *dst)
{
    *dst = *src;
}

int upload_segsrc(gca3d_context *ctx, gca3d_cloud *const *clouds, int P, SegSrc **out)
{
    std::vector<SegSrc> h(P);
    for (int i = 0; i < P; ++i)
        h[i] = SegSrc{clouds[i]->pos, clouds[i]->col, clouds[i]->has_normals ? clouds[i]->nrm : nullptr,
                      clouds[i]->d_count};
    SegSrc *d = ctx->arena.get<SegSrc>(P);
    if (!d)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "segsrc: scratch");
    GCA_CUDA(ctx, cudaMemcpyAsync(d, h.data(), sizeof(SegSrc) * P, cudaMemcpyHostToDevice, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream)); // h is a host temporary
    *out = d;
    return GCA3D_OK;
}

} // namespace

namespace gca3d
{
// a single-segment batch view of a cloud (no copy)
int cloud_batch(gca3d_context *ctx, gca3d_cloud *c, Batch &b)
{
    b.pos = c->pos;
    b.col = c->col;
    b.nrm = c->nrm;
    b.grd = c->grd;
    b.P = 1;
    b.cap = c->capacity;
    b.max_seg_cap = c->capacity;
    b.seg_off = ctx->arena.get<int32_t>(2);
    if (!b.seg_off)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "cloud_batch: scratch");
    return single_seg_offsets(ctx, c->d_count, b.seg_off);
}

int make_segsrc(gca3d_context *ctx, gca3d_cloud *const *clouds, int P, SegSrc **out)
{
    return upload_segsrc(ctx, clouds, P, out);
}
} // namespace gca3d

extern "C" {

int gca3d_voxel_downsample(gca3d_context *ctx, gca3d_cloud *in, float voxel, gca3d_cloud *out)
{
    if (!ctx || !in || !out || in == out)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "voxel_downsample: bad arguments");
    if (!(voxel > 0.0f) || !std::isfinite(voxel))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "voxel_downsample: voxel size must be > 0");
    if (out->capacity < in->capacity)
        return fail(ctx, GCA3D_ERR_CAPACITY, "voxel_downsample: output capacity below input capacity");
    ctx->arena.reset();
    SegSrc *d_src = nullptr;
    int st = upload_segsrc(ctx, &in, 1, &d_src);
    if (st)
        return st;
    Batch b;
    b.pos = out->pos;
    b.col = out->col;
    b.P = 1;
    b.cap = in->capacity;
    b.max_seg_cap = in->capacity;
    b.seg_off = ctx->arena.get<int32_t>(2);
    if (!b.seg_off)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "voxel_downsample: scratch");
    st = voxel_stage(ctx, d_src, 1, in->capacity, in->capacity, voxel, b);
    if (st)
        return st;
    k_set_count<<<1, 1, 0, ctx->stream>>>(b.seg_off + 1, out->d_count);
    GCA_CHECK_LAUNCH(ctx);
    out->has_normals = out->has_grad = false;
    return consume_device_error(ctx, "voxel_downsample");
}

int gca3d_estimate_normals(gca3d_context *ctx, gca3d_cloud *c, float radius, int max_nn)
{
    if (!ctx || !c || !(radius > 0.0f) || max_nn < 0)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "estimate_normals: bad arguments");
    int st = ensure_attr(ctx, c, true, false);
    if (st)
        return st;
    ctx->arena.reset();
    Batch b;
    if ((st = cloud_batch(ctx, c, b)))
        return st;
    Grid g;
    if ((st = grid_build(ctx, b, radius, kOriginPadF64, nullptr, g)))
        return st;
    if ((st = normals_stage(ctx, b, g, true, radius, max_nn, false, 0.0f, nullptr, nullptr, nullptr, c->nrm, nullptr)))
        return st;
    c->has_normals = true;
    c->has_grad = false;
    return consume_device_error(ctx, "estimate_normals");
}

int gca3d_color_gradient(gca3d_context *ctx, gca3d_cloud *c, float radius)
{
    if (!ctx || !c || !(radius > 0.0f))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "color_gradient: bad arguments");
    if (!c->has_normals)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "color_gradient: estimate normals first");
    int st = ensure_attr(ctx, c, false, true);
    if (st)
        return st;
    ctx->arena.reset();
    Batch b;
    if ((st = cloud_batch(ctx, c, b)))
        return st;
    Grid g;
    if ((st = grid_build(ctx, b, radius, kOriginPadF32, nullptr, g)))
        return st;
    if ((st = normals_stage(ctx, b, g, false, 0.0f, 0, true, radius, c->nrm, nullptr, nullptr, nullptr, c->grd)))
        return st;
    c->has_grad = true;
    c->grad_radius = radius;
    return consume_device_error(ctx, "color_gradient");
}

int gca3d_nn_search(gca3d_context *ctx, gca3d_cloud *query, gca3d_cloud *ref, float radius, int32_t *out_idx)
{
    if (!ctx || !query || !ref || !out_idx || !(radius > 0.0f))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "nn_search: bad arguments");
    ctx->arena.reset();
    Batch b;
    int st = cloud_batch(ctx, ref, b);
    if (st)
        return st;
    Grid g;
    if ((st = grid_build(ctx, b, radius, kOriginPadF32, nullptr, g)))
        return st;
    if ((st = nn_query(ctx, query->pos, query->d_count, query->capacity, g, radius, out_idx)))
        return st;
    return consume_device_error(ctx, "nn_search");
}

int gca3d_radius_search(gca3d_context *ctx, gca3d_cloud *query, gca3d_cloud *ref, float radius,
                        const float grid_min[3], int32_t *counts, int32_t *starts, int32_t *list, int64_t list_cap,
                        int64_t *total)
{
    if (!ctx || !query || !ref || !counts || !starts || !(radius > 0.0f) || (list_cap > 0 && !list))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "radius_search: bad arguments");
    ctx->arena.reset();
    Batch b;
    int st = cloud_batch(ctx, ref, b);
    if (st)
        return st;
    Grid g;
    if ((st = grid_build(ctx, b, radius, grid_min ? kOriginGiven : kOriginPadF64, grid_min, g)))
        return st;
    int32_t *d_total = ctx->arena.get<int32_t>(1);
    if (!d_total)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "radius_search: scratch");
    if ((st = radius_query(ctx, query->pos, query->d_count, query->capacity, g, radius, counts, starts, list,
                           list_cap, d_total)))
        return st;
    GCA_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, d_total, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (total)
        *total = ctx->h_pinned[0];
    st = consume_device_error(ctx, "radius_search");
    if (st == GCA3D_ERR_CAPACITY)
        ctx->last_error = "radius_search: list capacity below the total neighbour count";
    return st;
}

int gca3d_build_gauss_newton(gca3d_context *ctx, gca3d_cloud *src, gca3d_cloud *tgt, const int32_t *nn, float lambda,
                             double jtj[36], double jtr[6], double *r2)
{
    if (!ctx || !src || !tgt || !nn || !jtj || !jtr)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "build_gauss_newton: bad arguments");
    // cuda_color_icp_build_least_square.cu:438-452: lambda <= 1, target attributes present
    if (!(lambda <= 1.0f) || !(lambda >= 0.0f))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "build_gauss_newton: lambda must be in [0, 1]");
    if (!tgt->has_normals || !tgt->has_grad)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "build_gauss_newton: target needs normals and colour gradients");
    ctx->arena.reset();
    double S[kTermsPad];
    int st = build_gn(ctx, src, tgt, nn, lambda, S);
    if (st)
        return st;
    int u = 0;
    for (int a = 0; a < 6; ++a)
        for (int b = a; b < 6; ++b)
        {
            jtj[6 * a + b] = jtj[6 * b + a] = S[u];
            ++u;
        }
    for (int a = 0; a < 6; ++a)
        jtr[a] = S[21 + a];
    if (r2)
        *r2 = S[27];
    return GCA3D_OK;
}

int gca3d_abs_residual(gca3d_context *ctx, gca3d_cloud *src, gca3d_cloud *tgt, const int32_t *nn, float lambda,
                       float *out)
{
    if (!ctx || !src || !tgt || !nn || !out)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "abs_residual: bad arguments");
    if (!(lambda <= 1.0f) || !(lambda >= 0.0f))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "abs_residual: lambda must be in [0, 1]");
    if (!tgt->has_normals || !tgt->has_grad)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "abs_residual: target needs normals and colour gradients");
    int st = abs_residual(ctx, src, tgt, nn, lambda, out);
    if (st)
        return st;
    return GCA3D_OK;
}

} // extern "C"
