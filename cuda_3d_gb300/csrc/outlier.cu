// outlier.cu -- radius outlier removal, gather by index and the AoS view of a cloud.
//
// Radius outlier removal follows point_cloud::radius_outlier_removal
// (src/geometry/point_cloud.cu:238-280), check_if_enough_radius_nn_functor
// (src/geometry/cuda_nn_search.cu:416-542) and cuda_grid_radius_outliers_removal
// (:725-800): a grid of cell 2r with origin AABB min - 1.5 cells; per axis a point
// looks at its own cell and the neighbour on the side it is nearer to (the cell's
// lower corner computed fused as cell * c + origin, as the reference does), so
// 2 x 2 x 2 cells; it counts the points with d^2 < r^2, itself included, and
// survives with more than min_neighbors.  The reference stops counting once the
// threshold is passed, which does not change the outcome.  Survivors keep input
// order: flags, exclusive scan, scatter.  Here the grid is the row-hashed one
// (4 row probes, a 2-cell z window per row).
#include "grid_query.cuh"
#include "stages.cuh"

#include <algorithm>

using namespace gca3d;

namespace
{

struct Side
{
    int b, e; // neighbour offsets [b, e) on one axis
};

__device__ __forceinline__ Side near_side(float p, float o, float cell, int c, float radius)
{
    const float lo = __fmaf_rn(cell, (float)c, o);
    const float off = __fsub_rn(p, lo);
    return Side{off >= radius ? 0 : -1, off < radius ? 1 : 2};
}

__global__ void k_ror_flags(const float4 *__restrict__ pos, const int32_t *d_n, GridDev g, float radius, int min_nn,
                            int32_t *keep)
{
    const int n = *d_n;
    const KeyLayout L = *g.layout;
    const float3 o = g.gmin[0];
    const float cell = g.cell;
    const float rr = __fmul_rn(radius, radius);
    const int mx = (1 << L.bx) - 1, my = (1 << L.by) - 1;
    const uint32_t hmask = g.hmask;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float4 p = pos[i];
        const int cx = cell_of(p.x, o.x, cell), cy = cell_of(p.y, o.y, cell), cz = cell_of(p.z, o.z, cell);
        const Side sx = near_side(p.x, o.x, cell, cx, radius);
        const Side sy = near_side(p.y, o.y, cell, cy, radius);
        const Side sz = near_side(p.z, o.z, cell, cz, radius);
        const int zlo = cz + sz.b, zhi = cz + sz.e - 1;
        int count = 0;
        for (int dx = sx.b; dx < sx.e; ++dx)
            for (int dy = sy.b; dy < sy.e; ++dy)
            {
                const int x = cx + dx, y = cy + dy;
                if (x < 0 || x > mx || y < 0 || y > my)
                    continue;
                const unsigned long long rk = ((unsigned long long)x << L.by) | (unsigned long long)y;
                const uint32_t h = hash_u64(rk) & hmask;
                const ulonglong2 v = slot_load(g.slots, h);
                int2 r = make_int2(0, 0);
                if (v.x == rk)
                    r = make_int2((int)(uint32_t)v.y, (int)(uint32_t)(v.y >> 32));
                else if (v.x != kEmptyKey)
                    r = row_probe_rest(g.slots, hmask, rk, h);
                int a = r.x, b = r.y;
                while (a < b) // first point of the row with z cell >= zlo
                {
                    const int m = (a + b) >> 1;
                    if (__ldg(&g.scz[m]) < zlo)
                        a = m + 1;
                    else
                        b = m;
                }
                for (int t = a; t < r.y; ++t)
                {
                    const float4 q = __ldg(&g.spos[t]);
                    if (__float_as_int(q.w) > zhi)
                        break;
                    count += dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z) < rr;
                }
            }
        keep[i] = count > min_nn ? 1 : 0;
    }
}

__global__ void k_ror_scatter(const float4 *__restrict__ pos, const float4 *__restrict__ col, const int32_t *d_n,
                              const int32_t *keep, const int32_t *at, float4 *out_pos, float4 *out_col)
{
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (keep[i])
        {
            out_pos[at[i]] = pos[i];
            out_col[at[i]] = col[i];
        }
}

__global__ void k_select(const float4 *__restrict__ pos, const float4 *__restrict__ col,
                         const float4 *__restrict__ nrm, const int32_t *d_n, const int32_t *idx, int m,
                         float4 *out_pos, float4 *out_col, float4 *out_nrm, int32_t *out_n, int *d_err)
{
    const int n = *d_n;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        *out_n = m;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x)
    {
        const int i = idx[k];
        if (i < 0 || i >= n)
        {
            atomicOr(d_err, kErrInvalid);
            out_pos[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            out_col[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (out_nrm)
                out_nrm[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        out_pos[k] = pos[i];
        out_col[k] = col[i];
        if (out_nrm)
            out_nrm[k] = nrm[i];
    }
}

// the reference's 28-byte point record (geometry/type.hpp:65-70): float3
// coordinates, color3, 1-byte property (+3 padding)
struct PointAoS
{
    float x, y, z, r, g, b;
    uint8_t property, pad[3];
};
static_assert(sizeof(PointAoS) == 28, "point_t is 28 bytes");

__global__ void k_to_aos(const float4 *__restrict__ pos, const float4 *__restrict__ col,
                         const float4 *__restrict__ nrm, const int32_t *d_n, PointAoS *out, float *out_nrm,
                         uint8_t property)
{
    const int n = *d_n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float4 p = pos[i], c = col[i];
        PointAoS a;
        a.x = p.x, a.y = p.y, a.z = p.z, a.r = c.x, a.g = c.y, a.b = c.z;
        a.property = property;
        a.pad[0] = a.pad[1] = a.pad[2] = 0;
        out[i] = a;
        if (out_nrm)
        {
            const float4 v = nrm[i];
            out_nrm[3 * i] = v.x, out_nrm[3 * i + 1] = v.y, out_nrm[3 * i + 2] = v.z;
        }
    }
}

} // namespace

extern "C" {

int gca3d_radius_outlier_removal(gca3d_context *ctx, gca3d_cloud *in, float radius, int min_neighbors,
                                 gca3d_cloud *out)
{
    if (!ctx || !in || !out || in == out || !(radius > 0.0f) || min_neighbors < 0)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "radius_outlier_removal: bad arguments");
    if (out->capacity < in->capacity)
        return fail(ctx, GCA3D_ERR_CAPACITY, "radius_outlier_removal: output capacity below the input's");
    ctx->arena.reset();
    Batch b;
    int st = cloud_batch(ctx, in, b);
    if (st)
        return st;
    Grid g;
    if ((st = grid_build(ctx, b, 2.0f * radius, kOriginPadF32, nullptr, g)))
        return st;
    int32_t *keep = ctx->arena.get<int32_t>(std::max<int64_t>(in->capacity, 1));
    int32_t *at = ctx->arena.get<int32_t>(std::max<int64_t>(in->capacity, 1));
    if (!keep || !at)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "radius_outlier_removal: scratch");
    const int gs = std::min(grid_for(in->capacity), ctx->num_sms * 16);
    k_ror_flags<<<gs, kBlock, 0, ctx->stream>>>(in->pos, in->d_count, g.dev, radius, min_neighbors, keep);
    GCA_CHECK_LAUNCH(ctx);
    if ((st = exclusive_scan(ctx, keep, at, in->d_count, in->capacity, out->d_count)))
        return st;
    k_ror_scatter<<<gs, kBlock, 0, ctx->stream>>>(in->pos, in->col, in->d_count, keep, at, out->pos, out->col);
    GCA_CHECK_LAUNCH(ctx);
    out->has_normals = out->has_grad = false;
    return consume_device_error(ctx, "radius_outlier_removal");
}

int gca3d_cloud_select(gca3d_context *ctx, gca3d_cloud *in, const int32_t *idx, int64_t n, gca3d_cloud *out)
{
    if (!ctx || !in || !out || in == out || n < 0 || (n > 0 && !idx))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_select: bad arguments");
    if (n > out->capacity)
        return fail(ctx, GCA3D_ERR_CAPACITY, "cloud_select: output capacity below the index count");
    if (in->has_normals)
    {
        const int st = ensure_attr(ctx, out, true, false);
        if (st)
            return st;
    }
    ctx->arena.reset();
    int32_t *d_idx = ctx->arena.get<int32_t>(std::max<int64_t>(n, 1));
    if (!d_idx)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "cloud_select: scratch");
    if (n > 0)
        GCA_CUDA(ctx, cudaMemcpyAsync(d_idx, idx, sizeof(int32_t) * (size_t)n, cudaMemcpyDefault, ctx->stream));
    const int gs = std::min(grid_for(std::max<int64_t>(n, 1)), ctx->num_sms * 16);
    k_select<<<gs, kBlock, 0, ctx->stream>>>(in->pos, in->col, in->nrm, in->d_count, d_idx, (int)n, out->pos,
                                              out->col, in->has_normals ? out->nrm : nullptr, out->d_count,
                                              ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    out->has_normals = in->has_normals;
    out->has_grad = false;
    return consume_device_error(ctx, "cloud_select");
}

int gca3d_cloud_to_aos(gca3d_context *ctx, gca3d_cloud *cloud, void *d_points, float *d_normals)
{
    if (!ctx || !cloud || !d_points || (d_normals && !cloud->has_normals))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_to_aos: bad arguments");
    const int gs = std::min(grid_for(cloud->capacity), ctx->num_sms * 16);
    // point_property::active (geometry/type.hpp:15-20)
    k_to_aos<<<gs, kBlock, 0, ctx->stream>>>(cloud->pos, cloud->col, cloud->nrm, cloud->d_count,
                                              static_cast<PointAoS *>(d_points), d_normals, 1);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

} // extern "C"
