// cloud.cu -- context, scratch arena, cloud handles and the elementwise cloud
// kernels (pack/unpack, bounds, rigid transform, copy/append).
#include "internal.cuh"
#include "stages.cuh"

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstring>

namespace gca3d
{

// ---------------------------------------------------------------------------
// arena
// ---------------------------------------------------------------------------
void *Arena::take(size_t bytes)
{
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0)
        bytes = 256;
    while (cur < chunks.size())
    {
        Chunk &c = chunks[cur];
        if (c.size - c.used >= bytes)
        {
            void *p = c.ptr + c.used;
            c.used += bytes;
            return p;
        }
        ++cur;
    }
    if (frozen)
    {
        failed = true;
        return nullptr;
    }
    Chunk c;
    c.size = std::max(bytes, size_t(64) << 20);
    if (cudaMalloc(&c.ptr, c.size) != cudaSuccess)
    {
        cudaGetLastError();
        failed = true;
        return nullptr;
    }
    c.used = bytes;
    chunks.push_back(c);
    cur = chunks.size() - 1;
    return c.ptr;
}

void Arena::release()
{
    for (auto &c : chunks)
        if (c.ptr)
            cudaFree(c.ptr);
    chunks.clear();
    cur = 0;
}

int fail(gca3d_context *ctx, int status, const std::string &msg)
{
    if (ctx)
        ctx->last_error = msg;
    return status;
}

int cuda_fail(gca3d_context *ctx, cudaError_t e, const char *where)
{
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, m);
    return fail(ctx, GCA3D_ERR_CUDA, m);
}

int consume_device_error(gca3d_context *ctx, const char *where)
{
    int h = 0;
    GCA_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    h = ctx->h_pinned[0];
    if (!h)
        return GCA3D_OK;
    GCA_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    return device_error_status(ctx, h, where);
}

int device_error_status(gca3d_context *ctx, int h, const char *where)
{
    if (!h)
        return GCA3D_OK;
    if (h & kErrTimeout)
        return fail(ctx, GCA3D_ERR_TIMEOUT, std::string(where) + ": a look-back wait gave up");
    if (h & kErrKeyBits)
        return fail(ctx, GCA3D_ERR_CAPACITY, std::string(where) + ": extent / cell exceeds the key range");
    if (h & kErrCapacity)
        return fail(ctx, GCA3D_ERR_CAPACITY, std::string(where) + ": output capacity exceeded");
    if (h & kErrInvalid)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, std::string(where) + ": invalid value on the device");
    if (h & kErrBounds)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, std::string(where) + ": an index check failed (checked build)");
    return GCA3D_OK;
}

void prof_mark(gca3d_context *ctx, int kid)
{
    Profiler &P = ctx->prof;
    if (P.target != kid || kid == kKidNone)
        return;
    if (P.used == P.events.size())
    {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess)
            return;
        P.events.push_back(e);
    }
    cudaEventRecord(P.events[P.used++], ctx->stream);
}

int ensure_attr(gca3d_context *ctx, gca3d_cloud *c, bool normals, bool grad)
{
    size_t bytes = sizeof(float4) * (size_t)std::max<int64_t>(c->capacity, 1);
    if (normals && !c->nrm)
        GCA_CUDA(ctx, cudaMalloc(&c->nrm, bytes));
    if (grad && !c->grd)
        GCA_CUDA(ctx, cudaMalloc(&c->grd, bytes));
    return GCA3D_OK;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__global__ void k_pack(const float *__restrict__ xyz, const float *__restrict__ rgb, int n, float4 *pos,
                       float4 *col, int32_t *d_count)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0)
        *d_count = n;
    if (i >= n)
        return;
    float r = rgb ? rgb[3 * i] : 0.0f, g = rgb ? rgb[3 * i + 1] : 0.0f, b = rgb ? rgb[3 * i + 2] : 0.0f;
    pos[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], intensity_of(r, g, b));
    col[i] = make_float4(r, g, b, 0.0f);
}

// many clouds' uploads in one launch: descriptors by value (kUploadChunk per launch,
// under the 4 KB parameter limit); a block packs part of one cloud
constexpr int kUploadChunk = 64;
struct UploadDesc
{
    const float *xyz, *rgb;
    float4 *pos, *col;
    int32_t *d_count;
    int n, first; // points, first block
};
struct UploadBatch
{
    int count;
    UploadDesc d[kUploadChunk];
};

__global__ void k_pack_many(const __grid_constant__ UploadBatch B)
{
    // the block's cloud: the last one whose first block is <= blockIdx.x
    int lo = 0, hi = B.count - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (B.d[mid].first <= (int)blockIdx.x)
            lo = mid;
        else
            hi = mid - 1;
    }
    const UploadDesc &D = B.d[lo];
    const int i = ((int)blockIdx.x - D.first) * (int)blockDim.x + (int)threadIdx.x;
    if (i == 0)
        *D.d_count = D.n;
    if (i >= D.n)
        return;
    const float *rgb = D.rgb, *xyz = D.xyz;
    const float r = rgb ? rgb[3 * i] : 0.0f, g = rgb ? rgb[3 * i + 1] : 0.0f, b = rgb ? rgb[3 * i + 2] : 0.0f;
    D.pos[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], intensity_of(r, g, b));
    D.col[i] = make_float4(r, g, b, 0.0f);
}

__global__ void k_pack3(const float *__restrict__ v, int n, float4 *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = make_float4(v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.0f);
}

__global__ void k_unpack(const float4 *__restrict__ a, const int32_t *d_n, float *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *d_n)
        return;
    float4 p = a[i];
    out[3 * i] = p.x;
    out[3 * i + 1] = p.y;
    out[3 * i + 2] = p.z;
}

// per-segment bounds as ordered ints; grid.y = segment
__global__ void k_init_bounds(int *ord, int P)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * P)
        ord[i] = (i % 6) < 3 ? float_to_ordered(FLT_MAX) : float_to_ordered(-FLT_MAX);
}

__global__ void k_bounds(const float4 *__restrict__ pos, const int32_t *seg_off, int *ord)
{
    const int seg = blockIdx.y;
    const int b = seg_off[seg], e = seg_off[seg + 1];
    if (b + (int64_t)blockIdx.x * blockDim.x >= e)
        return;
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x)
    {
        float4 p = pos[i];
        mn[0] = fminf(mn[0], p.x), mn[1] = fminf(mn[1], p.y), mn[2] = fminf(mn[2], p.z);
        mx[0] = fmaxf(mx[0], p.x), mx[1] = fmaxf(mx[1], p.y), mx[2] = fmaxf(mx[2], p.z);
    }
    block_bounds_commit(mn, mx, ord + 6 * seg);
}

// single-segment offsets {0, n} from a device count
__global__ void k_single_seg(const int32_t *d_n, int32_t *seg_off)
{
    seg_off[0] = 0;
    seg_off[1] = *d_n;
}

__global__ void k_transform(float4 *pos, float4 *nrm, const int32_t *d_n, Pose34f T)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *d_n)
        return;
    // ((R0 x + R1 y) + R2 z) + t, unfused, as transform_point_functor's mat3x3 * mat3x1
    // + mat3x1 (src/geometry/geometry_util.cuh:133-149)
    float4 p = pos[i];
    float x = p.x, y = p.y, z = p.z;
    p.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T.m[0], x), __fmul_rn(T.m[1], y)), __fmul_rn(T.m[2], z)), T.m[3]);
    p.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T.m[4], x), __fmul_rn(T.m[5], y)), __fmul_rn(T.m[6], z)), T.m[7]);
    p.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T.m[8], x), __fmul_rn(T.m[9], y)), __fmul_rn(T.m[10], z)), T.m[11]);
    pos[i] = p;
    if (nrm)
    {
        float4 n = nrm[i];
        float a = n.x, b = n.y, c = n.z;
        n.x = T.m[0] * a + T.m[1] * b + T.m[2] * c;
        n.y = T.m[4] * a + T.m[5] * b + T.m[6] * c;
        n.z = T.m[8] * a + T.m[9] * b + T.m[10] * c;
        nrm[i] = n;
    }
}

__global__ void k_copy_cloud(const float4 *ps, const float4 *cs, const float4 *ns, const float4 *gs,
                             const int32_t *d_nsrc, int32_t *d_ndst, int offset_from_dst, float4 *pd,
                             float4 *cd, float4 *nd, float4 *gd, int64_t cap)
{
    const int n = *d_nsrc;
    const int off = offset_from_dst ? *d_ndst : 0;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && off + i < cap)
    {
        pd[off + i] = ps[i];
        cd[off + i] = cs[i];
        if (nd)
            nd[off + i] = ns ? ns[i] : make_float4(0, 0, 0, 0);
        if (gd)
            gd[off + i] = gs ? gs[i] : make_float4(0, 0, 0, 0);
    }
}

__global__ void k_set_count_after_copy(const int32_t *d_nsrc, int32_t *d_ndst, int append, int64_t cap,
                                       int *d_err)
{
    int64_t total = (int64_t)*d_nsrc + (append ? *d_ndst : 0);
    if (total > cap)
    {
        atomicOr(d_err, kErrCapacity);
        total = cap;
    }
    *d_ndst = (int32_t)total;
}

// ---------------------------------------------------------------------------
// stage helpers used across files
// ---------------------------------------------------------------------------
int seg_bounds(gca3d_context *ctx, const float4 *pos, const int32_t *seg_off, int P, int64_t max_seg_cap,
               int *ord)
{
    k_init_bounds<<<grid_for(6 * P), kBlock, 0, ctx->stream>>>(ord, P);
    GCA_CHECK_LAUNCH(ctx);
    int gx = std::min(grid_for(max_seg_cap, kBlock * 4), ctx->num_sms * 4);
    dim3 grid(gx, P);
    k_bounds<<<grid, kBlock, 0, ctx->stream>>>(pos, seg_off, ord);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

int single_seg_offsets(gca3d_context *ctx, const int32_t *d_n, int32_t *seg_off)
{
    k_single_seg<<<1, 1, 0, ctx->stream>>>(d_n, seg_off);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

Pose34f pose_to_f32(const double T[16])
{
    Pose34f P;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c)
            P.m[4 * r + c] = (float)T[4 * r + c];
    return P;
}

} // namespace gca3d

using namespace gca3d;

// ---------------------------------------------------------------------------
// C ABI: context and clouds
// ---------------------------------------------------------------------------
extern "C" {

const char *gca3d_status_string(int s)
{
    switch (s)
    {
    case GCA3D_OK:
        return "ok";
    case GCA3D_ERR_INVALID_VALUE:
        return "invalid value";
    case GCA3D_ERR_OUT_OF_MEMORY:
        return "out of memory";
    case GCA3D_ERR_NO_CORRESPONDENCES:
        return "no correspondences";
    case GCA3D_ERR_SINGULAR:
        return "singular system";
    case GCA3D_ERR_TIMEOUT:
        return "device wait timed out";
    case GCA3D_ERR_CUDA:
        return "CUDA error";
    case GCA3D_ERR_CAPACITY:
        return "capacity exceeded";
    case GCA3D_ERR_NOT_SUPPORTED:
        return "not supported";
    default:
        return "unknown status";
    }
}

int gca3d_create(int device, void *stream, gca3d_context **out)
{
    if (!out)
        return GCA3D_ERR_INVALID_VALUE;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    {
        cudaGetLastError();
        return GCA3D_ERR_INVALID_VALUE;
    }
    auto *ctx = new gca3d_context();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess)
    {
        delete ctx;
        return GCA3D_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (stream)
        ctx->stream = (cudaStream_t)stream;
    else
    {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        {
            delete ctx;
            return GCA3D_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    if (cudaMalloc(&ctx->d_err, 2 * sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_pinned, 64 * sizeof(int)) != cudaSuccess)
    {
        gca3d_destroy(ctx);
        return GCA3D_ERR_OUT_OF_MEMORY;
    }
    ctx->h_pinned[0] = 0;
    ctx->h_pinned[1] = kWaitLimitDefault;
    cudaMemcpyAsync(ctx->d_err, ctx->h_pinned, 2 * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    *out = ctx;
    return GCA3D_OK;
}

int gca3d_destroy(gca3d_context *ctx)
{
    if (!ctx)
        return GCA3D_ERR_INVALID_VALUE;
    cudaSetDevice(ctx->device);
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    ctx->arena.release();
    for (auto e : ctx->prof.events)
        cudaEventDestroy(e);
    if (ctx->d_err)
        cudaFree(ctx->d_err);
    if (ctx->h_pinned)
        cudaFreeHost(ctx->h_pinned);
    if (ctx->own_stream)
        cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GCA3D_OK;
}

int gca3d_synchronize(gca3d_context *ctx)
{
    if (!ctx)
        return GCA3D_ERR_INVALID_VALUE;
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return consume_device_error(ctx, "synchronize");
}

int gca3d_set_wait_limit(gca3d_context *ctx, int polls)
{
    if (!ctx || polls < 1)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "set_wait_limit: polls must be >= 1");
    cudaSetDevice(ctx->device);
    ctx->h_pinned[63] = polls;
    GCA_CUDA(ctx, cudaMemcpyAsync(ctx->d_err + 1, ctx->h_pinned + 63, sizeof(int), cudaMemcpyHostToDevice,
                                  ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GCA3D_OK;
}

int gca3d_get_wait_limit(gca3d_context *ctx, int *polls)
{
    if (!ctx || !polls)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "get_wait_limit: bad arguments");
    cudaSetDevice(ctx->device);
    GCA_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned + 63, ctx->d_err + 1, sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *polls = ctx->h_pinned[63];
    return GCA3D_OK;
}

const char *gca3d_last_error(gca3d_context *ctx)
{
    static thread_local std::string s;
    s = ctx ? ctx->last_error : std::string("no context");
    return s.c_str();
}

int64_t gca3d_kernel_launches(gca3d_context *ctx) { return ctx ? ctx->launches : -1; }

void *gca3d_stream(gca3d_context *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int gca3d_profile_begin(gca3d_context *ctx, const char *kernel)
{
    if (!ctx || !kernel)
        return GCA3D_ERR_INVALID_VALUE;
    static const char *names[kKidCount] = {"icp_iter", "sort_pass", "normals", "voxel_reduce", "grid_scatter",
                                           "frame"};
    ctx->prof.target = kKidNone;
    for (int k = 0; k < kKidCount; ++k)
        if (std::string(kernel) == names[k])
            ctx->prof.target = k;
    ctx->prof.used = 0;
    return ctx->prof.target == kKidNone ? fail(ctx, GCA3D_ERR_INVALID_VALUE, "profile: unknown kernel") : GCA3D_OK;
}

int gca3d_profile_read(gca3d_context *ctx, double *total_ms, int64_t *launches)
{
    if (!ctx || !total_ms || !launches)
        return GCA3D_ERR_INVALID_VALUE;
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double t = 0.0;
    for (size_t i = 0; i + 1 < ctx->prof.used; i += 2)
    {
        float ms = 0.0f;
        GCA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->prof.events[i], ctx->prof.events[i + 1]));
        t += ms;
    }
    *total_ms = t;
    *launches = (int64_t)(ctx->prof.used / 2);
    ctx->prof.target = kKidNone;
    ctx->prof.used = 0;
    return GCA3D_OK;
}

int gca3d_device_alloc(gca3d_context *ctx, int64_t bytes, void **ptr)
{
    if (!ctx || !ptr || bytes < 0)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "device_alloc: bad arguments");
    *ptr = nullptr;
    GCA_CUDA(ctx, cudaMalloc(ptr, (size_t)std::max<int64_t>(bytes, 1)));
    return GCA3D_OK;
}

int gca3d_device_free(gca3d_context *ctx, void *ptr)
{
    if (!ctx)
        return GCA3D_ERR_INVALID_VALUE;
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    GCA_CUDA(ctx, cudaFree(ptr));
    return GCA3D_OK;
}

int gca3d_copy(gca3d_context *ctx, void *dst, const void *src, int64_t bytes)
{
    if (!ctx || (bytes > 0 && (!dst || !src)) || bytes < 0)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "copy: bad arguments");
    if (bytes > 0)
        GCA_CUDA(ctx, cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GCA3D_OK;
}

int gca3d_cloud_create(gca3d_context *ctx, int64_t capacity, gca3d_cloud **out)
{
    if (!ctx || !out || capacity < 0 || capacity >= (int64_t(1) << 30))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_create: capacity must be in [0, 2^30)");
    *out = nullptr;
    auto *c = new gca3d_cloud();
    c->capacity = capacity;
    c->device = ctx->device;
    size_t bytes = sizeof(float4) * (size_t)std::max<int64_t>(capacity, 1);
    if (cudaMalloc(&c->pos, bytes) != cudaSuccess || cudaMalloc(&c->col, bytes) != cudaSuccess ||
        cudaMalloc(&c->d_count, sizeof(int32_t)) != cudaSuccess)
    {
        cudaGetLastError();
        gca3d_cloud_destroy(c);
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "cloud_create: cudaMalloc");
    }
    GCA_CUDA(ctx, cudaMemsetAsync(c->d_count, 0, sizeof(int32_t), ctx->stream));
    *out = c;
    return GCA3D_OK;
}

int gca3d_cloud_destroy(gca3d_cloud *c)
{
    if (!c)
        return GCA3D_ERR_INVALID_VALUE;
    cudaFree(c->pos);
    cudaFree(c->col);
    cudaFree(c->nrm);
    cudaFree(c->grd);
    cudaFree(c->d_count);
    delete c;
    return GCA3D_OK;
}

// the device address of a buffer the context's device can read in place: pinned
// (page-locked, mapped) host memory or memory of that device; null for anything
// else -- pageable or managed host memory, another device's memory -- which is
// copied through a staging buffer instead
static const float *device_readable(const gca3d_context *ctx, const float *p, bool *pinned_host = nullptr)
{
    if (pinned_host)
        *pinned_host = false;
    if (!p)
        return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    if (pinned_host)
        *pinned_host = a.type == cudaMemoryTypeHost;
    if (a.type == cudaMemoryTypeHost || (a.type == cudaMemoryTypeDevice && a.device == ctx->device))
        return static_cast<const float *>(a.devicePointer);
    return nullptr;
}

int gca3d_set_upload_mode(gca3d_context *ctx, int mode)
{
    if (!ctx || (mode != GCA3D_UPLOAD_IN_PLACE && mode != GCA3D_UPLOAD_COPY_ENGINE))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "set_upload_mode: unknown mode");
    ctx->upload_mode = mode;
    return GCA3D_OK;
}

int gca3d_cloud_upload(gca3d_context *ctx, gca3d_cloud *c, const float *xyz, const float *rgb, int64_t n)
{
    if (!ctx || !c || (!xyz && n > 0) || n < 0 || n > c->capacity)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_upload: bad arguments or n > capacity");
    if (n > 0)
    {
        // pinned host buffers (and device ones) are read by the packing kernel in place:
        // one transfer, no staging copy
        const float *dx = device_readable(ctx, xyz), *dc = rgb ? device_readable(ctx, rgb) : nullptr;
        if (dx && (!rgb || dc))
        {
            k_pack<<<grid_for(n), kBlock, 0, ctx->stream>>>(dx, dc, (int)n, c->pos, c->col, c->d_count);
            GCA_CHECK_LAUNCH(ctx);
            c->has_normals = c->has_grad = false;
            return GCA3D_OK;
        }
    }
    ctx->arena.reset();
    float *sx = ctx->arena.get<float>(3 * std::max<int64_t>(n, 1));
    float *sc = rgb ? ctx->arena.get<float>(3 * std::max<int64_t>(n, 1)) : nullptr;
    if (!sx || (rgb && !sc))
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "cloud_upload: staging");
    if (n > 0)
    {
        GCA_CUDA(ctx, cudaMemcpyAsync(sx, xyz, sizeof(float) * 3 * n, cudaMemcpyDefault, ctx->stream));
        if (rgb)
            GCA_CUDA(ctx, cudaMemcpyAsync(sc, rgb, sizeof(float) * 3 * n, cudaMemcpyDefault, ctx->stream));
    }
    k_pack<<<grid_for(n), kBlock, 0, ctx->stream>>>(sx, sc, (int)n, c->pos, c->col, c->d_count);
    GCA_CHECK_LAUNCH(ctx);
    c->has_normals = c->has_grad = false;
    return GCA3D_OK;
}

int gca3d_cloud_upload_many(gca3d_context *ctx, int count, gca3d_cloud *const *clouds, const float *const *xyz,
                            const float *const *rgb, const int64_t *n)
{
    if (!ctx || count < 0 || (count > 0 && (!clouds || !xyz || !n)))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_upload_many: bad arguments");
    for (int k = 0; k < count; ++k)
        if (!clouds[k] || (!xyz[k] && n[k] > 0) || n[k] < 0 || n[k] > clouds[k]->capacity)
            return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_upload_many: bad arguments or n > capacity");
    UploadBatch B;
    B.count = 0;
    int blocks = 0;
    // copy-engine mode: pinned sources are first copied into the context scratch
    const bool staged_mode = ctx->upload_mode == GCA3D_UPLOAD_COPY_ENGINE;
    if (staged_mode)
        ctx->arena.reset();
    auto stage = [&](const float *src, int64_t m, const float **dst) -> int {
        float *s = ctx->arena.get<float>(3 * std::max<int64_t>(m, 1));
        if (!s)
            return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "cloud_upload_many: staging");
        GCA_CUDA(ctx, cudaMemcpyAsync(s, src, sizeof(float) * 3 * m, cudaMemcpyHostToDevice, ctx->stream));
        *dst = s;
        return GCA3D_OK;
    };
    auto flush = [&]() -> int {
        if (B.count == 0)
            return GCA3D_OK;
        k_pack_many<<<blocks, kBlock, 0, ctx->stream>>>(B);
        GCA_CHECK_LAUNCH(ctx);
        B.count = 0;
        blocks = 0;
        return GCA3D_OK;
    };
    for (int k = 0; k < count; ++k)
    {
        gca3d_cloud *c = clouds[k];
        const float *ck = rgb ? rgb[k] : nullptr;
        bool hx = false, hc = false;
        const float *dx = n[k] > 0 ? device_readable(ctx, xyz[k], &hx) : nullptr;
        const float *dc = ck ? device_readable(ctx, ck, &hc) : nullptr;
        int st = GCA3D_OK;
        if (staged_mode && dx && (!ck || dc))
        {
            if (hx)
                st = stage(xyz[k], n[k], &dx);
            if (!st && hc)
                st = stage(ck, n[k], &dc);
            if (st)
                return st;
        }
        // the writes land in call order: queued in-place entries are packed before a
        // staged upload, and before a second entry for a cloud already queued (two
        // entries of one launch would race on the same cloud)
        bool queued = false;
        for (int j = 0; j < B.count; ++j)
            queued = queued || B.d[j].pos == c->pos;
        if (n[k] > 0 && (!dx || (ck && !dc)))
        {
            st = flush();
            if (!st)
                st = gca3d_cloud_upload(ctx, c, xyz[k], ck, n[k]); // pageable: staged on its own
        }
        else
        {
            if (B.count == kUploadChunk || queued)
                st = flush();
            if (!st)
            {
                B.d[B.count++] = UploadDesc{dx, dc, c->pos, c->col, c->d_count, (int)n[k], blocks};
                blocks += std::max(grid_for(n[k]), 1);
                c->has_normals = c->has_grad = false;
            }
        }
        if (st)
            return st;
    }
    return flush();
}

int gca3d_cloud_set_normals(gca3d_context *ctx, gca3d_cloud *c, const float *nrm, int64_t n)
{
    if (!ctx || !c || !nrm || n < 0 || n > c->capacity)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_set_normals: bad arguments");
    int st = ensure_attr(ctx, c, true, false);
    if (st)
        return st;
    ctx->arena.reset();
    float *s = ctx->arena.get<float>(3 * std::max<int64_t>(n, 1));
    if (!s)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "cloud_set_normals: staging");
    if (n > 0)
        GCA_CUDA(ctx, cudaMemcpyAsync(s, nrm, sizeof(float) * 3 * n, cudaMemcpyDefault, ctx->stream));
    k_pack3<<<grid_for(n), kBlock, 0, ctx->stream>>>(s, (int)n, c->nrm);
    GCA_CHECK_LAUNCH(ctx);
    c->has_normals = true;
    c->has_grad = false;
    return GCA3D_OK;
}

int gca3d_cloud_set_gradients(gca3d_context *ctx, gca3d_cloud *c, const float *grd, int64_t n)
{
    if (!ctx || !c || !grd || n < 0 || n > c->capacity)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_set_gradients: bad arguments");
    if (!c->has_normals)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_set_gradients: the cloud has no normals");
    int st = ensure_attr(ctx, c, false, true);
    if (st)
        return st;
    ctx->arena.reset();
    float *s = ctx->arena.get<float>(3 * std::max<int64_t>(n, 1));
    if (!s)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "cloud_set_gradients: staging");
    if (n > 0)
        GCA_CUDA(ctx, cudaMemcpyAsync(s, grd, sizeof(float) * 3 * n, cudaMemcpyDefault, ctx->stream));
    k_pack3<<<grid_for(n), kBlock, 0, ctx->stream>>>(s, (int)n, c->grd);
    GCA_CHECK_LAUNCH(ctx);
    c->has_grad = true;
    return GCA3D_OK;
}

int gca3d_cloud_capacity(const gca3d_cloud *c, int64_t *cap)
{
    if (!c || !cap)
        return GCA3D_ERR_INVALID_VALUE;
    *cap = c->capacity;
    return GCA3D_OK;
}

int gca3d_cloud_size(gca3d_context *ctx, gca3d_cloud *c, int64_t *n)
{
    if (!ctx || !c || !n)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_size: bad arguments");
    GCA_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, c->d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *n = ctx->h_pinned[0];
    return GCA3D_OK;
}

int gca3d_cloud_has_normals(const gca3d_cloud *c, int *has)
{
    if (!c || !has)
        return GCA3D_ERR_INVALID_VALUE;
    *has = c->has_normals ? 1 : 0;
    return GCA3D_OK;
}

int gca3d_cloud_download(gca3d_context *ctx, gca3d_cloud *c, float *xyz, float *rgb, float *nrm, float *grd,
                         int64_t cap, int64_t *n_out)
{
    if (!ctx || !c)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_download: bad arguments");
    int64_t n = 0;
    int st = gca3d_cloud_size(ctx, c, &n);
    if (st)
        return st;
    if (n_out)
        *n_out = n;
    if (n > cap && (xyz || rgb || nrm || grd))
        return fail(ctx, GCA3D_ERR_CAPACITY, "cloud_download: destination too small");
    if ((nrm && !c->nrm) || (grd && !c->grd))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud_download: cloud has no normals / gradients");
    ctx->arena.reset();
    float *s = ctx->arena.get<float>(3 * std::max<int64_t>(n, 1));
    if (!s)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "cloud_download: staging");
    const float4 *src[4] = {c->pos, c->col, c->nrm, c->grd};
    float *dst[4] = {xyz, rgb, nrm, grd};
    for (int k = 0; k < 4; ++k)
    {
        if (!dst[k] || n == 0)
            continue;
        k_unpack<<<grid_for(n), kBlock, 0, ctx->stream>>>(src[k], c->d_count, s);
        GCA_CHECK_LAUNCH(ctx);
        GCA_CUDA(ctx, cudaMemcpyAsync(dst[k], s, sizeof(float) * 3 * n, cudaMemcpyDefault, ctx->stream));
    }
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GCA3D_OK;
}

int gca3d_cloud_device_views(gca3d_cloud *c, void **pos, void **col, void **nrm, void **grd, int32_t **d_count)
{
    if (!c)
        return GCA3D_ERR_INVALID_VALUE;
    if (pos)
        *pos = c->pos;
    if (col)
        *col = c->col;
    if (nrm)
        *nrm = c->nrm;
    if (grd)
        *grd = c->grd;
    if (d_count)
        *d_count = c->d_count;
    return GCA3D_OK;
}

static int copy_impl(gca3d_context *ctx, const gca3d_cloud *src, gca3d_cloud *dst, bool append)
{
    if (!ctx || !src || !dst || src == dst)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "cloud copy: bad arguments");
    bool normals = src->has_normals && (append ? dst->has_normals : true);
    if (normals)
    {
        int st = ensure_attr(ctx, dst, true, false);
        if (st)
            return st;
    }
    k_copy_cloud<<<grid_for(src->capacity), kBlock, 0, ctx->stream>>>(
        src->pos, src->col, normals ? src->nrm : nullptr, nullptr, src->d_count, dst->d_count, append ? 1 : 0,
        dst->pos, dst->col, normals ? dst->nrm : nullptr, nullptr, dst->capacity);
    GCA_CHECK_LAUNCH(ctx);
    k_set_count_after_copy<<<1, 1, 0, ctx->stream>>>(src->d_count, dst->d_count, append ? 1 : 0, dst->capacity,
                                                    ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    dst->has_normals = normals;
    dst->has_grad = false;
    return consume_device_error(ctx, append ? "cloud_append" : "cloud_copy");
}

int gca3d_cloud_copy(gca3d_context *ctx, const gca3d_cloud *src, gca3d_cloud *dst)
{
    return copy_impl(ctx, src, dst, false);
}

int gca3d_cloud_append(gca3d_context *ctx, gca3d_cloud *dst, const gca3d_cloud *src)
{
    return copy_impl(ctx, src, dst, true);
}

int gca3d_bounds(gca3d_context *ctx, gca3d_cloud *c, float mn[3], float mx[3])
{
    if (!ctx || !c || !mn || !mx)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "bounds: bad arguments");
    ctx->arena.reset();
    int32_t *off = ctx->arena.get<int32_t>(2);
    int *ord = ctx->arena.get<int>(6);
    if (!off || !ord)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "bounds: scratch");
    int st = single_seg_offsets(ctx, c->d_count, off);
    if (!st)
        st = seg_bounds(ctx, c->pos, off, 1, c->capacity, ord);
    if (st)
        return st;
    GCA_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, ord, 6 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int a = 0; a < 3; ++a)
    {
        mn[a] = ordered_to_float_host(ctx->h_pinned[a]);
        mx[a] = ordered_to_float_host(ctx->h_pinned[3 + a]);
    }
    return GCA3D_OK;
}

int gca3d_transform(gca3d_context *ctx, gca3d_cloud *c, const double T[16])
{
    if (!ctx || !c || !T)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "transform: bad arguments");
    Pose34f P = pose_to_f32(T);
    k_transform<<<grid_for(c->capacity), kBlock, 0, ctx->stream>>>(c->pos, c->has_normals ? c->nrm : nullptr,
                                                                   c->d_count, P);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

} // extern "C"
