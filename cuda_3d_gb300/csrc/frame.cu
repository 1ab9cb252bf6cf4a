// frame.cu -- depth filter + back-projection + colour fetch + compaction, one kernel.
//
// reference: __adaptive_bilateral_filter / __bilateral_filter / __gaussian*
// (src/geometry/cuda_point_cloud_factory.cu:19-129), __kernel_make_pointcloud_Z16_BGR8
// (:189-267), cuda_make_point_cloud (:269-313) and remove_invalid_points
// (src/geometry/geometry_util.cuh:124-130).
//
// The reference writes an organised W x H array of 28-byte points, synchronises the
// device and compacts with thrust::remove_if.  Here a block owns one image row:
// it stages the 2R+1 depth rows around it in shared memory, filters and
// back-projects its pixels, ranks the valid ones in raster order with block scans,
// takes the row's output offset from the rows above by a warp-wide decoupled look-back (bounded
// spin) and writes the compacted SoA points directly.  Same arithmetic order as the
// reference (unfused multiply/add); the filter weights use det_expf below instead
// of expf, so the CPU oracle reproduces every output bit.
#include "stages.cuh"

#include <algorithm>

namespace gca3d
{

constexpr int kFrameThreads = 256;
constexpr int kRangeTable = 1024; // tabulated depth differences of the fixed filter
constexpr unsigned long long kRowAgg = 1ull << 62, kRowInc = 2ull << 62, kRowFlag = 3ull << 62;


// exp(x) in FP32: Cody-Waite reduction x = k ln2 + r (ln2 split into a 16-bit head
// and a tail so k * head is exact), degree-7 Taylor polynomial in Horner form, and
// 2^k applied in two exact power-of-two multiplies.  Only IEEE-rounded multiply
// and add, so the CPU oracle evaluates the identical sequence and the filtered
// depths (hence the colour lookups, which sit on pixel boundaries) agree bit for
// bit.  Within 2 ulp of exp(x) including the subnormal range.
__device__ __forceinline__ float det_expf(float x)
{
    if (x != x)
        return x;
    if (x > 88.72283935546875f)
        return __int_as_float(0x7f800000);
    if (x < -103.972084045410156f)
        return 0.0f;
    const float kf = rintf(__fmul_rn(x, 1.44269502162933349609f));
    const float r = __fsub_rn(__fsub_rn(x, __fmul_rn(kf, 0.693145751953125f)), __fmul_rn(kf, 1.428606765330187045e-06f));
    float p = 1.0f / 5040.0f;
    p = __fadd_rn(__fmul_rn(p, r), 1.0f / 720.0f);
    p = __fadd_rn(__fmul_rn(p, r), 1.0f / 120.0f);
    p = __fadd_rn(__fmul_rn(p, r), 1.0f / 24.0f);
    p = __fadd_rn(__fmul_rn(p, r), 1.0f / 6.0f);
    p = __fadd_rn(__fmul_rn(p, r), 0.5f);
    p = __fadd_rn(__fmul_rn(p, r), 1.0f);
    p = __fadd_rn(__fmul_rn(p, r), 1.0f);
    const int k = (int)kf;
    const int k1 = k / 2, k2 = k - k / 2;
    return __fmul_rn(__fmul_rn(p, __int_as_float((k1 + 127) << 23)), __int_as_float((k2 + 127) << 23));
}

__device__ __forceinline__ float gauss(float x, float s)
{
    return det_expf(__fdiv_rn(-__fmul_rn(x, x), __fmul_rn(s, s)));
}
__device__ __forceinline__ float gauss_sq(float x2, float s)
{
    return det_expf(__fdiv_rn(-x2, __fmul_rn(s, s)));
}

__global__ void __launch_bounds__(kFrameThreads) k_frame(const uint16_t *__restrict__ depth,
                                                         const uint8_t *__restrict__ bgr, FrameParams P,
                                                         float4 *out_pos, float4 *out_col, int32_t *d_count,
                                                         unsigned *tile_ctr, unsigned long long *status, int *d_err)
{
    extern __shared__ uint16_t s_depth[]; // (2R + 1) rows x w
    __shared__ unsigned s_tile;
    __shared__ int s_wsum[kFrameThreads / 32];
    __shared__ long long s_base;
    // the fixed filter's weights depend only on the tap offset (spatial) and on the
    // integer depth difference (range): both tabulated once per block, the same
    // function values as evaluating them per tap
    __shared__ float s_wsp[(2 * kMaxFilterRadius + 1) * (2 * kMaxFilterRadius + 1)];
    __shared__ float s_wrange[kRangeTable];
    const int R = P.mode == GCA3D_FILTER_FIXED ? P.radius : (P.mode == GCA3D_FILTER_ADAPTIVE ? 5 : 0);
    if (threadIdx.x == 0)
        s_tile = atomicAdd(tile_ctr, 1u);
    if (P.mode == GCA3D_FILTER_FIXED)
    {
        const int n = 2 * R + 1;
        for (int i = threadIdx.x; i < n * n; i += kFrameThreads)
        {
            const int dy = i / n - R, dx = i % n - R;
            s_wsp[i] = gauss_sq((float)(dx * dx + dy * dy), P.sigma_space);
        }
        for (int d = threadIdx.x; d < kRangeTable; d += kFrameThreads)
            s_wrange[d] = gauss((float)d, P.sigma_depth);
    }
    __syncthreads();
    const int y = (int)s_tile;
    if (y >= P.h)
        return;
    const int w = P.w;
    for (int r = -R; r <= R; ++r)
    {
        const int yy = y + r;
        uint16_t *row = s_depth + (r + R) * w;
        for (int x = threadIdx.x; x < w; x += kFrameThreads)
            row[x] = (yy >= 0 && yy < P.h) ? depth[(int64_t)yy * w + x] : (uint16_t)0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    long long row_count = 0;
    // pass over the row in chunks of kFrameThreads pixels, raster order = chunk-major
    const int nchunks = (w + kFrameThreads - 1) / kFrameThreads;
    float4 pp[kMaxFrameWidth / kFrameThreads], pc[kMaxFrameWidth / kFrameThreads];
    int valid[kMaxFrameWidth / kFrameThreads];
#pragma unroll
    for (int c = 0; c < kMaxFrameWidth / kFrameThreads; ++c)
    {
        valid[c] = 0;
        if (c >= nchunks)
            continue;
        const int x = c * kFrameThreads + threadIdx.x;
        if (x >= w)
            continue;
        const uint16_t d0 = s_depth[R * w + x];
        float fd = (float)d0;
        if (P.mode != GCA3D_FILTER_NONE)
        {
            const float dv = __fmul_rn((float)d0, P.depth_scale);
            if (!(dv < P.tmin || dv > P.tmax))
            {
                int rad;
                float ss, sd;
                if (P.mode == GCA3D_FILTER_FIXED)
                    rad = P.radius, ss = P.sigma_space, sd = P.sigma_depth;
                else
                {
                    unsigned step = (unsigned)__fdiv_rn(__fsub_rn(dv, P.tmin), 0.5f);
                    if (step > 5u)
                        step = 5u;
                    ss = __fadd_rn(8.0f, __fmul_rn((float)step, 1.0f));
                    sd = __fadd_rn(100.0f, __fmul_rn((float)step, 10.0f));
                    rad = (int)__fmul_rn(1.0f, (float)step);
                }
                float sw = 0.0f, sum = 0.0f;
                for (int dy = -rad; dy <= rad; ++dy)
                {
                    const uint16_t *row = s_depth + (R + dy) * w;
                    for (int dx = -rad; dx <= rad; ++dx)
                    {
                        const int nx = x + dx;
                        if (nx < 0 || nx >= w || y + dy < 0 || y + dy >= P.h)
                            continue;
                        const uint16_t nb = row[nx];
                        if (!nb)
                            continue;
                        const int diff = abs((int)d0 - (int)nb);
                        float wgt;
                        if (P.mode == GCA3D_FILTER_FIXED)
                            wgt = __fmul_rn(s_wsp[(dy + R) * (2 * R + 1) + dx + R],
                                            diff < kRangeTable ? s_wrange[diff] : gauss((float)diff, sd));
                        else
                            wgt = __fmul_rn(gauss_sq((float)(dx * dx + dy * dy), ss), gauss((float)diff, sd));
                        sw = __fadd_rn(sw, wgt);
                        sum = __fadd_rn(sum, __fmul_rn(wgt, (float)nb));
                    }
                }
                fd = __fdiv_rn(sum, sw);
            }
        }
        const float z = __fmul_rn(fd, P.depth_scale);
        if (z < P.tmin || z > P.tmax)
            continue;
        const float u = __fsub_rn((float)x, 0.5f), v = __fsub_rn((float)y, 0.5f);
        const float X = __fdiv_rn(__fmul_rn(__fsub_rn(u, P.cx), z), P.fx);
        const float Y = __fdiv_rn(__fmul_rn(__fsub_rn(v, P.cy), z), P.fy);
        const float cxp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(P.R[0], X), __fmul_rn(P.R[3], Y)), __fmul_rn(P.R[6], z)), P.t[0]);
        const float cyp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(P.R[1], X), __fmul_rn(P.R[4], Y)), __fmul_rn(P.R[7], z)), P.t[1]);
        const float czp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(P.R[2], X), __fmul_rn(P.R[5], Y)), __fmul_rn(P.R[8], z)), P.t[2]);
        const float cu = __fadd_rn(__fdiv_rn(__fmul_rn(cxp, P.cfx), czp), P.ccx);
        const float cv = __fadd_rn(__fdiv_rn(__fmul_rn(cyp, P.cfy), czp), P.ccy);
        const int tx = __float2int_rz(__fadd_rn(cu, 0.5f)), ty = __float2int_rz(__fadd_rn(cv, 0.5f));
        if (tx < 0 || tx >= w || ty < 0 || ty >= P.h)
            continue;
        const int64_t ci = 3 * ((int64_t)ty * w + tx);
        const float sc = 1.0f / 255.0f;
        const float r = __fmul_rn((float)bgr[ci + 2], sc), g = __fmul_rn((float)bgr[ci + 1], sc),
                    b = __fmul_rn((float)bgr[ci + 0], sc);
        pp[c] = make_float4(X, Y, z, intensity_of(r, g, b));
        pc[c] = make_float4(r, g, b, 0.0f);
        valid[c] = 1;
    }
    // ranks in raster order: per chunk a block scan of the valid flags
    int rank[kMaxFrameWidth / kFrameThreads];
#pragma unroll
    for (int c = 0; c < kMaxFrameWidth / kFrameThreads; ++c)
    {
        if (c >= nchunks)
            break;
        const unsigned bal = __ballot_sync(0xffffffffu, valid[c]);
        if (lane == 0)
            s_wsum[warp] = __popc(bal);
        __syncthreads();
        int before = 0, total = 0;
        for (int k = 0; k < kFrameThreads / 32; ++k)
        {
            if (k < warp)
                before += s_wsum[k];
            total += s_wsum[k];
        }
        rank[c] = (int)row_count + before + __popc(bal & ((1u << lane) - 1u));
        row_count += total;
        __syncthreads();
    }
    // decoupled look-back over rows, one warp: the 32 nearest predecessors' states are
    // read at once (each wait bounded), the nearest inclusive prefix is found by ballot
    // and the aggregates up to it are summed by the warp; only a window without an
    // inclusive state moves the look-back 32 rows further up
    if (warp == 0)
    {
        unsigned long long *st = status + y;
        long long excl = 0;
        if (lane == 0)
        {
            const unsigned long long v = (y == 0 ? kRowInc : kRowAgg) | (unsigned long long)row_count;
            asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(st), "l"(v) : "memory");
        }
        if (y > 0)
        {
            for (int top = y - 1;; top -= 32)
            {
                const int p = top - lane;
                unsigned long long s = kRowInc; // above row 0: an inclusive zero
                if (p >= 0)
                {
                    const uint32_t limit = wait_limit(d_err);
                    unsigned spins = 0;
                    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(s) : "l"(status + p) : "memory");
                    while ((s & kRowFlag) == 0)
                    {
                        if (++spins > limit)
                        {
                            atomicOr(d_err, kErrTimeout);
                            break; // a state that never came counts as the end of the look-back
                        }
                        if (spins > 64)
                            __nanosleep(64);
                        asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(s) : "l"(status + p) : "memory");
                    }
                }
                const unsigned inc = __ballot_sync(0xffffffffu, (s & kRowFlag) != kRowAgg);
                const int stop = inc ? __ffs(inc) - 1 : 31;
                long long v = lane <= stop ? (long long)(s & ~kRowFlag) : 0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    v += __shfl_xor_sync(0xffffffffu, v, o);
                excl += v;
                if (inc)
                    break;
            }
            if (lane == 0)
                asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(st),
                             "l"(kRowInc | (unsigned long long)(excl + row_count))
                             : "memory");
        }
        if (lane == 0)
        {
            s_base = excl;
            if (y == P.h - 1)
                *d_count = (int32_t)(excl + row_count);
        }
    }
    __syncthreads();
    const long long base = s_base;
#pragma unroll
    for (int c = 0; c < kMaxFrameWidth / kFrameThreads; ++c)
    {
        if (c >= nchunks)
            break;
        if (valid[c])
        {
            out_pos[base + rank[c]] = pp[c];
            out_col[base + rank[c]] = pc[c];
        }
    }
}

int frame_to_cloud(gca3d_context *ctx, const uint16_t *depth, const uint8_t *bgr, const FrameParams &P,
                   gca3d_cloud *out)
{
    unsigned *tile_ctr = ctx->arena.get<unsigned>(1);
    unsigned long long *status = ctx->arena.get<unsigned long long>(P.h);
    if (!tile_ctr || !status)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "frame_to_cloud: scratch");
    GCA_CUDA(ctx, cudaMemsetAsync(tile_ctr, 0, sizeof(unsigned), ctx->stream));
    GCA_CUDA(ctx, cudaMemsetAsync(status, 0, sizeof(unsigned long long) * P.h, ctx->stream));
    const int R = P.mode == GCA3D_FILTER_FIXED ? P.radius : (P.mode == GCA3D_FILTER_ADAPTIVE ? 5 : 0);
    const size_t smem = (size_t)(2 * R + 1) * P.w * sizeof(uint16_t);
    GCA_PROF_BEGIN(ctx, kKidFrame);
    k_frame<<<P.h, kFrameThreads, smem, ctx->stream>>>(depth, bgr, P, out->pos, out->col, out->d_count, tile_ctr,
                                                       status, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    GCA_PROF_END(ctx, kKidFrame);
    return GCA3D_OK;
}

} // namespace gca3d

using namespace gca3d;

namespace gca3d
{
// cuda_make_point_cloud (cuda_point_cloud_factory.cu:283-290): parameters present,
// depth_scale > 0; plus this kernel's limits (width, filter radius)
int frame_params(gca3d_context *ctx, int w, int h, const gca3d_intrinsics *di, const gca3d_intrinsics *ci,
                 const gca3d_extrinsics *d2c, float depth_scale, float tmin, float tmax, const gca3d_filter *filter,
                 FrameParams &P)
{
    if (!di || w <= 0 || h <= 0)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "frame_to_cloud: bad arguments");
    if (!(depth_scale > 0.0f))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "frame_to_cloud: depth_scale must be > 0");
    if (w > kMaxFrameWidth)
        return fail(ctx, GCA3D_ERR_NOT_SUPPORTED, "frame_to_cloud: width above 2048");
    P = FrameParams{};
    P.w = w, P.h = h;
    P.fx = di->fx, P.fy = di->fy, P.cx = di->cx, P.cy = di->cy;
    const gca3d_intrinsics *c = ci ? ci : di;
    P.cfx = c->fx, P.cfy = c->fy, P.ccx = c->cx, P.ccy = c->cy;
    for (int k = 0; k < 9; ++k)
        P.R[k] = d2c ? d2c->rotation[k] : (k % 4 == 0 ? 1.0f : 0.0f);
    for (int k = 0; k < 3; ++k)
        P.t[k] = d2c ? d2c->translation[k] : 0.0f;
    P.depth_scale = depth_scale, P.tmin = tmin, P.tmax = tmax;
    P.mode = filter ? filter->mode : GCA3D_FILTER_ADAPTIVE;
    P.radius = filter ? filter->radius : 0;
    P.sigma_space = filter ? filter->sigma_space : 0.0f;
    P.sigma_depth = filter ? filter->sigma_depth : 0.0f;
    if (P.mode < 0 || P.mode > 2 || (P.mode == GCA3D_FILTER_FIXED &&
                                     (P.radius < 0 || P.radius > kMaxFilterRadius || !(P.sigma_space > 0) ||
                                      !(P.sigma_depth > 0))))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "frame_to_cloud: bad filter parameters");
    return GCA3D_OK;
}
} // namespace gca3d

extern "C" int gca3d_frame_to_cloud(gca3d_context *ctx, const uint16_t *depth, const uint8_t *bgr, int w, int h,
                                    const gca3d_intrinsics *di, const gca3d_intrinsics *ci,
                                    const gca3d_extrinsics *d2c, float depth_scale, float tmin, float tmax,
                                    const gca3d_filter *filter, gca3d_cloud *out)
{
    if (!ctx || !depth || !bgr || !out)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "frame_to_cloud: bad arguments");
    FrameParams P;
    int st = frame_params(ctx, w, h, di, ci, d2c, depth_scale, tmin, tmax, filter, P);
    if (st)
        return st;
    if ((int64_t)w * h > out->capacity)
        return fail(ctx, GCA3D_ERR_CAPACITY, "frame_to_cloud: output capacity below w * h");
    ctx->arena.reset();
    if ((st = frame_to_cloud(ctx, depth, bgr, P, out)))
        return st;
    out->has_normals = out->has_grad = false;
    return GCA3D_OK;
}
