// selfcheck.cu -- the short FP64 routines of the pose update (pose_math.cuh)
// against CUDA's IEEE division and sincos, on the device that runs them.
#include "pose_math.cuh"

#include <algorithm>

namespace gca3d
{

__device__ __forceinline__ void max_into(double *slot, double v)
{
    // non-negative doubles order as their bit patterns
    atomicMax(reinterpret_cast<unsigned long long *>(slot), (unsigned long long)__double_as_longlong(v));
}

__global__ void k_selfcheck_fp64(int n, double *out)
{
    constexpr double kEps = 2.220446049250313e-16;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const double f = (double)i / (double)n;
        const double d = exp2(-60.0 + 120.0 * f) * (1.0 + 0.37 * sin((double)i));
        const double q = 1.0 / d;
        max_into(&out[0], fabs(rcp_nr(d) - q) / (fabs(q) * kEps));
        const double x = -kSmallAngle + 2.0 * kSmallAngle * f;
        double s0, c0, s1, c1;
        sincos(x, &s0, &c0);
        sincos_small(x, s1, c1);
        if (s0 != 0.0)
            max_into(&out[1], fabs(s1 - s0) / (fabs(s0) * kEps));
        max_into(&out[2], fabs(c1 - c0) / (fabs(c0) * kEps));
        const double t = 0.05 + (kSmallAngle - 0.05) * f, t2 = t * t;
        double A, B, C;
        exp_coeffs_small(t2, A, B, C);
        double st, ct;
        sincos(t, &st, &ct);
        const double A0 = st / t, B0 = (1.0 - ct) / t2, C0 = (t - st) / (t2 * t);
        // the closed forms cancel: 1 - cos t and t - sin t keep about t^2 / 2 and t^2 / 6
        // of their operands, so their rounding error is within eps (4 + 8 / t^2)
        const double bound = kEps * (4.0 + 8.0 / t2);
        max_into(&out[3], fmax(fabs(A - A0) / A0, fmax(fabs(B - B0) / B0, fabs(C - C0) / C0)) / bound);
    }
}

} // namespace gca3d

using namespace gca3d;

extern "C" int gca3d_selfcheck_fp64(gca3d_context *ctx, int n, double out[4])
{
    if (!ctx || !out || n < 1)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "selfcheck: bad arguments");
    ctx->arena.reset();
    double *d_out = ctx->arena.get<double>(4);
    if (!d_out)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "selfcheck: scratch");
    GCA_CUDA(ctx, cudaMemsetAsync(d_out, 0, 4 * sizeof(double), ctx->stream));
    k_selfcheck_fp64<<<std::min((n + 255) / 256, ctx->num_sms * 8), 256, 0, ctx->stream>>>(n, d_out);
    GCA_CHECK_LAUNCH(ctx);
    GCA_CUDA(ctx, cudaMemcpyAsync(out, d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return consume_device_error(ctx, "selfcheck");
}
