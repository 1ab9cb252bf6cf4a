// vjp.cu -- K unrolled Gauss-Newton steps of the colored-ICP objective and their
// adjoint with respect to the initial pose, the source points and the source
// colours.  No reference counterpart; the per-point rows are those of
// compute_JTJ_JTr_and_r_gauss_newton_functor
// (src/registration/cuda_color_icp_build_least_square.cu:184-253) and the step is
// solve_JTJ_JTr (src/registration/eigen_solver.hpp:44-85) with the chosen map.
//
// Forward: the ICP kernels run K + 1 evaluations of one pair from T_0 = Exp(xi0)
// with the convergence test switched off; every evaluation keeps its
// correspondences in its own buffer, and the finalize of each records the pose it
// started from, the summed system and the step (IcpTrace).  Evaluation K only
// supplies T_K and the objective E = sum of weighted r_g^2 + r_c^2 at T_K.
//
// Backward, evaluation k from K down to 0, from nothing but the recorded poses and
// 6-vectors (the Jacobians are recomputed from the points, none is stored):
//   step adjoint (one thread, FP64): Ubar = Tbar_{k+1} T_k^T, xbar = dU/dx : Ubar,
//     y = H_k^-1 xbar, Tbar_k = U_k^T Tbar_{k+1}  (x = -H^-1 b gives
//     bbar = -y and Hbar = -y x^T);
//   point adjoint (FP32 per point): every row (j, r) of a correspondence gets
//     jbar = -y (j.x) - x (j.y) - r y  and  rbar = -(j.y) + 2 e r
//     (x = y = 0 and e = dE at evaluation K), pushed through j = w [p x dir; dir]
//     and r to pbar and to the source intensity; sbar = R_k^T pbar and
//     cbar = Ibar (0.2126, 0.7152, 0.0722); Tbar_k += sum over points of
//     pbar [s^T 1], compensated FP32 in the block and FP64 across blocks.
// Finally xi0bar = dExp(xi0)/dxi : Tbar_0.  Correspondences are held fixed: they
// are piecewise constant in the inputs.
#include "icp.cuh"
#include "pose_math.cuh"
#include "stages.cuh"

#include <cmath>
#include <vector>

using namespace gca3d;

namespace
{

constexpr int kVjpThreads = 256;
constexpr int kTb = 12; // entries of Tbar (rows 0-2 of the 4x4)
constexpr int kTbPad = 16;

struct Vec6
{
    double v[6];
};
struct Mat34
{
    double v[12];
};

__global__ void k_vjp_init(PairState *st, Vec6 xi0)
{
    if (threadIdx.x != 0)
        return;
    double T[16];
    pose_from_x_device(xi0.v, GCA3D_UPDATE_SE3_EXP, T);
    for (int k = 0; k < 16; ++k)
        st[0].T[k] = T[k];
}

__global__ void k_vjp_seed(Mat34 dT, double *Tbar)
{
    if (threadIdx.x < kTb)
        Tbar[threadIdx.x] = dT.v[threadIdx.x];
}

// adjoint of T_{k+1} = U(x_k) T_k and of x_k = -H_k^-1 b_k
__global__ void k_vjp_step(const IcpTrace *tr, int map, const double *Tbar_next, double *Tbar, double *y,
                           int *status)
{
    if (threadIdx.x != 0)
        return;
    double U[16], dU[6][12], Ub[12], S[27], yy[6];
    pose_from_x_device(tr->x, map, U);
    pose_jacobian_device(tr->x, map, dU);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 4; ++b)
        {
            double s = 0.0;
            for (int c = 0; c < 4; ++c)
                s += Tbar_next[4 * a + c] * tr->T[4 * b + c];
            Ub[4 * a + b] = s;
        }
    for (int m = 0; m < 6; ++m)
    {
        double s = 0.0;
        for (int k = 0; k < 12; ++k)
            s += Ub[k] * dU[m][k];
        S[21 + m] = -s; // solve6_device returns -H^-1 (rhs): y = H^-1 xbar
    }
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 4; ++c)
        {
            double s = 0.0;
            for (int b = 0; b < 3; ++b)
                s += U[4 * b + a] * Tbar_next[4 * b + c];
            Tbar[4 * a + c] = s;
        }
    for (int k = 0; k < 21; ++k)
        S[k] = tr->S[k];
    const int singular = solve6_device(S, yy);
    for (int m = 0; m < 6; ++m)
        y[m] = yy[m];
    if (singular || tr->status)
        *status = 1;
}

__device__ __forceinline__ void two_sum_add(float &s, float &e, float x)
{
    const float t = s + x;
    const float bp = t - s;
    e += (s - (t - bp)) + (x - bp);
    s = t;
}

// adjoint of one row j = w [p x dir; dir], r: adds to pbar, returns rbar
__device__ __forceinline__ float row_adjoint(const float J[6], float r, float3 dir, float w, const float *x,
                                             const float *y, float e, float3 &pb)
{
    float jx = 0.0f, jy = 0.0f;
#pragma unroll
    for (int a = 0; a < 6; ++a)
    {
        jx += J[a] * x[a];
        jy += J[a] * y[a];
    }
    const float bx = -y[0] * jx - x[0] * jy - r * y[0];
    const float by = -y[1] * jx - x[1] * jy - r * y[1];
    const float bz = -y[2] * jx - x[2] * jy - r * y[2];
    const float rb = -jy + 2.0f * e * r;
    // d<jbar, p x dir> = <dp, dir x jbar>
    pb.x += w * (dir.y * bz - dir.z * by) + rb * w * dir.x;
    pb.y += w * (dir.z * bx - dir.x * bz) + rb * w * dir.y;
    pb.z += w * (dir.x * by - dir.y * bx) + rb * w * dir.z;
    return rb;
}

__global__ void __launch_bounds__(kVjpThreads)
    k_vjp_points(const float4 *__restrict__ src_pos, const int32_t *d_ns, const float4 *__restrict__ tpos,
                 const float4 *__restrict__ attr0, const float4 *__restrict__ attr1, const int2 *__restrict__ corr,
                 const IcpTrace *tr, bool step, const double *y, float e, float slg, float slc, float *dxyz,
                 float *drgb, double *partials, unsigned *ticket, double *Tbar)
{
    __shared__ float s_T[12], s_x[6], s_y[6];
    __shared__ float s_s[kVjpThreads / 32][kTb], s_e[kVjpThreads / 32][kTb];
    __shared__ int s_last;
    if (threadIdx.x < 12)
        s_T[threadIdx.x] = (float)tr->T[threadIdx.x];
    if (threadIdx.x < 6)
    {
        s_x[threadIdx.x] = step ? (float)tr->x[threadIdx.x] : 0.0f;
        s_y[threadIdx.x] = step ? (float)y[threadIdx.x] : 0.0f;
    }
    __syncthreads();
    const int ns = *d_ns;
    float acc[kTb], err[kTb];
#pragma unroll
    for (int k = 0; k < kTb; ++k)
        acc[k] = err[k] = 0.0f;
    for (int i = blockIdx.x * kVjpThreads + threadIdx.x; i < ns; i += gridDim.x * kVjpThreads)
    {
        const int2 c = corr[i];
        if (c.x < 0)
            continue;
        const float4 s4 = src_pos[i];
        const float3 p = apply_pose(s_T, s4);
        const float4 q = __ldg(&tpos[c.x]);
        const float4 a0 = __ldg(&attr0[c.x]);
        const float4 a1 = __ldg(&attr1[c.x]);
        const float3 n = make_float3(a0.x, a0.y, a0.z), d = make_float3(a1.x, a1.y, a1.z);
        GNTerms t;
        gn_terms(p, s4.w, make_float3(q.x, q.y, q.z), a0.w, n, d, slg, slc, t);
        const float nd = n.x * d.x + n.y * d.y + n.z * d.z;
        const float3 dt = make_float3(d.x - nd * n.x, d.y - nd * n.y, d.z - nd * n.z);
        float3 pb = make_float3(0.0f, 0.0f, 0.0f);
        row_adjoint(t.Jg, t.rg, n, slg, s_x, s_y, e, pb);
        const float rbc = row_adjoint(t.Jc, t.rc, dt, slc, s_x, s_y, e, pb);
        const float Ib = -rbc * slc;
        // p = R s + t
        dxyz[3 * i + 0] += s_T[0] * pb.x + s_T[4] * pb.y + s_T[8] * pb.z;
        dxyz[3 * i + 1] += s_T[1] * pb.x + s_T[5] * pb.y + s_T[9] * pb.z;
        dxyz[3 * i + 2] += s_T[2] * pb.x + s_T[6] * pb.y + s_T[10] * pb.z;
        drgb[3 * i + 0] += Ib * 0.2126f;
        drgb[3 * i + 1] += Ib * 0.7152f;
        drgb[3 * i + 2] += Ib * 0.0722f;
        const float pv[3] = {pb.x, pb.y, pb.z}, sv[3] = {s4.x, s4.y, s4.z};
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
#pragma unroll
            for (int cc = 0; cc < 3; ++cc)
                two_sum_add(acc[4 * r + cc], err[4 * r + cc], pv[r] * sv[cc]);
            two_sum_add(acc[4 * r + 3], err[4 * r + 3], pv[r]);
        }
    }
    // warp, then cross-warp two-sum reduction; one FP64 value per term and block
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < kTb; ++k)
        {
            const float s2 = __shfl_down_sync(0xffffffffu, acc[k], o);
            const float e2 = __shfl_down_sync(0xffffffffu, err[k], o);
            err[k] += e2;
            two_sum_add(acc[k], err[k], s2);
        }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < kTb; ++k)
        {
            s_s[warp][k] = acc[k];
            s_e[warp][k] = err[k];
        }
    __syncthreads();
    if (threadIdx.x < kTb)
    {
        float v = s_s[0][threadIdx.x], ev = s_e[0][threadIdx.x];
        for (int w = 1; w < kVjpThreads / 32; ++w)
        {
            ev += s_e[w][threadIdx.x];
            two_sum_add(v, ev, s_s[w][threadIdx.x]);
        }
        partials[(size_t)blockIdx.x * kTbPad + threadIdx.x] = (double)v + (double)ev;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
        s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last)
        return;
    if (threadIdx.x < kTb)
    {
        double v = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b)
            v += __ldcg(partials + (size_t)b * kTbPad + threadIdx.x);
        Tbar[threadIdx.x] += v;
    }
    if (threadIdx.x == 0)
        *ticket = 0u;
}

__global__ void k_vjp_finish(Vec6 xi0, const double *Tbar0, double *dxi)
{
    if (threadIdx.x != 0)
        return;
    double dX[6][12];
    pose_jacobian_device(xi0.v, GCA3D_UPDATE_SE3_EXP, dX);
    for (int m = 0; m < 6; ++m)
    {
        double s = 0.0;
        for (int k = 0; k < 12; ++k)
            s += Tbar0[k] * dX[m][k];
        dxi[m] = s;
    }
}

} // namespace

extern "C" int gca3d_color_icp_vjp(gca3d_context *ctx, gca3d_cloud *src, gca3d_cloud *tgt,
                                   const gca3d_vjp_params *p, const double xi0[6], const double dT[16], double dE,
                                   double T_out[16], double *E_out, double dxi0[6], float *d_dxyz, float *d_drgb,
                                   int32_t *d_corr)
{
    if (!ctx || !src || !tgt || !p || !xi0)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp vjp: null argument");
    if (p->K < 1 || p->K > GCA3D_VJP_MAX_STEPS || !(p->max_corr > 0.0f) || !(p->lambda >= 0.0f && p->lambda <= 1.0f) ||
        (p->update_map != GCA3D_UPDATE_EULER_ZYX && p->update_map != GCA3D_UPDATE_SE3_EXP))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp vjp: bad parameters (1 <= K <= 64, max_corr > 0)");
    if (!tgt->has_normals || !tgt->has_grad)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp vjp: the target needs normals and colour gradients");
    if (dT && (!dxi0 || !d_dxyz || !d_drgb))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp vjp: gradient outputs missing");
    const int K = p->K;
    ctx->arena.reset();
    // the point counts (the caller gets host results, so one read-back is due anyway)
    GCA_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, src->d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx,
             cudaMemcpyAsync(ctx->h_pinned + 1, tgt->d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int64_t ns = ctx->h_pinned[0], nt = ctx->h_pinned[1];
    if (ns <= 0 || nt <= 0)
        return fail(ctx, GCA3D_ERR_NO_CORRESPONDENCES, "icp vjp: empty cloud");

    Batch bs, bt;
    int st;
    if ((st = cloud_batch(ctx, src, bs)) || (st = cloud_batch(ctx, tgt, bt)))
        return st;
    Grid g;
    if ((st = grid_build(ctx, bt, p->max_corr, kOriginPadF32, nullptr, g)))
        return st;
    const int max_blocks = std::max(div_up(src->capacity, kIcpChunk), 1);
    const int max_blocks_nn = std::max(div_up(src->capacity, kNNChunk), 1);
    float4 *attr0 = ctx->arena.get<float4>(g.cap);
    float4 *attr1 = ctx->arena.get<float4>(g.cap);
    PairState *pst = ctx->arena.get<PairState>(1);
    int *bmap = ctx->arena.get<int>(3);
    int *bmap_nn = ctx->arena.get<int>(3);
    double *partials = ctx->arena.get<double>((size_t)max_blocks * kTermsPad);
    int2 *corr = ctx->arena.get<int2>((size_t)(K + 1) * src->capacity);
    const NNCerts cert{ctx->arena.get<float4>(src->capacity), ctx->arena.get<int>(src->capacity)};
    IcpTrace *trace = ctx->arena.get<IcpTrace>(K + 1);
    unsigned *fticket = ctx->arena.get<unsigned>(1);
    if (!attr0 || !attr1 || !pst || !bmap || !bmap_nn || !partials || !corr || !cert.pos || !cert.t || !trace ||
        !fticket)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "icp vjp: scratch");
    if ((st = gather_attrs(ctx, bt, g, tgt->nrm, tgt->grd, attr0, attr1)))
        return st;

    // forward: K steps plus the evaluation at T_K
    Vec6 x0;
    for (int m = 0; m < 6; ++m)
        x0.v[m] = xi0[m];
    if ((st = icp_state_init(ctx, pst, 1, nullptr)))
        return st;
    k_vjp_init<<<1, 32, 0, ctx->stream>>>(pst, x0);
    GCA_CHECK_LAUNCH(ctx);
    const IcpShape shape;
    if ((st = icp_setup(ctx, pst, 1, bs.seg_off, bt.seg_off, bmap, bmap_nn, 0, shape.nn_chunk)))
        return st;
    IcpScale prm;
    prm.max_corr = p->max_corr;
    prm.sqrt_lg = sqrtf(p->lambda);
    prm.sqrt_lc = sqrtf(1.0f - p->lambda);
    prm.update_map = p->update_map;
    prm.rot_eps = -1.0; // never converged: exactly K steps
    prm.trans_eps = -1.0;
    prm.trace = trace;
    prm.trace_cap = K + 1;
    GCA_CUDA(ctx, cudaMemsetAsync(fticket, 0, sizeof(unsigned), ctx->stream));
    IcpLoop loop;
    loop.ticket = fticket;
    for (int k = 0; k <= K; ++k)
        if ((st = icp_iteration(ctx, bs, g, attr0, attr1, pst, bmap, max_blocks, bmap_nn, max_blocks_nn, partials,
                                corr + (size_t)k * src->capacity, cert, prm, true,
                                d_corr ? d_corr + (size_t)k * ns : nullptr, loop, shape)))
            return st;

    // backward
    int *d_status = nullptr;
    double *d_dxi = nullptr;
    if (dT)
    {
        const int nbv = std::max(std::min(div_up(ns, kVjpThreads), ctx->num_sms * 4), 1);
        double *Tbar = ctx->arena.get<double>((size_t)(K + 1) * kTb);
        double *ybuf = ctx->arena.get<double>((size_t)K * 6);
        double *vpart = ctx->arena.get<double>((size_t)nbv * kTbPad);
        unsigned *ticket = ctx->arena.get<unsigned>(1);
        d_status = ctx->arena.get<int>(1);
        d_dxi = ctx->arena.get<double>(6);
        if (!Tbar || !ybuf || !vpart || !ticket || !d_status || !d_dxi)
            return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "icp vjp: scratch");
        GCA_CUDA(ctx, cudaMemsetAsync(d_dxyz, 0, sizeof(float) * 3 * (size_t)ns, ctx->stream));
        GCA_CUDA(ctx, cudaMemsetAsync(d_drgb, 0, sizeof(float) * 3 * (size_t)ns, ctx->stream));
        GCA_CUDA(ctx, cudaMemsetAsync(ticket, 0, sizeof(unsigned), ctx->stream));
        GCA_CUDA(ctx, cudaMemsetAsync(d_status, 0, sizeof(int), ctx->stream));
        Mat34 seed;
        for (int k = 0; k < kTb; ++k)
            seed.v[k] = dT[k];
        k_vjp_seed<<<1, 32, 0, ctx->stream>>>(seed, Tbar + (size_t)K * kTb);
        GCA_CHECK_LAUNCH(ctx);
        const float slg = prm.sqrt_lg, slc = prm.sqrt_lc;
        k_vjp_points<<<nbv, kVjpThreads, 0, ctx->stream>>>(bs.pos, bs.seg_off + 1, g.dev.spos, attr0, attr1,
                                                            corr + (size_t)K * src->capacity, trace + K, false,
                                                            nullptr, (float)dE, slg, slc, d_dxyz, d_drgb, vpart,
                                                            ticket, Tbar + (size_t)K * kTb);
        GCA_CHECK_LAUNCH(ctx);
        for (int k = K - 1; k >= 0; --k)
        {
            k_vjp_step<<<1, 32, 0, ctx->stream>>>(trace + k, p->update_map, Tbar + (size_t)(k + 1) * kTb,
                                                  Tbar + (size_t)k * kTb, ybuf + 6 * k, d_status);
            GCA_CHECK_LAUNCH(ctx);
            k_vjp_points<<<nbv, kVjpThreads, 0, ctx->stream>>>(
                bs.pos, bs.seg_off + 1, g.dev.spos, attr0, attr1, corr + (size_t)k * src->capacity, trace + k,
                true, ybuf + 6 * k, 0.0f, slg, slc, d_dxyz, d_drgb, vpart, ticket, Tbar + (size_t)k * kTb);
            GCA_CHECK_LAUNCH(ctx);
        }
        k_vjp_finish<<<1, 32, 0, ctx->stream>>>(x0, Tbar, d_dxi);
        GCA_CHECK_LAUNCH(ctx);
    }

    std::vector<IcpTrace> h(K + 1);
    double h_dxi[6] = {0, 0, 0, 0, 0, 0};
    int h_status = 0;
    GCA_CUDA(ctx, cudaMemcpyAsync(h.data(), trace, sizeof(IcpTrace) * (K + 1), cudaMemcpyDeviceToHost, ctx->stream));
    if (dT)
    {
        GCA_CUDA(ctx, cudaMemcpyAsync(h_dxi, d_dxi, sizeof h_dxi, cudaMemcpyDeviceToHost, ctx->stream));
        GCA_CUDA(ctx, cudaMemcpyAsync(&h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    }
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if ((st = consume_device_error(ctx, "icp vjp")))
        return st;
    if (T_out)
        for (int k = 0; k < 16; ++k)
            T_out[k] = h[K].T[k];
    if (E_out)
        *E_out = h[K].S[27];
    if (dT)
        for (int m = 0; m < 6; ++m)
            dxi0[m] = h_dxi[m];
    for (int k = 0; k <= K; ++k)
        if (h[k].S[28] == 0.0)
            return fail(ctx, GCA3D_ERR_NO_CORRESPONDENCES, "icp vjp: an evaluation had no correspondences");
    bool singular = h_status != 0;
    for (int k = 0; k < K; ++k)
        singular |= h[k].status != 0;
    if (singular)
        return fail(ctx, GCA3D_ERR_SINGULAR, "icp vjp: a step's system was singular");
    return GCA3D_OK;
}
