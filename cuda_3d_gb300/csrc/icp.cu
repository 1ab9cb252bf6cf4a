// icp.cu -- colored ICP iteration (Park et al. 2017) for a batch of pairs.
//
// reference: color_icp::align (src/registration/color_icp.cu:151-234),
// compute_JTJ_JTr_and_r_gauss_newton_functor
// (src/registration/cuda_color_icp_build_least_square.cu:134-254) and
// solve_JTJ_JTr<true> (src/registration/eigen_solver.hpp:44-85).
//
// Three launches per Gauss-Newton iteration cover every pair (two with the fused
// finalize).  A block owns a chunk of one pair's source points.  k_icp_nn transforms
// them by the pair's current pose and finds the nearest target point inside max_corr
// (row-hashed grid, ties to the smaller index); it keeps few registers so many warps
// hide the latency of the neighbour walk, and it skips the walk for points whose
// certificate from an earlier search of the scale still decides the answer
// (grid_query.cuh).  k_icp_accum builds the geometric and photometric residuals and
// their 6-vector Jacobians in FP32 and accumulates the 21 + 6 + 1 system terms plus
// the correspondence count and squared distances.  Accumulation is compensated FP32
// inside the block (two-sum per thread and per shuffle level) and FP64 across warps
// and blocks.  k_icp_finalize (one block per pair) -- or, fused, the last accumulate
// block of the pair to finish (atomic ticket, no waiting) -- sums the pair's block
// partials in FP64 in block order, solves the 6x6 system by FP64 LDL^T, maps the step
// to SE(3) (Euler ZYX as the reference, or the exponential), composes the pose in
// FP64 and applies the reference's convergence test; a converged pair skips the
// remaining launches.  The source cloud is never rewritten: the pose is applied on
// the fly.
#include "grid_query.cuh"
#include "icp.cuh"
#include "pose_math.cuh"
#include "stages.cuh"

#include <algorithm>

namespace gca3d
{

// accumulator of kTerms values.  A thread sums its own few points (kIcpChunk /
// kIcpThreads = 4) in plain FP32; with Comp every combination above that -- the
// shuffle tree, the cross-warp sum -- is an error-free two-sum carrying an FP32
// error term, so the block sum is compensated where its error would grow.
template <bool Comp> struct Acc
{
    float s[kTerms];
    float e[kTerms];
    __device__ void zero()
    {
#pragma unroll
        for (int k = 0; k < kTerms; ++k)
            s[k] = 0.0f, e[k] = 0.0f;
    }
    __device__ __forceinline__ void add(int k, float x) { s[k] += x; }
    __device__ __forceinline__ void add_terms(const GNTerms &o, float d2)
    {
        int u = 0;
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int b = a; b < 6; ++b)
                add(u++, o.Jg[a] * o.Jg[b] + o.Jc[a] * o.Jc[b]);
#pragma unroll
        for (int a = 0; a < 6; ++a)
            add(21 + a, o.Jg[a] * o.rg + o.Jc[a] * o.rc);
        add(27, o.rg * o.rg + o.rc * o.rc);
        add(28, 1.0f);
        add(29, d2);
    }
    // warp reduce-scatter by recursive halving: at the level of offset o a lane keeps
    // half of its current terms (the upper half when its lane bit o is set) and adds
    // the partner's copy of that half (xor o), sending the other half; 16 + 8 + 4 + 2 +
    // 1 exchanges per value instead of 5 per term.  Lane t < kTerms ends with term t
    // (value vs, error ve; terms 30 and 31 are zero padding).  The thread sums are
    // plain, so the first level has no error terms to exchange.
    __device__ __forceinline__ void warp_reduce_scatter(float &vs, float &ve) const
    {
        const unsigned full = 0xffffffffu;
        const int lane = threadIdx.x & 31;
        auto add2 = [](float a, float b, float ea, float eb, float &t, float &et) {
            if (Comp)
            {
                t = a + b;
                const float bp = t - a;
                et = ea + eb + ((a - (t - bp)) + (b - bp));
            }
            else
            {
                t = a + b;
                et = 0.0f;
            }
        };
        float s16[16], e16[16];
        {
            const bool up = lane & 16;
#pragma unroll
            for (int k = 0; k < 16; ++k)
            {
                const float lo = s[k], hi = k + 16 < kTerms ? s[k + 16] : 0.0f;
                const float keep = up ? hi : lo, send = up ? lo : hi;
                add2(keep, __shfl_xor_sync(full, send, 16), 0.0f, 0.0f, s16[k], e16[k]);
            }
        }
        float s8[8], e8[8];
        {
            const bool up = lane & 8;
#pragma unroll
            for (int k = 0; k < 8; ++k)
            {
                const float keep = up ? s16[k + 8] : s16[k], send = up ? s16[k] : s16[k + 8];
                const float ekeep = up ? e16[k + 8] : e16[k], esend = up ? e16[k] : e16[k + 8];
                add2(keep, __shfl_xor_sync(full, send, 8), ekeep, Comp ? __shfl_xor_sync(full, esend, 8) : 0.0f,
                     s8[k], e8[k]);
            }
        }
        float s4[4], e4[4];
        {
            const bool up = lane & 4;
#pragma unroll
            for (int k = 0; k < 4; ++k)
            {
                const float keep = up ? s8[k + 4] : s8[k], send = up ? s8[k] : s8[k + 4];
                const float ekeep = up ? e8[k + 4] : e8[k], esend = up ? e8[k] : e8[k + 4];
                add2(keep, __shfl_xor_sync(full, send, 4), ekeep, Comp ? __shfl_xor_sync(full, esend, 4) : 0.0f,
                     s4[k], e4[k]);
            }
        }
        float s2[2], e2[2];
        {
            const bool up = lane & 2;
#pragma unroll
            for (int k = 0; k < 2; ++k)
            {
                const float keep = up ? s4[k + 2] : s4[k], send = up ? s4[k] : s4[k + 2];
                const float ekeep = up ? e4[k + 2] : e4[k], esend = up ? e4[k] : e4[k + 2];
                add2(keep, __shfl_xor_sync(full, send, 2), ekeep, Comp ? __shfl_xor_sync(full, esend, 2) : 0.0f,
                     s2[k], e2[k]);
            }
        }
        {
            const bool up = lane & 1;
            const float keep = up ? s2[1] : s2[0], send = up ? s2[0] : s2[1];
            const float ekeep = up ? e2[1] : e2[0], esend = up ? e2[0] : e2[1];
            add2(keep, __shfl_xor_sync(full, send, 1), ekeep, Comp ? __shfl_xor_sync(full, esend, 1) : 0.0f, vs,
                 ve);
        }
    }
    __device__ __forceinline__ double value(int k) const
    {
        return Comp ? (double)s[k] + (double)e[k] : (double)s[k];
    }
};

// sum of the block's kTerms values into part[kTerms].  Compensated: the per-warp
// (value, error) pairs are combined across warps by two-sum in FP32 and each of the
// 30 results is converted to FP64 once per block (FP64 issue is ~1/64 of FP32 on
// this part, so per-warp conversions would cost more than the sums).  Plain: FP32.
template <bool Comp>
__device__ __forceinline__ void block_reduce_store(Acc<Comp> &acc, double *part)
{
    __shared__ float s_s[kIcpThreads / 32][kTerms];
    __shared__ float s_e[kIcpThreads / 32][kTerms];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float vs, ve;
    acc.warp_reduce_scatter(vs, ve); // lane k holds term k
    if (lane < kTerms)
    {
        s_s[warp][lane] = vs;
        s_e[warp][lane] = ve;
    }
    __syncthreads();
    if (threadIdx.x < kTerms)
    {
        const int k = threadIdx.x;
        float v = s_s[0][k], e = Comp ? s_e[0][k] : 0.0f;
        for (int w = 1; w < kIcpThreads / 32; ++w)
        {
            const float x = s_s[w][k];
            if (Comp)
            {
                const float t = v + x;
                const float bp = t - v;
                e += s_e[w][k] + ((v - (t - bp)) + (x - bp));
                v = t;
            }
            else
                v += x;
        }
        part[k] = Comp ? (double)v + (double)e : (double)v;
    }
}

__device__ __forceinline__ int find_pair(const int *bmap, int P, int b)
{
    if (b >= bmap[P])
        return -1;
    int lo = 0, hi = P - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (bmap[mid] <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// exclusive prefix over the block's kIcpThreads threads of two per-thread counts: each
// thread gets its own prefixes back in a and b, and every thread the two totals
__device__ __forceinline__ void block_prefix2(int &a, int &b, int &ta, int &tb)
{
    __shared__ int s_a[kIcpThreads], s_b[kIcpThreads];
    __shared__ int s_ta, s_tb;
    s_a[threadIdx.x] = a;
    s_b[threadIdx.x] = b;
    __syncthreads();
    if (threadIdx.x < 32)
    {
        // 8 per lane, then across the warp
        constexpr int kPer = kIcpThreads / 32;
        const int l = threadIdx.x;
        int va[kPer], vb[kPer], sa = 0, sb = 0;
#pragma unroll
        for (int k = 0; k < kPer; ++k)
        {
            va[k] = s_a[l * kPer + k];
            vb[k] = s_b[l * kPer + k];
            sa += va[k];
            sb += vb[k];
        }
        int ia = sa, ib = sb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int ya = __shfl_up_sync(0xffffffffu, ia, o), yb = __shfl_up_sync(0xffffffffu, ib, o);
            if (l >= o)
                ia += ya, ib += yb;
        }
        int ra = ia - sa, rb = ib - sb;
#pragma unroll
        for (int k = 0; k < kPer; ++k)
        {
            s_a[l * kPer + k] = ra;
            s_b[l * kPer + k] = rb;
            ra += va[k];
            rb += vb[k];
        }
        if (l == 31)
        {
            s_ta = ra;
            s_tb = rb;
        }
    }
    __syncthreads();
    a = s_a[threadIdx.x];
    b = s_b[threadIdx.x];
    ta = s_ta;
    tb = s_tb;
}

// per-scale setup: block map, per-pair counts, reset of the per-scale flags; the
// pairs split over the block's threads, the maps by a block prefix
__global__ void __launch_bounds__(kIcpThreads) k_icp_setup(PairState *st, int P, const int32_t *src_off,
                                                           const int32_t *tgt_off, int *bmap, int *bmap_nn, int scale,
                                                           int nn_chunk)
{
    __shared__ int s_nact;
    if (threadIdx.x == 0)
        s_nact = 0;
    __syncthreads();
    const int chunk = kIcpChunk;
    const int per = (P + kIcpThreads - 1) / kIcpThreads;
    const int p0 = min(P, (int)threadIdx.x * per), p1 = min(P, p0 + per);
    int b = 0, bn = 0, na = 0;
    for (int p = p0; p < p1; ++p)
    {
        PairState &S = st[p];
        const int ns = src_off[p + 1] - src_off[p];
        const int nt = tgt_off[p + 1] - tgt_off[p];
        const int nb = (ns > 0 && nt > 0) ? (ns + chunk - 1) / chunk : 0;
        const int nbn = (ns > 0 && nt > 0) ? (ns + nn_chunk - 1) / nn_chunk : 0;
        b += nb;
        bn += nbn;
        na += nb > 0;
        S.nblocks = nb;
        S.nblocks_nn = nbn;
        S.nsrc = ns;
        S.ntgt = nt;
        S.ticket = 0;
        S.active = nb > 0 ? 1 : 0;
        S.converged = 0;
        if (scale == 0)
        {
            S.iters = 0;
            S.status = 0;
            for (int k = 0; k < GCA3D_MAX_SCALES; ++k)
                S.scale_iters[k] = S.scale_nsrc[k] = S.scale_ntgt[k] = 0;
        }
        S.scale = scale;
        S.nn_warm = 0;
        S.scale_nsrc[scale] = ns;
        S.scale_ntgt[scale] = nt;
        if (nb == 0)
        {
            S.status = GCA3D_ERR_NO_CORRESPONDENCES;
            S.rmse_ref = S.fitness = S.inlier_rmse = 0.0;
        }
    }
    if (na)
        atomicAdd(&s_nact, na);
    int tb, tbn;
    block_prefix2(b, bn, tb, tbn);
    for (int p = p0; p < p1; ++p)
    {
        bmap[p] = b;
        bmap_nn[p] = bn;
        b += st[p].nblocks;
        bn += st[p].nblocks_nn;
    }
    if (threadIdx.x == 0)
    {
        bmap[P] = tb;
        bmap[P + 1] = s_nact; // pairs the fused accumulate finalizes this iteration
        bmap_nn[P] = tbn;
        bmap_nn[P + 1] = 0; // the correspondence kernel's work queue
    }
}

__global__ void k_state_init(PairState *st, int P, const double *T_init)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P)
        return;
    for (int k = 0; k < 16; ++k)
        st[p].T[k] = T_init ? T_init[16 * p + k] : (k % 5 == 0 ? 1.0 : 0.0);
    st[p].iters = 0;
    st[p].status = 0;
    st[p].rmse_ref = st[p].fitness = st[p].inlier_rmse = 0.0;
}

// work item w -> (pair, chunk) of the pair's source points; the pair's pose as
// FP32 in shared memory.  Every thread of the block must call it (it synchronises).
// Blocks take items in a strided order, so blocks running at the same time work
// on neighbouring points and share their target rows in L2.
struct BlockPair
{
    int pair, start, end;
};

__device__ __forceinline__ BlockPair item_pair(int w, const int32_t *src_off, const PairState *st, const int *bmap,
                                               int P, int chunk, float *s_T, int *s_pair)
{
    __syncthreads(); // the previous item's readers of s_T / s_pair are done
    if (threadIdx.x == 0)
    {
        int p = find_pair(bmap, P, w);
        if (p >= 0 && !st[p].active)
            p = -1;
        *s_pair = p;
        if (p >= 0)
            for (int k = 0; k < 12; ++k)
                s_T[k] = (float)st[p].T[k];
    }
    __syncthreads();
    BlockPair b;
    b.pair = *s_pair;
    b.start = b.end = 0;
    if (b.pair >= 0)
    {
        b.start = src_off[b.pair] + (w - bmap[b.pair]) * chunk;
        b.end = min(b.start + chunk, src_off[b.pair + 1]);
    }
    return b;
}

// step 1 of an iteration: the correspondence of every active source point
// (grid position and squared distance, -1 when none within max_corr).
// Phase 1, one thread per point: from the second iteration of a scale on, a point
// whose certificate from its last search still holds (it has not moved far enough
// for another target point to overtake its nearest one, grid_query.cuh) takes its
// correspondence without a search.  Phase 2, four lanes per point over the block's
// list of the others: the search, shrunk to the cells that overlap the ball
// through the last nearest point when that one is within max_corr (the ball holds
// the nearest point and all its ties); it renews the point's certificate.
__global__ void __launch_bounds__(kIcpThreads, 5) k_icp_nn(const float4 *__restrict__ src_pos, const int32_t *src_off,
                                                        GridDev g, const PairState *st, const int *bmap, int P,
                                                        float max_corr, int2 *corr, NNCerts cert, int32_t *nn_out,
                                                        int nn_chunk, int *queue, const int *stop_iter, int stop_at)
{
    // a search queued behind the iteration that spent the scale's budget has nothing to do
    if (stop_iter && *stop_iter >= stop_at)
        return;
    __shared__ int s_pair, s_w;
    __shared__ float s_T[12];
    __shared__ int s_list[kNNChunkMax];
    __shared__ int4 s_box[kNNChunkMax]; // x0, y0, zlo, nx | ny << 8 | nz << 16 of the search box
    __shared__ float4 s_p[kNNChunkMax]; // the transformed point
    __shared__ int s_cnt;
    const KeyLayout L = *g.layout;
    const float rr = __fmul_rn(max_corr, max_corr);
    const int items = bmap[P];
    const int lane = threadIdx.x & 31;
    for (int first = 1;; first = 0)
    {
    // a block's first work item is its own index, the later ones come from the
    // iteration's queue: blocks that draw quick items (mostly certified points) take
    // more of them
    __syncthreads();
    if (threadIdx.x == 0)
        s_w = first ? (int)blockIdx.x : (int)gridDim.x + atomicAdd(queue, 1);
    __syncthreads();
    const int w = s_w;
    if (w >= items)
        break;
    const BlockPair b = item_pair(w, src_off, st, bmap, P, nn_chunk, s_T, &s_pair);
    if (b.pair < 0)
        continue;
    if (threadIdx.x == 0)
        s_cnt = 0;
    __syncthreads();
    const float3 o = g.gmin[b.pair];
    const int tbase = g.seg_off[b.pair];
    const bool warm = st[b.pair].nn_warm;
    for (int base = b.start; base < b.end; base += kIcpThreads)
    {
        const int i = base + (int)threadIdx.x;
        bool need = false;
        float3 p;
        CellBox B;
        if (i < b.end)
        {
            p = apply_pose(s_T, src_pos[i]);
            need = nn_full_box(g, L, o, p, B);
            if (!need)
            {
                // outside the grid's range: no candidates
                corr[i] = make_int2(-1, __float_as_int(rr));
                if (nn_out)
                    nn_out[i] = -1;
                cert.pos[i] = make_float4(p.x, p.y, p.z, 0.0f);
                cert.t[i] = -1;
            }
        }
        if (need && warm)
        {
            const int t1 = cert.t[i];
            int t;
            float d2;
            if (nn_certified(g, o, p, B, cert.pos[i], t1, rr, t, d2))
            {
                need = false;
                corr[i] = make_int2(t, __float_as_int(d2));
                if (nn_out)
                    nn_out[i] = t >= 0 ? __ldg(&g.sidx[t]) - tbase : -1;
            }
            else if (t1 >= 0)
            {
                // the ball through the last nearest point holds the nearest point and its ties
                const float4 q = __ldg(&g.spos[t1]);
                const float u2 = dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z);
                if (u2 < rr)
                    nn_shrink_box(g, o, p, sqrtf(u2), B);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, need);
        int at = 0;
        if (lane == 0 && m)
            at = atomicAdd(&s_cnt, __popc(m));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (need)
        {
            const int k = at + __popc(m & ((1u << lane) - 1u));
            s_list[k] = i;
            s_box[k] = make_int4(B.x0, B.y0, B.zlo, B.nx | (B.ny << 8) | ((B.zhi - B.zlo + 1) << 16));
            s_p[k] = make_float4(p.x, p.y, p.z, 0.0f);
        }
    }
    __syncthreads();
    const int n = s_cnt;
    // four lanes per listed point (uniform trip count for the whole block)
    for (int base = 0; base < n; base += kIcpThreads / kSub)
    {
        const int k = base + (int)(threadIdx.x / kSub);
        const bool valid = k < n;
        const int kk = valid ? k : 0;
        NNBest2 best;
        {
            const int4 bx = s_box[kk];
            const float4 p4 = s_p[kk];
            const CellBox B{bx.x, bx.w & 0xff, bx.y, (bx.w >> 8) & 0xff, bx.z, bx.z + (bx.w >> 16) - 1};
            best = nn_search_box2(g, L, b.pair, B, make_float3(p4.x, p4.y, p4.z), valid);
        }
        if (valid && (threadIdx.x & (kSub - 1)) == 0)
        {
            // the point, its box and the grid origin read again (volatile: not kept
            // live in registers through the search)
            const volatile int *vl = s_list;
            const volatile int *vb = reinterpret_cast<const volatile int *>(&s_box[kk]);
            const volatile float *vp = reinterpret_cast<const volatile float *>(&s_p[kk]);
            const int i = vl[kk];
            const int bw = vb[3];
            const CellBox B{vb[0], bw & 0xff, vb[1], (bw >> 8) & 0xff, vb[2], vb[2] + (bw >> 16) - 1};
            const float3 p = make_float3(vp[0], vp[1], vp[2]);
            const float3 og = g.gmin[b.pair];
            const bool hit = best.t >= 0 && best.d2 < rr;
            corr[i] = make_int2(hit ? best.t : -1, __float_as_int(hit ? best.d2 : rr));
            if (nn_out)
                nn_out[i] = hit ? __ldg(&g.sidx[best.t]) - tbase : -1;
            cert.pos[i] = make_float4(p.x, p.y, p.z, cert_bound(g, og, p, B, best.s2));
            cert.t[i] = best.t;
        }
    }
    }
}

// one pair's finalize, by one whole block: the pair's block partials summed in FP64
// in block order, the 6x6 solve, the step map, the FP64 pose update and the
// reference's convergence test (color_icp.cu:216-228).  The partials are read from
// L2: in the fused accumulate other blocks of the same launch wrote them.
template <bool Comp>
__device__ __forceinline__ void finalize_pair_body(PairState *st, int P, int pair, const int *bmap,
                                                   const double *partials, const IcpScale &prm)
{
    PairState &Ps = st[pair];
    __shared__ double s_red[kIcpThreads / 32][kTermsPad];
    const int nb = Ps.nblocks, bstart = bmap[pair];
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    if (lane < kTerms)
    {
        constexpr int kW = kIcpThreads / 32;
        const double *src = partials + (size_t)bstart * kTermsPad + lane;
        if (Comp)
        {
            // four running sums (blocks grp + 8 (4 q + r), r = 0..3), added in a fixed order
            double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
            int j = grp;
            for (; j + 3 * kW < nb; j += 4 * kW)
            {
                v0 += __ldcg(src + (size_t)j * kTermsPad);
                v1 += __ldcg(src + (size_t)(j + kW) * kTermsPad);
                v2 += __ldcg(src + (size_t)(j + 2 * kW) * kTermsPad);
                v3 += __ldcg(src + (size_t)(j + 3 * kW) * kTermsPad);
            }
            for (; j < nb; j += kW)
                v0 += __ldcg(src + (size_t)j * kTermsPad);
            s_red[grp][lane] = (v0 + v1) + (v2 + v3);
        }
        else
        {
            float vf = 0.0f;
            for (int j = grp; j < nb; j += kW)
                vf += (float)__ldcg(src + (size_t)j * kTermsPad);
            s_red[grp][lane] = (double)vf;
        }
    }
    __syncthreads();
    __shared__ double s_S[kTermsPad];
    if (threadIdx.x < kTerms)
    {
        const int k = threadIdx.x;
        double v = 0.0;
        float vf = 0.0f;
        for (int w = 0; w < kIcpThreads / 32; ++w)
        {
            if (Comp)
                v += s_red[w][k];
            else
                vf += (float)s_red[w][k];
        }
        s_S[k] = Comp ? v : (double)vf;
    }
    __syncthreads();
    const int warp = grp;
    if (warp == 0)
    {
        // solve, step map and composition over the lanes of warp 0
        double x[6];
        const int singular = solve6_warp(s_S, x);
        const double Ti = pose_from_x_warp(x, prm.update_map); // lanes 0..15: Ti[lane]
        const int r = (lane >> 2) & 3, c = lane & 3;
        const double Told = lane < 16 ? Ps.T[lane] : 0.0;
        double v = 0.0;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            v += __shfl_sync(0xffffffffu, Ti, 4 * r + k) * __shfl_sync(0xffffffffu, Told, 4 * k + c);
        const double t00 = __shfl_sync(0xffffffffu, Ti, 0), t11 = __shfl_sync(0xffffffffu, Ti, 5),
                     t22 = __shfl_sync(0xffffffffu, Ti, 10), t03 = __shfl_sync(0xffffffffu, Ti, 3),
                     t13 = __shfl_sync(0xffffffffu, Ti, 7), t23 = __shfl_sync(0xffffffffu, Ti, 11);
        const int iters = Ps.iters;
        if (prm.trace && iters < prm.trace_cap)
        {
            IcpTrace &tr = prm.trace[(size_t)iters * P + pair];
            if (lane < 16)
                tr.T[lane] = Told;
            if (lane < kTerms)
                tr.S[lane] = s_S[lane];
            if (lane == 0)
            {
#pragma unroll
                for (int q = 0; q < 6; ++q)
                    tr.x[q] = x[q];
                tr.status = singular;
            }
        }
        __syncwarp();
        if (lane < 16)
            Ps.T[lane] = v;
        if (lane == 0)
        {
            if (s_S[28] == 0.0)
                Ps.status = GCA3D_ERR_NO_CORRESPONDENCES;
            else if (singular && Ps.status == 0)
                Ps.status = GCA3D_ERR_SINGULAR;
            Ps.iters = iters + 1;
            Ps.scale_iters[Ps.scale] += 1;
            Ps.nn_warm = 1;
            const double cth = 0.5 * (t00 + t11 + t22 - 1.0);
            const double tsq = t03 * t03 + t13 * t13 + t23 * t23;
            if (cth >= 1.0 - prm.rot_eps && tsq <= prm.trans_eps)
            {
                Ps.converged = 1;
                Ps.active = 0;
            }
        }
    }
    else if (warp == 1)
    {
        // the statistics, on their own warp (one division per lane)
        const double ns = (double)Ps.nsrc;
        const int m = lane % 3;
        const double num = m == 0 ? s_S[27] : (m == 1 ? s_S[28] : s_S[29]);
        const double den = m == 2 ? s_S[28] : ns;
        double q = num / den;
        if (m == 2)
            q = s_S[28] > 0.0 ? sqrt(q) : 0.0;
        if (lane == 0)
            Ps.rmse_ref = q;
        else if (lane == 1)
            Ps.fitness = q;
        else if (lane == 2)
            Ps.inlier_rmse = q;
    }
}

// the work maps over the pairs still active (the next iteration's NN and accumulate
// launches get no items for converged pairs), their count and, in a captured
// schedule, the loop condition.  Run by one whole block once every pair of the
// iteration is finalized.
__device__ __forceinline__ void rebuild_maps_body(PairState *st, int P, int *bmap, int *bmap_nn, const IcpLoop &loop)
{
    __shared__ int s_nact;
    if (threadIdx.x == 0)
        s_nact = 0;
    __syncthreads();
    const int per = (P + kIcpThreads - 1) / kIcpThreads;
    const int p0 = min(P, (int)threadIdx.x * per), p1 = min(P, p0 + per);
    int a = 0, an = 0, na = 0;
    for (int q = p0; q < p1; ++q)
        if (__ldcg(&st[q].active))
        {
            a += st[q].nblocks;
            an += st[q].nblocks_nn;
            ++na;
        }
    if (na)
        atomicAdd(&s_nact, na);
    int ta, tn;
    block_prefix2(a, an, ta, tn);
    if (threadIdx.x == 0)
    {
        bmap[P] = ta;
        bmap[P + 1] = s_nact;
        bmap_nn[P] = tn;
        bmap_nn[P + 1] = 0;
        *loop.ticket = 0u;
        if (loop.iter)
        {
            const int it = ++(*loop.iter);
            cudaGraphSetConditional(loop.handle, (tn > 0 && it < loop.max_iter) ? 1u : 0u);
        }
    }
    for (int q = p0; q < p1; ++q)
    {
        bmap[q] = a;
        bmap_nn[q] = an;
        if (__ldcg(&st[q].active))
        {
            a += st[q].nblocks;
            an += st[q].nblocks_nn;
        }
    }
}

// the same two steps as calls, for the fused accumulate: compiled apart from the
// accumulation loop, whose registers they would otherwise crowd (the separate finalize
// kernel inlines the bodies)
template <bool Comp>
__device__ __noinline__ void finalize_pair(PairState *st, int P, int pair, const int *bmap, const double *partials,
                                           IcpScale prm)
{
    finalize_pair_body<Comp>(st, P, pair, bmap, partials, prm);
}

__device__ __noinline__ void rebuild_maps(PairState *st, int P, int *bmap, int *bmap_nn, IcpLoop loop)
{
    rebuild_maps_body(st, P, bmap, bmap_nn, loop);
}

// step 2: residuals, Jacobians, block sums (one partial per block); three resident
// blocks per SM (80 registers: the 30 sums and two points' gathers in flight).
// Fused: after storing its partial a block takes the pair's ticket, and the pair's
// last block runs the pair's finalize; the last pair to be finalized rebuilds the
// work maps.  A block that starts after that rebuild finds no item: within a scale
// the active set only shrinks, so the next item count is at most this one, and every
// block below this count has work left until the rebuild.
template <bool Comp, bool Fused>
__global__ void __launch_bounds__(kIcpThreads, 3) k_icp_accum(const float4 *__restrict__ src_pos, const int32_t *src_off,
                                                           const float4 *__restrict__ tpos,
                                                           const float4 *__restrict__ attr0,
                                                           const float4 *__restrict__ attr1,
                                                           const int2 *__restrict__ corr, PairState *st,
                                                           int *bmap, int *bmap_nn, int P, double *partials,
                                                           float slg, float slc, const int32_t *d_nt, int *err,
                                                           IcpScale prm, IcpLoop loop)
{
    __shared__ int s_pair;
    __shared__ float s_T[12];
    __shared__ int s_fin;
    const int items = bmap[P];
    const int nact = Fused ? bmap[P + 1] : 0;
    if (Fused && items == 0)
    {
        // no active pair: nothing to finalize, but the maps and the loop condition are set
        if (blockIdx.x == 0)
            rebuild_maps(st, P, bmap, bmap_nn, loop);
        return;
    }
    for (int w = blockIdx.x; w < items; w += gridDim.x)
    {
    const BlockPair b = item_pair(w, src_off, st, bmap, P, kIcpChunk, s_T, &s_pair);
    if (b.pair < 0)
        continue;
    Acc<Comp> acc;
    acc.zero();
    // a thread's points two at a time, all their loads issued before either is used
    // (the sums still run over the points in ascending order)
    constexpr int kPer = kIcpChunk / kIcpThreads;
#pragma unroll
    for (int j0 = 0; j0 < kPer; j0 += 2)
    {
        int2 c[2];
        float4 s4[2], q[2], a0[2], a1[2];
#pragma unroll
        for (int j = 0; j < 2; ++j)
        {
            const int i = b.start + (int)threadIdx.x + kIcpThreads * (j0 + j);
            c[j] = i < b.end ? corr[i] : make_int2(-1, 0);
            if (c[j].x >= 0 && !GCA_INDEX_OK(c[j].x, *d_nt, err))
                c[j].x = -1;
            if (c[j].x >= 0)
            {
                s4[j] = src_pos[i];
                q[j] = __ldg(&tpos[c[j].x]);
                a0[j] = __ldg(&attr0[c[j].x]);
                a1[j] = __ldg(&attr1[c[j].x]);
            }
        }
#pragma unroll
        for (int j = 0; j < 2; ++j)
        {
            if (c[j].x < 0)
                continue;
            const float3 p = apply_pose(s_T, s4[j]);
            GNTerms terms;
            gn_terms(p, s4[j].w, make_float3(q[j].x, q[j].y, q[j].z), a0[j].w, make_float3(a0[j].x, a0[j].y, a0[j].z),
                     make_float3(a1[j].x, a1[j].y, a1[j].z), slg, slc, terms);
            acc.add_terms(terms, __int_as_float(c[j].y));
        }
    }
    block_reduce_store<Comp>(acc, partials + (size_t)w * kTermsPad);
    if (Fused)
    {
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0)
            s_fin = atomicAdd(&st[b.pair].ticket, 1u) == (unsigned)(st[b.pair].nblocks - 1);
        __syncthreads();
        if (s_fin)
        {
            __threadfence();
            finalize_pair<Comp>(st, P, b.pair, bmap, partials, prm);
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0)
            {
                st[b.pair].ticket = 0u;
                s_fin = P == 1 || atomicAdd(loop.ticket, 1u) == (unsigned)(nact - 1);
            }
            __syncthreads();
            if (s_fin)
            {
                __threadfence();
                rebuild_maps(st, P, bmap, bmap_nn, loop);
            }
        }
    }
    }
}

// the finalize as a launch of its own (one block per pair); the last block to
// finish rebuilds the work maps
template <bool Comp>
__global__ void __launch_bounds__(kIcpThreads) k_icp_finalize(PairState *st, int P, int *bmap, int *bmap_nn,
                                                              const double *partials, IcpScale prm, IcpLoop loop)
{
    __shared__ int s_last;
    if (st[blockIdx.x].active)
        finalize_pair_body<Comp>(st, P, blockIdx.x, bmap, partials, prm);
    if (gridDim.x > 1)
    {
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0)
            s_last = atomicAdd(loop.ticket, 1u) == gridDim.x - 1;
    }
    else if (threadIdx.x == 0)
        s_last = 1; // one pair: this block is the last, and its own writes are visible after the barrier
    __syncthreads();
    if (!s_last)
        return;
    rebuild_maps_body(st, P, bmap, bmap_nn, loop);
}

IcpShape icp_shape(const gca3d_tuning &t)
{
    IcpShape s;
    if (t.nn_item_points == 64 || t.nn_item_points == 128 || t.nn_item_points == 256 || t.nn_item_points == 512)
        s.nn_chunk = t.nn_item_points;
    if (t.nn_blocks_per_sm > 0)
        s.nn_bps = std::min(t.nn_blocks_per_sm, 64);
    if (t.accum_blocks_per_sm > 0)
        s.acc_bps = std::min(t.accum_blocks_per_sm, 64);
    s.fused = t.fused_finalize != 0;
    return s;
}

int icp_setup(gca3d_context *ctx, PairState *st, int P, const int32_t *src_off, const int32_t *tgt_off, int *bmap,
              int *bmap_nn, int scale, int nn_chunk)
{
    k_icp_setup<<<1, kIcpThreads, 0, ctx->stream>>>(st, P, src_off, tgt_off, bmap, bmap_nn, scale, nn_chunk);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

int icp_state_init(gca3d_context *ctx, PairState *st, int P, const double *d_Tinit)
{
    k_state_init<<<grid_for(P, 128), 128, 0, ctx->stream>>>(st, P, d_Tinit);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

int icp_search(gca3d_context *ctx, const Batch &src, const Grid &g, PairState *st, int *bmap_nn, int max_blocks_nn,
               int2 *corr, const NNCerts &cert, const IcpScale &prm, int32_t *nn_out, const IcpLoop *guard,
               const IcpShape &shape)
{
    // work-item loop: enough blocks to fill the SMs a few times over, never more than
    // the items the capacity can produce
    const int grid_nn = std::max(std::min(max_blocks_nn, ctx->num_sms * shape.nn_bps), 1);
    GCA_PROF_BEGIN(ctx, kKidIcpIter);
    k_icp_nn<<<grid_nn, kIcpThreads, 0, ctx->stream>>>(src.pos, src.seg_off, g.dev, st, bmap_nn, src.P, prm.max_corr,
                                                       corr, cert, nn_out, shape.nn_chunk, bmap_nn + src.P + 1,
                                                       guard ? guard->iter : nullptr, guard ? guard->max_iter : 0);
    GCA_CHECK_LAUNCH(ctx);
    GCA_PROF_END(ctx, kKidIcpIter);
    return GCA3D_OK;
}

int icp_update(gca3d_context *ctx, const Batch &src, const Grid &g, const float4 *attr0, const float4 *attr1,
               PairState *st, int *bmap, int max_blocks, int *bmap_nn, double *partials, const int2 *corr,
               const IcpScale &prm, bool compensated, const IcpLoop &loop, const IcpShape &shape)
{
    if (!loop.ticket)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: iteration without a finalize ticket");
    const int grid_acc = std::max(std::min(max_blocks, ctx->num_sms * shape.acc_bps), 1);
    GCA_PROF_BEGIN(ctx, kKidIcpIter);
    const int32_t *d_nt = g.dev.d_n;
    if (shape.fused)
    {
        if (compensated)
            k_icp_accum<true, true><<<grid_acc, kIcpThreads, 0, ctx->stream>>>(
                src.pos, src.seg_off, g.dev.spos, attr0, attr1, corr, st, bmap, bmap_nn, src.P, partials,
                prm.sqrt_lg, prm.sqrt_lc, d_nt, ctx->d_err, prm, loop);
        else
            k_icp_accum<false, true><<<grid_acc, kIcpThreads, 0, ctx->stream>>>(
                src.pos, src.seg_off, g.dev.spos, attr0, attr1, corr, st, bmap, bmap_nn, src.P, partials,
                prm.sqrt_lg, prm.sqrt_lc, d_nt, ctx->d_err, prm, loop);
        GCA_CHECK_LAUNCH(ctx);
    }
    else
    {
        if (compensated)
            k_icp_accum<true, false><<<grid_acc, kIcpThreads, 0, ctx->stream>>>(
                src.pos, src.seg_off, g.dev.spos, attr0, attr1, corr, st, bmap, bmap_nn, src.P, partials,
                prm.sqrt_lg, prm.sqrt_lc, d_nt, ctx->d_err, prm, loop);
        else
            k_icp_accum<false, false><<<grid_acc, kIcpThreads, 0, ctx->stream>>>(
                src.pos, src.seg_off, g.dev.spos, attr0, attr1, corr, st, bmap, bmap_nn, src.P, partials,
                prm.sqrt_lg, prm.sqrt_lc, d_nt, ctx->d_err, prm, loop);
        GCA_CHECK_LAUNCH(ctx);
        if (compensated)
            k_icp_finalize<true><<<src.P, kIcpThreads, 0, ctx->stream>>>(st, src.P, bmap, bmap_nn, partials, prm,
                                                                         loop);
        else
            k_icp_finalize<false><<<src.P, kIcpThreads, 0, ctx->stream>>>(st, src.P, bmap, bmap_nn, partials, prm,
                                                                          loop);
        GCA_CHECK_LAUNCH(ctx);
    }
    GCA_PROF_END(ctx, kKidIcpIter);
    return GCA3D_OK;
}

int icp_iteration(gca3d_context *ctx, const Batch &src, const Grid &g, const float4 *attr0, const float4 *attr1,
                  PairState *st, int *bmap, int max_blocks, int *bmap_nn, int max_blocks_nn, double *partials,
                  int2 *corr, const NNCerts &cert, const IcpScale &prm, bool compensated, int32_t *nn_out,
                  const IcpLoop &loop, const IcpShape &shape)
{
    if (!loop.ticket)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "icp: iteration without a finalize ticket");
    int st_ = icp_search(ctx, src, g, st, bmap_nn, max_blocks_nn, corr, cert, prm, nn_out, nullptr, shape);
    if (!st_)
        st_ = icp_update(ctx, src, g, attr0, attr1, st, bmap, max_blocks, bmap_nn, partials, corr, prm, compensated,
                         loop, shape);
    return st_;
}

// ---------------------------------------------------------------------------
// system for given correspondences (cuda_build_gauss_newton_color_icp) and the
// per-point |r_g| + |r_c| (cuda_compute_abs_residual_color_icp)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kIcpThreads) k_build_gn(const float4 *__restrict__ sp, const int32_t *d_ns,
                                                          const float4 *__restrict__ tp, const float4 *__restrict__ tn,
                                                          const float4 *__restrict__ tg, const int32_t *nn,
                                                          float slg, float slc, double *partials,
                                                          unsigned *ticket, double *out, const int32_t *d_nt,
                                                          int *d_err)
{
    const int ns = *d_ns;
    const int nt = d_nt ? *d_nt : INT_MAX;
    Acc<true> acc;
    acc.zero();
    for (int i = blockIdx.x * kIcpThreads + threadIdx.x; i < ns; i += gridDim.x * kIcpThreads)
    {
        const int j = nn[i];
        if (j < 0)
            continue;
        if (j >= nt)
        {
            atomicOr(d_err, kErrInvalid);
            continue;
        }
        const float4 s4 = sp[i], q = tp[j], n = tn[j], d = tg[j];
        GNTerms t;
        gn_terms(make_float3(s4.x, s4.y, s4.z), s4.w, make_float3(q.x, q.y, q.z), q.w, make_float3(n.x, n.y, n.z),
                 make_float3(d.x, d.y, d.z), slg, slc, t);
        const float dx = q.x - s4.x, dy = q.y - s4.y, dz = q.z - s4.z;
        acc.add_terms(t, dx * dx + dy * dy + dz * dz);
    }
    block_reduce_store<true>(acc, partials + (size_t)blockIdx.x * kTermsPad);
    __threadfence();
    __syncthreads();
    __shared__ int s_last;
    if (threadIdx.x == 0)
        s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last)
        return;
    if (threadIdx.x < kTerms)
    {
        double v = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b)
            v += __ldcg(partials + (size_t)b * kTermsPad + threadIdx.x);
        out[threadIdx.x] = v;
    }
    if (threadIdx.x == 0)
        *ticket = 0;
}

__global__ void k_abs_residual(const float4 *__restrict__ sp, const int32_t *d_ns, const float4 *__restrict__ tp,
                               const float4 *__restrict__ tn, const float4 *__restrict__ tg, const int32_t *nn,
                               float slg, float slc, float *out, const int32_t *d_nt, int *d_err)
{
    const int ns = *d_ns;
    const int nt = *d_nt;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x)
    {
        const int j = nn[i];
        if (j < 0 || j >= nt)
        {
            if (j >= nt)
                atomicOr(d_err, kErrInvalid); // an index beyond the target
            out[i] = 0.0f;
            continue;
        }
        const float4 s4 = sp[i], q = tp[j], n = tn[j], d = tg[j];
        GNTerms t;
        gn_terms(make_float3(s4.x, s4.y, s4.z), s4.w, make_float3(q.x, q.y, q.z), q.w, make_float3(n.x, n.y, n.z),
                 make_float3(d.x, d.y, d.z), slg, slc, t);
        out[i] = fabsf(t.rg) + fabsf(t.rc);
    }
}

int build_gn(gca3d_context *ctx, const gca3d_cloud *src, const gca3d_cloud *tgt, const int32_t *nn, float lambda,
             double *out30)
{
    const int blocks = std::min(grid_for(src->capacity, kIcpThreads * 4), ctx->num_sms * 2);
    double *partials = ctx->arena.get<double>((size_t)blocks * kTermsPad);
    unsigned *ticket = ctx->arena.get<unsigned>(1);
    double *d_out = ctx->arena.get<double>(kTermsPad);
    if (!partials || !ticket || !d_out)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "build_gn: scratch");
    GCA_CUDA(ctx, cudaMemsetAsync(ticket, 0, sizeof(unsigned), ctx->stream));
    k_build_gn<<<blocks, kIcpThreads, 0, ctx->stream>>>(src->pos, src->d_count, tgt->pos, tgt->nrm, tgt->grd, nn,
                                                        sqrtf(lambda), sqrtf(1.0f - lambda), partials, ticket, d_out,
                                                        tgt->d_count, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    GCA_CUDA(ctx, cudaMemcpyAsync(out30, d_out, sizeof(double) * kTerms, cudaMemcpyDeviceToHost, ctx->stream));
    GCA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return consume_device_error(ctx, "build_gauss_newton: a correspondence index lies beyond the target");
}

int abs_residual(gca3d_context *ctx, const gca3d_cloud *src, const gca3d_cloud *tgt, const int32_t *nn, float lambda,
                 float *out)
{
    k_abs_residual<<<grid_for(src->capacity), kBlock, 0, ctx->stream>>>(
        src->pos, src->d_count, tgt->pos, tgt->nrm, tgt->grd, nn, sqrtf(lambda), sqrtf(1.0f - lambda), out,
        tgt->d_count, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    return consume_device_error(ctx, "abs_residual: a correspondence index lies beyond the target");
}

} // namespace gca3d
