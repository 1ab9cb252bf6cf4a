// grid.cu -- uniform grid over a batch of point sets and its queries.
//
// reference: the grid build in src/geometry/cuda_nn_search.cu:573-608 (cell id, radix
// sort, reduce_by_key, dense cell table rebuilt per call), nn_search_functor
// (:113-214) and the radius-list passes (:216-414, 622-723).
//
// GB300 layout: points are physically reordered into cell order (float4 with the z
// cell in .w), so a query streams contiguous memory.  Instead of a dense
// nx*ny*nz table the grid keeps a hash of the occupied (segment, x, y) rows ->
// [start, end) in the sorted arrays; a 27-cell neighbourhood is 9 row lookups and
// 9 contiguous scans over z.  Cells, rows and the scan order (x, then y, then z,
// then ascending original index) are the reference's, so radius lists come out in
// the reference's order for the same grid origin.  Memory is O(points), not
// O(bounding-box volume).
#include "grid_query.cuh"
#include "stages.cuh"

#include <algorithm>

namespace gca3d
{

__global__ void k_grid_layout(const int *ord, int P, float cell, int mode, float3 given, float3 *origin,
                              KeyLayout *lay, int *d_err)
{
    __shared__ uint32_t s_max[3];
    if (threadIdx.x < 3)
        s_max[threadIdx.x] = 1;
    __syncthreads();
    for (int s = threadIdx.x; s < P; s += blockDim.x)
    {
        float mn[3], mx[3], o[3];
        for (int a = 0; a < 3; ++a)
        {
            mn[a] = ordered_to_float(ord[6 * s + a]);
            mx[a] = ordered_to_float(ord[6 * s + 3 + a]);
        }
        const float g[3] = {given.x, given.y, given.z};
        for (int a = 0; a < 3; ++a)
        {
            if (mode == kOriginGiven)
                o[a] = g[a];
            else if (mode == kOriginPadF64)
                o[a] = (float)__dsub_rn((double)mn[a], __dmul_rn(1.5, (double)cell));
            else
                o[a] = __fsub_rn(mn[a], __fmul_rn(1.5f, cell));
        }
        origin[s] = make_float3(o[0], o[1], o[2]);
        if (!(mx[0] >= mn[0]))
            continue; // empty segment
        for (int a = 0; a < 3; ++a)
        {
            int lo = cell_of(mn[a], o[a], cell);
            int hi = cell_of(mx[a], o[a], cell);
            if (lo < 0 || hi >= (1 << 21))
            {
                atomicOr(d_err, kErrKeyBits);
                hi = (1 << 21) - 1;
            }
            atomicMax(&s_max[a], (uint32_t)max(hi, 1));
        }
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        KeyLayout L;
        L.bseg = bitlen_u32((uint32_t)(P - 1));
        L.bx = bitlen_u32(s_max[0]);
        L.by = bitlen_u32(s_max[1]);
        L.bz = bitlen_u32(s_max[2]);
        L.total_bits = L.bseg + L.bx + L.by + L.bz;
        L.morton = 0;
        if (L.total_bits > 64)
            atomicOr(d_err, kErrKeyBits);
        *lay = L;
    }
}

__global__ void k_grid_keys(const float4 *__restrict__ pos, const int32_t *seg_off, const float3 *origin,
                            const KeyLayout *lay, float cell, uint64_t *keys, int32_t *vals, int ib_cap, int *d_ib,
                            int *d_kshift)
{
    const int seg = blockIdx.y;
    const int b = seg_off[seg], e = seg_off[seg + 1];
    const KeyLayout L = *lay;
    const int ib = packed_index_bits(L.total_bits, ib_cap);
    if (seg == 0 && blockIdx.x == 0 && threadIdx.x == 0)
        *d_ib = *d_kshift = ib;
    const float3 o = origin[seg];
    const uint64_t mask_x = (1ull << L.bx) - 1, mask_y = (1ull << L.by) - 1, mask_z = (1ull << L.bz) - 1;
    for (int i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x)
    {
        float4 p = pos[i];
        // clamp defends the key fields against points outside the declared origin
        uint64_t cx = (uint64_t)max(cell_of(p.x, o.x, cell), 0) & mask_x;
        uint64_t cy = (uint64_t)max(cell_of(p.y, o.y, cell), 0) & mask_y;
        uint64_t cz = (uint64_t)max(cell_of(p.z, o.z, cell), 0) & mask_z;
        sort_store(keys, vals, i, ((uint64_t)seg << (L.bx + L.by + L.bz)) | (cx << (L.by + L.bz)) | (cy << L.bz) | cz,
                   ib);
    }
}

__global__ void k_grid_scatter(SortBuffers sb, const int32_t *d_n, const KeyLayout *lay, const float4 *__restrict__ pos,
                               float4 *spos, int32_t *sidx, float *sint, int *scz, uint64_t *skey, int *err)
{
    const int n = *d_n;
    const SortedView sv = sorted_view(sb);
    const KeyLayout L = *lay;
    const uint64_t mz = (1ull << L.bz) - 1;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        uint64_t k = sv.key(s);
        int g = sv.val(s);
        if (!GCA_INDEX_OK(g, n, err))
            continue;
        float4 p = pos[g];
        spos[s] = make_float4(p.x, p.y, p.z, __int_as_float((int)(k & mz)));
        sidx[s] = g;
        sint[s] = p.w;
        scz[s] = (int)(k & mz);
        skey[s] = k;
    }
}

__global__ void k_hash_insert(const uint64_t *skey, const int32_t *d_n, const KeyLayout *lay, RowSlot *slots,
                              uint32_t hmask, int *d_err)
{
    const int n = *d_n;
    const int bz = lay->bz;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        const unsigned long long rk = skey[s] >> bz;
        if (s > 0 && (skey[s - 1] >> bz) == rk)
            continue;
        // the end of the row (the keys are sorted): galloping from s, then bisection
        // of (lo, hi], where lo is in the row and hi is past it or n
        int lo = s, hi = s + 1, step = 1;
        while (hi < n && (skey[hi] >> bz) == rk)
        {
            lo = hi;
            step <<= 1;
            hi = s + step;
        }
        hi = min(hi, n);
        while (hi - lo > 1)
        {
            const int m = (lo + hi) >> 1;
            if ((skey[m] >> bz) == rk)
                lo = m;
            else
                hi = m;
        }
        const int e = hi;
        uint32_t h = hash_u64(rk) & hmask;
        bool done = false;
        for (uint32_t probe = 0; probe <= hmask; ++probe)
        {
            const unsigned long long prev = atomicCAS(&slots[h].key, kEmptyKey, rk);
            if (prev == kEmptyKey || prev == rk)
            {
                slots[h].start = s;
                slots[h].end = e;
                done = true;
                break;
            }
            h = (h + 1) & hmask;
        }
        if (!done)
            atomicOr(d_err, kErrCapacity);
    }
}

int grid_build(gca3d_context *ctx, const Batch &b, float cell, int origin_mode, const float *host_origin,
               Grid &g)
{
    if (!(cell > 0.0f))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "grid cell must be > 0");
    if (origin_mode == kOriginGiven && (!host_origin || b.P != 1))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "grid: a given origin needs one segment");
    Arena &A = ctx->arena;
    const int P = b.P;
    const int64_t cap = std::max<int64_t>(b.cap, 1);
    uint32_t hcap = 1024;
    while ((int64_t)hcap < 2 * cap)
        hcap <<= 1;
    g.cap = cap;
    g.P = P;
    g.hcap = hcap;
    GridDev &d = g.dev;
    d.cell = cell;
    d.inv_cell = 1.0f / cell;
    d.gmin = A.get<float3>(P);
    d.layout = A.get<KeyLayout>(1);
    d.spos = A.get<float4>(cap);
    d.sidx = A.get<int32_t>(cap);
    d.sint = A.get<float>(cap);
    d.scz = A.get<int>(cap);
    d.skey = A.get<uint64_t>(cap);
    d.slots = A.get<RowSlot>(hcap);
    d.hmask = hcap - 1;
    d.seg_off = b.seg_off;
    d.d_n = b.seg_off + P;
    d.err = ctx->d_err;
    int *ord = A.get<int>(6 * P);
    SortBuffers sb;
    sb.keys[0] = A.get<uint64_t>(cap);
    sb.keys[1] = A.get<uint64_t>(cap);
    sb.vals[0] = A.get<int32_t>(cap);
    sb.vals[1] = A.get<int32_t>(cap);
    sb.d_sel = A.get<int>(1);
    sb.d_ib = A.get<int>(1);
    sb.d_kshift = A.get<int>(1);
    if (!d.gmin || !d.layout || !d.spos || !d.sidx || !d.sint || !d.scz || !d.skey || !d.slots || !ord || !sb.keys[1] ||
        !sb.vals[1] || !sb.d_sel || !sb.d_ib || !sb.d_kshift)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "grid_build: scratch");
    cudaStream_t s = ctx->stream;
    int st = seg_bounds(ctx, b.pos, b.seg_off, P, b.max_seg_cap, ord);
    if (st)
        return st;
    float3 given = host_origin ? make_float3(host_origin[0], host_origin[1], host_origin[2]) : make_float3(0, 0, 0);
    k_grid_layout<<<1, 256, 0, s>>>(ord, P, cell, origin_mode, given, d.gmin, d.layout, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    const int gx = std::min(grid_for(b.max_seg_cap, kBlock * 4), ctx->num_sms * 4);
    k_grid_keys<<<dim3(gx, P), kBlock, 0, s>>>(b.pos, b.seg_off, d.gmin, d.layout, cell, sb.keys[0], sb.vals[0],
                                               index_bits(cap), sb.d_ib, sb.d_kshift);
    GCA_CHECK_LAUNCH(ctx);
    const int32_t *d_n = b.seg_off + P;
    st = radix_sort(ctx, sb, b.seg_off, P, cap, b.max_seg_cap, 64);
    if (st)
        return st;
    const int gs = std::min(grid_for(cap), ctx->num_sms * 8);
    GCA_PROF_BEGIN(ctx, kKidGridScatter);
    k_grid_scatter<<<gs, kBlock, 0, s>>>(sb, d_n, d.layout, b.pos, d.spos, d.sidx, d.sint, d.scz, d.skey, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    GCA_PROF_END(ctx, kKidGridScatter);
    GCA_CUDA(ctx, cudaMemsetAsync(d.slots, 0xFF, sizeof(RowSlot) * hcap, s));
    k_hash_insert<<<gs, kBlock, 0, s>>>(d.skey, d_n, d.layout, d.slots, d.hmask, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

// ---------------------------------------------------------------------------
// queries against a single-segment grid
// ---------------------------------------------------------------------------
__global__ void k_nn_query(const float4 *__restrict__ q, const int32_t *d_nq, GridDev g, float radius, int32_t *out)
{
    const int nq = *d_nq;
    const KeyLayout L = *g.layout;
    const float3 o = g.gmin[0];
    const float rr = __fmul_rn(radius, radius);
    const int per_block = blockDim.x / kSub;
    for (int base = blockIdx.x * per_block; base < nq; base += gridDim.x * per_block)
    {
        const int i = base + (int)(threadIdx.x / kSub);
        const bool valid = i < nq;
        const float4 p = q[valid ? i : 0];
        const NNBest best = nn_search_sub(g, L, 0, o, make_float3(p.x, p.y, p.z), rr, valid);
        if (valid && (threadIdx.x & (kSub - 1)) == 0)
            out[i] = best.t >= 0 ? g.sidx[best.t] : -1;
    }
}

__global__ void k_radius_count(const float4 *__restrict__ q, const int32_t *d_nq, GridDev g, float radius,
                               int32_t *counts)
{
    const int nq = *d_nq;
    const KeyLayout L = *g.layout;
    const float3 o = g.gmin[0];
    const float rr = __fmul_rn(radius, radius);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x)
    {
        float4 p = q[i];
        int c = 0;
        grid_visit(g, L, 0, o, make_float3(p.x, p.y, p.z), [&](int t, float4 c4) {
            if (dist2_ref(c4.x, c4.y, c4.z, p.x, p.y, p.z) < rr)
                ++c;
        });
        counts[i] = c;
    }
}

__global__ void k_radius_fill(const float4 *__restrict__ q, const int32_t *d_nq, GridDev g, float radius,
                              const int32_t *starts, int32_t *list, int64_t cap, int *d_err)
{
    const int nq = *d_nq;
    const KeyLayout L = *g.layout;
    const float3 o = g.gmin[0];
    const float rr = __fmul_rn(radius, radius);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x)
    {
        float4 p = q[i];
        int64_t w = starts[i];
        grid_visit(g, L, 0, o, make_float3(p.x, p.y, p.z), [&](int t, float4 c4) {
            if (dist2_ref(c4.x, c4.y, c4.z, p.x, p.y, p.z) < rr)
            {
                if (w < cap)
                    list[w] = g.sidx[t];
                else
                    atomicOr(d_err, kErrCapacity);
                ++w;
            }
        });
    }
}

int nn_query(gca3d_context *ctx, const float4 *qpos, const int32_t *d_nq, int64_t qcap, const Grid &g, float radius,
             int32_t *out_idx)
{
    const int gs = std::min(grid_for(qcap, kBlock / kSub), ctx->num_sms * 16);
    k_nn_query<<<gs, kBlock, 0, ctx->stream>>>(qpos, d_nq, g.dev, radius, out_idx);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

int radius_query(gca3d_context *ctx, const float4 *qpos, const int32_t *d_nq, int64_t qcap, const Grid &g,
                 float radius, int32_t *counts, int32_t *starts, int32_t *list, int64_t list_cap, int32_t *d_total)
{
    const int gs = std::min(grid_for(qcap), ctx->num_sms * 16);
    k_radius_count<<<gs, kBlock, 0, ctx->stream>>>(qpos, d_nq, g.dev, radius, counts);
    GCA_CHECK_LAUNCH(ctx);
    int st = exclusive_scan(ctx, counts, starts, d_nq, qcap, d_total);
    if (st)
        return st;
    k_radius_fill<<<gs, kBlock, 0, ctx->stream>>>(qpos, d_nq, g.dev, radius, starts, list, list_cap, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

} // namespace gca3d
