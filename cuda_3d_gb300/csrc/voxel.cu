// voxel.cu -- batched voxel-grid downsampling.
//
// reference: cuda_voxel_grid_downsample (src/geometry/cuda_voxel_grid_down_sample.cu:123-161)
// and point_cloud::voxel_grid_down_sample (src/geometry/point_cloud.cu:198-229).
//
// Per segment (cloud) the key is floor((p - aabb_min) / v) per axis, as the
// reference computes it.  The three axis keys of every segment are packed, with the
// segment index above them, into one 64-bit key whose numeric order is the
// reference's lexicographic (kx, ky, kz) order; one stable radix sort then orders
// all segments at once.  A voxel's sum runs sequentially over its points in
// ascending original index (the sort is stable), so the downsampled set is
// bit-exact against the oracle; the mean is xyz / n and rgb * (1 / n) as in
// src/geometry/type.hpp:58-62.
#include "stages.cuh"

#include <algorithm>

namespace gca3d
{

int batch_alloc(gca3d_context *ctx, Batch &b, int P, int64_t cap, int64_t max_seg_cap, bool nrm, bool grd)
{
    Arena &A = ctx->arena;
    b.P = P;
    b.cap = cap;
    b.max_seg_cap = max_seg_cap;
    int64_t c = std::max<int64_t>(cap, 1);
    b.pos = A.get<float4>(c);
    b.col = A.get<float4>(c);
    b.nrm = nrm ? A.get<float4>(c) : nullptr;
    b.grd = grd ? A.get<float4>(c) : nullptr;
    b.seg_off = A.get<int32_t>(P + 1);
    if (!b.pos || !b.col || (nrm && !b.nrm) || (grd && !b.grd) || !b.seg_off)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "batch_alloc: scratch");
    return GCA3D_OK;
}

// exclusive prefix of the segment sizes (one block)
__global__ void k_src_prefix(const SegSrc *src, int P, int32_t *off)
{
    __shared__ int32_t s_base;
    if (threadIdx.x == 0)
        s_base = 0;
    __syncthreads();
    for (int c0 = 0; c0 < P; c0 += blockDim.x)
    {
        int i = c0 + threadIdx.x;
        int v = i < P ? *src[i].d_n : 0;
        // block inclusive scan (Hillis-Steele over 256)
        __shared__ int32_t s[256];
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 256; o <<= 1)
        {
            int32_t y = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < P)
            off[i] = s_base + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 255)
            s_base += s[255];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        off[P] = s_base;
}

__global__ void k_src_bounds_init(int *ord, int P)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * P)
        ord[i] = (i % 6) < 3 ? float_to_ordered(3.402823466e38f) : float_to_ordered(-3.402823466e38f);
}

__global__ void k_src_bounds(const SegSrc *src, int *ord)
{
    const int seg = blockIdx.y;
    const int n = *src[seg].d_n;
    if ((int64_t)blockIdx.x * blockDim.x >= n)
        return;
    const float4 *pos = src[seg].pos;
    float mn[3] = {3.402823466e38f, 3.402823466e38f, 3.402823466e38f};
    float mx[3] = {-3.402823466e38f, -3.402823466e38f, -3.402823466e38f};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        float4 p = pos[i];
        mn[0] = fminf(mn[0], p.x), mn[1] = fminf(mn[1], p.y), mn[2] = fminf(mn[2], p.z);
        mx[0] = fmaxf(mx[0], p.x), mx[1] = fmaxf(mx[1], p.y), mx[2] = fmaxf(mx[2], p.z);
    }
    block_bounds_commit(mn, mx, ord + 6 * seg);
}

// key layout shared by all segments; per-segment origin = unpadded aabb min.  With
// morton (and room in 64 bits) the three axis keys are bit-interleaved below the
// segment index instead: the voxels then come out in Z-order, so runs of
// consecutive output points are compact in space (the correspondence search of the
// ICP stages a block's target cells once for such a run).
__global__ void k_voxel_layout(const int *ord, int P, float voxel, bool morton, int sub_bits, float3 *origin,
                               KeyLayout *lay, int *d_err)
{
    __shared__ uint32_t s_max[3];
    if (threadIdx.x < 3)
        s_max[threadIdx.x] = 0;
    __syncthreads();
    for (int s = threadIdx.x; s < P; s += blockDim.x)
    {
        float mn[3], mx[3];
        for (int a = 0; a < 3; ++a)
        {
            mn[a] = ordered_to_float(ord[6 * s + a]);
            mx[a] = ordered_to_float(ord[6 * s + 3 + a]);
        }
        origin[s] = make_float3(mn[0], mn[1], mn[2]);
        if (!(mx[0] >= mn[0])) // empty segment
            continue;
        for (int a = 0; a < 3; ++a)
        {
            int k = cell_of(mx[a], mn[a], voxel);
            if (k < 0 || k >= (1 << 21))
            {
                atomicOr(d_err, kErrKeyBits);
                k = (1 << 21) - 1;
            }
            atomicMax(&s_max[a], (uint32_t)k);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        KeyLayout L;
        L.bseg = bitlen_u32((uint32_t)(P - 1));
        L.bx = max(1, bitlen_u32(s_max[0]));
        L.by = max(1, bitlen_u32(s_max[1]));
        L.bz = max(1, bitlen_u32(s_max[2]));
        L.total_bits = L.bseg + L.bx + L.by + L.bz;
        L.morton = 0;
        const int b = max(L.bx, max(L.by, L.bz));
        if (morton && L.bseg + 3 * b + sub_bits <= 64)
        {
            L.bx = L.by = L.bz = b;
            L.total_bits = L.bseg + 3 * b;
            L.morton = 1;
        }
        // sub-cell bits for finer scales ride below a Z-order key
        if (L.total_bits + sub_bits > 64 || (sub_bits && !L.morton))
            atomicOr(d_err, kErrKeyBits);
        *lay = L;
    }
}

// the bits of v (up to 21) at every third position (bit interleaving by masks)
__device__ __forceinline__ uint64_t spread3(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__global__ void k_voxel_keys(const SegSrc *src, const int32_t *off, const float3 *origin, const KeyLayout *lay,
                             float voxel, SubLevels sub, uint64_t *keys, int32_t *vals, int ib_cap, int *d_ib,
                             int *d_kshift, int *d_err)
{
    const int seg = blockIdx.y;
    const int n = *src[seg].d_n;
    const int base = off[seg];
    const KeyLayout L = *lay;
    const int sb = 3 * sub.n;
    const int ib = packed_index_bits(L.total_bits + sb, ib_cap);
    if (seg == 0 && blockIdx.x == 0 && threadIdx.x == 0)
    {
        *d_ib = ib;
        *d_kshift = ib + sb;
    }
    const float3 o = origin[seg];
    const float4 *pos = src[seg].pos;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        float4 p = pos[i];
        uint64_t kx = (uint32_t)cell_of(p.x, o.x, voxel), ky = (uint32_t)cell_of(p.y, o.y, voxel),
                 kz = (uint32_t)cell_of(p.z, o.z, voxel);
        uint64_t key = ((uint64_t)seg << (L.bx + L.by + L.bz)) |
                       (L.morton ? (spread3(kx) << 2) | (spread3(ky) << 1) | spread3(kz)
                                 : (kx << (L.by + L.bz)) | (ky << L.bz) | kz);
        // each finer scale's cells, as that scale computes them: with its voxel half the
        // previous one, its quotient is exactly twice the previous one, so each axis adds
        // one bit (x, y, z -- the next three bits of the finer Z-order key)
        for (int l = 0; l < sub.n; ++l)
        {
            const uint64_t fx = (uint32_t)cell_of(p.x, o.x, sub.voxel[l]), fy = (uint32_t)cell_of(p.y, o.y, sub.voxel[l]),
                           fz = (uint32_t)cell_of(p.z, o.z, sub.voxel[l]);
            const uint64_t bx = fx - 2 * kx, by = fy - 2 * ky, bz = fz - 2 * kz;
            if ((bx | by | bz) > 1)
                atomicOr(d_err, kErrInvalid);
            key = (key << 3) | ((bx & 1) << 2) | ((by & 1) << 1) | (bz & 1);
            kx = fx, ky = fy, kz = fz;
        }
        sort_store(keys, vals, base + i, key, ib);
    }
}

// segment offsets of the output; empty segments start where the next one does
__global__ void k_seg_first_to_offsets(const int32_t *seg_first, int P, const int32_t *d_m, int32_t *off)
{
    if (threadIdx.x != 0)
        return;
    int32_t next = *d_m;
    off[P] = next;
    for (int s = P - 1; s >= 0; --s)
    {
        if (seg_first[s] >= 0)
            next = seg_first[s];
        off[s] = next;
    }
}

__global__ void k_voxel_reduce(const SegSrc *src, const int32_t *in_off, SortBuffers sb, const int32_t *starts,
                               const int32_t *d_m, const KeyLayout *lay, float4 *opos, float4 *ocol, int *err)
{
    const int m = *d_m;
    const SortedView sv = sorted_view(sb);
    const KeyLayout L = *lay;
    const int segshift = L.bx + L.by + L.bz;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < m; v += gridDim.x * blockDim.x)
    {
        const int s = starts[v], e = starts[v + 1];
        const int seg = L.bseg ? (int)(sv.key(s) >> segshift) : 0;
        const int base = in_off[seg];
        const float4 *ps = src[seg].pos;
        const float4 *cs = src[seg].col;
        int g = sv.val(s) - base;
        if (!GCA_INDEX_OK(g, in_off[seg + 1] - base, err))
            continue;
        float4 p = ps[g], c = cs[g];
        float sx = p.x, sy = p.y, sz = p.z, cr = c.x, cg = c.y, cb = c.z;
        for (int j = s + 1; j < e; ++j)
        {
            g = sv.val(j) - base;
            if (!GCA_INDEX_OK(g, in_off[seg + 1] - base, err))
                break;
            p = ps[g];
            c = cs[g];
            sx = __fadd_rn(sx, p.x);
            sy = __fadd_rn(sy, p.y);
            sz = __fadd_rn(sz, p.z);
            cr = __fadd_rn(cr, c.x);
            cg = __fadd_rn(cg, c.y);
            cb = __fadd_rn(cb, c.z);
        }
        const float fn = (float)(e - s);
        const float inv = __fdiv_rn(1.0f, fn);
        const float r = __fmul_rn(cr, inv), gg = __fmul_rn(cg, inv), b = __fmul_rn(cb, inv);
        opos[v] = make_float4(__fdiv_rn(sx, fn), __fdiv_rn(sy, fn), __fdiv_rn(sz, fn), intensity_of(r, gg, b));
        ocol[v] = make_float4(r, gg, b, 0.0f);
    }
}

// One finer scale from the previous one's sorted order: within each previous voxel's run
// the elements are split, stably, by the next three sub-cell bits below the key, which
// orders them by (finer key, index) -- what a full sort by the finer key gives.  One
// thread per previous voxel (a handful of points each); the output goes to the other
// buffer, and the finer scale's view and layout are written beside the previous ones.
__global__ void k_voxel_refine(SortBuffers sb, const int32_t *starts, const int32_t *d_m, const KeyLayout *lay_in,
                               int *d_sel_out, int *d_kshift_out, KeyLayout *lay_out)
{
    const int sel = *sb.d_sel;
    const int ks = *sb.d_kshift - 3; // the finer key's lowest bit
    const bool packed = *sb.d_ib != 0;
    const uint64_t *kin = sb.keys[sel];
    uint64_t *kout = sb.keys[sel ^ 1];
    const int32_t *vin = sb.vals[sel];
    int32_t *vout = sb.vals[sel ^ 1];
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        *d_sel_out = sel ^ 1;
        *d_kshift_out = ks;
        KeyLayout L = *lay_in;
        L.bx += 1, L.by += 1, L.bz += 1;
        L.total_bits += 3;
        *lay_out = L;
    }
    const int m = *d_m;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < m; v += gridDim.x * blockDim.x)
    {
        const int s = starts[v], e = starts[v + 1];
        if (e - s < 256)
        {
            // a run of fewer than 256 keys: the eight sub-cell counts are the bytes of one
            // register, and one multiplication by 0x0101..01 gives their running sums
            // (byte b of the product: the keys of sub-cells 0..b; shifted one byte up: the
            // keys of the sub-cells below b), all below 256, so no byte carries
            uint64_t c = 0;
            for (int j = s; j < e; ++j)
                c += 1ull << (8 * (int)((kin[j] >> ks) & 7));
            uint64_t at = (c * 0x0101010101010101ull) << 8;
            for (int j = s; j < e; ++j)
            {
                const uint64_t w = kin[j];
                const int sh = 8 * (int)((w >> ks) & 7);
                const int o = s + (int)((at >> sh) & 255u);
                at += 1ull << sh;
                kout[o] = w;
                if (!packed)
                    vout[o] = vin[j];
            }
            continue;
        }
        int off[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int j = s; j < e; ++j)
            ++off[(kin[j] >> ks) & 7];
        int run = s;
#pragma unroll
        for (int b = 0; b < 8; ++b)
        {
            const int c = off[b];
            off[b] = run;
            run += c;
        }
        for (int j = s; j < e; ++j)
        {
            const uint64_t w = kin[j];
            const int o = off[(w >> ks) & 7]++;
            kout[o] = w;
            if (!packed)
                vout[o] = vin[j];
        }
    }
}

// the runs of equal keys (voxels) of the sorted view and their sums: the part of a voxel
// stage after its order is known
static int voxel_reduce_stage(gca3d_context *ctx, const SegSrc *d_src, int P, int64_t total_cap,
                              const int32_t *in_off, const SortBuffers &sb, const KeyLayout *lay, Batch &out,
                              int32_t *starts, int32_t *d_m)
{
    Arena &A = ctx->arena;
    const int64_t cap = std::max<int64_t>(total_cap, 1);
    int32_t *seg_count = A.get<int32_t>(P);
    if (!seg_count)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "voxel_stage: scratch");
    cudaStream_t s = ctx->stream;
    const int32_t *d_n = in_off + P;
    const int gs = std::min(grid_for(total_cap), ctx->num_sms * 8);
    GCA_CUDA(ctx, cudaMemsetAsync(seg_count, 0xFF, sizeof(int32_t) * P, s));
    int st = run_scan(ctx, sb, d_n, cap, lay, starts, seg_count, d_m);
    if (st)
        return st;
    GCA_PROF_BEGIN(ctx, kKidVoxelReduce);
    k_voxel_reduce<<<gs, kBlock, 0, s>>>(d_src, in_off, sb, starts, d_m, lay, out.pos, out.col, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    GCA_PROF_END(ctx, kKidVoxelReduce);
    k_seg_first_to_offsets<<<1, 32, 0, s>>>(seg_count, P, d_m, out.seg_off);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

int voxel_refine(gca3d_context *ctx, const SegSrc *d_src, VoxelChain &c, Batch &out)
{
    if (c.used >= c.levels)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "voxel_refine: no finer scale carried");
    Arena &A = ctx->arena;
    const int64_t cap = std::max<int64_t>(c.total_cap, 1);
    SortBuffers sb = c.sb;
    sb.d_sel = A.get<int>(1);
    sb.d_kshift = A.get<int>(1);
    KeyLayout *lay = A.get<KeyLayout>(1);
    int32_t *starts = A.get<int32_t>(cap + 1);
    int32_t *d_m = A.get<int32_t>(1);
    if (!sb.d_sel || !sb.d_kshift || !lay || !starts || !d_m)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "voxel_refine: scratch");
    if (!out.pos)
    {
        int st = batch_alloc(ctx, out, c.P, c.total_cap, c.max_seg_cap, false, false);
        if (st)
            return st;
    }
    const int gs = std::min(grid_for(c.total_cap), ctx->num_sms * 8);
    k_voxel_refine<<<gs, kBlock, 0, ctx->stream>>>(c.sb, c.starts, c.d_m, c.lay, sb.d_sel, sb.d_kshift, lay);
    GCA_CHECK_LAUNCH(ctx);
    int st = voxel_reduce_stage(ctx, d_src, c.P, c.total_cap, c.in_off, sb, lay, out, starts, d_m);
    if (st)
        return st;
    c.sb = sb;
    c.lay = lay;
    c.starts = starts;
    c.d_m = d_m;
    c.used += 1;
    return GCA3D_OK;
}

int voxel_stage(gca3d_context *ctx, const SegSrc *d_src, int P, int64_t total_cap, int64_t max_seg_cap,
                float voxel, Batch &out, bool morton, const SubLevels *finer, VoxelChain *chain)
{
    if (!(voxel > 0.0f))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "voxel size must be > 0");
    Arena &A = ctx->arena;
    const int64_t cap = std::max<int64_t>(total_cap, 1);
    int32_t *in_off = A.get<int32_t>(P + 1);
    int *ord = A.get<int>(6 * P);
    float3 *origin = A.get<float3>(P);
    KeyLayout *lay = A.get<KeyLayout>(1);
    SortBuffers sb;
    sb.keys[0] = A.get<uint64_t>(cap);
    sb.keys[1] = A.get<uint64_t>(cap);
    sb.vals[0] = A.get<int32_t>(cap);
    sb.vals[1] = A.get<int32_t>(cap);
    sb.d_sel = A.get<int>(1);
    sb.d_ib = A.get<int>(1);
    sb.d_kshift = A.get<int>(1);
    int32_t *starts = A.get<int32_t>(cap + 1);
    int32_t *d_m = A.get<int32_t>(1);
    if (!in_off || !ord || !origin || !lay || !sb.keys[1] || !sb.vals[1] || !sb.d_sel || !sb.d_ib || !sb.d_kshift ||
        !starts || !d_m)
        return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "voxel_stage: scratch");
    const SubLevels sub = finer ? *finer : SubLevels{};
    if (sub.n < 0 || sub.n > kMaxSubLevels || (sub.n && !morton))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "voxel_stage: finer scales need Z-order keys");
    if (!out.pos)
    {
        int st = batch_alloc(ctx, out, P, total_cap, max_seg_cap, false, false);
        if (st)
            return st;
    }
    cudaStream_t s = ctx->stream;
    k_src_prefix<<<1, 256, 0, s>>>(d_src, P, in_off);
    GCA_CHECK_LAUNCH(ctx);
    k_src_bounds_init<<<grid_for(6 * P), kBlock, 0, s>>>(ord, P);
    GCA_CHECK_LAUNCH(ctx);
    const int gx = std::min(grid_for(max_seg_cap, kBlock * 4), ctx->num_sms * 4);
    k_src_bounds<<<dim3(gx, P), kBlock, 0, s>>>(d_src, ord);
    GCA_CHECK_LAUNCH(ctx);
    k_voxel_layout<<<1, 256, 0, s>>>(ord, P, voxel, morton, 3 * sub.n, origin, lay, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    k_voxel_keys<<<dim3(gx, P), kBlock, 0, s>>>(d_src, in_off, origin, lay, voxel, sub, sb.keys[0], sb.vals[0],
                                                index_bits(cap), sb.d_ib, sb.d_kshift, ctx->d_err);
    GCA_CHECK_LAUNCH(ctx);
    int st = radix_sort(ctx, sb, in_off, P, total_cap, max_seg_cap, 64);
    if (st)
        return st;
    st = voxel_reduce_stage(ctx, d_src, P, total_cap, in_off, sb, lay, out, starts, d_m);
    if (st)
        return st;
    if (chain)
    {
        chain->sb = sb;
        chain->in_off = in_off;
        chain->starts = starts;
        chain->d_m = d_m;
        chain->lay = lay;
        chain->levels = sub.n;
        chain->used = 0;
        chain->P = P;
        chain->total_cap = total_cap;
        chain->max_seg_cap = max_seg_cap;
    }
    return GCA3D_OK;
}

// copy segments into a contiguous batch (no downsampling)
__global__ void k_gather(const SegSrc *src, const int32_t *off, float4 *pos, float4 *col, float4 *nrm)
{
    const int seg = blockIdx.y;
    const int n = *src[seg].d_n;
    const int base = off[seg];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        pos[base + i] = src[seg].pos[i];
        col[base + i] = src[seg].col[i];
        if (nrm)
            nrm[base + i] = src[seg].nrm ? src[seg].nrm[i] : make_float4(0, 0, 0, 0);
    }
}

int gather_stage(gca3d_context *ctx, const SegSrc *d_src, int P, int64_t max_seg_cap, Batch &out,
                 bool with_normals)
{
    if (with_normals && !out.nrm)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "gather_stage: batch has no normal storage");
    k_src_prefix<<<1, 256, 0, ctx->stream>>>(d_src, P, out.seg_off);
    GCA_CHECK_LAUNCH(ctx);
    const int gx = std::min(grid_for(max_seg_cap, kBlock * 4), ctx->num_sms * 4);
    k_gather<<<dim3(gx, P), kBlock, 0, ctx->stream>>>(d_src, out.seg_off, out.pos, out.col,
                                                     with_normals ? out.nrm : nullptr);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

} // namespace gca3d
