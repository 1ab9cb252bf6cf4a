// grid_query.cuh -- device-side traversal of the row-hashed uniform grid.
#pragma once

#include "internal.cuh"

namespace gca3d
{

// the 9 rows (x offset, then y offset) around a point: [start, end) in the sorted
// arrays, and the z-cell window [lo, hi]
struct GridRows
{
    int2 r[9];
    int lo, hi;
};

// Probe all 9 rows with independent 16-byte loads (one round of memory latency for
// the common case where the first slot answers), then resolve the rare collisions.
// Returns false when p lies outside the grid's key range.
__device__ __forceinline__ bool grid_rows(const GridDev &g, const KeyLayout &L, int seg, float3 o, float3 p,
                                          GridRows &R)
{
    const int cx = cell_of(p.x, o.x, g.cell), cy = cell_of(p.y, o.y, g.cell), cz = cell_of(p.z, o.z, g.cell);
    const int mx = (1 << L.bx) - 1, my = (1 << L.by) - 1, mz = (1 << L.bz) - 1;
    if (cx < -1 || cx > mx + 1 || cy < -1 || cy > my + 1 || cz < -1 || cz > mz + 1)
        return false;
    const unsigned long long segbits = (unsigned long long)seg << (L.bx + L.by);
    unsigned long long rk[9];
    uint32_t h[9];
    ulonglong2 v[9];
    const uint32_t hmask = g.hmask;
#pragma unroll
    for (int k = 0; k < 9; ++k)
    {
        const int x = cx + k / 3 - 1, y = cy + k % 3 - 1;
        const bool ok = x >= 0 && x <= mx && y >= 0 && y <= my;
        rk[k] = ok ? (segbits | ((unsigned long long)x << L.by) | (unsigned long long)y) : kEmptyKey;
        h[k] = hash_u64(rk[k]) & hmask;
        v[k] = ok ? slot_load(g.slots, h[k]) : make_ulonglong2(kEmptyKey, 0ull);
    }
#pragma unroll
    for (int k = 0; k < 9; ++k)
    {
        if (rk[k] != kEmptyKey && v[k].x == rk[k])
            R.r[k] = make_int2((int)(uint32_t)v[k].y, (int)(uint32_t)(v[k].y >> 32));
        else if (rk[k] != kEmptyKey && v[k].x != kEmptyKey)
            R.r[k] = row_probe_rest(g.slots, hmask, rk[k], h[k]);
        else
            R.r[k] = make_int2(0, 0);
    }
    R.lo = cz - 1;
    R.hi = cz + 1;
    return true;
}

// visit the points of the probed rows whose z cell lies in [lo, hi], in the
// reference's scan order (x offset, then y offset, then z, then ascending original
// index; nn_search_functor, src/geometry/cuda_nn_search.cu:164-206).  f(t, spos[t]).
template <class F> __device__ __forceinline__ void grid_scan(const GridDev &g, const GridRows &R, F &&f)
{
#pragma unroll
    for (int k = 0; k < 9; ++k)
    {
        int t = R.r[k].x;
        const int e = R.r[k].y;
        if (t >= e)
            continue;
        if (e - t > 16)
        {
            int a = t, b = e;
            while (a < b)
            {
                const int m = (a + b) >> 1;
                if (__ldg(&g.scz[m]) < R.lo)
                    a = m + 1;
                else
                    b = m;
            }
            t = a;
        }
        for (; t < e; ++t)
        {
            const float4 q = __ldg(&g.spos[t]);
            const int qz = __float_as_int(q.w);
            if (qz < R.lo)
                continue;
            if (qz > R.hi)
                break;
            f(t, q);
        }
    }
}

template <class F>
__device__ __forceinline__ void grid_visit(const GridDev &g, const KeyLayout &L, int seg, float3 o, float3 p, F &&f)
{
    GridRows R;
    if (grid_rows(g, L, seg, o, p, R))
        grid_scan(g, R, f);
}

struct NNBest
{
    float d2;
    int t;
};

// nearest grid point with d^2 < rr; ties on d^2 go to the smaller original index
__device__ __forceinline__ NNBest nn_search_one(const GridDev &g, const KeyLayout &L, int seg, float3 o, float3 p,
                                                float rr)
{
    NNBest b{rr, -1};
    grid_visit(g, L, seg, o, p, [&](int t, float4 q) {
        const float d2 = dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z);
        if (d2 < b.d2 || (d2 == b.d2 && b.t >= 0 && __ldg(&g.sidx[t]) < __ldg(&g.sidx[b.t])))
        {
            b.d2 = d2;
            b.t = t;
        }
    });
    return b;
}

// ---------------------------------------------------------------------------
// 4 lanes per query: lane `sub` of a 4-lane group probes and scans rows
// sub, sub + 4, sub + 8 of the 9, so the dependent chain of a query is a third
// as long; the group combines its partial results with width-4 shuffles.
// ---------------------------------------------------------------------------
constexpr int kSub = 4;

struct SubRows
{
    int2 r[3];
    int lo, hi;
};

template <class F> __device__ __forceinline__ void grid_scan_sub(const GridDev &g, const SubRows &R, F &&f)
{
#pragma unroll
    for (int j = 0; j < 3; ++j)
    {
        int t = R.r[j].x;
        const int e = R.r[j].y;
        if (t >= e)
            continue;
        if (e - t > 8)
        {
            int a = t, b = e;
            while (a < b)
            {
                const int m = (a + b) >> 1;
                if (__ldg(&g.scz[m]) < R.lo)
                    a = m + 1;
                else
                    b = m;
            }
            t = a;
        }
        for (; t < e; ++t)
        {
            const float4 q = __ldg(&g.spos[t]);
            const int qz = __float_as_int(q.w);
            if (qz < R.lo)
                continue;
            if (qz > R.hi)
                break;
            f(t, q);
        }
    }
}

// the cells [x0, x0 + nx) x [y0, y0 + ny) x [zlo, zhi] of a search
struct CellBox
{
    int x0, nx, y0, ny, zlo, zhi;
};

// the rows of a box, split over the 4 lanes of a group as grid_rows_sub does
__device__ __forceinline__ void grid_rows_box(const GridDev &g, const KeyLayout &L, int seg, const CellBox &B,
                                              int sub, SubRows &R)
{
    const int mx = (1 << L.bx) - 1, my = (1 << L.by) - 1;
    const unsigned long long segbits = (unsigned long long)seg << (L.bx + L.by);
    const int nrows = B.nx * B.ny;
    unsigned long long rk[3];
    uint32_t h[3];
    ulonglong2 v[3];
    const uint32_t hmask = g.hmask;
#pragma unroll
    for (int j = 0; j < 3; ++j)
    {
        const int k = sub + kSub * j;
        const int x = B.x0 + k / B.ny, y = B.y0 + k % B.ny;
        const bool ok = k < nrows && x >= 0 && x <= mx && y >= 0 && y <= my;
        rk[j] = ok ? (segbits | ((unsigned long long)x << L.by) | (unsigned long long)y) : kEmptyKey;
        h[j] = hash_u64(rk[j]) & hmask;
        v[j] = ok ? slot_load(g.slots, h[j]) : make_ulonglong2(kEmptyKey, 0ull);
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)
    {
        R.r[j] = make_int2(0, 0);
        if (rk[j] != kEmptyKey && v[j].x == rk[j])
            R.r[j] = make_int2((int)(uint32_t)v[j].y, (int)(uint32_t)(v[j].y >> 32));
        else if (rk[j] != kEmptyKey && v[j].x != kEmptyKey)
            R.r[j] = row_probe_rest(g.slots, hmask, rk[j], h[j]);
    }
    R.lo = B.zlo;
    R.hi = B.zhi;
}

// the 3 x 3 x 3 cells around p's cell; false when p lies outside the grid's range
__device__ __forceinline__ bool nn_full_box(const GridDev &g, const KeyLayout &L, float3 o, float3 p, CellBox &B)
{
    const int cx = cell_of(p.x, o.x, g.cell), cy = cell_of(p.y, o.y, g.cell), cz = cell_of(p.z, o.z, g.cell);
    const int mx = (1 << L.bx) - 1, my = (1 << L.by) - 1, mz = (1 << L.bz) - 1;
    B = CellBox{cx - 1, 3, cy - 1, 3, cz - 1, cz + 1};
    return !(cx < -1 || cx > mx + 1 || cy < -1 || cy > my + 1 || cz < -1 || cz > mz + 1);
}

// shrink a full box to the cells that overlap the ball of radius u around p.  u
// bounds the distance of the nearest point (a known candidate lies at that
// distance), so the nearest point -- and every point that could tie with it -- is
// in the smaller box.  u is inflated for the rounding of the distance and of p -/+ u;
// cell_of is monotonic, so the cell range of the ball contains the cells of all its
// points.
__device__ __forceinline__ void nn_shrink_box(const GridDev &g, float3 o, float3 p, float u, CellBox &B)
{
    const float ui = u * 1.00002f + 1e-6f * (1.0f + fabsf(p.x) + fabsf(p.y) + fabsf(p.z));
    const int x0 = max(cell_of(__fsub_rn(p.x, ui), o.x, g.cell), B.x0);
    const int x1 = min(cell_of(__fadd_rn(p.x, ui), o.x, g.cell), B.x0 + 2);
    const int y0 = max(cell_of(__fsub_rn(p.y, ui), o.y, g.cell), B.y0);
    const int y1 = min(cell_of(__fadd_rn(p.y, ui), o.y, g.cell), B.y0 + 2);
    B.zlo = max(cell_of(__fsub_rn(p.z, ui), o.z, g.cell), B.zlo);
    B.zhi = min(cell_of(__fadd_rn(p.z, ui), o.z, g.cell), B.zhi);
    // the ball contains p, so every range contains p's own cell: never empty
    B.x0 = x0, B.nx = x1 - x0 + 1;
    B.y0 = y0, B.ny = y1 - y0 + 1;
}

// the nearest grid point with d^2 < rr inside box B over the whole 4-lane group;
// every lane of the group returns the same answer (ties on d^2 go to the smaller
// original index).  All 32 lanes of the warp must call it (invalid lanes pass
// valid = false).
__device__ __forceinline__ NNBest nn_search_box(const GridDev &g, const KeyLayout &L, int seg, const CellBox &B,
                                                float3 p, float rr, bool valid)
{
    const int sub = threadIdx.x & (kSub - 1);
    NNBest b{rr, -1};
    SubRows R;
    if (valid)
    {
        grid_rows_box(g, L, seg, B, sub, R);
        grid_scan_sub(g, R, [&](int t, float4 q) {
            const float d2 = dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z);
            if (d2 < b.d2 || (d2 == b.d2 && b.t >= 0 && __ldg(&g.sidx[t]) < __ldg(&g.sidx[b.t])))
            {
                b.d2 = d2;
                b.t = t;
            }
        });
    }
#pragma unroll
    for (int off = 1; off < kSub; off <<= 1)
    {
        const float od2 = __shfl_xor_sync(0xffffffffu, b.d2, off, kSub);
        const int ot = __shfl_xor_sync(0xffffffffu, b.t, off, kSub);
        if (ot >= 0 && (b.t < 0 || od2 < b.d2 || (od2 == b.d2 && __ldg(&g.sidx[ot]) < __ldg(&g.sidx[b.t]))))
        {
            b.d2 = od2;
            b.t = ot;
        }
    }
    return b;
}

// the nearest grid point with d^2 < rr in the 27 cells around p (4-lane group)
__device__ __forceinline__ NNBest nn_search_sub(const GridDev &g, const KeyLayout &L, int seg, float3 o, float3 p,
                                                float rr, bool valid)
{
    CellBox B;
    const bool in = nn_full_box(g, L, o, p, B);
    return nn_search_box(g, L, seg, B, p, rr, valid && in);
}

} // namespace gca3d
