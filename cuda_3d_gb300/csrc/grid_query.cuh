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

// a position in [t, e] at most 8 before the first one whose z cell is >= lo (the
// row is sorted by z cell): a 4-way search, its three probes loaded together
__device__ __forceinline__ int row_seek_z(const int *scz, int t, int e, int lo)
{
    int a = t, n = e - t; // the first z cell >= lo is in [a, a + n]
    while (n > 8)
    {
        const int s = n >> 2;
        const int c1 = __ldg(&scz[a + s]), c2 = __ldg(&scz[a + 2 * s]), c3 = __ldg(&scz[a + 3 * s]);
        if (c3 < lo)
        {
            a += 3 * s + 1;
            n -= 3 * s + 1;
        }
        else if (c2 < lo)
        {
            a += 2 * s + 1;
            n = s - 1;
        }
        else if (c1 < lo)
        {
            a += s + 1;
            n = s - 1;
        }
        else
            n = s;
    }
    return a;
}

// visit the points of row [t, e) whose z cell lies in [lo, hi] in order, reading
// Batch candidates per load round (their loads overlap instead of each waiting for
// the test of the one before).  f(t, spos[t]).
template <int Batch, class F>
__device__ __forceinline__ void row_scan(const GridDev &g, int t, int e, int lo, int hi, F &&f)
{
    if (t >= e)
        return;
    if (!GCA_INDEX_OK(t, *g.d_n, g.err) || !GCA_INDEX_OK(e - 1, *g.d_n, g.err))
        return;
    if (e - t > 8)
        t = row_seek_z(g.scz, t, e, lo);
    for (bool more = true; more && t < e; t += Batch)
    {
        float4 q[Batch];
#pragma unroll
        for (int u = 0; u < Batch; ++u)
            q[u] = t + u < e ? __ldg(&g.spos[t + u]) : make_float4(0.0f, 0.0f, 0.0f, __int_as_float(0x7fffffff));
#pragma unroll
        for (int u = 0; u < Batch; ++u)
        {
            const int qz = __float_as_int(q[u].w);
            more = more && qz <= hi;
            if (more && qz >= lo)
                f(t + u, q[u]);
        }
    }
}

// visit the points of the probed rows whose z cell lies in [lo, hi], in the
// reference's scan order (x offset, then y offset, then z, then ascending original
// index; nn_search_functor, src/geometry/cuda_nn_search.cu:164-206).  f(t, spos[t]).
template <int Batch = 1, class F> __device__ __forceinline__ void grid_scan(const GridDev &g, const GridRows &R, F &&f)
{
#pragma unroll
    for (int k = 0; k < 9; ++k)
        row_scan<Batch>(g, R.r[k].x, R.r[k].y, R.lo, R.hi, f);
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

// ---------------------------------------------------------------------------
// 4 lanes per query: lane `sub` of a 4-lane group probes and scans rows
// sub, sub + 4, sub + 8 of the 9, so the dependent chain of a query is a third
// as long; the group combines its partial results with width-4 shuffles.
// ---------------------------------------------------------------------------
constexpr int kSub = 4;
constexpr int kSubRows = (9 + kSub - 1) / kSub; // rows per lane

struct SubRows
{
    int2 r[kSubRows];
    int lo, hi;
};

// scan the rows in order, kScanBatch candidates per load round
constexpr int kScanBatch = 4;
template <class F> __device__ __forceinline__ void grid_scan_sub(const GridDev &g, const SubRows &R, F &&f)
{
#pragma unroll
    for (int j = 0; j < kSubRows; ++j)
        row_scan<kScanBatch>(g, R.r[j].x, R.r[j].y, R.lo, R.hi, f);
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
    unsigned long long rk[kSubRows];
    uint32_t h[kSubRows];
    ulonglong2 v[kSubRows];
    const uint32_t hmask = g.hmask;
#pragma unroll
    for (int j = 0; j < kSubRows; ++j)
    {
        const int k = sub + kSub * j;
        // k / ny for k < 9 and ny <= 3 by a multiply: (k * ceil(256 / ny)) >> 8
        const int kx = (k * (B.ny == 1 ? 256 : (B.ny == 2 ? 128 : 86))) >> 8;
        const int x = B.x0 + kx, y = B.y0 + (k - kx * B.ny);
        const bool ok = k < nrows && x >= 0 && x <= mx && y >= 0 && y <= my;
        rk[j] = ok ? (segbits | ((unsigned long long)x << L.by) | (unsigned long long)y) : kEmptyKey;
        h[j] = hash_u64(rk[j]) & hmask;
        v[j] = ok ? slot_load(g.slots, h[j]) : make_ulonglong2(kEmptyKey, 0ull);
    }
#pragma unroll
    for (int j = 0; j < kSubRows; ++j)
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

// cell bounds without a division: the cell that cell_of assigns to any value v'
// >= v (resp. <= v) is at least lo_cell(v) (resp. at most hi_cell(v)).  The quotient
// by the reciprocal is within 3 rounding units of (v - o) / cell and the binning
// itself (sub, div) within 2, so a slack of 1e-6 (|a| + 3) cells covers both.
__device__ __forceinline__ int lo_cell(float v, float o, float inv)
{
    const float a = (v - o) * inv;
    return __float2int_rd(a - 1e-6f * (fabsf(a) + 3.0f));
}
__device__ __forceinline__ int hi_cell(float v, float o, float inv)
{
    const float a = (v - o) * inv;
    return __float2int_rd(a + 1e-6f * (fabsf(a) + 3.0f));
}

// shrink a full box to the cells that overlap the ball of radius u around p.  u
// bounds the distance of the nearest point (a known candidate lies at that
// distance), so the nearest point -- and every point that could tie with it -- is
// in the smaller box.  u is inflated for the rounding of the distance and of p -/+ u;
// lo_cell / hi_cell bound the cells of every point of the ball.
__device__ __forceinline__ void nn_shrink_box(const GridDev &g, float3 o, float3 p, float u, CellBox &B)
{
    const float ui = u * 1.00002f + 1e-6f * (1.0f + fabsf(p.x) + fabsf(p.y) + fabsf(p.z));
    const float inv = g.inv_cell;
    const int x0 = max(lo_cell(__fsub_rn(p.x, ui), o.x, inv), B.x0);
    const int x1 = min(hi_cell(__fadd_rn(p.x, ui), o.x, inv), B.x0 + 2);
    const int y0 = max(lo_cell(__fsub_rn(p.y, ui), o.y, inv), B.y0);
    const int y1 = min(hi_cell(__fadd_rn(p.y, ui), o.y, inv), B.y0 + 2);
    B.zlo = max(lo_cell(__fsub_rn(p.z, ui), o.z, inv), B.zlo);
    B.zhi = min(hi_cell(__fadd_rn(p.z, ui), o.z, inv), B.zhi);
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

// ---------------------------------------------------------------------------
// Correspondence certificates.  A search at position ps also yields a lower bound
// G on the distance from ps to every target point other than the nearest one t1:
// the second-smallest squared distance it saw, and the radius of the ball that the
// searched cells contain (points outside were not seen).  While the source point
// moves by delta from ps, no other point can come closer than G - delta, so a
// fresh distance to t1 below that proves t1 is still the unique nearest point.
// Every FP32 rounding on the way is covered by relative slack of a few 1e-6
// (distances are computed to within 6 units of 2^-24).
// ---------------------------------------------------------------------------
struct NNCerts
{
    float4 *pos; // ps (the transformed source point of the last search), w = G
    int *t;      // t1: the nearest point that search found at any distance, -1 for none
};

struct NNBest2
{
    float d2; // nearest (any distance), +inf when the searched cells are empty
    int t;
    float s2; // second-smallest squared distance, +inf when fewer than two points
};

// radius R of the ball around p whose points all lie in cells of box B: the
// distance from p to the box's faces, less a slack that covers the rounding of
// that distance and of the binning (cell_of is within 2 rounding units of
// (v - o) / cell); 0 when nothing positive remains
__device__ __forceinline__ float box_cover(const GridDev &g, float3 o, float3 p, const CellBox &B)
{
    const float c = g.cell;
    auto axis = [c](float pv, float ov, int lo, int n) {
        const float d = pv - ov;
        const float slack = 2e-6f * (fabsf(d) + fabsf(ov) + 3.0f * c);
        return fminf(d - (float)lo * c, (float)(lo + n) * c - d) - slack;
    };
    const float r = fminf(fminf(axis(p.x, o.x, B.x0, B.nx), axis(p.y, o.y, B.y0, B.ny)),
                          axis(p.z, o.z, B.zlo, B.zhi - B.zlo + 1));
    return r > 0.0f ? r * 0.99999f : 0.0f;
}

// the nearest grid point inside box B at any distance (ties to the smaller original
// index, as nn_search_box) and the second-smallest squared distance, over the
// 4-lane group; all 32 lanes of the warp call it
__device__ __forceinline__ NNBest2 nn_search_box2(const GridDev &g, const KeyLayout &L, int seg, const CellBox &B,
                                                  float3 p, bool valid)
{
    const int sub = threadIdx.x & (kSub - 1);
    NNBest2 b{INFINITY, -1, INFINITY};
    SubRows R;
    if (valid)
    {
        grid_rows_box(g, L, seg, B, sub, R);
        grid_scan_sub(g, R, [&](int t, float4 q) {
            const float d2 = dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z);
            if (b.t < 0 || d2 < b.d2 || (d2 == b.d2 && __ldg(&g.sidx[t]) < __ldg(&g.sidx[b.t])))
            {
                b.s2 = b.d2;
                b.d2 = d2;
                b.t = t;
            }
            else
                b.s2 = fminf(b.s2, d2);
        });
    }
#pragma unroll
    for (int off = 1; off < kSub; off <<= 1)
    {
        const float od2 = __shfl_xor_sync(0xffffffffu, b.d2, off, kSub);
        const int ot = __shfl_xor_sync(0xffffffffu, b.t, off, kSub);
        const float os2 = __shfl_xor_sync(0xffffffffu, b.s2, off, kSub);
        if (ot >= 0 && (b.t < 0 || od2 < b.d2 || (od2 == b.d2 && __ldg(&g.sidx[ot]) < __ldg(&g.sidx[b.t]))))
        {
            b.s2 = fminf(os2, b.d2);
            b.d2 = od2;
            b.t = ot;
        }
        else
            b.s2 = fminf(b.s2, od2);
    }
    return b;
}

// G of a search at p over box B (see NNCerts)
__device__ __forceinline__ float cert_bound(const GridDev &g, float3 o, float3 p, const CellBox &B, float s2)
{
    float G = box_cover(g, o, p, B);
    if (s2 < INFINITY)
        G = fminf(G, sqrtf(s2) * 0.999998f);
    return G;
}

// the correspondence of p from a certificate (ps, G, t1), without a search; false
// when the certificate does not decide it.  On true, t is what the search over the
// 27 cells around p gives (nearest with d^2 < rr, ties to the smaller index, -1 for
// none) and d2 its squared distance.
__device__ __forceinline__ bool nn_certified(const GridDev &g, float3 o, float3 p, const CellBox &B, float4 cp,
                                             int t1, float rr, int &t, float &d2)
{
    const float dx = p.x - cp.x, dy = p.y - cp.y, dz = p.z - cp.z;
    const float delta = sqrtf(dx * dx + dy * dy + dz * dz) * 1.000002f;
    const float m = cp.w - delta; // every other point is at least this far from p
    if (!(m > 1e-6f))
        return false;
    const float m2 = m * m * 0.999996f; // below the FP32 squared distance of every other point
    if (t1 < 0)
    {
        if (!(m2 >= rr * 1.000001f))
            return false;
        t = -1;
        d2 = rr;
        return true;
    }
    const float4 q = __ldg(&g.spos[t1]);
    const float dq = dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z);
    if (!(dq < m2))
        return false;
    d2 = dq;
    if (!(dq < rr))
    {
        t = -1; // t1 is the nearest and it is beyond max_corr
        d2 = rr;
        return true;
    }
    // t1 must also be one of the candidates of the 27-cell search around p
    const int qx = cell_of(q.x, o.x, g.cell), qy = cell_of(q.y, o.y, g.cell), qz = __float_as_int(q.w);
    if (qx < B.x0 || qx >= B.x0 + B.nx || qy < B.y0 || qy >= B.y0 + B.ny || qz < B.zlo || qz > B.zhi)
        return false;
    t = t1;
    return true;
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
