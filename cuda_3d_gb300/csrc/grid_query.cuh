// grid_query.cuh -- device-side traversal of the row-hashed uniform grid.
#pragma once

#include "internal.cuh"

namespace gca3d
{

// visit the grid points of the 27 cells around p in the reference's scan order
// (x offset, then y offset, then z, then ascending original index; the order of
// nn_search_functor, src/geometry/cuda_nn_search.cu:164-206).  f(t, spos[t]).
template <class F>
__device__ __forceinline__ void grid_visit(const GridDev &g, const KeyLayout &L, int seg, float3 o, float3 p, F &&f)
{
    const int cx = cell_of(p.x, o.x, g.cell), cy = cell_of(p.y, o.y, g.cell), cz = cell_of(p.z, o.z, g.cell);
    const int mx = (1 << L.bx) - 1, my = (1 << L.by) - 1, mz = (1 << L.bz) - 1;
    if (cx < -1 || cx > mx + 1 || cy < -1 || cy > my + 1 || cz < -1 || cz > mz + 1)
        return;
    const unsigned long long segbits = (unsigned long long)seg << (L.bx + L.by);
    const int lo = cz - 1, hi = cz + 1;
    for (int dx = -1; dx <= 1; ++dx)
    {
        const int x = cx + dx;
        if (x < 0 || x > mx)
            continue;
        for (int dy = -1; dy <= 1; ++dy)
        {
            const int y = cy + dy;
            if (y < 0 || y > my)
                continue;
            const unsigned long long rk = segbits | ((unsigned long long)x << L.by) | (unsigned long long)y;
            const int2 r = row_lookup(g.hkeys, g.hvals, g.hmask, rk);
            int t = r.x;
            const int e = r.y;
            if (t >= e)
                continue;
            if (e - t > 16)
            {
                int a = t, b = e;
                while (a < b)
                {
                    int m = (a + b) >> 1;
                    if (__float_as_int(__ldg(&g.spos[m].w)) < lo)
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
                if (qz < lo)
                    continue;
                if (qz > hi)
                    break;
                f(t, q);
            }
        }
    }
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

} // namespace gca3d
