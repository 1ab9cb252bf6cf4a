// pose_math.cuh -- FP64 6x6 solve, pose maps and the per-correspondence rows of
// the colored-ICP objective, shared by the ICP kernels and their adjoint.
#pragma once

#include "internal.cuh"

namespace gca3d
{

// ---------------------------------------------------------------------------
// FP64 6x6 solve and pose maps (device; the oracle restates the same steps)
// ---------------------------------------------------------------------------
// exact selects on the bit patterns: a conditional written with ?: over a set of
// static indices is turned back into a runtime index by the compiler, which moves
// the array to local memory
__device__ __forceinline__ double bsel(bool s, double a, double b)
{
    const long long m = -(long long)s;
    return __longlong_as_double((__double_as_longlong(a) & m) | (__double_as_longlong(b) & ~m));
}
__device__ __forceinline__ int isel(bool s, int a, int b)
{
    const int m = -(int)s;
    return (a & m) | (b & ~m);
}

// Every loop is unrolled and every array index is a compile-time constant: the
// pivot's row / column exchange is a conditional swap (bsel) against each candidate
// row, so the matrix stays in registers (the solve is one thread's dependent FP64
// chain on the ICP critical path; in local memory it cost several times more).
__device__ inline int solve6_device(const double *S /* 21 upper + 6 rhs */, double x[6])
{
    constexpr double kTiny = 2.2250738585072014e-308;
    double A[6][6], b[6], D[6];
    int perm[6];
    int status = 0;
    {
        int u = 0;
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = i; j < 6; ++j)
            {
                A[i][j] = A[j][i] = S[u];
                ++u;
            }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        b[i] = -S[21 + i];
        perm[i] = i;
        if (!isfinite(b[i]))
            status = 1;
#pragma unroll
        for (int j = 0; j < 6; ++j)
            if (!isfinite(A[i][j]))
                status = 1;
    }
    if (status)
    {
#pragma unroll
        for (int i = 0; i < 6; ++i)
            x[i] = 0.0;
        return 1;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k)
    {
        // symmetric pivot: the largest remaining diagonal entry (first one on ties)
        int piv = k;
        double best = fabs(A[k][k]);
#pragma unroll
        for (int i = k + 1; i < 6; ++i)
        {
            const double v = fabs(A[i][i]);
            if (v > best)
            {
                best = v;
                piv = i;
            }
        }
#pragma unroll
        for (int i = k + 1; i < 6; ++i)
        {
            const bool sw = piv == i;
#pragma unroll
            for (int j = 0; j < 6; ++j)
            {
                const double t = A[k][j];
                A[k][j] = bsel(sw, A[i][j], t);
                A[i][j] = bsel(sw, t, A[i][j]);
            }
#pragma unroll
            for (int j = 0; j < 6; ++j)
            {
                const double t = A[j][k];
                A[j][k] = bsel(sw, A[j][i], t);
                A[j][i] = bsel(sw, t, A[j][i]);
            }
            const int tp = perm[k];
            perm[k] = isel(sw, perm[i], tp);
            perm[i] = isel(sw, tp, perm[i]);
        }
        D[k] = A[k][k];
        if (fabs(D[k]) <= kTiny)
        {
            status = 1;
#pragma unroll
            for (int i = k + 1; i < 6; ++i)
                A[i][k] = 0.0;
        }
        else
        {
            // one reciprocal per pivot: FP64 division is a long dependent sequence
            const double inv = 1.0 / D[k];
#pragma unroll
            for (int i = k + 1; i < 6; ++i)
                A[i][k] *= inv;
#pragma unroll
            for (int i = k + 1; i < 6; ++i)
#pragma unroll
                for (int j = k + 1; j <= i; ++j)
                {
                    A[i][j] -= A[i][k] * A[j][k] * D[k];
                    A[j][i] = A[i][j];
                }
        }
    }
    double y[6], z[6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 6; ++q)
            s = bsel(perm[i] == q, b[q], s);
#pragma unroll
        for (int j = 0; j < i; ++j)
            s -= A[i][j] * y[j];
        y[i] = s;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i)
        y[i] = fabs(D[i]) > kTiny ? y[i] / D[i] : 0.0;
#pragma unroll
    for (int i = 5; i >= 0; --i)
    {
        double s = y[i];
#pragma unroll
        for (int j = i + 1; j < 6; ++j)
            s -= A[j][i] * z[j];
        z[i] = s;
    }
#pragma unroll
    for (int q = 0; q < 6; ++q)
    {
        double v = 0.0;
#pragma unroll
        for (int i = 0; i < 6; ++i)
            v = bsel(perm[i] == q, z[i], v);
        x[q] = v;
    }
    return status;
}

// ---------------------------------------------------------------------------
// Warp-parallel restatements of solve6_device and pose_from_x_device for the
// per-iteration finalize.  FP64 issues at a small fraction of the FP32 rate on
// this part, so a single thread's dependent FP64 chain costs tens of
// microseconds; spread over the lanes of a warp, the chain is the depth of the
// computation instead of its length.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int tri_lane(int i, int j) { return i * (i + 1) / 2 + j; } // i >= j

// Short FP64 chains for the warp-parallel solve and step map, where each dependent
// FP64 operation costs tens of nanoseconds.
//
// rcp_nr: 1/d by Newton-Raphson, two steps (e = 1 - d r, r += r e; each step squares
// the relative error) from the approximate reciprocal rcp.approx.ftz.f64 (about
// 2^-20).  Within one unit in the last place of 1/d for normal d whose reciprocal
// is normal (0 for a reciprocal below the normal range); half the latency of the
// IEEE division.
__device__ __forceinline__ double rcp_nr(double d)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
    double e = fma(-d, r, 1.0);
    r = fma(r, e, r);
    e = fma(-d, r, 1.0);
    return fma(r, e, r);
}

// sin x and cos x for |x| <= kSmallAngle from their Taylor series (Horner in x^2,
// through x^13 and x^14; the first omitted terms are below 1e-18 relative)
constexpr double kSmallAngle = 0.25;
__device__ __forceinline__ void sincos_small(double x, double &s, double &c)
{
    const double z = x * x;
    double ps = 1.0 / 6227020800.0; // 1/13!
    double pc = 1.0 / 87178291200.0; // 1/14!
    ps = fma(ps, -z, 1.0 / 39916800.0);
    pc = fma(pc, -z, 1.0 / 479001600.0);
    ps = fma(ps, -z, 1.0 / 362880.0);
    pc = fma(pc, -z, 1.0 / 3628800.0);
    ps = fma(ps, -z, 1.0 / 5040.0);
    pc = fma(pc, -z, 1.0 / 40320.0);
    ps = fma(ps, -z, 1.0 / 120.0);
    pc = fma(pc, -z, 1.0 / 720.0);
    ps = fma(ps, -z, 1.0 / 6.0);
    pc = fma(pc, -z, 1.0 / 24.0);
    pc = fma(pc, -z, 0.5);
    s = fma(-x * z, ps, x);
    c = fma(-z, pc, 1.0);
}

// the coefficients of the SO(3) / SE(3) exponential, A = sin t / t,
// B = (1 - cos t) / t^2, C = (t - sin t) / t^3, as series in t2 = t^2 for
// t2 <= kSmallAngle^2 (A = sum (-t2)^n / (2n+1)!, B = sum (-t2)^n / (2n+2)!,
// C = sum (-t2)^n / (2n+3)!, n <= 6; the first omitted terms are below 1e-19)
__device__ __forceinline__ void exp_coeffs_small(double t2, double &A, double &B, double &C)
{
    double a = 1.0 / 6227020800.0, b = 1.0 / 87178291200.0, c = 1.0 / 1307674368000.0; // 1/13!, 1/14!, 1/15!
    a = fma(a, -t2, 1.0 / 39916800.0);
    b = fma(b, -t2, 1.0 / 479001600.0);
    c = fma(c, -t2, 1.0 / 6227020800.0);
    a = fma(a, -t2, 1.0 / 362880.0);
    b = fma(b, -t2, 1.0 / 3628800.0);
    c = fma(c, -t2, 1.0 / 39916800.0);
    a = fma(a, -t2, 1.0 / 5040.0);
    b = fma(b, -t2, 1.0 / 40320.0);
    c = fma(c, -t2, 1.0 / 362880.0);
    a = fma(a, -t2, 1.0 / 120.0);
    b = fma(b, -t2, 1.0 / 720.0);
    c = fma(c, -t2, 1.0 / 5040.0);
    a = fma(a, -t2, 1.0 / 6.0);
    b = fma(b, -t2, 1.0 / 24.0);
    c = fma(c, -t2, 1.0 / 120.0);
    A = fma(a, -t2, 1.0);
    B = fma(b, -t2, 0.5);
    C = fma(c, -t2, 1.0 / 6.0);
}

// solve6_device over one warp (same symmetric pivots, factorisation and
// substitutions; the backward substitution sums in the opposite order, and the
// reciprocals of the pivots are rcp_nr's).  Lane
// tri_lane(i, j) < 21 holds A[i][j] of the lower triangle, lanes 21..26 the
// right-hand side.  All 32 lanes call it; every lane returns the status and x.
__device__ inline int solve6_warp(const double *S /* 21 upper + 6 rhs */, double x[6])
{
    constexpr double kTiny = 2.2250738585072014e-308;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int li = 0;
    while (li < 5 && tri_lane(li + 1, 0) <= lane)
        ++li;
    const int lj = lane - tri_lane(li, 0);
    const bool mat = lane < 21, diag = mat && li == lj;
    double a = 0.0;
    if (mat)
        a = S[lj * 6 - lj * (lj - 1) / 2 + (li - lj)]; // upper-packed (lj, li)
    else if (lane < 27)
        a = -S[lane];
    const bool bad = lane < 27 && !isfinite(a);
#pragma unroll
    for (int q = 0; q < 6; ++q)
        x[q] = 0.0;
    if (__any_sync(full, bad))
        return 1;
    unsigned perm = 0x543210u; // 4 bits per entry
    int status = 0;
#pragma unroll
    for (int k = 0; k < 6; ++k)
    {
        // every diagonal lane's reciprocal, computed while the pivot is searched (the
        // chosen one is broadcast below, so the division is off the pivot's chain)
        const double ra = diag ? rcp_nr(a) : 0.0;
        // symmetric pivot: the largest remaining diagonal entry (first one on ties);
        // magnitudes compared as the bit patterns of |A[i][i]|
        const long long mag = diag ? (__double_as_longlong(a) & 0x7fffffffffffffffll) : -1ll;
        int piv = k;
        long long best = __shfl_sync(full, mag, tri_lane(k, k));
#pragma unroll
        for (int i = k + 1; i < 6; ++i)
        {
            const long long v = __shfl_sync(full, mag, tri_lane(i, i));
            if (v > best)
            {
                best = v;
                piv = i;
            }
        }
        if (piv != k)
        {
            const int si = li == k ? piv : (li == piv ? k : li), sj = lj == k ? piv : (lj == piv ? k : lj);
            const int src = mat ? tri_lane(max(si, sj), min(si, sj)) : lane;
            a = __shfl_sync(full, a, src);
            const unsigned pk = (perm >> (4 * k)) & 15u, pp = (perm >> (4 * piv)) & 15u;
            perm = (perm & ~((15u << (4 * k)) | (15u << (4 * piv)))) | (pp << (4 * k)) | (pk << (4 * piv));
        }
        const double Dk = __shfl_sync(full, a, tri_lane(k, k));
        const double rk = __shfl_sync(full, ra, tri_lane(piv, piv)); // 1 / Dk (before the swap)
        const bool lcol = mat && lj == k && li > k;
        if (fabs(Dk) <= kTiny)
        {
            status = 1;
            if (lcol)
                a = 0.0;
        }
        else
        {
            const double inv = rk; // one reciprocal per pivot
            if (lcol)
                a *= inv;
            const bool upd = mat && lj > k;
            const double lik = __shfl_sync(full, a, upd ? tri_lane(li, k) : lane);
            const double ljk = __shfl_sync(full, a, upd ? tri_lane(lj, k) : lane);
            if (upd)
                a -= lik * ljk * Dk;
        }
    }
    // L y = P b (the diagonal lanes accumulate), then y / D
    const int pi = (int)((perm >> (4 * li)) & 15u);
    double acc = __shfl_sync(full, a, diag ? 21 + pi : lane);
#pragma unroll
    for (int j = 0; j < 5; ++j)
    {
        const double yj = __shfl_sync(full, acc, tri_lane(j, j));
        const double lij = __shfl_sync(full, a, diag && li > j ? tri_lane(li, j) : lane);
        if (diag && li > j)
            acc -= lij * yj;
    }
    if (diag)
        acc = fabs(a) > kTiny ? acc * rcp_nr(a) : 0.0;
    // L^T z = y, by columns from the last
#pragma unroll
    for (int j = 5; j > 0; --j)
    {
        const double zj = __shfl_sync(full, acc, tri_lane(j, j));
        const double lji = __shfl_sync(full, a, diag && li < j ? tri_lane(j, li) : lane);
        if (diag && li < j)
            acc -= lji * zj;
    }
    // x[perm[i]] = z[i]
    unsigned invp = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
        invp |= (unsigned)i << (4 * ((perm >> (4 * i)) & 15u));
#pragma unroll
    for (int q = 0; q < 6; ++q)
    {
        const int iq = (int)((invp >> (4 * q)) & 15u);
        x[q] = __shfl_sync(full, acc, tri_lane(iq, iq));
    }
    return status;
}

// pose_from_x_device over one warp: every lane returns Ti[lane] for lane < 16
// (row-major 4x4), the same formulas with one matrix entry per lane.  The three
// sines and cosines of the Euler map are on separate lanes (sincos_small up to
// kSmallAngle); the exponential's coefficients are exp_coeffs_small's series up to
// a rotation of kSmallAngle, else three divisions on separate lanes.
__device__ inline double pose_from_x_warp(const double x[6], int map)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int r = (lane >> 2) & 3, c = lane & 3; // the Ti entry of this lane
    const int rr = min(r, 2), cc = min(c, 2);  // its 3x3 entry (clamped for the 4th row / column)
    double Rrc, tr;
    if (map == GCA3D_UPDATE_EULER_ZYX)
    {
        const int m = lane % 3;
        const double xm = m == 0 ? x[0] : (m == 1 ? x[1] : x[2]);
        double sn, cs;
        if (fabs(xm) <= kSmallAngle)
            sincos_small(xm, sn, cs);
        else
            sincos(xm, &sn, &cs);
        const double sa = __shfl_sync(full, sn, 0), ca = __shfl_sync(full, cs, 0);
        const double sb = __shfl_sync(full, sn, 1), cb = __shfl_sync(full, cs, 1);
        const double sc = __shfl_sync(full, sn, 2), ccz = __shfl_sync(full, cs, 2);
        // R = Rz(x2) Ry(x1) Rx(x0), entry (rr, cc) as u * v * w + g0 * g1 with
        // operands picked per lane (one uniform FP64 expression, no divergence)
        const int e = 3 * rr + cc;
        const double u = rr == 0 ? ccz : (rr == 1 ? sc : (cc == 0 ? -sb : cb));
        const double v = e == 0 || e == 3 ? cb : (e == 6 ? 1.0 : (rr == 2 ? (cc == 1 ? sa : ca) : sb));
        const double w = cc == 0 || rr == 2 ? 1.0 : (cc == 1 ? sa : ca);
        const double g0 = cc == 0 || rr == 2 ? 0.0 : (e == 1 ? -sc : (e == 2 ? sc : (e == 4 ? ccz : -ccz)));
        const double g1 = cc == 0 || rr == 2 ? 0.0 : (cc == 1 ? ca : sa);
        Rrc = u * v * w + g0 * g1;
        tr = rr == 0 ? x[3] : (rr == 1 ? x[4] : x[5]);
    }
    else
    {
        const double w0 = x[0], w1 = x[1], w2 = x[2];
        const double th2 = w0 * w0 + w1 * w1 + w2 * w2;
        double A, B, C;
        if (th2 <= kSmallAngle * kSmallAngle)
            exp_coeffs_small(th2, A, B, C); // no root, sine or division on the chain
        else
        {
            const double th = sqrt(th2);
            double sn, cs;
            sincos(th, &sn, &cs);
            // the three coefficient divisions on three lanes
            const int m = lane % 3;
            const double num = m == 0 ? sn : (m == 1 ? 1.0 - cs : th - sn);
            const double den = m == 0 ? th : (m == 1 ? th2 : th2 * th);
            const double q = num * rcp_nr(den);
            A = __shfl_sync(full, q, 0);
            B = __shfl_sync(full, q, 1);
            C = __shfl_sync(full, q, 2);
        }
        const double K[3][3] = {{0, -w2, w1}, {w2, 0, -w0}, {-w1, w0, 0}};
        auto Kat = [&](int i, int j) { return i == 0 ? (j == 0 ? K[0][0] : j == 1 ? K[0][1] : K[0][2])
                                             : i == 1 ? (j == 0 ? K[1][0] : j == 1 ? K[1][1] : K[1][2])
                                                      : (j == 0 ? K[2][0] : j == 1 ? K[2][1] : K[2][2]); };
        const double Kij = Kat(rr, cc);
        const double k2 = Kat(rr, 0) * Kat(0, cc) + Kat(rr, 1) * Kat(1, cc) + Kat(rr, 2) * Kat(2, cc);
        const double I = rr == cc ? 1.0 : 0.0;
        Rrc = I + A * Kij + B * k2;
        const double Vrc = I + B * Kij + C * k2; // this lane's V entry (rr, cc)
        // t[rr] = V[rr][0] x3 + V[rr][1] x4 + V[rr][2] x5, V from the lanes 4 rr + 0..2
        const double v0 = __shfl_sync(full, Vrc, 4 * rr), v1 = __shfl_sync(full, Vrc, 4 * rr + 1),
                     v2 = __shfl_sync(full, Vrc, 4 * rr + 2);
        tr = v0 * x[3] + v1 * x[4] + v2 * x[5];
    }
    if (r == 3)
        return c == 3 ? 1.0 : 0.0;
    return c == 3 ? tr : Rrc;
}

__device__ inline void pose_from_x_device(const double x[6], int map, double T[16])
{
    double R[3][3], t[3];
    if (map == GCA3D_UPDATE_EULER_ZYX)
    {
        double sa, ca, sb, cb, sc, cc;
        sincos(x[0], &sa, &ca);
        sincos(x[1], &sb, &cb);
        sincos(x[2], &sc, &cc);
        R[0][0] = cc * cb;
        R[0][1] = cc * sb * sa - sc * ca;
        R[0][2] = cc * sb * ca + sc * sa;
        R[1][0] = sc * cb;
        R[1][1] = sc * sb * sa + cc * ca;
        R[1][2] = sc * sb * ca - cc * sa;
        R[2][0] = -sb;
        R[2][1] = cb * sa;
        R[2][2] = cb * ca;
        t[0] = x[3], t[1] = x[4], t[2] = x[5];
    }
    else
    {
        const double w0 = x[0], w1 = x[1], w2 = x[2];
        const double th2 = w0 * w0 + w1 * w1 + w2 * w2, th = sqrt(th2);
        double A, B, C;
        if (th < 1e-4)
        {
            A = 1.0 - th2 / 6.0 + th2 * th2 / 120.0;
            B = 0.5 - th2 / 24.0 + th2 * th2 / 720.0;
            C = 1.0 / 6.0 - th2 / 120.0 + th2 * th2 / 5040.0;
        }
        else
        {
            double s, c;
            sincos(th, &s, &c);
            A = s / th;
            B = (1.0 - c) / th2;
            C = (th - s) / (th2 * th);
        }
        const double K[3][3] = {{0, -w2, w1}, {w2, 0, -w0}, {-w1, w0, 0}};
        double V[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
            {
                double k2 = K[i][0] * K[0][j] + K[i][1] * K[1][j] + K[i][2] * K[2][j];
                double I = i == j ? 1.0 : 0.0;
                R[i][j] = I + A * K[i][j] + B * k2;
                V[i][j] = I + B * K[i][j] + C * k2;
            }
        for (int i = 0; i < 3; ++i)
            t[i] = V[i][0] * x[3] + V[i][1] * x[4] + V[i][2] * x[5];
    }
    for (int i = 0; i < 3; ++i)
    {
        for (int j = 0; j < 3; ++j)
            T[4 * i + j] = R[i][j];
        T[4 * i + 3] = t[i];
    }
    T[12] = T[13] = T[14] = 0.0;
    T[15] = 1.0;
}

// dU/dx_m of the pose map as 3x4 row-major blocks (the adjoint of a step).
// Euler ZYX: U = Rz(x2) Ry(x1) Rx(x0), t = x3..5.  SE(3) exponential:
// R = I + A K + B K^2, t = (I + B K + C K^2) v with K = [w]x, differentiated
// through A, B, C as functions of theta^2 (series below theta = 1e-2).
__device__ inline void mat3_mul(const double *A, const double *B, double *C)
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}

__device__ inline void pose_jacobian_device(const double x[6], int map, double dU[6][12])
{
    for (int m = 0; m < 6; ++m)
        for (int k = 0; k < 12; ++k)
            dU[m][k] = 0.0;
    if (map == GCA3D_UPDATE_EULER_ZYX)
    {
        double sa, ca, sb, cb, sc, cc;
        sincos(x[0], &sa, &ca);
        sincos(x[1], &sb, &cb);
        sincos(x[2], &sc, &cc);
        const double Rx[9] = {1, 0, 0, 0, ca, -sa, 0, sa, ca}, dRx[9] = {0, 0, 0, 0, -sa, -ca, 0, ca, -sa};
        const double Ry[9] = {cb, 0, sb, 0, 1, 0, -sb, 0, cb}, dRy[9] = {-sb, 0, cb, 0, 0, 0, -cb, 0, -sb};
        const double Rz[9] = {cc, -sc, 0, sc, cc, 0, 0, 0, 1}, dRz[9] = {-sc, -cc, 0, cc, -sc, 0, 0, 0, 0};
        for (int m = 0; m < 3; ++m)
        {
            double M1[9], M2[9];
            mat3_mul(m == 2 ? dRz : Rz, m == 1 ? dRy : Ry, M1);
            mat3_mul(M1, m == 0 ? dRx : Rx, M2);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    dU[m][4 * i + j] = M2[3 * i + j];
        }
        for (int i = 0; i < 3; ++i)
            dU[3 + i][4 * i + 3] = 1.0;
        return;
    }
    const double w[3] = {x[0], x[1], x[2]}, v[3] = {x[3], x[4], x[5]};
    const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2], th = sqrt(th2);
    double A, B, C, Ad, Bd, Cd;
    if (th < 1e-2)
    {
        const double t4 = th2 * th2, t6 = t4 * th2;
        A = 1.0 - th2 / 6.0 + t4 / 120.0 - t6 / 5040.0;
        B = 0.5 - th2 / 24.0 + t4 / 720.0 - t6 / 40320.0;
        C = 1.0 / 6.0 - th2 / 120.0 + t4 / 5040.0 - t6 / 362880.0;
        Ad = -1.0 / 6.0 + th2 / 60.0 - t4 / 1680.0;
        Bd = -1.0 / 24.0 + th2 / 360.0 - t4 / 13440.0;
        Cd = -1.0 / 120.0 + th2 / 2520.0 - t4 / 120960.0;
    }
    else
    {
        double s, c;
        sincos(th, &s, &c);
        A = s / th;
        B = (1.0 - c) / th2;
        C = (th - s) / (th2 * th);
        Ad = (th * c - s) / (2.0 * th2 * th);
        Bd = (th * s - 2.0 * (1.0 - c)) / (2.0 * th2 * th2);
        Cd = ((1.0 - c) * th - 3.0 * (th - s)) / (2.0 * th2 * th2 * th);
    }
    const double K[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
    double K2[9];
    mat3_mul(K, K, K2);
    for (int m = 0; m < 3; ++m)
    {
        double G[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}; // [e_m]x
        if (m == 0)
            G[5] = -1, G[7] = 1;
        else if (m == 1)
            G[2] = 1, G[6] = -1;
        else
            G[1] = -1, G[3] = 1;
        double GK[9], KG[9];
        mat3_mul(G, K, GK);
        mat3_mul(K, G, KG);
        double dV[9];
        for (int k = 0; k < 9; ++k)
        {
            const double sym = GK[k] + KG[k];
            dU[m][4 * (k / 3) + k % 3] = 2.0 * w[m] * Ad * K[k] + A * G[k] + 2.0 * w[m] * Bd * K2[k] + B * sym;
            dV[k] = 2.0 * w[m] * Bd * K[k] + B * G[k] + 2.0 * w[m] * Cd * K2[k] + C * sym;
        }
        for (int i = 0; i < 3; ++i)
            dU[m][4 * i + 3] = dV[3 * i] * v[0] + dV[3 * i + 1] * v[1] + dV[3 * i + 2] * v[2];
    }
    for (int m = 0; m < 3; ++m)
        for (int i = 0; i < 3; ++i)
            dU[3 + m][4 * i + 3] = (i == m ? 1.0 : 0.0) + B * K[3 * i + m] + C * K2[3 * i + m];
}

// ---------------------------------------------------------------------------
// per-correspondence terms (cuda_color_icp_build_least_square.cu:184-253)
// ---------------------------------------------------------------------------
struct GNTerms
{
    float Jg[6], Jc[6];
    float rg, rc;
};

__device__ __forceinline__ void gn_terms(float3 p, float Is, float3 q, float Iq, float3 n, float3 d, float slg,
                                         float slc, GNTerms &o)
{
    const float rg_ = (p.x - q.x) * n.x + (p.y - q.y) * n.y + (p.z - q.z) * n.z;
    o.Jg[0] = slg * (p.y * n.z - p.z * n.y);
    o.Jg[1] = slg * (p.z * n.x - p.x * n.z);
    o.Jg[2] = slg * (p.x * n.y - p.y * n.x);
    o.Jg[3] = slg * n.x;
    o.Jg[4] = slg * n.y;
    o.Jg[5] = slg * n.z;
    o.rg = slg * rg_;
    // d^T (I - n n^T)
    const float nd = n.x * d.x + n.y * d.y + n.z * d.z;
    const float tx = d.x - nd * n.x, ty = d.y - nd * n.y, tz = d.z - nd * n.z;
    o.Jc[0] = slc * (p.y * tz - p.z * ty);
    o.Jc[1] = slc * (p.z * tx - p.x * tz);
    o.Jc[2] = slc * (p.x * ty - p.y * tx);
    o.Jc[3] = slc * tx;
    o.Jc[4] = slc * ty;
    o.Jc[5] = slc * tz;
    // photometric residual on the tangent plane
    const float px = p.x - rg_ * n.x, py = p.y - rg_ * n.y, pz = p.z - rg_ * n.z;
    const float Iproj = Iq + (d.x * (px - q.x) + d.y * (py - q.y) + d.z * (pz - q.z));
    o.rc = slc * (Iproj - Is);
}

// FP32 pose (row-major 3x4) applied to a point, as explicit fused multiply-adds
// x' = fma(r0, x, fma(r1, y, fma(r2, z, t))) so that a CPU check can reproduce it
__device__ __forceinline__ float3 apply_pose(const float *T, float4 s)
{
    return make_float3(__fmaf_rn(T[0], s.x, __fmaf_rn(T[1], s.y, __fmaf_rn(T[2], s.z, T[3]))),
                       __fmaf_rn(T[4], s.x, __fmaf_rn(T[5], s.y, __fmaf_rn(T[6], s.z, T[7]))),
                       __fmaf_rn(T[8], s.x, __fmaf_rn(T[9], s.y, __fmaf_rn(T[10], s.z, T[11]))));
}

} // namespace gca3d
