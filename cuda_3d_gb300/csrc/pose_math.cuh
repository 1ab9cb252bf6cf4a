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
