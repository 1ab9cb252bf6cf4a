// normals.cu -- fused PCA normals and colour gradients over a grid's own points.
//
// reference: cuda_estimate_normals (src/geometry/cuda_estimate_normals.cu:46-199) and
// compute_color_gradient_functor (src/registration/cuda_compute_color_gradient.cu:13-90).
//
// The reference materialises CSR neighbour lists, expands them to per-neighbour
// moment vectors and reduces by key.  Here one thread walks its 27-cell
// neighbourhood in the grid (points already in cell order) and accumulates in
// registers; no lists exist.  Moments are taken about the query point, so the
// FP32 covariance does not cancel at metre-scale coordinates (the reference's
// E[xx^T] - E[x]E[x]^T does).  The 3x3 eigen-problem is solved in closed form in
// FP32; points whose two smallest eigenvalues are close (a few dozen per frame)
// are queued and redone by a second kernel with the covariance rebuilt in FP64
// and a closed-form FP64 eigen-solve, one warp per point (FP64 issues at a small
// fraction of the FP32 rate here, so the work is spread over lanes, and a
// divergent fallback inside the FP32 kernel would stall whole warps).  A third
// kernel computes the gradients.  The gradient follows the reference's
// system: tangent-plane least squares, (knn - 1)^2 n n^T orthogonality term,
// 1e-6 ridge, LDL^T solve (in the tangent/normal basis, see solve_gradient_system).
#include "grid_query.cuh"
#include "stages.cuh"

#include <algorithm>

namespace gca3d
{

constexpr int kMaxNN = 64;

// FP64 eigenvector of the smallest eigenvalue of a symmetric 3x3 whose two smallest
// eigenvalues may be close (the points the FP32 pass queues).  The largest
// eigenvalue is then well separated: it comes from the trigonometric formula and
// its eigenvector v1 from the largest cross product of the rows of A - l1 I.  The
// other two eigenvectors span the plane orthogonal to v1; in an orthonormal basis
// (u, w) of that plane A is a 2x2 symmetric matrix, which one rotation (the
// Jacobi rotation of the oracle's sweeps) diagonalises exactly.  The result is
// accurate to eps / gap like the sweeps, at about a quarter of their FP64
// instructions (FP64 issues at a small fraction of the FP32 rate here, and this is
// one thread's dependent chain).  An isotropic matrix gives (1, 0, 0), as the
// sweeps do (no rotation, first of equal diagonal entries).
__device__ void smallest_eigvec_f64(const double A[3][3], double out[3])
{
    double m = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j)
            m = fmax(m, fabs(A[i][j]));
    out[0] = 1.0, out[1] = 0.0, out[2] = 0.0;
    if (!(m > 0.0))
        return;
    const double inv = 1.0 / m;
    const double a00 = A[0][0] * inv, a01 = A[0][1] * inv, a02 = A[0][2] * inv;
    const double a11 = A[1][1] * inv, a12 = A[1][2] * inv, a22 = A[2][2] * inv;
    const double q = (a00 + a11 + a22) * (1.0 / 3.0);
    const double b00 = a00 - q, b11 = a11 - q, b22 = a22 - q;
    const double p2 = (b00 * b00 + b11 * b11 + b22 * b22 + 2.0 * (a01 * a01 + a02 * a02 + a12 * a12)) * (1.0 / 6.0);
    if (!(p2 > 0.0))
        return;
    const double p = sqrt(p2);
    const double det = b00 * (b11 * b22 - a12 * a12) - a01 * (a01 * b22 - a12 * a02) + a02 * (a01 * a12 - b11 * a02);
    const double r = fmin(fmax(det / (2.0 * p2 * p), -1.0), 1.0);
    const double l1 = q + 2.0 * p * cos(acos(r) * (1.0 / 3.0));
    // v1: the null vector of A - l1 I
    const double r0[3] = {a00 - l1, a01, a02}, r1[3] = {a01, a11 - l1, a12}, r2[3] = {a02, a12, a22 - l1};
    auto cross = [](const double *x, const double *y, double *z) {
        z[0] = x[1] * y[2] - x[2] * y[1];
        z[1] = x[2] * y[0] - x[0] * y[2];
        z[2] = x[0] * y[1] - x[1] * y[0];
    };
    double c0[3], c1[3], c2[3];
    cross(r0, r1, c0);
    cross(r0, r2, c1);
    cross(r1, r2, c2);
    const double d0 = c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2];
    const double d1 = c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2];
    const double d2 = c2[0] * c2[0] + c2[1] * c2[1] + c2[2] * c2[2];
    const double *c = c0;
    double dm = d0;
    if (d1 > dm)
        c = c1, dm = d1;
    if (d2 > dm)
        c = c2, dm = d2;
    if (!(dm > 0.0))
        return;
    const double il = 1.0 / sqrt(dm);
    const double v1[3] = {c[0] * il, c[1] * il, c[2] * il};
    // orthonormal basis (u, w) of the plane orthogonal to v1
    double u[3];
    if (fabs(v1[0]) > fabs(v1[1]))
    {
        const double iu = 1.0 / sqrt(v1[0] * v1[0] + v1[2] * v1[2]);
        u[0] = -v1[2] * iu, u[1] = 0.0, u[2] = v1[0] * iu;
    }
    else
    {
        const double iu = 1.0 / sqrt(v1[1] * v1[1] + v1[2] * v1[2]);
        u[0] = 0.0, u[1] = v1[2] * iu, u[2] = -v1[1] * iu;
    }
    double w[3];
    cross(v1, u, w);
    const double Au[3] = {a00 * u[0] + a01 * u[1] + a02 * u[2], a01 * u[0] + a11 * u[1] + a12 * u[2],
                          a02 * u[0] + a12 * u[1] + a22 * u[2]};
    const double Aw[3] = {a00 * w[0] + a01 * w[1] + a02 * w[2], a01 * w[0] + a11 * w[1] + a12 * w[2],
                          a02 * w[0] + a12 * w[1] + a22 * w[2]};
    const double m00 = u[0] * Au[0] + u[1] * Au[1] + u[2] * Au[2];
    const double m01 = u[0] * Aw[0] + u[1] * Aw[1] + u[2] * Aw[2];
    const double m11 = w[0] * Aw[0] + w[1] * Aw[1] + w[2] * Aw[2];
    double e[3];
    if (m01 == 0.0)
    {
        const double *s = m00 <= m11 ? u : w;
        e[0] = s[0], e[1] = s[1], e[2] = s[2];
    }
    else
    {
        // rotation by (c, s): eigenvalue m00 - t m01 on c u - s w, m11 + t m01 on s u + c w
        const double theta = (m11 - m00) / (2.0 * m01);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double cr = 1.0 / sqrt(t * t + 1.0), sr = t * cr;
        if (m00 - t * m01 <= m11 + t * m01)
            for (int k = 0; k < 3; ++k)
                e[k] = cr * u[k] - sr * w[k];
        else
            for (int k = 0; k < 3; ++k)
                e[k] = sr * u[k] + cr * w[k];
    }
    const double ie = 1.0 / sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    out[0] = e[0] * ie, out[1] = e[1] * ie, out[2] = e[2] * ie;
}

// closed-form symmetric 3x3 eigen-system (trigonometric eigenvalues, eigenvector
// of the smallest one from cross products of the rows of A - lambda I).
// Returns false when the smallest eigenvalue is not well separated.
__device__ bool smallest_eigvec_f32(float a00, float a01, float a02, float a11, float a12, float a22, float3 &n)
{
    float m = fmaxf(fmaxf(fmaxf(fabsf(a00), fabsf(a01)), fmaxf(fabsf(a02), fabsf(a11))), fmaxf(fabsf(a12), fabsf(a22)));
    if (!(m > 0.0f))
        return false;
    const float inv = 1.0f / m;
    a00 *= inv, a01 *= inv, a02 *= inv, a11 *= inv, a12 *= inv, a22 *= inv;
    const float q = (a00 + a11 + a22) * (1.0f / 3.0f);
    const float b00 = a00 - q, b11 = a11 - q, b22 = a22 - q;
    const float off = a01 * a01 + a02 * a02 + a12 * a12;
    const float p2 = (b00 * b00 + b11 * b11 + b22 * b22 + 2.0f * off) * (1.0f / 6.0f);
    if (!(p2 > 0.0f))
        return false;
    const float p = sqrtf(p2);
    const float det = b00 * (b11 * b22 - a12 * a12) - a01 * (a01 * b22 - a12 * a02) + a02 * (a01 * a12 - b11 * a02);
    float r = det / (2.0f * p2 * p);
    r = fminf(fmaxf(r, -1.0f), 1.0f);
    const float phi = acosf(r) * (1.0f / 3.0f);
    const float lmax = q + 2.0f * p * cosf(phi);
    float lmin = q + 2.0f * p * cosf(phi + 2.0943951023931957f);
    const float lmid = 3.0f * q - lmax - lmin;
    if (!(lmid - lmin > 1e-3f * (lmax - lmin)))
        return false;
    // One Newton step on det(A - l I) = 0 from the trigonometric lmin.  Where two
    // eigenvalues are close, r is near +-1 and acos(r) is ill-conditioned, so lmin
    // carries an error of order sqrt(eps) p; the cross products below turn an error d in
    // lmin into an angle of about d / (lmid - lmin).  With B = A - lmin I the step is
    // lmin += det(B) / (sum of the principal 2x2 minors of B), the minors' sum being
    // -d/dl det(A - l I); it is about (lmid - lmin)(lmax - lmin) > 0 here.
    {
        const float c0 = a00 - lmin, c1 = a11 - lmin, c2 = a22 - lmin;
        const float m2 = (c0 * c1 - a01 * a01) + (c0 * c2 - a02 * a02) + (c1 * c2 - a12 * a12);
        const float dB = c0 * (c1 * c2 - a12 * a12) - a01 * (a01 * c2 - a12 * a02) + a02 * (a01 * a12 - c1 * a02);
        if (m2 > 0.0f)
            lmin += dB / m2;
    }
    const float3 r0 = make_float3(a00 - lmin, a01, a02);
    const float3 r1 = make_float3(a01, a11 - lmin, a12);
    const float3 r2 = make_float3(a02, a12, a22 - lmin);
    const float3 c0 = make_float3(r0.y * r1.z - r0.z * r1.y, r0.z * r1.x - r0.x * r1.z, r0.x * r1.y - r0.y * r1.x);
    const float3 c1 = make_float3(r0.y * r2.z - r0.z * r2.y, r0.z * r2.x - r0.x * r2.z, r0.x * r2.y - r0.y * r2.x);
    const float3 c2 = make_float3(r1.y * r2.z - r1.z * r2.y, r1.z * r2.x - r1.x * r2.z, r1.x * r2.y - r1.y * r2.x);
    const float d0 = c0.x * c0.x + c0.y * c0.y + c0.z * c0.z;
    const float d1 = c1.x * c1.x + c1.y * c1.y + c1.z * c1.z;
    const float d2 = c2.x * c2.x + c2.y * c2.y + c2.z * c2.z;
    float3 c = c0;
    float d = d0;
    if (d1 > d)
        c = c1, d = d1;
    if (d2 > d)
        c = c2, d = d2;
    if (!(d > 1e-20f))
        return false;
    const float il = rsqrtf(d);
    n = make_float3(c.x * il, c.y * il, c.z * il);
    return true;
}

// LDL^T solve of a symmetric 3x3 (little_3x3_ldlt_solve.cuh:6-67 factorisation)
__device__ __forceinline__ float3 ldlt3(float A00, float A01, float A02, float A11, float A12, float A22, float b0,
                                        float b1, float b2)
{
    const float D0 = A00, L10 = A01 / D0, L20 = A02 / D0;
    const float D1 = A11 - L10 * L10 * D0;
    const float L21 = (A12 - L10 * L20 * D0) / D1;
    const float D2 = A22 - L20 * L20 * D0 - L21 * L21 * D1;
    float x0 = b0, x1 = b1 - L10 * x0, x2 = b2 - L20 * x0 - L21 * x1;
    x0 /= D0, x1 /= D1, x2 /= D2;
    x1 -= L21 * x2;
    x0 -= L10 * x1 + L20 * x2;
    return make_float3(x0, x1, x2);
}

// The colour-gradient system of compute_color_gradient_functor
// (cuda_compute_color_gradient.cu:57-88):  (sum v v^T + w n n^T + 1e-6 I) d = sum v dI
// with w = (knn - 1)^2.  The w n n^T term is ~1e4-1e5 times the tangent entries, so
// the xyz-basis LDL^T loses most FP32 digits.  The same system is solved in the
// orthonormal basis (t1, t2, n): there the large term sits on the last diagonal
// entry only and the tangent block factors first, at full FP32 accuracy.
__device__ __forceinline__ float3 solve_gradient_system(float A00, float A01, float A02, float A11, float A12,
                                                        float A22, float b0, float b1, float b2, float3 n, float w)
{
    const float nn = n.x * n.x + n.y * n.y + n.z * n.z;
    if (!(nn > 0.0f))
        return ldlt3(A00 + 1.0e-6f, A01, A02, A11 + 1.0e-6f, A12, A22 + 1.0e-6f, b0, b1, b2);
    float3 t1;
    if (fabsf(n.x) > fabsf(n.y))
    {
        const float il = rsqrtf(n.x * n.x + n.z * n.z);
        t1 = make_float3(-n.z * il, 0.0f, n.x * il);
    }
    else
    {
        const float il = rsqrtf(n.y * n.y + n.z * n.z);
        t1 = make_float3(0.0f, n.z * il, -n.y * il);
    }
    const float3 t2 = make_float3(n.y * t1.z - n.z * t1.y, n.z * t1.x - n.x * t1.z, n.x * t1.y - n.y * t1.x);
    const float3 e[3] = {t1, t2, n};
    float3 Ae[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        Ae[k] = make_float3(A00 * e[k].x + A01 * e[k].y + A02 * e[k].z, A01 * e[k].x + A11 * e[k].y + A12 * e[k].z,
                            A02 * e[k].x + A12 * e[k].y + A22 * e[k].z);
    auto dot3 = [](float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; };
    const float m00 = dot3(e[0], Ae[0]) + 1.0e-6f, m01 = dot3(e[0], Ae[1]), m02 = dot3(e[0], Ae[2]);
    const float m11 = dot3(e[1], Ae[1]) + 1.0e-6f, m12 = dot3(e[1], Ae[2]);
    const float m22 = dot3(e[2], Ae[2]) + w * nn + 1.0e-6f;
    const float3 b = make_float3(b0, b1, b2);
    const float3 y = ldlt3(m00, m01, m02, m11, m12, m22, dot3(e[0], b), dot3(e[1], b), dot3(e[2], b));
    return make_float3(y.x * t1.x + y.y * t2.x + y.z * n.x, y.x * t1.y + y.y * t2.y + y.z * n.y,
                       y.x * t1.z + y.y * t2.z + y.z * n.z);
}

struct NbrEntry
{
    float d2;
    int idx; // batch index (original order)
    int t;   // grid position
};

// the max_nn nearest neighbours inside rn2 (distance, then index), ascending
__device__ __forceinline__ int select_knn(const GridDev &g, const GridRows &R, float3 p, float rn2, int max_nn,
                                          NbrEntry *list)
{
    int cnt = 0;
    grid_scan(g, R, [&](int t, float4 q) {
        const float d2 = dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z);
        if (!(d2 < rn2))
            return;
        const int idx = g.sidx[t];
        if (cnt == max_nn)
        {
            const NbrEntry &w = list[cnt - 1];
            if (!(d2 < w.d2 || (d2 == w.d2 && idx < w.idx)))
                return;
            --cnt;
        }
        int j = cnt;
        while (j > 0 && (list[j - 1].d2 > d2 || (list[j - 1].d2 == d2 && list[j - 1].idx > idx)))
        {
            list[j] = list[j - 1];
            --j;
        }
        list[j] = NbrEntry{d2, idx, t};
        ++cnt;
    });
    return cnt;
}

struct NormalOut
{
    float4 *attr0;    // grid order {n, intensity}, or null
    float4 *nrm_out;  // original order {n, 0}, or null
    int *degen_count; // near-degenerate points, appended for the FP64 pass
    int *degen_list;
    // fused colour gradients (when grad_r2 > 0): outputs as k_gradient's, and the
    // gradient moments of the queued points (three float4 per queue slot)
    float grad_r2;
    float4 *attr1, *grd_out;
    float4 *degen_mom;
};

// The colour gradient from moments about the point p: G = sum d d^T (xx, xy, xz, yy,
// yz, zz) and m = sum d (I_q - I_p) over the points within the gradient radius
// (knn of them, p included), d = q - p.  The reference's system (sum v v^T +
// (knn - 1)^2 n n^T + 1e-6 I) x = sum v dI with v = d - (d . n) n has sum v v^T =
// P G P and sum v dI = P m (P = I - n n^T), so the neighbours need not be walked
// again once n is known.  In the orthonormal basis (t1, t2, n) of
// solve_gradient_system the projected terms have no normal row or column: the
// tangent block is t^T G t, the normal entry (knn - 1)^2 |n|^2 + 1e-6, and the
// right-hand side (t1 . m, t2 . m, 0).
__device__ __forceinline__ float3 gradient_from_moments(float g0, float g1, float g2, float g3, float g4, float g5,
                                                        float3 m, int knn, float3 n)
{
    const float G[6] = {g0, g1, g2, g3, g4, g5};
    if (knn < 5)
        return make_float3(0.0f, 0.0f, 0.0f);
    const float w = (float)((knn - 1) * (knn - 1));
    const float nn = n.x * n.x + n.y * n.y + n.z * n.z;
    if (!(nn > 0.0f))
        return ldlt3(G[0] + 1.0e-6f, G[1], G[2], G[3] + 1.0e-6f, G[4], G[5] + 1.0e-6f, m.x, m.y, m.z);
    float3 t1;
    if (fabsf(n.x) > fabsf(n.y))
    {
        const float il = rsqrtf(n.x * n.x + n.z * n.z);
        t1 = make_float3(-n.z * il, 0.0f, n.x * il);
    }
    else
    {
        const float il = rsqrtf(n.y * n.y + n.z * n.z);
        t1 = make_float3(0.0f, n.z * il, -n.y * il);
    }
    const float3 t2 = make_float3(n.y * t1.z - n.z * t1.y, n.z * t1.x - n.x * t1.z, n.x * t1.y - n.y * t1.x);
    auto Gx = [&](float3 v) {
        return make_float3(G[0] * v.x + G[1] * v.y + G[2] * v.z, G[1] * v.x + G[3] * v.y + G[4] * v.z,
                           G[2] * v.x + G[4] * v.y + G[5] * v.z);
    };
    auto dot3 = [](float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; };
    const float3 Gt1 = Gx(t1), Gt2 = Gx(t2);
    const float3 y = ldlt3(dot3(t1, Gt1) + 1.0e-6f, dot3(t1, Gt2), 0.0f, dot3(t2, Gt2) + 1.0e-6f, 0.0f,
                           w * nn + 1.0e-6f, dot3(t1, m), dot3(t2, m), 0.0f);
    return make_float3(y.x * t1.x + y.y * t2.x + y.z * n.x, y.x * t1.y + y.y * t2.y + y.z * n.y,
                       y.x * t1.z + y.y * t2.z + y.z * n.z);
}

__device__ __forceinline__ void store_gradient(const NormalOut &O, int s, int gi, float3 gr)
{
    if (O.attr1)
        O.attr1[s] = make_float4(gr.x, gr.y, gr.z, 0.0f);
    if (O.grd_out)
        O.grd_out[gi] = make_float4(gr.x, gr.y, gr.z, 0.0f);
}

__device__ __forceinline__ void store_normal(const NormalOut &O, int s, int gi, float3 n, float Ip)
{
    if (O.attr0)
        O.attr0[s] = make_float4(n.x, n.y, n.z, Ip);
    if (O.nrm_out)
        O.nrm_out[gi] = make_float4(n.x, n.y, n.z, 0.0f);
}

// the sums of one point's walk: first and second moments of the neighbours inside the
// normal radius (k of them), and the gradient moments G, m inside the gradient radius
// (gk of them), all about the point
struct PointMoments
{
    float s1x, s1y, s1z, sxx, sxy, sxz, syy, syz, szz;
    float gxx, gxy, gxz, gyy, gyz, gzz, mx, my, mz;
    int k, gk;
};

// what follows a point's walk: the FP32 eigen-solve (or the queue for the FP64 pass),
// the orientation, the gradient and the stores.  Compiled once and called by every
// instantiation of the walk, so that the results round alike whichever walk summed
// the moments.
__device__ __noinline__ void finish_point(const int32_t *sidx, NormalOut O, int s, float Ip, PointMoments M, bool grad)
{
    float3 nrm = make_float3(0.0f, 0.0f, 0.0f);
    if (M.k >= 3)
    {
        const float ik = 1.0f / (float)M.k;
        const float ux = M.s1x * ik, uy = M.s1y * ik, uz = M.s1z * ik;
        if (!smallest_eigvec_f32(M.sxx * ik - ux * ux, M.sxy * ik - ux * uy, M.sxz * ik - ux * uz,
                                 M.syy * ik - uy * uy, M.syz * ik - uy * uz, M.szz * ik - uz * uz, nrm))
        {
            const int slot = atomicAdd(O.degen_count, 1);
            O.degen_list[slot] = s;
            if (grad)
            {
                O.degen_mom[3 * slot] = make_float4(M.gxx, M.gxy, M.gxz, M.gyy);
                O.degen_mom[3 * slot + 1] = make_float4(M.gyz, M.gzz, M.mx, M.my);
                O.degen_mom[3 * slot + 2] = make_float4(M.mz, __int_as_float(M.gk), 0.0f, 0.0f);
            }
            return; // written by the FP64 pass
        }
        // orient against (0, 0, -1) (cuda_estimate_normals.cu:131-151)
        if (nrm.z > 0.0f)
            nrm = make_float3(-nrm.x, -nrm.y, -nrm.z);
    }
    const int gi = sidx[s];
    store_normal(O, s, gi, nrm, Ip);
    if (grad)
        store_gradient(O, s, gi,
                       gradient_from_moments(M.gxx, M.gxy, M.gxz, M.gyy, M.gyz, M.gzz, make_float3(M.mx, M.my, M.mz),
                                             M.gk, nrm));
}

// pass 1: PCA normal per grid point in FP32 -- moments about the query point,
// closed-form eigen-system; points whose smallest eigenvalue is not separated by
// 1e-3 of the spread are queued for the FP64 pass.  With Grad the same walk sums
// the gradient moments (gradient_from_moments), and the gradient follows the
// normal (for queued points, the FP64 pass computes it from the stored moments).
// candidates a thread reads per load round in its row walk: one, because the 19
// moment sums already fill the registers (wider rounds spill on the multi-scale
// batches)
constexpr int kNormScanBatch = 1;

template <bool Grad, bool SameR>
__global__ void __launch_bounds__(256, 4) k_normals32(GridDev g, const int32_t *d_n, float rn, int max_nn, NormalOut O)
{
    const int n = *d_n;
    const KeyLayout L = *g.layout;
    const int segshift = L.bx + L.by + L.bz;
    const float rn2 = __fmul_rn(rn, rn);
    NbrEntry list[kMaxNN];
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        const float4 p4 = g.spos[s];
        const float3 p = make_float3(p4.x, p4.y, p4.z);
        const int seg = L.bseg ? (int)(g.skey[s] >> segshift) : 0;
        const float Ip = g.sint[s];
        GridRows R;
        const bool inside = grid_rows(g, L, seg, g.gmin[seg], p, R);
        float s1x = 0, s1y = 0, s1z = 0, sxx = 0, sxy = 0, sxz = 0, syy = 0, syz = 0, szz = 0;
        float gxx = 0, gxy = 0, gxz = 0, gyy = 0, gyz = 0, gzz = 0, mx = 0, my = 0, mz = 0;
        int k = 0, gk = 0;
        // the products are added by fused multiply-adds, written out so that every
        // instantiation rounds the sums alike
        auto acc = [&](float4 q) {
            const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
            s1x += dx, s1y += dy, s1z += dz;
            sxx = fmaf(dx, dx, sxx), sxy = fmaf(dx, dy, sxy), sxz = fmaf(dx, dz, sxz);
            syy = fmaf(dy, dy, syy), syz = fmaf(dy, dz, syz), szz = fmaf(dz, dz, szz);
            ++k;
        };
        // every neighbour inside the radius; only when there are more than max_nn
        // are the max_nn nearest selected instead (most points have fewer, and then
        // the two sets are the same)
        if (inside)
            grid_scan<kNormScanBatch>(g, R, [&](int t, float4 q) {
                const float d2 = dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z);
                if (d2 < rn2)
                {
                    acc(q);
                    if (SameR)
                    {
                        // equal radii: G is the second-moment sum just taken, only m is new
                        const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
                        const float dI = g.sint[t] - Ip;
                        mx = fmaf(dx, dI, mx), my = fmaf(dy, dI, my), mz = fmaf(dz, dI, mz);
                    }
                }
                if (Grad && !SameR && d2 < O.grad_r2)
                {
                    const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
                    const float dI = g.sint[t] - Ip;
                    gxx = fmaf(dx, dx, gxx), gxy = fmaf(dx, dy, gxy), gxz = fmaf(dx, dz, gxz);
                    gyy = fmaf(dy, dy, gyy), gyz = fmaf(dy, dz, gyz), gzz = fmaf(dz, dz, gzz);
                    mx = fmaf(dx, dI, mx), my = fmaf(dy, dI, my), mz = fmaf(dz, dI, mz);
                    ++gk;
                }
            });
        if (SameR)
        {
            gxx = sxx, gxy = sxy, gxz = sxz, gyy = syy, gyz = syz, gzz = szz;
            gk = k;
        }
        if (inside && max_nn > 0 && k > max_nn)
        {
            s1x = s1y = s1z = sxx = sxy = sxz = syy = syz = szz = 0.0f;
            k = 0;
            const int cnt = select_knn(g, R, p, rn2, max_nn, list);
            for (int j = 0; j < cnt; ++j)
                acc(g.spos[list[j].t]);
        }
        finish_point(g.sidx, O, s, Ip,
                     PointMoments{s1x, s1y, s1z, sxx, sxy, sxz, syy, syz, szz, gxx, gxy, gxz, gyy, gyz, gzz, mx,
                                  my, mz, k, gk},
                     Grad);
    }
}

// pass 2: the queued near-degenerate points (a few dozen per frame), one warp per
// point: lanes 0..8 walk one row each of the 27-cell neighbourhood and write the
// points inside the radius to shared memory at deterministic positions (row
// counts, then their prefix); with max_nn the max_nn nearest (distance, then
// index) are kept by rank; the FP64 moments about the point are summed per lane
// and across the warp in a fixed order, and lane 0 solves the eigen-problem in
// closed form.  A neighbourhood larger than the shared list (kN64Cand points)
// falls back to one lane walking the rows itself.
constexpr int kN64Cand = 256;

__global__ void __launch_bounds__(128) k_normals64(GridDev g, float rn, int max_nn, NormalOut O)
{
    __shared__ float s_d2[4][kN64Cand];
    __shared__ int s_t[4][kN64Cand];
    const int n = *O.degen_count;
    const KeyLayout L = *g.layout;
    const int segshift = L.bx + L.by + L.bz;
    const float rn2 = __fmul_rn(rn, rn);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    for (int j = blockIdx.x * 4 + warp; j < n; j += gridDim.x * 4)
    {
        const int s = O.degen_list[j];
        const float4 p4 = g.spos[s];
        const float3 p = make_float3(p4.x, p4.y, p4.z);
        const int seg = L.bseg ? (int)(g.skey[s] >> segshift) : 0;
        GridRows R;
        grid_rows(g, L, seg, g.gmin[seg], p, R);
        // the z window of this lane's row
        int t0 = 0, e = 0;
        if (lane < 9)
        {
            t0 = R.r[0].x, e = R.r[0].y;
#pragma unroll
            for (int k = 1; k < 9; ++k)
                if (lane == k)
                    t0 = R.r[k].x, e = R.r[k].y;
            int a = t0, b = e;
            while (a < b)
            {
                const int m = (a + b) >> 1;
                if (__ldg(&g.scz[m]) < R.lo)
                    a = m + 1;
                else
                    b = m;
            }
            t0 = a;
        }
        auto inside = [&](int t, float &d2) {
            const float4 q = __ldg(&g.spos[t]);
            const int qz = __float_as_int(q.w);
            d2 = dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z);
            return qz <= R.hi && d2 < rn2;
        };
        int cnt = 0;
        for (int t = t0; t < e; ++t)
        {
            float d2;
            if (__float_as_int(__ldg(&g.spos[t]).w) > R.hi)
                break;
            if (inside(t, d2))
                ++cnt;
        }
        int off = cnt;
#pragma unroll
        for (int d = 1; d < 16; d <<= 1)
        {
            const int y = __shfl_up_sync(full, off, d);
            if (lane >= d)
                off += y;
        }
        const int total = __shfl_sync(full, off, 8);
        off -= cnt;
        double S1[3] = {0.0, 0.0, 0.0}, S2[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        int k = 0;
        auto acc = [&](float4 q) {
            const double dx = (double)q.x - (double)p.x, dy = (double)q.y - (double)p.y, dz = (double)q.z - (double)p.z;
            S1[0] += dx, S1[1] += dy, S1[2] += dz;
            S2[0] += dx * dx, S2[1] += dx * dy, S2[2] += dx * dz;
            S2[3] += dy * dy, S2[4] += dy * dz, S2[5] += dz * dz;
            ++k;
        };
        if (total <= kN64Cand)
        {
            int w = off;
            for (int t = t0; t < e; ++t)
            {
                float d2;
                if (__float_as_int(__ldg(&g.spos[t]).w) > R.hi)
                    break;
                if (inside(t, d2))
                {
                    s_d2[warp][w] = d2;
                    s_t[warp][w] = t;
                    ++w;
                }
            }
            __syncwarp();
            const bool select = max_nn > 0 && total > max_nn;
            for (int c = lane; c < total; c += 32)
            {
                const float dc = s_d2[warp][c];
                const int tc = s_t[warp][c];
                bool keep = true;
                if (select)
                {
                    int rank = 0;
                    for (int o = 0; o < total; ++o)
                    {
                        const float d2o = s_d2[warp][o];
                        rank += d2o < dc || (d2o == dc && __ldg(&g.sidx[s_t[warp][o]]) < __ldg(&g.sidx[tc]));
                    }
                    keep = rank < max_nn;
                }
                if (keep)
                    acc(__ldg(&g.spos[tc]));
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1)
            {
#pragma unroll
                for (int i = 0; i < 3; ++i)
                    S1[i] += __shfl_xor_sync(full, S1[i], d);
#pragma unroll
                for (int i = 0; i < 6; ++i)
                    S2[i] += __shfl_xor_sync(full, S2[i], d);
                k += __shfl_xor_sync(full, k, d);
            }
            __syncwarp(); // the list is rewritten by the next point
        }
        else if (lane == 0)
        {
            // a neighbourhood larger than the shared list: one lane, as the FP32 pass
            grid_scan(g, R, [&](int t, float4 q) {
                if (dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z) < rn2)
                    acc(q);
            });
            if (max_nn > 0 && k > max_nn)
            {
                NbrEntry list[kMaxNN];
                S1[0] = S1[1] = S1[2] = 0.0;
                for (int i = 0; i < 6; ++i)
                    S2[i] = 0.0;
                k = 0;
                const int cnt2 = select_knn(g, R, p, rn2, max_nn, list);
                for (int i = 0; i < cnt2; ++i)
                    acc(g.spos[list[i].t]);
            }
        }
        if (lane == 0)
        {
            const double kk = (double)k;
            const double mu[3] = {S1[0] / kk, S1[1] / kk, S1[2] / kk};
            double C[3][3];
            C[0][0] = S2[0] / kk - mu[0] * mu[0];
            C[0][1] = C[1][0] = S2[1] / kk - mu[0] * mu[1];
            C[0][2] = C[2][0] = S2[2] / kk - mu[0] * mu[2];
            C[1][1] = S2[3] / kk - mu[1] * mu[1];
            C[1][2] = C[2][1] = S2[4] / kk - mu[1] * mu[2];
            C[2][2] = S2[5] / kk - mu[2] * mu[2];
            double v[3];
            smallest_eigvec_f64(C, v);
            float3 nrm = make_float3((float)v[0], (float)v[1], (float)v[2]);
            if (nrm.z > 0.0f)
                nrm = make_float3(-nrm.x, -nrm.y, -nrm.z);
            const int gi = g.sidx[s];
            store_normal(O, s, gi, nrm, g.sint[s]);
            if (O.degen_mom)
            {
                const float4 m0 = O.degen_mom[3 * j], m1 = O.degen_mom[3 * j + 1], m2 = O.degen_mom[3 * j + 2];
                store_gradient(O, s, gi,
                               gradient_from_moments(m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, make_float3(m1.z, m1.w, m2.x),
                                                     __float_as_int(m2.y), nrm));
            }
        }
        __syncwarp();
    }
}

// pass 3: colour gradient per grid point (the reference's system, solved in the
// tangent/normal basis); the normal comes from grid-order attr0 or from an
// original-order array
__global__ void __launch_bounds__(256) k_gradient(GridDev g, const int32_t *d_n, float rg, const float4 *nrm_grid,
                                                  const float4 *nrm_orig, float4 *attr1, float4 *grd_out)
{
    const int n = *d_n;
    const KeyLayout L = *g.layout;
    const int segshift = L.bx + L.by + L.bz;
    const float rg2 = __fmul_rn(rg, rg);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        const float4 p4 = g.spos[s];
        const float3 p = make_float3(p4.x, p4.y, p4.z);
        const int gi = g.sidx[s];
        const float Ip = g.sint[s];
        const int seg = L.bseg ? (int)(g.skey[s] >> segshift) : 0;
        const float4 n4 = nrm_grid ? nrm_grid[s] : nrm_orig[gi];
        const float3 nrm = make_float3(n4.x, n4.y, n4.z);
        int knn = 0;
        float A00 = 0, A01 = 0, A02 = 0, A11 = 0, A12 = 0, A22 = 0, b0 = 0, b1 = 0, b2 = 0;
        grid_visit(g, L, seg, g.gmin[seg], p, [&](int t, float4 q) {
            if (!(dist2_ref(q.x, q.y, q.z, p.x, p.y, p.z) < rg2))
                return;
            ++knn;
            if (t == s)
                return;
            const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
            const float sp = dx * nrm.x + dy * nrm.y + dz * nrm.z;
            const float vx = dx - sp * nrm.x, vy = dy - sp * nrm.y, vz = dz - sp * nrm.z;
            const float dI = g.sint[t] - Ip;
            A00 += vx * vx, A01 += vx * vy, A02 += vx * vz;
            A11 += vy * vy, A12 += vy * vz, A22 += vz * vz;
            b0 += vx * dI, b1 += vy * dI, b2 += vz * dI;
        });
        float3 grad = make_float3(0.0f, 0.0f, 0.0f);
        if (knn >= 5)
            grad = solve_gradient_system(A00, A01, A02, A11, A12, A22, b0, b1, b2, nrm,
                                         (float)((knn - 1) * (knn - 1)));
        if (attr1)
            attr1[s] = make_float4(grad.x, grad.y, grad.z, 0.0f);
        if (grd_out)
            grd_out[gi] = make_float4(grad.x, grad.y, grad.z, 0.0f);
    }
}

// ICP target records in another grid's order: {normal, intensity}, {gradient, 0}
__global__ void k_gather_attrs(GridDev g, const int32_t *d_n, const float4 *__restrict__ nrm,
                               const float4 *__restrict__ grd, float4 *attr0, float4 *attr1)
{
    const int n = *d_n;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        const int gi = g.sidx[s];
        const float4 a = nrm[gi], d = grd[gi];
        attr0[s] = make_float4(a.x, a.y, a.z, g.sint[s]);
        attr1[s] = make_float4(d.x, d.y, d.z, 0.0f);
    }
}

int gather_attrs(gca3d_context *ctx, const Batch &b, const Grid &g, const float4 *nrm, const float4 *grd,
                 float4 *attr0, float4 *attr1)
{
    const int gs = std::min(grid_for(g.cap), ctx->num_sms * 8);
    k_gather_attrs<<<gs, kBlock, 0, ctx->stream>>>(g.dev, b.seg_off + b.P, nrm, grd, attr0, attr1);
    GCA_CHECK_LAUNCH(ctx);
    return GCA3D_OK;
}

// grid-order {normal, intensity} records from original-order normals
__global__ void k_attr0_from(GridDev g, const int32_t *d_n, const float4 *__restrict__ nrm, float4 *attr0)
{
    const int n = *d_n;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        const float4 a = nrm[g.sidx[s]];
        attr0[s] = make_float4(a.x, a.y, a.z, g.sint[s]);
    }
}

int normals_stage(gca3d_context *ctx, const Batch &b, const Grid &g, bool do_normals, float normal_radius, int max_nn,
                  bool do_grad, float grad_radius, const float4 *in_nrm, float4 *attr0, float4 *attr1,
                  float4 *nrm_out, float4 *grd_out)
{
    if (max_nn > kMaxNN)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "normals: max_nn above 64 is not supported");
    if (do_normals && !(normal_radius > 0.0f && normal_radius <= g.dev.cell))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "normals: radius must be in (0, grid cell]");
    if (do_grad && !(grad_radius > 0.0f && grad_radius <= g.dev.cell))
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "gradient: radius must be in (0, grid cell]");
    if (!do_normals && !in_nrm)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "gradient: normals needed");
    if (do_grad && do_normals && !attr0 && !nrm_out)
        return fail(ctx, GCA3D_ERR_INVALID_VALUE, "gradient: the normals must be stored");
    const int32_t *d_n = b.seg_off + b.P;
    const int gs = std::min(grid_for(g.cap), ctx->num_sms * 8);
    GCA_PROF_BEGIN(ctx, kKidNormals);
    if (do_normals)
    {
        NormalOut O;
        O.attr0 = attr0;
        O.nrm_out = nrm_out;
        O.degen_count = ctx->arena.get<int>(1);
        O.degen_list = ctx->arena.get<int>(std::max<int64_t>(g.cap, 1));
        // the gradients in the same walk
        O.grad_r2 = do_grad ? grad_radius * grad_radius : 0.0f;
        O.attr1 = do_grad ? attr1 : nullptr;
        O.grd_out = do_grad ? grd_out : nullptr;
        O.degen_mom = do_grad ? ctx->arena.get<float4>(3 * (size_t)std::max<int64_t>(g.cap, 1)) : nullptr;
        if (!O.degen_count || !O.degen_list || (do_grad && !O.degen_mom))
            return fail(ctx, GCA3D_ERR_OUT_OF_MEMORY, "normals: scratch");
        GCA_CUDA(ctx, cudaMemsetAsync(O.degen_count, 0, sizeof(int), ctx->stream));
        // equal radii (the usual case): the gradient's second moments are the normal's
        if (do_grad && O.grad_r2 == normal_radius * normal_radius)
            k_normals32<true, true><<<gs, 256, 0, ctx->stream>>>(g.dev, d_n, normal_radius, max_nn, O);
        else if (do_grad)
            k_normals32<true, false><<<gs, 256, 0, ctx->stream>>>(g.dev, d_n, normal_radius, max_nn, O);
        else
            k_normals32<false, false><<<gs, 256, 0, ctx->stream>>>(g.dev, d_n, normal_radius, max_nn, O);
        GCA_CHECK_LAUNCH(ctx);
        // one warp per queued point and a long dependent FP64 chain per point: as many
        // resident blocks as the registers allow, to overlap the chains
        static const int blocks64 = [] {
            int b = 0;
            return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_normals64, 128, 0) == cudaSuccess && b > 0 ? b
                                                                                                            : 2;
        }();
        k_normals64<<<ctx->num_sms * blocks64, 128, 0, ctx->stream>>>(g.dev, normal_radius, max_nn, O);
        GCA_CHECK_LAUNCH(ctx);
    }
    if (do_grad && !do_normals)
    {
        const float4 *ng = do_normals ? attr0 : nullptr;
        const float4 *no = do_normals ? (attr0 ? nullptr : nrm_out) : in_nrm;
        k_gradient<<<gs, 256, 0, ctx->stream>>>(g.dev, d_n, grad_radius, ng, no, attr1, grd_out);
        GCA_CHECK_LAUNCH(ctx);
    }
    else if (!do_grad && attr1)
        GCA_CUDA(ctx, cudaMemsetAsync(attr1, 0, sizeof(float4) * g.cap, ctx->stream));
    if (!do_normals && attr0)
    {
        k_attr0_from<<<gs, 256, 0, ctx->stream>>>(g.dev, d_n, in_nrm, attr0);
        GCA_CHECK_LAUNCH(ctx);
    }
    GCA_PROF_END(ctx, kKidNormals);
    return GCA3D_OK;
}

} // namespace gca3d
