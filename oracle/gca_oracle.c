/*
 * gca_oracle.c -- CPU oracle for the RGB-D registration path.
 *
 * TEST INFRASTRUCTURE ONLY (see gca_oracle.h).  Every function cites the
 * reference file:line it restates.  Reference paths are relative to the
 * XssZuiNB/CUDA_3D source tree (src/...).
 *
 * Build with -ffp-contract=off: the FP32 flavour must not fuse multiply-adds,
 * so that its results are reproducible on x86-64 and aarch64 alike.
 */
#include "gca_oracle.h"
#include "det_expf.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;

void orc_set_threads(int n)
{
    g_threads = n < 1 ? 1 : n;
}

int orc_get_threads(void)
{
    return g_threads;
}

#ifdef _OPENMP
#define ORC_PAR _Pragma("omp parallel for schedule(dynamic, 256) num_threads(g_threads)")
#else
#define ORC_PAR
#endif

/* ------------------------------------------------------------------ */
/* small float3 helpers in the reference's operation order             */
/* (util/math.cuh:27-110: dot = x*x' + y*y' + z*z', left to right)     */
/* ------------------------------------------------------------------ */
typedef struct { float x, y, z; } f3;

static inline f3 f3m(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f3 f3sub(f3 a, f3 b) { return f3m(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 f3add(f3 a, f3 b) { return f3m(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 f3mul(f3 a, float s) { return f3m(a.x * s, a.y * s, a.z * s); }
static inline f3 f3div(f3 a, float s) { return f3m(a.x / s, a.y / s, a.z / s); }
static inline float f3dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 f3cross(f3 a, f3 b)
{
    return f3m(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline f3 f3load(const float *p, int64_t i) { return f3m(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

typedef struct { double x, y, z; } d3;
static inline d3 d3m(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 d3sub(d3 a, d3 b) { return d3m(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 d3mul(d3 a, double s) { return d3m(a.x * s, a.y * s, a.z * s); }
static inline double d3dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 d3cross(d3 a, d3 b)
{
    return d3m(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline d3 d3loadf(const float *p, int64_t i)
{
    return d3m((double)p[3 * i], (double)p[3 * i + 1], (double)p[3 * i + 2]);
}

/* geometry/type.hpp:45-51 */
float orc_intensity(float r, float g, float b)
{
    return (float)(0.2126 * (double)r + 0.7152 * (double)g + 0.0722 * (double)b);
}

/* geometry/geometry_util.cuh:88-105 (thrust::reduce with min/max functors) */
void orc_aabb(const float *xyz, int64_t n, int flt_min_bug, float mn[3], float mx[3])
{
    for (int a = 0; a < 3; ++a) {
        mn[a] = FLT_MAX;
        mx[a] = flt_min_bug ? FLT_MIN : -FLT_MAX;
    }
    for (int64_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            float v = xyz[3 * i + a];
            mn[a] = v < mn[a] ? v : mn[a];
            mx[a] = v > mx[a] ? v : mx[a];
        }
}

/* ------------------------------------------------------------------ */
/* a1-a3: depth filter + back-projection                               */
/* ------------------------------------------------------------------ */

/* exp(x) as the frame kernel evaluates it (det_expf.h: Cody-Waite reduction and a
 * degree-7 Taylor polynomial, at most 2 ulp from exp(x)) */
static inline float orc_expf(float x) { return gca_det_expf(x); }

float orc_exp32(float x) { return orc_expf(x); }

/* __gaussian / __gaussian_square (cuda_point_cloud_factory.cu:19-27) */
static inline float gauss(float x, float sigma) { return orc_expf(-(x * x) / (sigma * sigma)); }
static inline float gauss_sq(float x2, float sigma) { return orc_expf(-x2 / (sigma * sigma)); }

/* zero-skipping bilateral filter (cuda_point_cloud_factory.cu:64-98) */
static float bilateral(const uint16_t *in, int w, int h, int x, int y, uint16_t centre,
                       int radius, float sigma_space, float sigma_depth)
{
    float sum_w = 0.0f, sum = 0.0f;
    for (int dy = -radius; dy <= radius; ++dy)
        for (int dx = -radius; dx <= radius; ++dx) {
            int nx = x + dx, ny = y + dy;
            if (nx < 0 || nx >= w || ny < 0 || ny >= h)
                continue;
            uint16_t nb = in[(int64_t)ny * w + nx];
            if (!nb)
                continue;
            int diff = (int)centre - (int)nb;
            if (diff < 0)
                diff = -diff;
            float wgt = gauss_sq((float)(dx * dx + dy * dy), sigma_space) * gauss((float)diff, sigma_depth);
            sum_w += wgt;
            sum += wgt * (float)nb;
        }
    return sum / sum_w;
}

/* __adaptive_bilateral_filter (cuda_point_cloud_factory.cu:100-129): 5 steps of
 * 0.5 m, sigma_space 8 + step px, sigma_depth 100 + 10 step depth units,
 * radius = step.  The fixed mode uses the same code with a given radius. */
static float filter_pixel(const uint16_t *in, int w, int h, float depth_scale, int x, int y,
                          float tmin, float tmax, int mode, int fr, float fss, float fsd)
{
    uint16_t d = in[(int64_t)y * w + x];
    float dv = (float)d * depth_scale;
    if (dv < tmin || dv > tmax)
        return (float)d;
    if (mode == ORC_FILTER_FIXED)
        return bilateral(in, w, h, x, y, d, fr, fss, fsd);
    uint32_t step = (uint32_t)((dv - tmin) / 0.5f);
    if (step > 5u)
        step = 5u;
    float ss = 8.0f + (float)step * 1.0f;
    float sd = 100.0f + (float)step * 10.0f;
    float r = 1.0f * (float)step;
    return bilateral(in, w, h, x, y, d, (int)r, ss, sd);
}

/* float -> int truncation with the GPU's conversion semantics (NaN -> 0,
 * saturation), which (int) in C leaves undefined */
static inline int f2i_rz(float x)
{
    if (x != x)
        return 0;
    if (x >= 2147483647.0f)
        return 2147483647;
    if (x <= -2147483648.0f)
        return (-2147483647 - 1);
    return (int)x;
}

/* __kernel_make_pointcloud_Z16_BGR8 (cuda_point_cloud_factory.cu:189-267) and
 * remove_invalid_points (geometry_util.cuh:124-130, stable) */
int64_t orc_make_point_cloud(const uint16_t *depth, const uint8_t *bgr, int w, int h,
                             const orc_intrinsics *di, const orc_intrinsics *ci,
                             const orc_extrinsics *e, float depth_scale, float tmin, float tmax,
                             int filter_mode, int fixed_radius, float fixed_sigma_space,
                             float fixed_sigma_depth, float *out_xyz, float *out_rgb,
                             float *out_depth)
{
    int64_t npx = (int64_t)w * h;
    float *tmp = (float *)malloc(sizeof(float) * 6 * (size_t)npx);
    unsigned char *valid = (unsigned char *)malloc((size_t)npx);
    ORC_PAR
    for (int64_t i = 0; i < npx; ++i) {
        int x = (int)(i % w), y = (int)(i / w);
        float fd;
        if (filter_mode == ORC_FILTER_NONE)
            fd = (float)depth[i];
        else
            fd = filter_pixel(depth, w, h, depth_scale, x, y, tmin, tmax, filter_mode,
                              fixed_radius, fixed_sigma_space, fixed_sigma_depth);
        if (out_depth)
            out_depth[i] = fd;
        float z = fd * depth_scale;
        valid[i] = 0;
        if (z < tmin || z > tmax)
            continue;
        float u = (float)x - 0.5f, v = (float)y - 0.5f;
        float X = (u - di->cx) * z / di->fx;
        float Y = (v - di->cy) * z / di->fy;
        const float *R = e->rotation, *t = e->translation;
        float cx = R[0] * X + R[3] * Y + R[6] * z + t[0];
        float cy = R[1] * X + R[4] * Y + R[7] * z + t[1];
        float cz = R[2] * X + R[5] * Y + R[8] * z + t[2];
        float cu = (cx * ci->fx / cz) + ci->cx;
        float cv = (cy * ci->fy / cz) + ci->cy;
        int tx = f2i_rz(cu + 0.5f), ty = f2i_rz(cv + 0.5f);
        if (tx < 0 || tx >= w || ty < 0 || ty >= h)
            continue;
        int64_t c = 3 * ((int64_t)ty * w + tx);
        float s = 1.0f / 255.0f;
        tmp[6 * i + 0] = X;
        tmp[6 * i + 1] = Y;
        tmp[6 * i + 2] = z;
        tmp[6 * i + 3] = (float)bgr[c + 2] * s; /* r */
        tmp[6 * i + 4] = (float)bgr[c + 1] * s; /* g */
        tmp[6 * i + 5] = (float)bgr[c + 0] * s; /* b */
        valid[i] = 1;
    }
    int64_t m = 0;
    for (int64_t i = 0; i < npx; ++i) {
        if (!valid[i])
            continue;
        memcpy(out_xyz + 3 * m, tmp + 6 * i, 3 * sizeof(float));
        memcpy(out_rgb + 3 * m, tmp + 6 * i + 3, 3 * sizeof(float));
        ++m;
    }
    free(tmp);
    free(valid);
    return m;
}

/* ------------------------------------------------------------------ */
/* a4-a6: voxel downsample                                             */
/* ------------------------------------------------------------------ */
typedef struct { int32_t k[3]; int64_t idx; } vkey;

static int cmp_vkey(const void *a, const void *b)
{
    const vkey *x = (const vkey *)a, *y = (const vkey *)b;
    for (int i = 0; i < 3; ++i)
        if (x->k[i] != y->k[i])
            return x->k[i] < y->k[i] ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* compute_voxel_key_functor (cuda_voxel_grid_down_sample.cu:26-48): floor((p-min)/v) */
static inline int32_t floor_div_key(float p, float mn, float v) { return (int32_t)floorf((p - mn) / v); }

/* cuda_voxel_grid_downsample (cuda_voxel_grid_down_sample.cu:123-161): lexicographic
 * key sort (stable), per-voxel sums in ascending original index, xyz / n and
 * rgb * (1/n) (type.hpp:58-62). */
int64_t orc_voxel_downsample(const float *xyz, const float *rgb, int64_t n, const float mn[3],
                             float voxel, float *out_xyz, float *out_rgb, int32_t *out_count,
                             int32_t *out_key)
{
    if (n <= 0)
        return 0;
    vkey *keys = (vkey *)malloc(sizeof(vkey) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a)
            keys[i].k[a] = floor_div_key(xyz[3 * i + a], mn[a], voxel);
        keys[i].idx = i;
    }
    qsort(keys, (size_t)n, sizeof(vkey), cmp_vkey);
    int64_t m = 0;
    int64_t s = 0;
    while (s < n) {
        int64_t e = s + 1;
        while (e < n && keys[e].k[0] == keys[s].k[0] && keys[e].k[1] == keys[s].k[1] &&
               keys[e].k[2] == keys[s].k[2])
            ++e;
        int64_t i0 = keys[s].idx;
        float sx = xyz[3 * i0], sy = xyz[3 * i0 + 1], sz = xyz[3 * i0 + 2];
        float cr = rgb[3 * i0], cg = rgb[3 * i0 + 1], cb = rgb[3 * i0 + 2];
        for (int64_t j = s + 1; j < e; ++j) {
            int64_t i = keys[j].idx;
            sx = sx + xyz[3 * i];
            sy = sy + xyz[3 * i + 1];
            sz = sz + xyz[3 * i + 2];
            cr = cr + rgb[3 * i];
            cg = cg + rgb[3 * i + 1];
            cb = cb + rgb[3 * i + 2];
        }
        int32_t cnt = (int32_t)(e - s);
        float fn = (float)cnt;
        out_xyz[3 * m + 0] = sx / fn;
        out_xyz[3 * m + 1] = sy / fn;
        out_xyz[3 * m + 2] = sz / fn;
        float inv = 1.0f / fn;
        out_rgb[3 * m + 0] = cr * inv;
        out_rgb[3 * m + 1] = cg * inv;
        out_rgb[3 * m + 2] = cb * inv;
        if (out_count)
            out_count[m] = cnt;
        if (out_key)
            for (int a = 0; a < 3; ++a)
                out_key[3 * m + a] = keys[s].k[a];
        ++m;
        s = e;
    }
    free(keys);
    return m;
}

/* ------------------------------------------------------------------ */
/* a7-a10: uniform grid                                                */
/* ------------------------------------------------------------------ */
typedef struct {
    int64_t n;
    vkey *cells; /* sorted by (cx, cy, cz, idx) */
} ogrid;

static void grid_build(ogrid *g, const float *pts, int64_t n, const float gmin[3], float cell)
{
    g->n = n;
    g->cells = (vkey *)malloc(sizeof(vkey) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a)
            g->cells[i].k[a] = floor_div_key(pts[3 * i + a], gmin[a], cell);
        g->cells[i].idx = i;
    }
    qsort(g->cells, (size_t)n, sizeof(vkey), cmp_vkey);
}

static void grid_free(ogrid *g) { free(g->cells); }

/* first position whose cell is >= (x, y, z) */
static int64_t grid_lower(const ogrid *g, int32_t x, int32_t y, int32_t z)
{
    int64_t lo = 0, hi = g->n;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        const int32_t *k = g->cells[mid].k;
        int less = k[0] != x ? k[0] < x : (k[1] != y ? k[1] < y : k[2] < z);
        if (less)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

/* nn_search_functor (cuda_nn_search.cu:145-213): 27 cells in (i, j, k) order,
 * ascending original index inside a cell, d^2 = dx*dx + dy*dy + dz*dz with
 * d = neighbour - query, strict < r^2. */
void orc_nn_search(const float *q, int64_t nq, const float *r, int64_t nr, float radius,
                   const float gmin[3], int tie_mode, int32_t *out)
{
    ogrid g;
    grid_build(&g, r, nr, gmin, radius);
    float rr = radius * radius;
    ORC_PAR
    for (int64_t i = 0; i < nq; ++i) {
        f3 p = f3load(q, i);
        int32_t c[3];
        c[0] = floor_div_key(p.x, gmin[0], radius);
        c[1] = floor_div_key(p.y, gmin[1], radius);
        c[2] = floor_div_key(p.z, gmin[2], radius);
        float best = rr;
        int32_t bi = -1;
        for (int di = -1; di <= 1; ++di)
            for (int dj = -1; dj <= 1; ++dj)
                for (int dk = -1; dk <= 1; ++dk) {
                    int32_t x = c[0] + di, y = c[1] + dj, z = c[2] + dk;
                    for (int64_t s = grid_lower(&g, x, y, z); s < g.n; ++s) {
                        const vkey *e = &g.cells[s];
                        if (e->k[0] != x || e->k[1] != y || e->k[2] != z)
                            break;
                        f3 nb = f3load(r, e->idx);
                        float dx = nb.x - p.x, dy = nb.y - p.y, dz = nb.z - p.z;
                        float d2 = dx * dx + dy * dy + dz * dz;
                        if (tie_mode == ORC_TIE_SCAN_ORDER) {
                            if (d2 < best) {
                                best = d2;
                                bi = (int32_t)e->idx;
                            }
                        } else if (d2 < rr &&
                                   (bi < 0 || d2 < best || (d2 == best && e->idx < bi))) {
                            best = d2;
                            bi = (int32_t)e->idx;
                        }
                    }
                }
        out[i] = bi;
    }
    grid_free(&g);
}

/* visit every reference point within radius of q in scan order */
typedef void (*visit_fn)(void *ctx, int64_t j, float d2);

static int64_t grid_visit_radius(const ogrid *g, const float *r, f3 p, const float gmin[3],
                                 float radius, visit_fn fn, void *ctx)
{
    int32_t c[3];
    c[0] = floor_div_key(p.x, gmin[0], radius);
    c[1] = floor_div_key(p.y, gmin[1], radius);
    c[2] = floor_div_key(p.z, gmin[2], radius);
    int64_t cnt = 0;
    for (int di = -1; di <= 1; ++di)
        for (int dj = -1; dj <= 1; ++dj)
            for (int dk = -1; dk <= 1; ++dk) {
                int32_t x = c[0] + di, y = c[1] + dj, z = c[2] + dk;
                for (int64_t s = grid_lower(g, x, y, z); s < g->n; ++s) {
                    const vkey *e = &g->cells[s];
                    if (e->k[0] != x || e->k[1] != y || e->k[2] != z)
                        break;
                    f3 nb = f3load(r, e->idx);
                    float dx = nb.x - p.x, dy = nb.y - p.y, dz = nb.z - p.z;
                    float d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 < radius * radius) {
                        if (fn)
                            fn(ctx, e->idx, d2);
                        ++cnt;
                    }
                }
            }
    return cnt;
}

typedef struct { int32_t *list; int64_t pos; } list_ctx;
static void visit_append(void *ctx, int64_t j, float d2)
{
    (void)d2;
    list_ctx *c = (list_ctx *)ctx;
    c->list[c->pos++] = (int32_t)j;
}

/* cuda_search_radius_neighbors (cuda_nn_search.cu:622-723): count pass, exclusive
 * scan, fill pass, self included, no cap */
int64_t orc_radius_search(const float *q, int64_t nq, const float *r, int64_t nr, float radius,
                          const float gmin[3], int32_t *counts, int64_t *starts,
                          int32_t *list, int64_t list_cap)
{
    ogrid g;
    grid_build(&g, r, nr, gmin, radius);
    ORC_PAR
    for (int64_t i = 0; i < nq; ++i)
        counts[i] = (int32_t)grid_visit_radius(&g, r, f3load(q, i), gmin, radius, NULL, NULL);
    int64_t total = 0;
    for (int64_t i = 0; i < nq; ++i) {
        starts[i] = total;
        total += counts[i];
    }
    if (list && total <= list_cap) {
        ORC_PAR
        for (int64_t i = 0; i < nq; ++i) {
            list_ctx c = {list, starts[i]};
            grid_visit_radius(&g, r, f3load(q, i), gmin, radius, visit_append, &c);
        }
    }
    grid_free(&g);
    return total;
}

/* ------------------------------------------------------------------ */
/* a11: normals, reference flavour                                     */
/* ------------------------------------------------------------------ */

/* __compute_eigenvector_1 (util/fast_eigen_val_vec.cuh:13-32); rows of the
 * scaled matrix, upper entries used for the symmetric ones */
static f3 eig_vec1(const f3 rows[3], float e)
{
    f3 r1 = f3m(rows[0].x - e, rows[0].y, rows[0].z);
    f3 r2 = f3m(rows[0].y, rows[1].y - e, rows[1].z);
    f3 r3 = f3m(rows[0].z, rows[1].z, rows[2].z - e);
    f3 rxr[3] = {f3cross(r1, r2), f3cross(r1, r3), f3cross(r2, r3)};
    float dx = f3dot(rxr[0], rxr[0]), dy = f3dot(rxr[1], rxr[1]), dz = f3dot(rxr[2], rxr[2]);
    /* max_coeff (util/math.cuh:97-106) */
    int imax = (dx > fmaxf(dy, dz)) * 0 + (dy > fmaxf(dx, dz)) * 1 + (dz > fmaxf(dx, dy)) * 2;
    float md = imax == 0 ? dx : (imax == 1 ? dy : dz);
    return f3div(rxr[imax], sqrtf(md));
}

static f3 mat_rows_mul(const f3 rows[3], f3 v)
{
    return f3m(rows[0].x * v.x + rows[0].y * v.y + rows[0].z * v.z,
               rows[1].x * v.x + rows[1].y * v.y + rows[1].z * v.z,
               rows[2].x * v.x + rows[2].y * v.y + rows[2].z * v.z);
}

/* __compute_eigenvector_2 (util/fast_eigen_val_vec.cuh:34-108) */
static f3 eig_vec2(const f3 rows[3], f3 e1, float e2)
{
    float mabs = fmaxf(fabsf(e1.x), fabsf(e1.y));
    float inv_len = 1.0f / sqrtf(mabs * mabs + e1.z * e1.z);
    f3 U = (fabsf(e1.x) > fabsf(e1.y)) ? f3m(-e1.z, 0.0f, e1.x) : f3m(0.0f, e1.z, -e1.y);
    U = f3mul(U, inv_len);
    f3 V = f3cross(e1, U);
    f3 AU = mat_rows_mul(rows, U), AV = mat_rows_mul(rows, V);
    float m00 = f3dot(U, AU) - e2, m01 = f3dot(U, AV), m11 = f3dot(V, AV) - e2;
    float a00 = fabsf(m00), a01 = fabsf(m01), a11 = fabsf(m11);
    if (a00 >= a11) {
        if (fmaxf(a00, a01) > 0.0f) {
            if (a00 >= a01) {
                m01 /= m00;
                m00 = 1.0f / sqrtf(1.0f + m01 * m01);
                m01 *= m00;
            } else {
                m00 /= m01;
                m01 = 1.0f / sqrtf(1.0f + m00 * m00);
                m00 *= m01;
            }
            return f3sub(f3mul(U, m01), f3mul(V, m00));
        }
        return U;
    }
    if (fmaxf(a11, a01) > 0.0f) {
        if (a11 >= a01) {
            m01 /= m11;
            m11 = 1.0f / sqrtf(1.0f + m01 * m01);
            m01 *= m11;
        } else {
            m11 /= m01;
            m01 = 1.0f / sqrtf(1.0f + m11 * m11);
            m11 *= m01;
        }
        return f3sub(f3mul(U, m11), f3mul(V, m01));
    }
    return U;
}

/* fast_eigen_compute_3x3_symm (util/fast_eigen_val_vec.cuh:115-205): the closed-form
 * symmetric 3x3 eigensolver (trigonometric eigenvalues, cross-product eigenvectors) */
static void eig3_ref32(const float A[9], float eval[3], f3 evec[3])
{
    f3 rows[3] = {f3m(A[0], A[1], A[2]), f3m(A[3], A[4], A[5]), f3m(A[6], A[7], A[8])};
    float m1 = fmaxf(fmaxf(fabsf(rows[0].x), fabsf(rows[0].y)), fabsf(rows[0].z));
    float m2 = fmaxf(m1, fmaxf(fabsf(rows[1].y), fabsf(rows[1].z)));
    float amax = fmaxf(m2, fabsf(rows[2].z));
    if (amax == 0.0f) {
        eval[0] = eval[1] = eval[2] = 0.0f;
        evec[0] = f3m(1, 0, 0);
        evec[1] = f3m(0, 1, 0);
        evec[2] = f3m(0, 0, 1);
        return;
    }
    float inv = 1.0f / amax;
    for (int i = 0; i < 3; ++i)
        rows[i] = f3mul(rows[i], inv);
    float nrm = rows[0].y * rows[0].y + rows[0].z * rows[0].z + rows[1].z * rows[1].z;
    if (nrm > 0.0f) {
        float q = (rows[0].x + rows[1].y + rows[2].z) / 3.0f;
        float b00 = rows[0].x - q, b11 = rows[1].y - q, b22 = rows[2].z - q;
        float p = sqrtf((b00 * b00 + b11 * b11 + b22 * b22 + nrm * 2.0f) / 6.0f);
        float c00 = b11 * b22 - rows[1].z * rows[1].z;
        float c01 = rows[0].y * b22 - rows[1].z * rows[0].z;
        float c02 = rows[0].y * rows[1].z - b11 * rows[0].z;
        float det = (b00 * c00 - rows[0].y * c01 + rows[0].z * c02) / (p * p * p);
        float hd = det * 0.5f;
        hd = fminf(fmaxf(hd, -1.0f), 1.0f);
        float ang = acosf(hd) / 3.0f;
        const float two_thirds_pi = 2.09439510239319549f;
        float beta2 = cosf(ang) * 2.0f;
        float beta0 = cosf(ang + two_thirds_pi) * 2.0f;
        float beta1 = -(beta0 + beta2);
        float e1 = q + p * beta0, e2 = q + p * beta1, e3 = q + p * beta2;
        f3 v1, v2, v3;
        if (hd >= 0.0f) {
            v3 = eig_vec1(rows, e3);
            v2 = eig_vec2(rows, v3, e2);
            v1 = f3cross(v2, v3);
        } else {
            v1 = eig_vec1(rows, e1);
            v2 = eig_vec2(rows, v1, e2);
            v3 = f3cross(v1, v2);
        }
        eval[0] = e1 * amax;
        eval[1] = e2 * amax;
        eval[2] = e3 * amax;
        evec[0] = v1;
        evec[1] = v2;
        evec[2] = v3;
        return;
    }
    eval[0] = A[0];
    eval[1] = A[4];
    eval[2] = A[8];
    evec[0] = f3m(1, 0, 0);
    evec[1] = f3m(0, 1, 0);
    evec[2] = f3m(0, 0, 1);
}

typedef struct { const float *pts; float m[9]; int64_t cnt; } mom_ctx;
static void visit_moments(void *ctx, int64_t j, float d2)
{
    (void)d2;
    mom_ctx *c = (mom_ctx *)ctx;
    float x = c->pts[3 * j], y = c->pts[3 * j + 1], z = c->pts[3 * j + 2];
    float v[9] = {x, y, z, x * x, x * y, x * z, y * y, y * z, z * z};
    /* reduce_by_key over the CSR expansion: the first value starts the sum */
    if (c->cnt == 0)
        memcpy(c->m, v, sizeof v);
    else
        for (int k = 0; k < 9; ++k)
            c->m[k] = c->m[k] + v[k];
    c->cnt++;
}

/* cuda_estimate_normals (cuda_estimate_normals.cu:46-199): raw FP32 moments summed
 * in scan order, E[xx^T] - E[x]E[x]^T, strictly smallest eigenvalue's vector,
 * oriented against (0, 0, -1) */
void orc_normals_ref32(const float *xyz, int64_t n, float radius, const float gmin[3],
                       float *out)
{
    ogrid g;
    grid_build(&g, xyz, n, gmin, radius);
    ORC_PAR
    for (int64_t i = 0; i < n; ++i) {
        mom_ctx c;
        c.pts = xyz;
        c.cnt = 0;
        memset(c.m, 0, sizeof c.m);
        grid_visit_radius(&g, xyz, f3load(xyz, i), gmin, radius, visit_moments, &c);
        f3 nrm = f3m(0, 0, 0);
        if (c.cnt >= 3) {
            float fc = (float)c.cnt, cu[9];
            for (int k = 0; k < 9; ++k)
                cu[k] = c.m[k] / fc;
            float A[9];
            A[0] = cu[3] - cu[0] * cu[0];
            A[4] = cu[6] - cu[1] * cu[1];
            A[8] = cu[8] - cu[2] * cu[2];
            A[1] = A[3] = cu[4] - cu[0] * cu[1];
            A[2] = A[6] = cu[5] - cu[0] * cu[2];
            A[5] = A[7] = cu[7] - cu[1] * cu[2];
            float ev[3];
            f3 vec[3];
            eig3_ref32(A, ev, vec);
            if (ev[0] < ev[1] && ev[0] < ev[2])
                nrm = vec[0];
            else if (ev[1] < ev[0] && ev[1] < ev[2])
                nrm = vec[1];
            else
                nrm = vec[2];
            if (!(sqrtf(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z) > 0.0f))
                nrm = f3m(0, 0, 0);
        }
        /* align_normal_direction_functor (cuda_estimate_normals.cu:131-151) */
        if (sqrtf(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z) == 0.0f)
            nrm = f3m(0, 0, 0);
        else if (f3dot(nrm, f3m(0.0f, 0.0f, -1.0f)) < 0.0f)
            nrm = f3mul(nrm, -1.0f);
        out[3 * i] = nrm.x;
        out[3 * i + 1] = nrm.y;
        out[3 * i + 2] = nrm.z;
    }
    grid_free(&g);
}

/* ------------------------------------------------------------------ */
/* a11: normals, FP64 flavour                                          */
/* ------------------------------------------------------------------ */

/* cyclic Jacobi eigen-decomposition of a symmetric 3x3 (FP64) */
static void jacobi3(double a[3][3], double ev[3], double V[3][3])
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            V[i][j] = i == j;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off <= 1e-36 * diag || off == 0.0)
            break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (a[p][q] == 0.0)
                    continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < 3; ++i)
        ev[i] = a[i][i];
}

typedef struct { int64_t j; float d2; } nbr;
static int cmp_nbr(const void *a, const void *b)
{
    const nbr *x = (const nbr *)a, *y = (const nbr *)b;
    if (x->d2 != y->d2)
        return x->d2 < y->d2 ? -1 : 1;
    return x->j < y->j ? -1 : (x->j > y->j);
}

typedef struct { nbr *v; int64_t n, cap; } nbr_list;
static void visit_collect(void *ctx, int64_t j, float d2)
{
    nbr_list *l = (nbr_list *)ctx;
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 64;
        l->v = (nbr *)realloc(l->v, sizeof(nbr) * (size_t)l->cap);
    }
    l->v[l->n].j = j;
    l->v[l->n].d2 = d2;
    l->n++;
}

/* the FP64 normal: covariance about the neighbourhood mean, eigenvector of the
 * smallest eigenvalue, flipped so that n . (0, 0, -1) >= 0; fewer than 3
 * neighbours give the zero vector (cuda_estimate_normals.cu:89-93) */
void orc_normals_f64(const float *xyz, int64_t n, float radius, int max_nn, double *out)
{
    float amin[3], amax[3], gmin[3];
    orc_aabb(xyz, n, 0, amin, amax);
    for (int a = 0; a < 3; ++a)
        gmin[a] = amin[a] - 1.5f * radius;
    ogrid g;
    grid_build(&g, xyz, n, gmin, radius);
    ORC_PAR
    for (int64_t i = 0; i < n; ++i) {
        nbr_list l = {NULL, 0, 0};
        grid_visit_radius(&g, xyz, f3load(xyz, i), gmin, radius, visit_collect, &l);
        int64_t k = l.n;
        if (max_nn > 0 && k > max_nn) {
            qsort(l.v, (size_t)k, sizeof(nbr), cmp_nbr);
            k = max_nn;
        }
        double nx = 0, ny = 0, nz = 0;
        if (k >= 3) {
            double mu[3] = {0, 0, 0};
            for (int64_t t = 0; t < k; ++t)
                for (int a = 0; a < 3; ++a)
                    mu[a] += (double)xyz[3 * l.v[t].j + a];
            for (int a = 0; a < 3; ++a)
                mu[a] /= (double)k;
            double C[3][3] = {{0}};
            for (int64_t t = 0; t < k; ++t) {
                double d[3];
                for (int a = 0; a < 3; ++a)
                    d[a] = (double)xyz[3 * l.v[t].j + a] - mu[a];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        C[a][b] += d[a] * d[b];
            }
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    C[a][b] /= (double)k;
            double ev[3], V[3][3];
            jacobi3(C, ev, V);
            int s = 0;
            for (int a = 1; a < 3; ++a)
                if (ev[a] < ev[s])
                    s = a;
            nx = V[0][s];
            ny = V[1][s];
            nz = V[2][s];
            double len = sqrt(nx * nx + ny * ny + nz * nz);
            nx /= len;
            ny /= len;
            nz /= len;
            if (-nz < 0.0) {
                nx = -nx;
                ny = -ny;
                nz = -nz;
            }
        }
        out[3 * i] = nx;
        out[3 * i + 1] = ny;
        out[3 * i + 2] = nz;
        free(l.v);
    }
    grid_free(&g);
}

/* ------------------------------------------------------------------ */
/* a13: colour gradient                                                */
/* ------------------------------------------------------------------ */

/* ldlt_3x3 (util/little_3x3_ldlt_solve.cuh:6-67), A row-major, lower entries used */
static void ldlt3_solve32(const float A[9], const float b[3], float x[3])
{
    float D0 = A[0];
    float L10 = A[3] / D0;
    float L20 = A[6] / D0;
    float D1 = A[4] - L10 * L10 * D0;
    float L21 = (A[7] - L10 * L20 * D0) / D1;
    float D2 = A[8] - L20 * L20 * D0 - L21 * L21 * D1;
    x[0] = b[0];
    x[1] = b[1] - L10 * x[0];
    x[2] = b[2] - L20 * x[0] - L21 * x[1];
    x[0] /= D0;
    x[1] /= D1;
    x[2] /= D2;
    x[1] -= L21 * x[2];
    x[0] -= L10 * x[1] + L20 * x[2];
}

typedef struct {
    const float *pts, *rgb;
    int64_t self;
    f3 p, n;
    float Ip;
    float AtA[9], Atb[3];
} grad_ctx;

static void visit_grad32(void *ctx, int64_t j, float d2)
{
    (void)d2;
    grad_ctx *c = (grad_ctx *)ctx;
    if (j == c->self)
        return;
    f3 q = f3load(c->pts, j);
    f3 proj = f3sub(q, f3mul(c->n, f3dot(f3sub(q, c->p), c->n)));
    float Iq = orc_intensity(c->rgb[3 * j], c->rgb[3 * j + 1], c->rgb[3 * j + 2]);
    f3 v = f3sub(proj, c->p);
    float vv[3] = {v.x, v.y, v.z};
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            c->AtA[3 * a + b] = c->AtA[3 * a + b] + vv[a] * vv[b];
    float dI = Iq - c->Ip;
    for (int a = 0; a < 3; ++a)
        c->Atb[a] = c->Atb[a] + vv[a] * dI;
}

/* compute_color_gradient_functor (cuda_compute_color_gradient.cu:34-89) */
void orc_gradient_ref32(const float *xyz, const float *rgb, const float *nrm, int64_t n,
                        float radius, const float gmin[3], float *out)
{
    ogrid g;
    grid_build(&g, xyz, n, gmin, radius);
    ORC_PAR
    for (int64_t i = 0; i < n; ++i) {
        f3 p = f3load(xyz, i);
        int64_t knn = grid_visit_radius(&g, xyz, p, gmin, radius, NULL, NULL);
        out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = 0.0f;
        if (knn < 5)
            continue;
        grad_ctx c;
        c.pts = xyz;
        c.rgb = rgb;
        c.self = i;
        c.p = p;
        c.n = f3load(nrm, i);
        c.Ip = orc_intensity(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
        memset(c.AtA, 0, sizeof c.AtA);
        memset(c.Atb, 0, sizeof c.Atb);
        grid_visit_radius(&g, xyz, p, gmin, radius, visit_grad32, &c);
        float w = (float)((knn - 1) * (knn - 1));
        float nw[3] = {c.n.x * w, c.n.y * w, c.n.z * w};
        float nn[3] = {c.n.x, c.n.y, c.n.z};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                c.AtA[3 * a + b] = c.AtA[3 * a + b] + nw[a] * nn[b];
        c.AtA[0] += 1.0e-6f;
        c.AtA[4] += 1.0e-6f;
        c.AtA[8] += 1.0e-6f;
        ldlt3_solve32(c.AtA, c.Atb, out + 3 * i);
    }
    grid_free(&g);
}

/* FP64 colour gradient: same system (tangent-plane least squares, orthogonality
 * term (knn-1)^2 n n^T, 1e-6 ridge) solved in FP64 */
void orc_gradient_f64(const float *xyz, const float *rgb, const double *nrm, int64_t n,
                      float radius, double *out)
{
    float amin[3], amax[3], gmin[3];
    orc_aabb(xyz, n, 0, amin, amax);
    for (int a = 0; a < 3; ++a)
        gmin[a] = amin[a] - 1.5f * radius;
    ogrid g;
    grid_build(&g, xyz, n, gmin, radius);
    ORC_PAR
    for (int64_t i = 0; i < n; ++i) {
        nbr_list l = {NULL, 0, 0};
        grid_visit_radius(&g, xyz, f3load(xyz, i), gmin, radius, visit_collect, &l);
        out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = 0.0;
        if (l.n >= 5) {
            d3 p = d3loadf(xyz, i);
            d3 nv = d3m(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
            double Ip = (double)orc_intensity(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
            double A[3][3] = {{0}}, b[3] = {0, 0, 0};
            for (int64_t t = 0; t < l.n; ++t) {
                int64_t j = l.v[t].j;
                if (j == i)
                    continue;
                d3 q = d3loadf(xyz, j);
                d3 dq = d3sub(q, p);
                double s = d3dot(dq, nv);
                double v[3] = {dq.x - s * nv.x, dq.y - s * nv.y, dq.z - s * nv.z};
                double dI = (double)orc_intensity(rgb[3 * j], rgb[3 * j + 1], rgb[3 * j + 2]) - Ip;
                for (int a = 0; a < 3; ++a) {
                    for (int c = 0; c < 3; ++c)
                        A[a][c] += v[a] * v[c];
                    b[a] += v[a] * dI;
                }
            }
            double w = (double)((l.n - 1) * (l.n - 1));
            double nn[3] = {nv.x, nv.y, nv.z};
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c)
                    A[a][c] += w * nn[a] * nn[c];
            for (int a = 0; a < 3; ++a)
                A[a][a] += 1.0e-6;
            /* LDL^T (SPD) */
            double D0 = A[0][0], L10 = A[1][0] / D0, L20 = A[2][0] / D0;
            double D1 = A[1][1] - L10 * L10 * D0;
            double L21 = (A[2][1] - L10 * L20 * D0) / D1;
            double D2 = A[2][2] - L20 * L20 * D0 - L21 * L21 * D1;
            double y0 = b[0], y1 = b[1] - L10 * y0, y2 = b[2] - L20 * y0 - L21 * y1;
            double x2 = y2 / D2, x1 = y1 / D1 - L21 * x2, x0 = y0 / D0 - L10 * x1 - L20 * x2;
            out[3 * i] = x0;
            out[3 * i + 1] = x1;
            out[3 * i + 2] = x2;
        }
        free(l.v);
    }
    grid_free(&g);
}

/* ------------------------------------------------------------------ */
/* a14-a15: Gauss-Newton system, reference flavour                     */
/* ------------------------------------------------------------------ */

/* compute_JTJ_JTr_and_r_gauss_newton_functor (cuda_color_icp_build_least_square.cu:154-253) */
static void gn_point32(f3 p, float Is, f3 q, float It, f3 n, f3 d, float slg, float slc,
                       float J[2][6], float *rg, float *rc)
{
    float rg_ = f3dot(f3sub(p, q), n);
    f3 jr = f3mul(f3cross(p, n), slg);
    f3 jt = f3mul(n, slg);
    J[0][0] = jr.x; J[0][1] = jr.y; J[0][2] = jr.z;
    J[0][3] = jt.x; J[0][4] = jt.y; J[0][5] = jt.z;
    *rg = slg * rg_;
    /* dc_x_df = d^T (I - n n^T), summed over k from 0 (math.cuh:1712-1737) */
    float nv[3] = {n.x, n.y, n.z}, dv[3] = {d.x, d.y, d.z}, dc[3];
    for (int j = 0; j < 3; ++j) {
        float s = 0.0f;
        for (int k = 0; k < 3; ++k) {
            float M = (k == j ? 1.0f : 0.0f) - nv[k] * nv[j];
            s += dv[k] * M;
        }
        dc[j] = s;
    }
    f3 dcv = f3m(dc[0], dc[1], dc[2]);
    f3 cr = f3mul(f3cross(p, dcv), slc);
    f3 ct = f3mul(dcv, slc);
    J[1][0] = cr.x; J[1][1] = cr.y; J[1][2] = cr.z;
    J[1][3] = ct.x; J[1][4] = ct.y; J[1][5] = ct.z;
    f3 proj = f3sub(p, f3mul(n, rg_));
    float Iproj = It + f3dot(d, f3sub(proj, q));
    *rc = slc * (Iproj - Is);
}

void orc_build_gn_ref32(const float *sx, const float *srgb, int64_t ns, const float *tx,
                        const float *trgb, const float *tn, const float *tg, const int32_t *nn,
                        float lambda, float jtj[36], float jtr[6], float *r2)
{
    float slg = sqrtf(lambda), slc = sqrtf(1.0f - lambda);
    float A[36] = {0}, b[6] = {0}, e = 0.0f;
    for (int64_t i = 0; i < ns; ++i) {
        int32_t j = nn[i];
        if (j < 0)
            continue;
        float J[2][6], rg, rc;
        gn_point32(f3load(sx, i), orc_intensity(srgb[3 * i], srgb[3 * i + 1], srgb[3 * i + 2]),
                   f3load(tx, j), orc_intensity(trgb[3 * j], trgb[3 * j + 1], trgb[3 * j + 2]),
                   f3load(tn, j), f3load(tg, j), slg, slc, J, &rg, &rc);
        for (int a = 0; a < 6; ++a) {
            for (int c = 0; c < 6; ++c)
                A[6 * a + c] = A[6 * a + c] + (J[0][a] * J[0][c] + J[1][a] * J[1][c]);
            b[a] = b[a] + (J[0][a] * rg + J[1][a] * rc);
        }
        e = e + (rg * rg + rc * rc);
    }
    memcpy(jtj, A, sizeof A);
    memcpy(jtr, b, sizeof b);
    *r2 = e;
}

/* compute_residual_functor (cuda_color_icp_build_least_square.cu:33-80) */
void orc_abs_residual_ref32(const float *sx, const float *srgb, int64_t ns, const float *tx,
                            const float *trgb, const float *tn, const float *tg,
                            const int32_t *nn, float lambda, float *out)
{
    float slg = sqrtf(lambda), slc = sqrtf(1.0f - lambda);
    for (int64_t i = 0; i < ns; ++i) {
        int32_t j = nn[i];
        if (j < 0) {
            out[i] = 0.0f;
            continue;
        }
        f3 p = f3load(sx, i), q = f3load(tx, j), n = f3load(tn, j), d = f3load(tg, j);
        float rg_ = f3dot(f3sub(p, q), n);
        float rgw = slg * rg_;
        float Is = orc_intensity(srgb[3 * i], srgb[3 * i + 1], srgb[3 * i + 2]);
        float It = orc_intensity(trgb[3 * j], trgb[3 * j + 1], trgb[3 * j + 2]);
        f3 proj = f3sub(p, f3mul(n, rg_));
        float Ip = It + f3dot(d, f3sub(proj, q));
        float rcw = slc * (Ip - Is);
        out[i] = fabsf(rgw) + fabsf(rcw);
    }
}

/* ------------------------------------------------------------------ */
/* a16: 6x6 solve and pose maps                                        */
/* ------------------------------------------------------------------ */

/* LDL^T with symmetric diagonal pivoting, the factorisation Eigen's LDLT performs
 * (registration/eigen_solver.hpp:59-65); a vanishing pivot zeroes its component. */
int orc_solve6(const double jtj[36], const double jtr[6], double x[6])
{
    double A[6][6], b[6];
    int perm[6];
    int status = 0;
    for (int i = 0; i < 6; ++i) {
        for (int j = 0; j < 6; ++j)
            A[i][j] = jtj[6 * i + j];
        b[i] = -jtr[i];
        perm[i] = i;
        if (!isfinite(b[i]))
            status = 1;
        for (int j = 0; j < 6; ++j)
            if (!isfinite(A[i][j]))
                status = 1;
    }
    if (status) {
        for (int i = 0; i < 6; ++i)
            x[i] = 0.0;
        return 1;
    }
    double D[6];
    for (int k = 0; k < 6; ++k) {
        int piv = k;
        for (int i = k + 1; i < 6; ++i)
            if (fabs(A[i][i]) > fabs(A[piv][piv]))
                piv = i;
        if (piv != k) {
            for (int j = 0; j < 6; ++j) {
                double t = A[k][j];
                A[k][j] = A[piv][j];
                A[piv][j] = t;
            }
            for (int i = 0; i < 6; ++i) {
                double t = A[i][k];
                A[i][k] = A[i][piv];
                A[i][piv] = t;
            }
            int t = perm[k];
            perm[k] = perm[piv];
            perm[piv] = t;
        }
        D[k] = A[k][k];
        if (fabs(D[k]) <= DBL_MIN) {
            status = 1;
            for (int i = k + 1; i < 6; ++i)
                A[i][k] = 0.0;
            continue;
        }
        for (int i = k + 1; i < 6; ++i)
            A[i][k] /= D[k];
        for (int i = k + 1; i < 6; ++i)
            for (int j = k + 1; j <= i; ++j) {
                A[i][j] -= A[i][k] * A[j][k] * D[k];
                A[j][i] = A[i][j];
            }
    }
    double y[6];
    for (int i = 0; i < 6; ++i) {
        double s = b[perm[i]];
        for (int j = 0; j < i; ++j)
            s -= A[i][j] * y[j];
        y[i] = s;
    }
    for (int i = 0; i < 6; ++i)
        y[i] = fabs(D[i]) > DBL_MIN ? y[i] / D[i] : 0.0;
    double z[6];
    for (int i = 5; i >= 0; --i) {
        double s = y[i];
        for (int j = i + 1; j < 6; ++j)
            s -= A[j][i] * z[j];
        z[i] = s;
    }
    for (int i = 0; i < 6; ++i)
        x[perm[i]] = z[i];
    return status;
}

/* transform_vec6d_to_mat4f (registration/eigen_solver.hpp:30-40): R = Rz(x2) Ry(x1)
 * Rx(x0), t = x3..5.  SE3 exp: R = exp([w]x), t = V v (left Jacobian). */
void orc_pose_from_x(const double x[6], int update_map, double T[16])
{
    double R[3][3], t[3];
    if (update_map == ORC_UPDATE_EULER_ZYX) {
        double ca = cos(x[0]), sa = sin(x[0]);
        double cb = cos(x[1]), sb = sin(x[1]);
        double cc = cos(x[2]), sc = sin(x[2]);
        R[0][0] = cc * cb;
        R[0][1] = cc * sb * sa - sc * ca;
        R[0][2] = cc * sb * ca + sc * sa;
        R[1][0] = sc * cb;
        R[1][1] = sc * sb * sa + cc * ca;
        R[1][2] = sc * sb * ca - cc * sa;
        R[2][0] = -sb;
        R[2][1] = cb * sa;
        R[2][2] = cb * ca;
        t[0] = x[3];
        t[1] = x[4];
        t[2] = x[5];
    } else {
        double w[3] = {x[0], x[1], x[2]}, v[3] = {x[3], x[4], x[5]};
        double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
        double th = sqrt(th2);
        double A, B, C;
        if (th < 1e-4) {
            A = 1.0 - th2 / 6.0 + th2 * th2 / 120.0;
            B = 0.5 - th2 / 24.0 + th2 * th2 / 720.0;
            C = 1.0 / 6.0 - th2 / 120.0 + th2 * th2 / 5040.0;
        } else {
            A = sin(th) / th;
            B = (1.0 - cos(th)) / th2;
            C = (th - sin(th)) / (th2 * th);
        }
        double K[3][3] = {{0, -w[2], w[1]}, {w[2], 0, -w[0]}, {-w[1], w[0], 0}};
        double K2[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int k = 0; k < 3; ++k)
                    s += K[i][k] * K[k][j];
                K2[i][j] = s;
            }
        double V[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double I = i == j ? 1.0 : 0.0;
                R[i][j] = I + A * K[i][j] + B * K2[i][j];
                V[i][j] = I + B * K[i][j] + C * K2[i][j];
            }
        for (int i = 0; i < 3; ++i)
            t[i] = V[i][0] * v[0] + V[i][1] * v[1] + V[i][2] * v[2];
    }
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            T[4 * i + j] = R[i][j];
        T[4 * i + 3] = t[i];
    }
    T[12] = T[13] = T[14] = 0.0;
    T[15] = 1.0;
}

static void mat4_mul_d(const double A[16], const double B[16], double C[16])
{
    double R[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0;
            for (int k = 0; k < 4; ++k)
                s += A[4 * i + k] * B[4 * k + j];
            R[4 * i + j] = s;
        }
    memcpy(C, R, sizeof R);
}

/* ------------------------------------------------------------------ */
/* a17: colored ICP, FP64                                              */
/* ------------------------------------------------------------------ */
void orc_color_icp_f64(const float *sx, const float *srgb, int64_t ns, const float *tx,
                       const float *trgb, const double *tn, const double *tg, int64_t nt,
                       const orc_icp_params *P, const double T_init[16], orc_icp_result *res)
{
    double T[16];
    memcpy(T, T_init, sizeof T);
    memset(res, 0, sizeof *res);
    if (ns <= 0 || nt <= 0) {
        memcpy(res->T, T, sizeof T);
        res->status = 3;
        return;
    }
    float amin[3], amax[3], gmin[3];
    orc_aabb(tx, nt, 0, amin, amax);
    double cell = (double)P->max_corr;
    for (int a = 0; a < 3; ++a)
        gmin[a] = amin[a] - 1.5f * P->max_corr;
    /* target grid in FP64 cell coordinates (partition does not change the result
     * under the (distance, index) tie-break) */
    vkey *cells = (vkey *)malloc(sizeof(vkey) * (size_t)nt);
    for (int64_t j = 0; j < nt; ++j) {
        for (int a = 0; a < 3; ++a)
            cells[j].k[a] = (int32_t)floor(((double)tx[3 * j + a] - (double)gmin[a]) / cell);
        cells[j].idx = j;
    }
    qsort(cells, (size_t)nt, sizeof(vkey), cmp_vkey);
    ogrid g = {nt, cells};
    double *Is = (double *)malloc(sizeof(double) * (size_t)ns);
    double *It = (double *)malloc(sizeof(double) * (size_t)nt);
    for (int64_t i = 0; i < ns; ++i)
        Is[i] = orc_intensity(srgb[3 * i], srgb[3 * i + 1], srgb[3 * i + 2]);
    for (int64_t j = 0; j < nt; ++j)
        It[j] = orc_intensity(trgb[3 * j], trgb[3 * j + 1], trgb[3 * j + 2]);
    double slg = sqrt((double)P->lambda), slc = sqrt(1.0 - (double)P->lambda);
    double rr = cell * cell;
    int nthr = g_threads;
    double *part = (double *)calloc((size_t)nthr, sizeof(double) * 48);
    const float rrf = P->max_corr * P->max_corr;
    for (int it = 0; it < P->max_iter; ++it) {
        memset(part, 0, sizeof(double) * 48 * (size_t)nthr);
        float tf[12];
        for (int k = 0; k < 12; ++k)
            tf[k] = (float)T[k];
#ifdef _OPENMP
#pragma omp parallel num_threads(nthr)
#endif
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            double *acc = part + 48 * tid;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
            for (int64_t i = 0; i < ns; ++i) {
                d3 p0 = d3loadf(sx, i);
                d3 p;
                float pf[3] = {0.0f, 0.0f, 0.0f};
                if (P->search_f32) {
                    /* the GPU kernels' point: orc_apply_pose_f32 */
                    for (int r = 0; r < 3; ++r)
                        pf[r] = fmaf(tf[4 * r], sx[3 * i], fmaf(tf[4 * r + 1], sx[3 * i + 1],
                                                                fmaf(tf[4 * r + 2], sx[3 * i + 2], tf[4 * r + 3])));
                    p = d3m(pf[0], pf[1], pf[2]);
                } else {
                    p = d3m(T[0] * p0.x + T[1] * p0.y + T[2] * p0.z + T[3],
                            T[4] * p0.x + T[5] * p0.y + T[6] * p0.z + T[7],
                            T[8] * p0.x + T[9] * p0.y + T[10] * p0.z + T[11]);
                }
                int32_t c[3];
                c[0] = (int32_t)floor((p.x - (double)gmin[0]) / cell);
                c[1] = (int32_t)floor((p.y - (double)gmin[1]) / cell);
                c[2] = (int32_t)floor((p.z - (double)gmin[2]) / cell);
                double best = rr;
                float bestf = rrf;
                int64_t bi = -1;
                for (int di = -1; di <= 1; ++di)
                    for (int dj = -1; dj <= 1; ++dj)
                        for (int dk = -1; dk <= 1; ++dk) {
                            int32_t x = c[0] + di, y = c[1] + dj, z = c[2] + dk;
                            for (int64_t s = grid_lower(&g, x, y, z); s < g.n; ++s) {
                                const vkey *e = &g.cells[s];
                                if (e->k[0] != x || e->k[1] != y || e->k[2] != z)
                                    break;
                                if (P->search_f32) {
                                    /* unfused FP32 d^2 in the reference's order (q - p) */
                                    const float ex = tx[3 * e->idx] - pf[0], ey = tx[3 * e->idx + 1] - pf[1],
                                                ez = tx[3 * e->idx + 2] - pf[2];
                                    const float d2f = ex * ex + ey * ey + ez * ez;
                                    if (d2f < rrf && (bi < 0 || d2f < bestf || (d2f == bestf && e->idx < bi))) {
                                        bestf = d2f;
                                        bi = e->idx;
                                    }
                                    continue;
                                }
                                d3 q = d3loadf(tx, e->idx);
                                d3 dd = d3sub(q, p);
                                double d2 = d3dot(dd, dd);
                                if (d2 < rr && (bi < 0 || d2 < best || (d2 == best && e->idx < bi))) {
                                    best = d2;
                                    bi = e->idx;
                                }
                            }
                        }
                if (bi < 0)
                    continue;
                if (P->search_f32)
                    best = (double)bestf;
                d3 q = d3loadf(tx, bi);
                d3 n = d3m(tn[3 * bi], tn[3 * bi + 1], tn[3 * bi + 2]);
                d3 d = d3m(tg[3 * bi], tg[3 * bi + 1], tg[3 * bi + 2]);
                double rg = d3dot(d3sub(p, q), n);
                d3 proj = d3sub(p, d3mul(n, rg));
                double rc = It[bi] + d3dot(d, d3sub(proj, q)) - Is[i];
                double nd = d3dot(n, d);
                d3 dt = d3m(d.x - nd * n.x, d.y - nd * n.y, d.z - nd * n.z);
                d3 a1 = d3cross(p, n), a2 = d3cross(p, dt);
                double Jg[6] = {a1.x, a1.y, a1.z, n.x, n.y, n.z};
                double Jc[6] = {a2.x, a2.y, a2.z, dt.x, dt.y, dt.z};
                for (int k = 0; k < 6; ++k) {
                    Jg[k] *= slg;
                    Jc[k] *= slc;
                }
                double wg = slg * rg, wc = slc * rc;
                int u = 0;
                for (int a = 0; a < 6; ++a)
                    for (int b2 = a; b2 < 6; ++b2)
                        acc[u++] += Jg[a] * Jg[b2] + Jc[a] * Jc[b2];
                for (int a = 0; a < 6; ++a)
                    acc[21 + a] += Jg[a] * wg + Jc[a] * wc;
                acc[27] += wg * wg + wc * wc;
                acc[28] += 1.0;
                acc[29] += best;
            }
        }
        double S[30] = {0};
        for (int t = 0; t < nthr; ++t)
            for (int k = 0; k < 30; ++k)
                S[k] += part[48 * t + k];
        double jtj[36], jtr[6], x[6], Ti[16];
        int u = 0;
        for (int a = 0; a < 6; ++a)
            for (int b2 = a; b2 < 6; ++b2) {
                jtj[6 * a + b2] = S[u];
                jtj[6 * b2 + a] = S[u];
                ++u;
            }
        for (int a = 0; a < 6; ++a)
            jtr[a] = S[21 + a];
        res->rmse_ref = S[27] / (double)ns;
        res->fitness = S[28] / (double)ns;
        res->inlier_rmse = S[28] > 0 ? sqrt(S[29] / S[28]) : 0.0;
        if (orc_solve6(jtj, jtr, x))
            res->status = 4;
        orc_pose_from_x(x, P->update_map, Ti);
        mat4_mul_d(Ti, T, T);
        res->iterations = it + 1;
        double cth = 0.5 * (Ti[0] + Ti[5] + Ti[10] - 1.0);
        double tsq = Ti[3] * Ti[3] + Ti[7] * Ti[7] + Ti[11] * Ti[11];
        if (cth >= 1.0 - P->rot_eps && tsq <= P->trans_eps) {
            res->converged = 1;
            break;
        }
    }
    if (res->fitness == 0.0 && res->status == 0)
        res->status = 3;
    memcpy(res->T, T, sizeof T);
    free(part);
    free(Is);
    free(It);
    free(cells);
}

/* ------------------------------------------------------------------ */
/* a17-a18: colored ICP as the reference runs it                       */
/* ------------------------------------------------------------------ */

/* transform_point_functor (geometry_util.cuh:133-149): mat3x3 * mat3x1 (sum from 0)
 * + t, in place */
static void transform32(float *xyz, int64_t n, const float T[16])
{
    for (int64_t i = 0; i < n; ++i) {
        float p[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        for (int a = 0; a < 3; ++a) {
            float s = 0.0f;
            for (int k = 0; k < 3; ++k)
                s += T[4 * a + k] * p[k];
            xyz[3 * i + a] = s + T[4 * a + 3];
        }
    }
}

static void mat4_mul_f(const float A[16], const float B[16], float C[16])
{
    float R[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float s = 0.0f;
            for (int k = 0; k < 4; ++k)
                s += A[4 * i + k] * B[4 * k + j];
            R[4 * i + j] = s;
        }
    memcpy(C, R, sizeof R);
}

/* color_icp::align (registration/color_icp.cu:151-234) */
void orc_color_icp_ref32(const float *sx_in, const float *srgb, int64_t ns, const float *tx,
                         const float *trgb, const float *tn, const float *tg, int64_t nt,
                         int max_iter, float max_corr, const float T_init[16],
                         orc_icp_result *res)
{
    memset(res, 0, sizeof *res);
    float *sx = (float *)malloc(sizeof(float) * 3 * (size_t)(ns > 0 ? ns : 1));
    memcpy(sx, sx_in, sizeof(float) * 3 * (size_t)ns);
    float Tt[16];
    memcpy(Tt, T_init, sizeof Tt);
    transform32(sx, ns, T_init);
    int32_t *nn = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ns > 0 ? ns : 1));
    float tmin[3], tmax[3];
    orc_aabb(tx, nt, 1, tmin, tmax);
    const float lambda = 0.968f; /* color_icp.hpp:46 */
    const float trans_thr = 0.000001f, rot_thr = 1.0f - trans_thr;
    float jtj[36], jtr[6], r2 = 0.0f;
    for (int it = 0; it < max_iter && ns > 0; ++it) {
        /* point_cloud::nn_search (point_cloud.cu:506-557) bounds */
        float smin[3], smax[3], gmin[3];
        orc_aabb(sx, ns, 1, smin, smax);
        float pad = 1.5f * max_corr;
        for (int a = 0; a < 3; ++a)
            gmin[a] = (smin[a] < tmin[a] ? smin[a] : tmin[a]) - pad;
        orc_nn_search(sx, ns, tx, nt, max_corr, gmin, ORC_TIE_SCAN_ORDER, nn);
        orc_build_gn_ref32(sx, srgb, ns, tx, trgb, tn, tg, nn, lambda, jtj, jtr, &r2);
        double J[36], r[6], x[6], Td[16];
        for (int k = 0; k < 36; ++k)
            J[k] = jtj[k];
        for (int k = 0; k < 6; ++k)
            r[k] = jtr[k];
        float Ti[16];
        if (orc_solve6(J, r, x)) {
            for (int k = 0; k < 16; ++k)
                Ti[k] = (k % 5 == 0) ? 1.0f : 0.0f;
            res->status = 4;
        } else {
            orc_pose_from_x(x, ORC_UPDATE_EULER_ZYX, Td);
            for (int k = 0; k < 16; ++k)
                Ti[k] = (float)Td[k];
        }
        /* fitness / inlier rmse of this system */
        int64_t inl = 0;
        double dsum = 0;
        for (int64_t i = 0; i < ns; ++i)
            if (nn[i] >= 0) {
                ++inl;
                float dx = tx[3 * nn[i]] - sx[3 * i], dy = tx[3 * nn[i] + 1] - sx[3 * i + 1],
                      dz = tx[3 * nn[i] + 2] - sx[3 * i + 2];
                dsum += (double)(dx * dx + dy * dy + dz * dz);
            }
        res->fitness = (double)inl / (double)ns;
        res->inlier_rmse = inl ? sqrt(dsum / (double)inl) : 0.0;
        transform32(sx, ns, Ti);
        mat4_mul_f(Ti, Tt, Tt);
        res->iterations = it + 1;
        float cth = (float)(0.5 * (double)(Ti[0] + Ti[5] + Ti[10] - 1.0f));
        float tsq = Ti[3] * Ti[3] + Ti[7] * Ti[7] + Ti[11] * Ti[11];
        if (cth >= rot_thr && tsq <= trans_thr) {
            res->converged = 1;
            break;
        }
    }
    res->rmse_ref = ns > 0 ? (double)(r2 / (float)ns) : 0.0;
    for (int k = 0; k < 16; ++k)
        res->T[k] = Tt[k];
    free(sx);
    free(nn);
}

/* ------------------------------------------------------------------ */
/* a21: K unrolled Gauss-Newton steps of the colored-ICP objective and  */
/* their adjoint (no reference counterpart; FP64).  The per-point rows  */
/* follow compute_JTJ_JTr_and_r_gauss_newton_functor                    */
/* (cuda_color_icp_build_least_square.cu:184-253); the step follows     */
/* solve_JTJ_JTr (eigen_solver.hpp:44-85) with the chosen pose map.     */
/* ------------------------------------------------------------------ */

/* d U(x) / d x_m as 3x4 row-major blocks, for both pose maps */
void orc_pose_jacobian(const double x[6], int update_map, double dU[6][12])
{
    memset(dU, 0, sizeof(double) * 72);
    if (update_map == ORC_UPDATE_EULER_ZYX) {
        double ca = cos(x[0]), sa = sin(x[0]), cb = cos(x[1]), sb = sin(x[1]);
        double cc = cos(x[2]), sc = sin(x[2]);
        double Rx[9] = {1, 0, 0, 0, ca, -sa, 0, sa, ca}, dRx[9] = {0, 0, 0, 0, -sa, -ca, 0, ca, -sa};
        double Ry[9] = {cb, 0, sb, 0, 1, 0, -sb, 0, cb}, dRy[9] = {-sb, 0, cb, 0, 0, 0, -cb, 0, -sb};
        double Rz[9] = {cc, -sc, 0, sc, cc, 0, 0, 0, 1}, dRz[9] = {-sc, -cc, 0, cc, -sc, 0, 0, 0, 0};
        const double *f[3][3] = {{Rz, Ry, dRx}, {Rz, dRy, Rx}, {dRz, Ry, Rx}};
        for (int m = 0; m < 3; ++m) {
            double M1[9], M2[9];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double s = 0;
                    for (int k = 0; k < 3; ++k)
                        s += f[m][0][3 * i + k] * f[m][1][3 * k + j];
                    M1[3 * i + j] = s;
                }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double s = 0;
                    for (int k = 0; k < 3; ++k)
                        s += M1[3 * i + k] * f[m][2][3 * k + j];
                    M2[3 * i + j] = s;
                }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    dU[m][4 * i + j] = M2[3 * i + j];
        }
        for (int i = 0; i < 3; ++i)
            dU[3 + i][4 * i + 3] = 1.0;
        return;
    }
    /* SE(3) exponential: R = I + A K + B K^2, t = (I + B K + C K^2) v with
     * K = [w]x; A, B, C and their derivatives with respect to theta^2 */
    double w[3] = {x[0], x[1], x[2]}, v[3] = {x[3], x[4], x[5]};
    double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2], th = sqrt(th2);
    double A, B, C, Ad, Bd, Cd;
    if (th < 1e-2) {
        double t4 = th2 * th2, t6 = t4 * th2;
        A = 1.0 - th2 / 6.0 + t4 / 120.0 - t6 / 5040.0;
        B = 0.5 - th2 / 24.0 + t4 / 720.0 - t6 / 40320.0;
        C = 1.0 / 6.0 - th2 / 120.0 + t4 / 5040.0 - t6 / 362880.0;
        Ad = -1.0 / 6.0 + th2 / 60.0 - t4 / 1680.0;
        Bd = -1.0 / 24.0 + th2 / 360.0 - t4 / 13440.0;
        Cd = -1.0 / 120.0 + th2 / 2520.0 - t4 / 120960.0;
    } else {
        double s = sin(th), c = cos(th);
        A = s / th;
        B = (1.0 - c) / th2;
        C = (th - s) / (th2 * th);
        Ad = (th * c - s) / (2.0 * th2 * th);
        Bd = (th * s - 2.0 * (1.0 - c)) / (2.0 * th2 * th2);
        Cd = ((1.0 - c) * th - 3.0 * (th - s)) / (2.0 * th2 * th2 * th);
    }
    double K[3][3] = {{0, -w[2], w[1]}, {w[2], 0, -w[0]}, {-w[1], w[0], 0}};
    double K2[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k)
                s += K[i][k] * K[k][j];
            K2[i][j] = s;
        }
    for (int m = 0; m < 3; ++m) {
        double G[3][3] = {{0}};
        /* [e_m]x */
        if (m == 0) { G[1][2] = -1; G[2][1] = 1; }
        if (m == 1) { G[0][2] = 1; G[2][0] = -1; }
        if (m == 2) { G[0][1] = -1; G[1][0] = 1; }
        double GK[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int k = 0; k < 3; ++k)
                    s += G[i][k] * K[k][j] + K[i][k] * G[k][j];
                GK[i][j] = s;
            }
        double dR[3][3], dV[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                dR[i][j] = 2.0 * w[m] * Ad * K[i][j] + A * G[i][j] + 2.0 * w[m] * Bd * K2[i][j] + B * GK[i][j];
                dV[i][j] = 2.0 * w[m] * Bd * K[i][j] + B * G[i][j] + 2.0 * w[m] * Cd * K2[i][j] + C * GK[i][j];
            }
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j)
                dU[m][4 * i + j] = dR[i][j];
            dU[m][4 * i + 3] = dV[i][0] * v[0] + dV[i][1] * v[1] + dV[i][2] * v[2];
        }
    }
    for (int m = 0; m < 3; ++m)
        for (int i = 0; i < 3; ++i)
            dU[3 + m][4 * i + 3] = (i == m ? 1.0 : 0.0) + B * K[i][m] + C * K2[i][m];
}

/* the two weighted rows of one correspondence (FP64) */
typedef struct {
    double Jg[6], Jc[6], rg, rc;
    d3 n, dt; /* normal and the tangential colour gradient (I - n n^T) d */
} orc_rows;

static void rows_f64(d3 p, double Is, d3 q, double Iq, d3 n, d3 d, double slg, double slc, orc_rows *o)
{
    double rg = d3dot(d3sub(p, q), n);
    double nd = d3dot(n, d);
    d3 dt = d3m(d.x - nd * n.x, d.y - nd * n.y, d.z - nd * n.z);
    d3 a1 = d3cross(p, n), a2 = d3cross(p, dt);
    double Jg[6] = {a1.x, a1.y, a1.z, n.x, n.y, n.z};
    double Jc[6] = {a2.x, a2.y, a2.z, dt.x, dt.y, dt.z};
    for (int k = 0; k < 6; ++k) {
        o->Jg[k] = slg * Jg[k];
        o->Jc[k] = slc * Jc[k];
    }
    o->rg = slg * rg;
    o->rc = slc * (Iq + d3dot(dt, d3sub(p, q)) - Is);
    o->n = n;
    o->dt = dt;
}

typedef struct {
    const double *sx, *srgb;
    int64_t ns;
    const float *tx;
    const double *tn, *tg;
    double *It;
    int64_t nt;
    double slg, slc;
    float gmin[3];
    double cell, rr;
    ogrid g; /* FP64 cell coordinates, (distance, index) tie-break */
} unroll_ctx;

static d3 pose_apply(const double T[16], d3 s)
{
    return d3m(T[0] * s.x + T[1] * s.y + T[2] * s.z + T[3], T[4] * s.x + T[5] * s.y + T[6] * s.z + T[7],
               T[8] * s.x + T[9] * s.y + T[10] * s.z + T[11]);
}

static int64_t nn_f64(const unroll_ctx *u, d3 p)
{
    int32_t c[3];
    c[0] = (int32_t)floor((p.x - (double)u->gmin[0]) / u->cell);
    c[1] = (int32_t)floor((p.y - (double)u->gmin[1]) / u->cell);
    c[2] = (int32_t)floor((p.z - (double)u->gmin[2]) / u->cell);
    double best = u->rr;
    int64_t bi = -1;
    for (int di = -1; di <= 1; ++di)
        for (int dj = -1; dj <= 1; ++dj)
            for (int dk = -1; dk <= 1; ++dk) {
                int32_t x = c[0] + di, y = c[1] + dj, z = c[2] + dk;
                for (int64_t s = grid_lower(&u->g, x, y, z); s < u->g.n; ++s) {
                    const vkey *e = &u->g.cells[s];
                    if (e->k[0] != x || e->k[1] != y || e->k[2] != z)
                        break;
                    d3 dd = d3sub(d3loadf(u->tx, e->idx), p);
                    double d2 = d3dot(dd, dd);
                    if (d2 < u->rr && (bi < 0 || d2 < best || (d2 == best && e->idx < bi))) {
                        best = d2;
                        bi = e->idx;
                    }
                }
            }
    return bi;
}

static void unroll_open(unroll_ctx *u, const double *sx, const double *srgb, int64_t ns, const float *tx,
                        const float *trgb, const double *tn, const double *tg, int64_t nt,
                        const orc_unroll_params *p, int need_grid)
{
    memset(u, 0, sizeof *u);
    u->sx = sx, u->srgb = srgb, u->ns = ns, u->tx = tx, u->tn = tn, u->tg = tg, u->nt = nt;
    u->slg = sqrt((double)p->lambda);
    u->slc = sqrt(1.0 - (double)p->lambda);
    u->It = (double *)malloc(sizeof(double) * (size_t)(nt > 0 ? nt : 1));
    for (int64_t j = 0; j < nt; ++j)
        u->It[j] = orc_intensity(trgb[3 * j], trgb[3 * j + 1], trgb[3 * j + 2]);
    u->cell = (double)p->max_corr;
    u->rr = u->cell * u->cell;
    if (need_grid && nt > 0) {
        float amin[3], amax[3];
        orc_aabb(tx, nt, 0, amin, amax);
        for (int a = 0; a < 3; ++a)
            u->gmin[a] = amin[a] - 1.5f * p->max_corr;
        u->g.n = nt;
        u->g.cells = (vkey *)malloc(sizeof(vkey) * (size_t)nt);
        for (int64_t j = 0; j < nt; ++j) {
            for (int a = 0; a < 3; ++a)
                u->g.cells[j].k[a] = (int32_t)floor(((double)tx[3 * j + a] - (double)u->gmin[a]) / u->cell);
            u->g.cells[j].idx = j;
        }
        qsort(u->g.cells, (size_t)nt, sizeof(vkey), cmp_vkey);
    }
}

static void unroll_close(unroll_ctx *u)
{
    free(u->It);
    free(u->g.cells);
}

/* source intensity as an exact FP64 function of the colour (smooth in the colour) */
static const double kIw[3] = {0.2126, 0.7152, 0.0722};
static double src_intensity(const unroll_ctx *u, int64_t i)
{
    return kIw[0] * u->srgb[3 * i] + kIw[1] * u->srgb[3 * i + 1] + kIw[2] * u->srgb[3 * i + 2];
}

static int corr_rows(const unroll_ctx *u, int64_t i, int64_t j, d3 p, orc_rows *o)
{
    if (j < 0 || j >= u->nt)
        return 0;
    d3 q = d3loadf(u->tx, j);
    d3 n = d3m(u->tn[3 * j], u->tn[3 * j + 1], u->tn[3 * j + 2]);
    d3 d = d3m(u->tg[3 * j], u->tg[3 * j + 1], u->tg[3 * j + 2]);
    rows_f64(p, src_intensity(u, i), q, u->It[j], n, d, u->slg, u->slc, o);
    return 1;
}

/* one evaluation at pose T: correspondences (frozen from cin or searched and
 * written to cout), system S[28] = 21 upper JTJ + 6 JTr + sum r^2 */
static void unroll_eval(const unroll_ctx *u, const double T[16], const int32_t *cin, int32_t *cout, double S[28])
{
    memset(S, 0, sizeof(double) * 28);
    for (int64_t i = 0; i < u->ns; ++i) {
        d3 p = pose_apply(T, d3m(u->sx[3 * i], u->sx[3 * i + 1], u->sx[3 * i + 2]));
        int64_t j = cin ? cin[i] : nn_f64(u, p);
        if (cout)
            cout[i] = (int32_t)j;
        orc_rows o;
        if (!corr_rows(u, i, j, p, &o))
            continue;
        int k = 0;
        for (int a = 0; a < 6; ++a)
            for (int b = a; b < 6; ++b)
                S[k++] += o.Jg[a] * o.Jg[b] + o.Jc[a] * o.Jc[b];
        for (int a = 0; a < 6; ++a)
            S[21 + a] += o.Jg[a] * o.rg + o.Jc[a] * o.rc;
        S[27] += o.rg * o.rg + o.rc * o.rc;
    }
}

static void sys_to_full(const double S[28], double H[36], double b[6])
{
    int k = 0;
    for (int a = 0; a < 6; ++a)
        for (int c = a; c < 6; ++c) {
            H[6 * a + c] = H[6 * c + a] = S[k];
            ++k;
        }
    for (int a = 0; a < 6; ++a)
        b[a] = S[21 + a];
}

/* forward of the unrolled steps; Ts receives the K + 1 poses, xs the K steps,
 * Ss the K + 1 systems (each may be NULL) */
static double unroll_forward(const unroll_ctx *u, const orc_unroll_params *p, const double xi0[6],
                             const int32_t *cin, int32_t *cout, double *Ts, double *xs, double *Ss, int *status)
{
    double T[16], S[28];
    orc_pose_from_x(xi0, ORC_UPDATE_SE3_EXP, T);
    *status = 0;
    for (int k = 0; k <= p->K; ++k) {
        unroll_eval(u, T, cin ? cin + (size_t)k * u->ns : NULL, cout ? cout + (size_t)k * u->ns : NULL, S);
        if (Ts)
            memcpy(Ts + 16 * k, T, sizeof T);
        if (Ss)
            memcpy(Ss + 28 * k, S, sizeof S);
        if (k == p->K)
            break;
        double H[36], b[6], x[6], U[16];
        sys_to_full(S, H, b);
        if (orc_solve6(H, b, x))
            *status = 1;
        if (xs)
            memcpy(xs + 6 * k, x, sizeof x);
        orc_pose_from_x(x, p->update_map, U);
        mat4_mul_d(U, T, T);
    }
    return S[27];
}

double orc_icp_unrolled_f64(const double *sx, const double *srgb, int64_t ns, const float *tx, const float *trgb,
                            const double *tn, const double *tg, int64_t nt, const orc_unroll_params *p,
                            const double xi0[6], const int32_t *corr_in, int32_t *corr_out, double T_out[16])
{
    unroll_ctx u;
    unroll_open(&u, sx, srgb, ns, tx, trgb, tn, tg, nt, p, corr_in == NULL);
    double *Ts = (double *)malloc(sizeof(double) * 16 * (size_t)(p->K + 1));
    int status;
    double E = unroll_forward(&u, p, xi0, corr_in, corr_out, Ts, NULL, NULL, &status);
    if (T_out)
        memcpy(T_out, Ts + 16 * p->K, sizeof(double) * 16);
    free(Ts);
    unroll_close(&u);
    return E;
}

/* adjoint of one evaluation at pose T with correspondences c: the rows' adjoints
 * are  jbar = -y (j.x) - x (j.y) - r y  and  rbar = -(j.y) + 2 e r  (x = y = 0 for
 * the objective, e = 0 for a step).  Adds to dxyz, drgb and Tbar (3x4). */
static void unroll_point_adjoint(const unroll_ctx *u, const double T[16], const int32_t *c, const double x[6],
                                 const double y[6], double e, double *dxyz, double *drgb, double Tbar[12])
{
    for (int64_t i = 0; i < u->ns; ++i) {
        d3 s = d3m(u->sx[3 * i], u->sx[3 * i + 1], u->sx[3 * i + 2]);
        d3 p = pose_apply(T, s);
        orc_rows o;
        if (!corr_rows(u, i, c[i], p, &o))
            continue;
        d3 pb = d3m(0, 0, 0);
        double Ib = 0.0;
        for (int row = 0; row < 2; ++row) {
            const double *J = row ? o.Jc : o.Jg;
            double r = row ? o.rc : o.rg, w = row ? u->slc : u->slg;
            d3 dir = row ? o.dt : o.n;
            double jx = 0, jy = 0;
            for (int a = 0; a < 6; ++a) {
                jx += J[a] * x[a];
                jy += J[a] * y[a];
            }
            d3 jb = d3m(-y[0] * jx - x[0] * jy - r * y[0], -y[1] * jx - x[1] * jy - r * y[1],
                        -y[2] * jx - x[2] * jy - r * y[2]);
            double rb = -jy + 2.0 * e * r;
            /* J top = w (p x dir): d<jb, p x dir> = <dp, dir x jb> */
            d3 cr = d3cross(dir, jb);
            pb = d3m(pb.x + w * cr.x + rb * w * dir.x, pb.y + w * cr.y + rb * w * dir.y,
                     pb.z + w * cr.z + rb * w * dir.z);
            if (row)
                Ib += -rb * w;
        }
        /* p = R s + t */
        dxyz[3 * i + 0] += T[0] * pb.x + T[4] * pb.y + T[8] * pb.z;
        dxyz[3 * i + 1] += T[1] * pb.x + T[5] * pb.y + T[9] * pb.z;
        dxyz[3 * i + 2] += T[2] * pb.x + T[6] * pb.y + T[10] * pb.z;
        for (int a = 0; a < 3; ++a)
            drgb[3 * i + a] += Ib * kIw[a];
        double pv[3] = {pb.x, pb.y, pb.z}, sv[3] = {s.x, s.y, s.z};
        for (int r = 0; r < 3; ++r) {
            for (int cidx = 0; cidx < 3; ++cidx)
                Tbar[4 * r + cidx] += pv[r] * sv[cidx];
            Tbar[4 * r + 3] += pv[r];
        }
    }
}

/* adjoint of T' = U(x) T through the step map and the solve: from Tbar' (3x4)
 * to xbar, then y = H^-1 xbar; Tbar <- U^T Tbar' (rows 0-2) */
static int unroll_step_adjoint(const double T[16], const double x[6], const double S[28], int map,
                               const double Tbar_next[12], double Tbar[12], double y[6])
{
    double U[16], dU[6][12], Ub[12], xb[6];
    orc_pose_from_x(x, map, U);
    orc_pose_jacobian(x, map, dU);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 4; ++b) {
            double s = 0;
            for (int c = 0; c < 4; ++c)
                s += Tbar_next[4 * a + c] * T[4 * b + c];
            Ub[4 * a + b] = s;
        }
    for (int m = 0; m < 6; ++m) {
        double s = 0;
        for (int k = 0; k < 12; ++k)
            s += Ub[k] * dU[m][k];
        xb[m] = s;
    }
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 4; ++c) {
            double s = 0;
            for (int b = 0; b < 3; ++b)
                s += U[4 * b + a] * Tbar_next[4 * b + c];
            Tbar[4 * a + c] = s;
        }
    double H[36], bb[6], nxb[6];
    sys_to_full(S, H, bb);
    for (int m = 0; m < 6; ++m)
        nxb[m] = -xb[m];
    return orc_solve6(H, nxb, y); /* y = -H^-1 (-xbar) */
}

int orc_icp_unrolled_vjp_f64(const double *sx, const double *srgb, int64_t ns, const float *tx, const float *trgb,
                             const double *tn, const double *tg, int64_t nt, const orc_unroll_params *p,
                             const double xi0[6], const int32_t *corr, const double dT[16], double dE,
                             double dxi0[6], double *dxyz, double *drgb)
{
    unroll_ctx u;
    unroll_open(&u, sx, srgb, ns, tx, trgb, tn, tg, nt, p, 0);
    const int K = p->K;
    double *Ts = (double *)malloc(sizeof(double) * 16 * (size_t)(K + 1));
    double *xs = (double *)malloc(sizeof(double) * 6 * (size_t)(K > 0 ? K : 1));
    double *Ss = (double *)malloc(sizeof(double) * 28 * (size_t)(K + 1));
    int status;
    unroll_forward(&u, p, xi0, corr, NULL, Ts, xs, Ss, &status);
    memset(dxyz, 0, sizeof(double) * 3 * (size_t)ns);
    memset(drgb, 0, sizeof(double) * 3 * (size_t)ns);
    double Tbar[12], Tprev[12], y[6];
    const double zero6[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 12; ++k)
        Tbar[k] = dT[k];
    unroll_point_adjoint(&u, Ts + 16 * K, corr + (size_t)K * ns, zero6, zero6, dE, dxyz, drgb, Tbar);
    for (int k = K - 1; k >= 0; --k) {
        status |= unroll_step_adjoint(Ts + 16 * k, xs + 6 * k, Ss + 28 * k, p->update_map, Tbar, Tprev, y);
        unroll_point_adjoint(&u, Ts + 16 * k, corr + (size_t)k * ns, xs + 6 * k, y, 0.0, dxyz, drgb, Tprev);
        memcpy(Tbar, Tprev, sizeof Tbar);
    }
    double dX[6][12];
    orc_pose_jacobian(xi0, ORC_UPDATE_SE3_EXP, dX);
    for (int m = 0; m < 6; ++m) {
        double s = 0;
        for (int k = 0; k < 12; ++k)
            s += Tbar[k] * dX[m][k];
        dxi0[m] = s;
    }
    free(Ts);
    free(xs);
    free(Ss);
    unroll_close(&u);
    return status;
}

/* ------------------------------------------------------------------ */
/* radius outlier removal (point_cloud.cu:238-280,                     */
/* cuda_nn_search.cu:416-542,725-800): cell 2r, origin min - 1.5 cells; */
/* per axis the own cell and the nearer neighbour (lower corner fused   */
/* cell * c + origin); count d^2 < r^2 with d = q - p, self included;   */
/* keep when the count exceeds min_nn; survivors in input order.        */
/* ------------------------------------------------------------------ */
int64_t orc_radius_outlier_removal(const float *xyz, const float *rgb, int64_t n, float radius, int min_nn,
                                   float *out_xyz, float *out_rgb)
{
    if (n <= 0)
        return 0;
    float mn[3], mx[3], gmin[3];
    orc_aabb(xyz, n, 1, mn, mx);
    const float cell = 2.0f * radius, pad = 1.5f * cell, rr = radius * radius;
    for (int a = 0; a < 3; ++a)
        gmin[a] = mn[a] - pad;
    ogrid g;
    grid_build(&g, xyz, n, gmin, cell);
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) {
        f3 p = f3load(xyz, i);
        float pv[3] = {p.x, p.y, p.z};
        int32_t c[3];
        int b[3], e[3];
        for (int a = 0; a < 3; ++a) {
            c[a] = floor_div_key(pv[a], gmin[a], cell);
            float lo = fmaf(cell, (float)c[a], gmin[a]);
            float off = pv[a] - lo;
            b[a] = off >= radius ? 0 : -1;
            e[a] = off < radius ? 1 : 2;
        }
        int count = 0;
        for (int dx = b[0]; dx < e[0]; ++dx)
            for (int dy = b[1]; dy < e[1]; ++dy)
                for (int dz = b[2]; dz < e[2]; ++dz) {
                    int32_t x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                    for (int64_t s = grid_lower(&g, x, y, z); s < g.n; ++s) {
                        const vkey *k = &g.cells[s];
                        if (k->k[0] != x || k->k[1] != y || k->k[2] != z)
                            break;
                        f3 q = f3load(xyz, k->idx);
                        float ddx = q.x - p.x, ddy = q.y - p.y, ddz = q.z - p.z;
                        float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                        count += d2 < rr;
                    }
                }
        if (count > min_nn) {
            for (int a = 0; a < 3; ++a) {
                out_xyz[3 * m + a] = xyz[3 * i + a];
                out_rgb[3 * m + a] = rgb[3 * i + a];
            }
            ++m;
        }
    }
    grid_free(&g);
    return m;
}

/* the GPU ICP kernels' FP32 pose application, x' = fma(r0, x, fma(r1, y, fma(r2, z, t)))
 * with T the row-major 3x4 pose rounded to float */
void orc_apply_pose_f32(const double T[16], const float *xyz, int64_t n, float *out)
{
    float t[12];
    for (int k = 0; k < 12; ++k)
        t[k] = (float)T[k];
    for (int64_t i = 0; i < n; ++i) {
        const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        for (int r = 0; r < 3; ++r)
            out[3 * i + r] = fmaf(t[4 * r], x, fmaf(t[4 * r + 1], y, fmaf(t[4 * r + 2], z, t[4 * r + 3])));
    }
}
