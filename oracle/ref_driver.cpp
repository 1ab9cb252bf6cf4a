/*
 * ref_driver.cpp -- C entry points around the reference's own host-compiled
 * Thrust code (XssZuiNB/CUDA_3D, serial CPP backend).  Checker only: used to
 * generate the golden fixtures that pin the oracle.  The bound computations that
 * live in the reference's point_cloud class are restated here with citations.
 */
#include "geometry/cuda_estimate_normals.cuh"
#include "geometry/cuda_nn_search.cuh"
#include "geometry/cuda_voxel_grid_down_sample.cuh"
#include "geometry/geometry_util.cuh"
#include "geometry/type.hpp"
#include "registration/cuda_color_icp_build_least_square.cuh"
#include "registration/cuda_compute_color_gradient.cuh"

#include <thrust/host_vector.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

namespace
{
thrust::device_vector<gca::point_t> to_points(const float *xyz, const float *rgb, int64_t n)
{
    thrust::host_vector<gca::point_t> h(n);
    for (int64_t i = 0; i < n; ++i)
    {
        gca::point_t p;
        p.coordinates = make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        p.color = gca::color3{rgb ? rgb[3 * i] : 0.0f, rgb ? rgb[3 * i + 1] : 0.0f,
                              rgb ? rgb[3 * i + 2] : 0.0f};
        p.property = gca::point_property::inactive;
        h[i] = p;
    }
    return thrust::device_vector<gca::point_t>(h);
}

thrust::device_vector<float3> to_f3(const float *v, int64_t n)
{
    thrust::host_vector<float3> h(n);
    for (int64_t i = 0; i < n; ++i)
        h[i] = make_float3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    return thrust::device_vector<float3>(h);
}
} // namespace

extern "C" {

/* geometry_util.cuh:88-105 */
void ref_aabb(const float *xyz, int64_t n, float mn[3], float mx[3])
{
    auto pts = to_points(xyz, nullptr, n);
    auto b = gca::cuda_compute_min_max_bound(pts);
    mn[0] = b.first.x, mn[1] = b.first.y, mn[2] = b.first.z;
    mx[0] = b.second.x, mx[1] = b.second.y, mx[2] = b.second.z;
}

/* point_cloud::voxel_grid_down_sample (point_cloud.cu:198-229) */
int64_t ref_voxel_downsample(const float *xyz, const float *rgb, int64_t n, float voxel,
                             float *out_xyz, float *out_rgb)
{
    auto pts = to_points(xyz, rgb, n);
    auto b = gca::cuda_compute_min_max_bound(pts);
    auto res = gca::cuda_voxel_grid_downsample(pts, b.first, voxel);
    thrust::host_vector<gca::point_t> h(res);
    for (size_t i = 0; i < h.size(); ++i)
    {
        out_xyz[3 * i] = h[i].coordinates.x;
        out_xyz[3 * i + 1] = h[i].coordinates.y;
        out_xyz[3 * i + 2] = h[i].coordinates.z;
        out_rgb[3 * i] = h[i].color.r;
        out_rgb[3 * i + 1] = h[i].color.g;
        out_rgb[3 * i + 2] = h[i].color.b;
    }
    return (int64_t)h.size();
}

/* point_cloud::nn_search (point_cloud.cu:506-557): grid spans the union of both
 * bounds padded by 1.5 r (float) */
int ref_nn_search(const float *q, int64_t nq, const float *r, int64_t nr, float radius,
                  int32_t *out, float gmin_out[3])
{
    auto Q = to_points(q, nullptr, nq);
    auto R = to_points(r, nullptr, nr);
    auto bq = gca::cuda_compute_min_max_bound(Q);
    auto br = gca::cuda_compute_min_max_bound(R);
    float pad = 1.5f * radius;
    float3 mn = make_float3(std::min(bq.first.x, br.first.x) - pad,
                            std::min(bq.first.y, br.first.y) - pad,
                            std::min(bq.first.z, br.first.z) - pad);
    float3 mx = make_float3(std::max(bq.second.x, br.second.x) + pad,
                            std::max(bq.second.y, br.second.y) + pad,
                            std::max(bq.second.z, br.second.z) + pad);
    thrust::device_vector<gca::index_t> res(nq);
    auto err = gca::cuda_nn_search(res, Q, R, mn, mx, radius);
    thrust::host_vector<gca::index_t> h(res);
    for (int64_t i = 0; i < nq; ++i)
        out[i] = h[i];
    gmin_out[0] = mn.x, gmin_out[1] = mn.y, gmin_out[2] = mn.z;
    return (int)err;
}

/* point_cloud::estimate_normals bounds (point_cloud.cu:145-181): the padding is a
 * double (1.5 * r) and the result is narrowed to float */
static void normals_bounds(const thrust::device_vector<gca::point_t> &pts, float radius,
                           float3 &mn, float3 &mx)
{
    auto b = gca::cuda_compute_min_max_bound(pts);
    auto padding = 1.5 * radius;
    mn = make_float3(b.first.x - padding, b.first.y - padding, b.first.z - padding);
    mx = make_float3(b.second.x + padding, b.second.y + padding, b.second.z + padding);
}

/* cuda_search_radius_neighbors with the estimate_normals bounds */
int64_t ref_radius_search(const float *xyz, int64_t n, float radius, int32_t *counts,
                          int32_t *starts, int32_t *list, int64_t cap, float gmin_out[3])
{
    auto pts = to_points(xyz, nullptr, n);
    float3 mn, mx;
    normals_bounds(pts, radius, mn, mx);
    thrust::device_vector<gca::index_t> all;
    thrust::device_vector<thrust::pair<gca::index_t, gca::counter_t>> pairs;
    gca::cuda_search_radius_neighbors(all, pairs, pts, mn, mx, radius);
    thrust::host_vector<gca::index_t> ha(all);
    thrust::host_vector<thrust::pair<gca::index_t, gca::counter_t>> hp(pairs);
    for (int64_t i = 0; i < n; ++i)
    {
        starts[i] = hp[i].first;
        counts[i] = hp[i].second;
    }
    for (size_t i = 0; i < ha.size() && (int64_t)i < cap; ++i)
        list[i] = ha[i];
    gmin_out[0] = mn.x, gmin_out[1] = mn.y, gmin_out[2] = mn.z;
    return (int64_t)ha.size();
}

int ref_estimate_normals(const float *xyz, int64_t n, float radius, float *out,
                         float gmin_out[3])
{
    auto pts = to_points(xyz, nullptr, n);
    float3 mn, mx;
    normals_bounds(pts, radius, mn, mx);
    thrust::device_vector<float3> res(n);
    auto err = gca::cuda_estimate_normals(res, pts, mn, mx, radius);
    thrust::host_vector<float3> h(res);
    for (int64_t i = 0; i < n; ++i)
        out[3 * i] = h[i].x, out[3 * i + 1] = h[i].y, out[3 * i + 2] = h[i].z;
    gmin_out[0] = mn.x, gmin_out[1] = mn.y, gmin_out[2] = mn.z;
    return (int)err;
}

/* color_icp::compute_color_gradient_target bounds (color_icp.cu:50-87): float padding */
int ref_color_gradient(const float *xyz, const float *rgb, const float *nrm, int64_t n,
                       float radius, float *out, float gmin_out[3])
{
    auto pts = to_points(xyz, rgb, n);
    auto normals = to_f3(nrm, n);
    auto b = gca::cuda_compute_min_max_bound(pts);
    float p = 1.5f * radius;
    float3 mn = b.first - make_float3(p, p, p);
    float3 mx = b.second + make_float3(p, p, p);
    thrust::device_vector<float3> res;
    auto err = gca::cuda_compute_color_gradient(res, pts, normals, mn, mx, radius);
    thrust::host_vector<float3> h(res);
    for (int64_t i = 0; i < n; ++i)
        out[3 * i] = h[i].x, out[3 * i + 1] = h[i].y, out[3 * i + 2] = h[i].z;
    gmin_out[0] = mn.x, gmin_out[1] = mn.y, gmin_out[2] = mn.z;
    return (int)err;
}

/* cuda_build_gauss_newton_color_icp (cuda_color_icp_build_least_square.cu:431-474) */
int ref_build_gn(const float *sx, const float *srgb, int64_t ns, const float *tx,
                 const float *trgb, const float *tn, const float *tg, int64_t nt,
                 const int32_t *nn, float lambda, float jtj[36], float jtr[6], float *r2)
{
    auto S = to_points(sx, srgb, ns);
    auto T = to_points(tx, trgb, nt);
    auto N = to_f3(tn, nt);
    auto G = to_f3(tg, nt);
    thrust::device_vector<gca::index_t> idx(nn, nn + ns);
    mat6x6 A;
    mat6x1 b;
    float e;
    auto err = gca::cuda_build_gauss_newton_color_icp(A, b, e, S, T, N, G, idx, lambda);
    for (int i = 0; i < 6; ++i)
    {
        for (int j = 0; j < 6; ++j)
            jtj[6 * i + j] = A(i, j);
        jtr[i] = b(i);
    }
    *r2 = e;
    return (int)err;
}

/* cuda_compute_abs_residual_color_icp (cuda_color_icp_build_least_square.cu:310-350) */
int ref_abs_residual(const float *sx, const float *srgb, int64_t ns, const float *tx,
                     const float *trgb, const float *tn, const float *tg, int64_t nt,
                     const int32_t *nn, float lambda, float *out)
{
    auto S = to_points(sx, srgb, ns);
    auto T = to_points(tx, trgb, nt);
    auto N = to_f3(tn, nt);
    auto G = to_f3(tg, nt);
    thrust::device_vector<gca::index_t> idx(nn, nn + ns);
    thrust::device_vector<float> res(ns);
    auto err = gca::cuda_compute_abs_residual_color_icp(res, S, T, N, G, idx, lambda);
    thrust::host_vector<float> h(res);
    for (int64_t i = 0; i < ns; ++i)
        out[i] = h[i];
    return (int)err;
}

/* cuda_transform_point (geometry_util.cuh:133-149, 167-171) */
void ref_transform(float *xyz, int64_t n, const float T[16])
{
    auto pts = to_points(xyz, nullptr, n);
    mat4x4 M;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            M(i, j) = T[4 * i + j];
    gca::cuda_transform_point(pts, M);
    thrust::host_vector<gca::point_t> h(pts);
    for (int64_t i = 0; i < n; ++i)
    {
        xyz[3 * i] = h[i].coordinates.x;
        xyz[3 * i + 1] = h[i].coordinates.y;
        xyz[3 * i + 2] = h[i].coordinates.z;
    }
}

/* point_cloud::radius_outlier_removal (point_cloud.cu:368-412): cell side 2 r,
 * padding 1.5 cell (float) */
int64_t ref_radius_outlier_removal(const float *xyz, const float *rgb, int64_t n, float radius,
                                   int min_nn, float *out_xyz, float *out_rgb)
{
    auto pts = to_points(xyz, rgb, n);
    auto b = gca::cuda_compute_min_max_bound(pts);
    float cell = 2.0f * radius;
    float pad = 1.5f * cell;
    float3 mn = make_float3(b.first.x - pad, b.first.y - pad, b.first.z - pad);
    float3 mx = make_float3(b.second.x + pad, b.second.y + pad, b.second.z + pad);
    thrust::device_vector<gca::point_t> res;
    gca::cuda_grid_radius_outliers_removal(res, pts, mn, mx, cell, radius, min_nn);
    thrust::host_vector<gca::point_t> h(res);
    for (size_t i = 0; i < h.size(); ++i)
    {
        out_xyz[3 * i] = h[i].coordinates.x;
        out_xyz[3 * i + 1] = h[i].coordinates.y;
        out_xyz[3 * i + 2] = h[i].coordinates.z;
        out_rgb[3 * i] = h[i].color.r;
        out_rgb[3 * i + 1] = h[i].color.g;
        out_rgb[3 * i + 2] = h[i].color.b;
    }
    return (int64_t)h.size();
}
}

/* the reference's error printer (util/cuda_util.cuh:64-72) names the CUDA runtime's
 * error-string function; the host build has no runtime, so it gets a fixed text */
extern "C" const char *cudaGetErrorString(cudaError_t)
{
    return "cuda error (host build of the reference)";
}
