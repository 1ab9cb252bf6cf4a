// gca_compat_cloud.hpp -- gca::cuda_*_frame, gca::cuda_camera_param and
// gca::point_cloud over the C ABI (see gca_compat_core.hpp for the conventions).
#pragma once

#include "gca_compat_core.hpp"

#include <limits>

namespace gca
{

// cuda_container/cuda_container.hpp:12-64: a frame in device memory
template <typename T, int C> class compat_frame
{
public:
    compat_frame(uint32_t w, uint32_t h) : m_w(w), m_h(h), m_data((size_t)w * h * C) {}
    compat_frame(const T *frame, uint32_t w, uint32_t h) : compat_frame(w, h) { upload(frame, w, h); }
    void upload(const T *src, uint32_t w, uint32_t h)
    {
        if (w != m_w || h != m_h)
        {
            m_w = w, m_h = h;
            m_data.resize((size_t)w * h * C);
        }
        if (src && m_data.size())
            gca3d_copy(detail::ctx(), m_data.data(), src, (int64_t)(m_data.size() * sizeof(T)));
    }
    void clear()
    {
        m_data = device_vector<T>();
        m_w = m_h = 0;
    }
    uint32_t w() const { return m_w; }
    uint32_t h() const { return m_h; }
    const device_vector<T> &vec() const { return m_data; }

private:
    uint32_t m_w, m_h;
    device_vector<T> m_data;
};

class cuda_color_frame : public compat_frame<uint8_t, 3>
{
public:
    using compat_frame::compat_frame;
    uint32_t get_color_frame_width() const { return w(); }
    uint32_t get_color_frame_height() const { return h(); }
    const device_vector<uint8_t> &get_color_frame_vec() const { return vec(); }
};

class cuda_depth_frame : public compat_frame<uint16_t, 1>
{
public:
    using compat_frame::compat_frame;
    uint32_t get_depth_frame_width() const { return w(); }
    uint32_t get_depth_frame_height() const { return h(); }
    const device_vector<uint16_t> &get_depth_frame_vec() const { return vec(); }
};

// cuda_container/cuda_container.hpp:65-113.  The pointer getters return host
// copies (the reference hands out device pointers for its kernels).
class cuda_camera_param
{
public:
    cuda_camera_param() = default;
    cuda_camera_param(const intrinsics &depth_intrin, const intrinsics &color_intrin,
                      const extrinsics &depth2color_extrin, const extrinsics &color2depth_extrin, uint32_t width,
                      uint32_t height, float depth_scale, frame_format depth_format = Z16,
                      frame_format color_format = BGR8)
        : m_depth_intrin(depth_intrin), m_color_intrin(color_intrin), m_d2c(depth2color_extrin),
          m_c2d(color2depth_extrin), m_width(width), m_height(height), m_depth_scale(depth_scale),
          m_depth_format(depth_format), m_color_format(color_format)
    {
    }
    bool set(const intrinsics &in, param_type t)
    {
        if (t == depth_intrinsics)
            m_depth_intrin = in;
        else if (t == color_intrinsics)
            m_color_intrin = in;
        else
            return false;
        return true;
    }
    bool set(const extrinsics &ex, param_type t)
    {
        if (t == depth2color_extrinsics)
            m_d2c = ex;
        else if (t == color2depth_extrinsics)
            m_c2d = ex;
        else
            return false;
        return true;
    }
    bool set(uint32_t length, param_type t)
    {
        if (t == width)
            m_width = length;
        else if (t == height)
            m_height = length;
        else
            return false;
        return true;
    }
    bool set(float scale)
    {
        m_depth_scale = scale;
        return true;
    }
    const intrinsics *get_depth_intrinsics_ptr() const { return &m_depth_intrin; }
    const intrinsics *get_color_intrinsics_ptr() const { return &m_color_intrin; }
    const extrinsics *get_depth2color_extrinsics_ptr() const { return &m_d2c; }
    const extrinsics *get_color2depth_extrinsics_ptr() const { return &m_c2d; }
    uint32_t get_width() const { return m_width; }
    uint32_t get_height() const { return m_height; }
    float get_depth_scale() const { return m_depth_scale; }
    frame_format get_depth_frame_format() const { return m_depth_format; }
    frame_format get_color_frame_format() const { return m_color_format; }

private:
    intrinsics m_depth_intrin{}, m_color_intrin{};
    extrinsics m_d2c{{1, 0, 0, 0, 1, 0, 0, 0, 1}, {0, 0, 0}}, m_c2d{{1, 0, 0, 0, 1, 0, 0, 0, 1}, {0, 0, 0}};
    uint32_t m_width = 0, m_height = 0;
    float m_depth_scale = 0.001f;
    frame_format m_depth_format = Z16, m_color_format = BGR8;
};

class color_icp;

// geometry/point_cloud.hpp:20-140 (clustering, plane removal and segmentation are
// not part of this library)
class point_cloud
{
public:
    point_cloud() = default;
    // n points at the origin, black (the reference's n default points)
    explicit point_cloud(size_t n_points)
    {
        if (!alloc(n_points))
            return;
        std::vector<float> zero(3 * n_points, 0.0f);
        detail::ok(gca3d_cloud_upload(detail::ctx(), m_cloud.get(), zero.data(), zero.data(), (int64_t)n_points),
                   "gca: point_cloud(n)");
    }
    point_cloud(const point_cloud &o) { *this = o; }
    point_cloud &operator=(const point_cloud &o)
    {
        if (this == &o)
            return *this;
        invalidate();
        m_has_normals = false;
        if (!o.m_cloud)
        {
            m_cloud.reset();
            return *this;
        }
        if (!alloc(o.capacity()))
            return *this;
        if (detail::ok(gca3d_cloud_copy(detail::ctx(), o.m_cloud.get(), m_cloud.get()), "gca: copy"))
            m_has_normals = o.m_has_normals;
        return *this;
    }
    // appends other (the reference's operator+ also appends to *this)
    point_cloud &operator+(const point_cloud &other) { return *this += other; }
    point_cloud &operator+=(const point_cloud &other)
    {
        if (!other.m_cloud || other.points_number() == 0)
            return *this;
        const size_t n = points_number(), m = other.points_number();
        if (!m_cloud || capacity() < n + m)
        {
            point_cloud grown;
            if (!grown.alloc(std::max(n + m, 2 * capacity())))
                return *this;
            if (m_cloud && n)
                gca3d_cloud_copy(detail::ctx(), m_cloud.get(), grown.m_cloud.get());
            grown.m_has_normals = n ? m_has_normals : other.m_has_normals;
            m_cloud = grown.m_cloud;
            if (!n)
                m_has_normals = other.m_has_normals;
        }
        invalidate();
        detail::ok(gca3d_cloud_append(detail::ctx(), m_cloud.get(), other.m_cloud.get()), "gca: append");
        int h = 0;
        gca3d_cloud_has_normals(m_cloud.get(), &h);
        m_has_normals = h != 0;
        return *this;
    }
    point_cloud &operator+=(point_cloud &&other) { return *this += static_cast<const point_cloud &>(other); }

    void download(std::vector<point_t> &dst) const { dst = download(); }
    std::vector<point_t> download() const
    {
        const size_t n = points_number();
        std::vector<point_t> out(n);
        if (!n)
            return out;
        std::vector<float> xyz(3 * n), rgb(3 * n);
        int64_t got = 0;
        gca3d_cloud_download(detail::ctx(), m_cloud.get(), xyz.data(), rgb.data(), nullptr, nullptr, (int64_t)n,
                             &got);
        for (size_t i = 0; i < n; ++i)
        {
            out[i].coordinates = make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
            out[i].color = color3{rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]};
            out[i].property = active;
        }
        return out;
    }
    std::vector<float3> download_normals() const
    {
        const size_t n = m_has_normals ? points_number() : 0;
        std::vector<float3> out(n);
        if (!n)
            return out;
        std::vector<float> v(3 * n);
        int64_t got = 0;
        gca3d_cloud_download(detail::ctx(), m_cloud.get(), nullptr, nullptr, v.data(), nullptr, (int64_t)n, &got);
        for (size_t i = 0; i < n; ++i)
            out[i] = make_float3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        return out;
    }

    bool has_points() const { return points_number() > 0; }
    bool has_normals() const { return m_has_normals; }
    size_t points_number() const
    {
        int64_t n = 0;
        if (m_cloud)
            gca3d_cloud_size(detail::ctx(), m_cloud.get(), &n);
        return (size_t)n;
    }

    // point_cloud.cu:145-181: returns true at once when normals exist
    bool estimate_normals(float search_radius)
    {
        if (m_has_normals)
            return true;
        if (!m_cloud || !(search_radius > 0.0f))
        {
            detail::warn("gca: estimate_normals needs points and a radius > 0", nullptr);
            return false;
        }
        invalidate();
        if (!detail::ok(gca3d_estimate_normals(detail::ctx(), m_cloud.get(), search_radius, 0),
                        "gca: estimate_normals"))
            return false;
        m_has_normals = true;
        return true;
    }

    // the 28-byte records, materialised on first use after a change
    const device_vector<point_t> &get_points() const
    {
        materialise();
        return m_aos;
    }
    const device_vector<float3> &get_normals() const
    {
        materialise();
        return m_aos_normals;
    }
    const float3 &get_min_bound() const
    {
        bounds();
        return m_min_bound;
    }
    // the true maximum (the reference's starts at FLT_MIN)
    const float3 &get_max_bound() const
    {
        bounds();
        return m_max_bound;
    }
    const float3 &get_centroid()
    {
        const auto pts = download();
        double s[3] = {0, 0, 0};
        for (const auto &p : pts)
            s[0] += p.coordinates.x, s[1] += p.coordinates.y, s[2] += p.coordinates.z;
        const double n = pts.empty() ? 1.0 : (double)pts.size();
        m_centroid = make_float3((float)(s[0] / n), (float)(s[1] / n), (float)(s[2] / n));
        return m_centroid;
    }

    // point_cloud.cu:93-105
    void transform(const mat4x4 &T)
    {
        if (!m_cloud)
            return;
        double d[16];
        for (int k = 0; k < 16; ++k)
            d[k] = T.m[k];
        invalidate();
        detail::ok(gca3d_transform(detail::ctx(), m_cloud.get(), d), "gca: transform");
    }

    // point_cloud.cu:198-229 (the result has no normals)
    std::shared_ptr<point_cloud> voxel_grid_down_sample(float voxel_size)
    {
        auto out = std::make_shared<point_cloud>();
        if (!m_cloud || !(voxel_size > 0.0f))
        {
            detail::warn("gca: voxel size must be > 0, an empty point cloud returned", nullptr);
            return out;
        }
        if (!out->alloc(capacity()))
            return out;
        if (!detail::ok(gca3d_voxel_downsample(detail::ctx(), m_cloud.get(), voxel_size, out->m_cloud.get()),
                        "gca: voxel_grid_down_sample"))
            return std::make_shared<point_cloud>();
        return out;
    }

    // point_cloud.cu:238-280
    std::shared_ptr<point_cloud> radius_outlier_removal(float radius, counter_t min_neighbors_in_radius)
    {
        auto out = std::make_shared<point_cloud>();
        if (!m_cloud || !(radius > 0.0f))
        {
            detail::warn("gca: radius must be > 0, an empty point cloud returned", nullptr);
            return out;
        }
        if (!out->alloc(capacity()))
            return out;
        if (!detail::ok(gca3d_radius_outlier_removal(detail::ctx(), m_cloud.get(), radius, min_neighbors_in_radius,
                                                     out->m_cloud.get()),
                        "gca: radius_outlier_removal"))
            return std::make_shared<point_cloud>();
        return out;
    }

    // point_cloud.cu:438-453 (indices on the device or the host)
    std::shared_ptr<point_cloud> create_new_by_index(const device_vector<index_t> &indices) const
    {
        return select(indices.data(), indices.size());
    }
    std::shared_ptr<point_cloud> create_new_by_index(const std::vector<index_t> &indices) const
    {
        return select(indices.data(), indices.size());
    }

    // point_cloud.cu:455-479: Z16 depth and BGR8 colour, adaptive bilateral filter
    static std::shared_ptr<point_cloud> create_from_rgbd(const cuda_depth_frame &depth, const cuda_color_frame &color,
                                                         const cuda_camera_param &param,
                                                         float threshold_min_in_meter = 0.0f,
                                                         float threshold_max_in_meter = 10.0f)
    {
        auto pc = std::make_shared<point_cloud>();
        if (param.get_depth_frame_format() != Z16 || param.get_color_frame_format() != BGR8)
        {
            detail::warn("gca: frame format is not supported, an empty point cloud returned", nullptr);
            return pc;
        }
        const uint32_t w = param.get_width(), h = param.get_height();
        if (!pc->alloc((size_t)w * h))
            return pc;
        const intrinsics &di = *param.get_depth_intrinsics_ptr(), &ci = *param.get_color_intrinsics_ptr();
        const extrinsics &e = *param.get_depth2color_extrinsics_ptr();
        gca3d_intrinsics a{di.fx, di.fy, di.cx, di.cy}, b{ci.fx, ci.fy, ci.cx, ci.cy};
        gca3d_extrinsics x;
        std::memcpy(x.rotation, e.rotation, sizeof x.rotation);
        std::memcpy(x.translation, e.translation, sizeof x.translation);
        if (!detail::ok(gca3d_frame_to_cloud(detail::ctx(), depth.get_depth_frame_vec().data(),
                                             color.get_color_frame_vec().data(), (int)w, (int)h, &a, &b, &x,
                                             param.get_depth_scale(), threshold_min_in_meter,
                                             threshold_max_in_meter, nullptr, pc->m_cloud.get()),
                        "gca: create_from_rgbd"))
            return std::make_shared<point_cloud>();
        return pc;
    }

    // point_cloud.cu:481-504 for any cloud whose .points[i] has x, y, z and 8-bit
    // r, g, b (pcl::PointCloud<pcl::PointXYZRGB> among them)
    template <typename Cloud> static std::shared_ptr<point_cloud> create_from_pcl(const Cloud &pcl_pc)
    {
        const size_t n = pcl_pc.points.size();
        std::vector<float> xyz(3 * n), rgb(3 * n);
        const float scale = 1.0f / 255.0f;
        for (size_t i = 0; i < n; ++i)
        {
            const auto &p = pcl_pc.points[i];
            xyz[3 * i] = p.x, xyz[3 * i + 1] = p.y, xyz[3 * i + 2] = p.z;
            rgb[3 * i] = (float)p.r * scale, rgb[3 * i + 1] = (float)p.g * scale, rgb[3 * i + 2] = (float)p.b * scale;
        }
        return create_from_xyzrgb(xyz, rgb);
    }
    // n x 3 positions and colours in [0, 1]
    static std::shared_ptr<point_cloud> create_from_xyzrgb(const std::vector<float> &xyz,
                                                           const std::vector<float> &rgb)
    {
        auto pc = std::make_shared<point_cloud>();
        const size_t n = xyz.size() / 3;
        if (!pc->alloc(n))
            return pc;
        detail::ok(gca3d_cloud_upload(detail::ctx(), pc->m_cloud.get(), xyz.data(),
                                      rgb.size() == xyz.size() ? rgb.data() : nullptr, (int64_t)n),
                   "gca: create_from_xyzrgb");
        return pc;
    }

    // point_cloud.cu:506-557: nearest reference point within radius, -1 if none
    static device_vector<index_t> nn_search(const point_cloud &query_pc, const point_cloud &reference_pc,
                                            float radius)
    {
        device_vector<index_t> out(query_pc.points_number());
        if (out.empty() || !reference_pc.m_cloud)
            return out;
        if (!detail::ok(gca3d_nn_search(detail::ctx(), query_pc.m_cloud.get(), reference_pc.m_cloud.get(), radius,
                                        out.data()),
                        "gca: nn_search"))
            return device_vector<index_t>();
        return out;
    }
    static void nn_search(std::vector<index_t> &result_nn_idx, point_cloud &query_pc, point_cloud &reference_pc,
                          float radius)
    {
        result_nn_idx = nn_search(query_pc, reference_pc, radius).download();
    }

    gca3d_cloud *handle() const { return m_cloud.get(); }

private:
    friend class color_icp;

    size_t capacity() const
    {
        int64_t c = 0;
        if (m_cloud)
            gca3d_cloud_capacity(m_cloud.get(), &c);
        return (size_t)c;
    }
    bool alloc(size_t capacity)
    {
        gca3d_cloud *c = nullptr;
        if (!detail::ok(gca3d_cloud_create(detail::ctx(), (int64_t)std::max<size_t>(capacity, 1), &c),
                        "gca: cloud_create"))
            return false;
        m_cloud = std::shared_ptr<gca3d_cloud>(c, [](gca3d_cloud *p) { gca3d_cloud_destroy(p); });
        invalidate();
        return true;
    }
    void invalidate()
    {
        m_aos_valid = false;
        m_has_bound = false;
    }
    void materialise() const
    {
        if (m_aos_valid)
            return;
        const size_t n = points_number();
        m_aos.resize(n);
        m_aos_normals.resize(m_has_normals ? n : 0);
        if (n)
            gca3d_cloud_to_aos(detail::ctx(), m_cloud.get(), m_aos.data(),
                               m_has_normals ? reinterpret_cast<float *>(m_aos_normals.data()) : nullptr);
        m_aos_valid = true;
    }
    void bounds() const
    {
        if (m_has_bound)
            return;
        float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
        if (m_cloud && points_number())
            gca3d_bounds(detail::ctx(), m_cloud.get(), mn, mx);
        m_min_bound = make_float3(mn[0], mn[1], mn[2]);
        m_max_bound = make_float3(mx[0], mx[1], mx[2]);
        m_has_bound = true;
    }
    std::shared_ptr<point_cloud> select(const index_t *idx, size_t n) const
    {
        auto out = std::make_shared<point_cloud>();
        if (!m_cloud || !out->alloc(n))
            return out;
        if (!detail::ok(gca3d_cloud_select(detail::ctx(), m_cloud.get(), idx, (int64_t)n, out->m_cloud.get()),
                        "gca: create_new_by_index"))
            return std::make_shared<point_cloud>();
        out->m_has_normals = m_has_normals;
        return out;
    }

    std::shared_ptr<gca3d_cloud> m_cloud;
    bool m_has_normals = false;
    mutable device_vector<point_t> m_aos;
    mutable device_vector<float3> m_aos_normals;
    mutable bool m_aos_valid = false;
    mutable bool m_has_bound = false;
    mutable float3 m_min_bound{0, 0, 0}, m_max_bound{0, 0, 0};
    float3 m_centroid{0, 0, 0};
};
} // namespace gca
