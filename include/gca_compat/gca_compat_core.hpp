// gca_compat_core.hpp -- the reference's C++ types (namespace gca) over the C ABI.
//
// Compatibility layer for code written against XssZuiNB/CUDA_3D's point-cloud and
// registration classes: the same class names, member functions, argument meaning
// and error behaviour (failures print a message and return false / an empty
// result; nothing throws).  Build with -I<repo>/include -I<repo>/include/gca_compat
// -I<cuda>/include and link libgca3d.so; no nvcc needed.
//
// Differences, all documented at the member: device arrays are gca::device_vector
// (size/data/download) instead of thrust::device_vector; create_from_pcl takes any
// cloud type with .points[i].{x, y, z, r, g, b} (PCL's PointXYZRGB qualifies) and
// there is a PCL-free create_from_xyzrgb; get_max_bound reports the true maximum
// (the reference starts its maximum at FLT_MIN).  Every thread gets its own
// library context on device GCA3D_DEVICE (default 0).
#pragma once

#include "gca3d.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <utility>
#include <vector>

#include <vector_functions.h>
#include <vector_types.h>

namespace gca
{
typedef int32_t index_t;
typedef int32_t counter_t;

// geometry/type.hpp:15-20
enum point_property : uint8_t
{
    invalid = 0,
    active = 1,
    inactive = 2
};

// geometry/type.hpp:21-63
struct color3
{
    float r;
    float g;
    float b;

    operator float3() const { return make_float3(r, g, b); }
    color3 operator+(const color3 &o) const { return color3{r + o.r, g + o.g, b + o.b}; }
    color3 &operator+=(const color3 &o)
    {
        r += o.r, g += o.g, b += o.b;
        return *this;
    }
    // luminance weights of the paper the reference cites, summed in double
    float to_intensity() const
    {
        return (float)(0.2126 * (double)r + 0.7152 * (double)g + 0.0722 * (double)b);
    }
    float get_average() const { return (float)(((double)r + (double)g + (double)b) / 3.0); }
    template <typename T> color3 operator/(T n) const
    {
        const float s = 1.0f / (float)n;
        return color3{r * s, g * s, b * s};
    }
};

// geometry/type.hpp:65-70: 28 bytes
struct point_t
{
    float3 coordinates;
    color3 color;
    point_property property;
};
static_assert(sizeof(point_t) == 28, "point_t is 28 bytes");

inline std::ostream &operator<<(std::ostream &os, const point_t &p)
{
    return os << "(" << p.coordinates.x << ", " << p.coordinates.y << ", " << p.coordinates.z << ") rgb("
              << p.color.r << ", " << p.color.g << ", " << p.color.b << ")";
}

// 4 x 4 float matrix, row-major, the subset of util/math.cuh's matNxM<4, 4> that
// registration code uses
struct mat4x4
{
    float m[16];

    mat4x4() { set_identity(); }
    float &operator()(int i, int j) { return m[4 * i + j]; }
    float operator()(int i, int j) const { return m[4 * i + j]; }
    void set_identity()
    {
        for (int k = 0; k < 16; ++k)
            m[k] = (k % 5 == 0) ? 1.0f : 0.0f;
    }
    static mat4x4 get_identity() { return mat4x4(); }
    mat4x4 operator*(const mat4x4 &o) const
    {
        mat4x4 r;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
            {
                float s = 0.0f;
                for (int k = 0; k < 4; ++k)
                    s += m[4 * i + k] * o.m[4 * k + j];
                r.m[4 * i + j] = s;
            }
        return r;
    }
};

namespace detail
{
inline void warn(const char *what, gca3d_context *ctx)
{
    std::cout << "\033[33m" << what << (ctx ? ": " : "") << (ctx ? gca3d_last_error(ctx) : "") << "\033[0m"
              << std::endl;
}

// one library context per host thread (the reference is single-threaded and
// synchronous; every call here is ordered on this context's stream)
inline gca3d_context *ctx()
{
    struct holder
    {
        gca3d_context *h = nullptr;
        bool tried = false;
        ~holder()
        {
            if (h)
                gca3d_destroy(h);
        }
    };
    thread_local holder c;
    if (!c.h && !c.tried)
    {
        c.tried = true;
        const char *dev = std::getenv("GCA3D_DEVICE");
        if (gca3d_create(dev ? std::atoi(dev) : 0, nullptr, &c.h) != GCA3D_OK)
        {
            c.h = nullptr;
            warn("gca: no device context", nullptr);
        }
    }
    return c.h;
}

inline bool ok(int st, const char *what)
{
    if (st == GCA3D_OK)
        return true;
    warn(what, ctx());
    return false;
}
} // namespace detail

// device array with the parts of thrust::device_vector that callers of the
// reference use: size, empty, data, and a copy to the host
template <typename T> class device_vector
{
public:
    device_vector() = default;
    explicit device_vector(size_t n) { resize(n); }
    device_vector(const device_vector &o) { *this = o; }
    device_vector(device_vector &&o) noexcept { swap(o); }
    device_vector &operator=(const device_vector &o)
    {
        if (this != &o)
        {
            resize(o.m_size);
            if (m_size)
                gca3d_copy(detail::ctx(), m_ptr, o.m_ptr, (int64_t)(m_size * sizeof(T)));
        }
        return *this;
    }
    device_vector &operator=(device_vector &&o) noexcept
    {
        swap(o);
        return *this;
    }
    ~device_vector() { release(); }

    size_t size() const { return m_size; }
    bool empty() const { return m_size == 0; }
    T *data() { return m_ptr; }
    const T *data() const { return m_ptr; }
    // contents are not kept
    void resize(size_t n)
    {
        if (n == m_size)
            return;
        release();
        if (n)
        {
            void *p = nullptr;
            if (!detail::ok(gca3d_device_alloc(detail::ctx(), (int64_t)(n * sizeof(T)), &p), "gca: device_alloc"))
                return;
            m_ptr = static_cast<T *>(p);
            m_size = n;
        }
    }
    std::vector<T> download() const
    {
        std::vector<T> h(m_size);
        if (m_size)
            gca3d_copy(detail::ctx(), h.data(), m_ptr, (int64_t)(m_size * sizeof(T)));
        return h;
    }
    void swap(device_vector &o) noexcept
    {
        std::swap(m_ptr, o.m_ptr);
        std::swap(m_size, o.m_size);
    }

private:
    void release()
    {
        if (m_ptr && detail::ctx())
            gca3d_device_free(detail::ctx(), m_ptr);
        m_ptr = nullptr;
        m_size = 0;
    }
    T *m_ptr = nullptr;
    size_t m_size = 0;
};

// camera/camera_param.hpp:5-37
struct intrinsics
{
    float fx;
    float fy;
    float cx;
    float cy;
};

struct extrinsics
{
    float rotation[9];
    float translation[3];
};

enum frame_format
{
    BGR8,
    RGB8,
    Z16
};

enum param_type
{
    depth_intrinsics,
    color_intrinsics,
    depth2color_extrinsics,
    color2depth_extrinsics,
    width,
    height,
    depth_scale
};
} // namespace gca
