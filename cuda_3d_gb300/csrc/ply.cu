// ply.cu -- PLY point files on the host (no device work, no context).
//
// The reference reads its fragment files through PCL (apps/test_color_icp.cpp:350,
// point_cloud::create_from_pcl, src/geometry/point_cloud.cu:481-504).  Here a small
// reader / writer covers the files such pipelines use: "format ascii 1.0" and
// "format binary_little_endian 1.0", a vertex element with x, y, z and optional
// nx, ny, nz and red, green, blue (8-bit, scaled by 1/255 as create_from_pcl does, or
// float); scalar properties of any PLY type are accepted and skipped when unused.
// List properties in the vertex element, big-endian files and elements before the
// vertex element that cannot be skipped (lists in binary files) are reported as
// GCA3D_ERR_NOT_SUPPORTED.
#include "gca3d.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace
{

enum PlyType
{
    kI8,
    kU8,
    kI16,
    kU16,
    kI32,
    kU32,
    kF32,
    kF64,
    kBad
};

PlyType ply_type(const std::string &t)
{
    if (t == "char" || t == "int8")
        return kI8;
    if (t == "uchar" || t == "uint8")
        return kU8;
    if (t == "short" || t == "int16")
        return kI16;
    if (t == "ushort" || t == "uint16")
        return kU16;
    if (t == "int" || t == "int32")
        return kI32;
    if (t == "uint" || t == "uint32")
        return kU32;
    if (t == "float" || t == "float32")
        return kF32;
    if (t == "double" || t == "float64")
        return kF64;
    return kBad;
}

int type_size(PlyType t)
{
    static const int s[] = {1, 1, 2, 2, 4, 4, 4, 8};
    return t == kBad ? 0 : s[t];
}

struct Prop
{
    std::string name;
    PlyType type = kBad;
    bool list = false;
};

struct Element
{
    std::string name;
    int64_t count = 0;
    std::vector<Prop> props;
};

struct Header
{
    bool binary = false;
    std::vector<Element> elements;
    std::streampos data = 0;
};

int read_header(std::ifstream &f, Header &h)
{
    std::string line;
    if (!std::getline(f, line) || line.compare(0, 3, "ply") != 0)
        return GCA3D_ERR_INVALID_VALUE;
    bool format = false;
    while (std::getline(f, line))
    {
        if (!line.empty() && line.back() == '\r')
            line.pop_back();
        std::istringstream ss(line);
        std::string key;
        ss >> key;
        if (key == "format")
        {
            std::string fmt;
            ss >> fmt;
            if (fmt == "ascii")
                h.binary = false;
            else if (fmt == "binary_little_endian")
                h.binary = true;
            else
                return GCA3D_ERR_NOT_SUPPORTED;
            format = true;
        }
        else if (key == "element")
        {
            Element e;
            ss >> e.name >> e.count;
            if (e.count < 0)
                return GCA3D_ERR_INVALID_VALUE;
            h.elements.push_back(e);
        }
        else if (key == "property")
        {
            if (h.elements.empty())
                return GCA3D_ERR_INVALID_VALUE;
            Prop p;
            std::string t;
            ss >> t;
            if (t == "list")
            {
                std::string ct, it;
                ss >> ct >> it >> p.name;
                p.list = true;
                p.type = ply_type(it);
            }
            else
            {
                p.type = ply_type(t);
                ss >> p.name;
            }
            if (p.type == kBad)
                return GCA3D_ERR_INVALID_VALUE;
            h.elements.back().props.push_back(p);
        }
        else if (key == "end_header")
        {
            h.data = f.tellg();
            return format ? GCA3D_OK : GCA3D_ERR_INVALID_VALUE;
        }
    }
    return GCA3D_ERR_INVALID_VALUE;
}

double load_le(const unsigned char *b, PlyType t)
{
    // assemble little-endian values byte by byte (host byte order does not matter)
    uint64_t u = 0;
    const int n = type_size(t);
    for (int i = n - 1; i >= 0; --i)
        u = (u << 8) | b[i];
    switch (t)
    {
    case kI8:
        return (double)(int8_t)(uint8_t)u;
    case kU8:
        return (double)(uint8_t)u;
    case kI16:
        return (double)(int16_t)(uint16_t)u;
    case kU16:
        return (double)(uint16_t)u;
    case kI32:
        return (double)(int32_t)(uint32_t)u;
    case kU32:
        return (double)(uint32_t)u;
    case kF32:
    {
        const uint32_t w = (uint32_t)u;
        float v;
        memcpy(&v, &w, 4);
        return (double)v;
    }
    case kF64:
    {
        double v;
        memcpy(&v, &u, 8);
        return v;
    }
    default:
        return 0.0;
    }
}

struct Layout
{
    int xyz[3] = {-1, -1, -1}, nrm[3] = {-1, -1, -1}, rgb[3] = {-1, -1, -1};
    bool rgb8 = true;
};

Layout vertex_layout(const Element &v)
{
    Layout L;
    static const char *xyz[] = {"x", "y", "z"}, *nrm[] = {"nx", "ny", "nz"}, *rgb[] = {"red", "green", "blue"};
    for (int i = 0; i < (int)v.props.size(); ++i)
        for (int a = 0; a < 3; ++a)
        {
            if (v.props[i].name == xyz[a])
                L.xyz[a] = i;
            if (v.props[i].name == nrm[a])
                L.nrm[a] = i;
            if (v.props[i].name == rgb[a])
            {
                L.rgb[a] = i;
                L.rgb8 = L.rgb8 && (v.props[i].type == kU8);
            }
        }
    return L;
}

bool has3(const int *k) { return k[0] >= 0 && k[1] >= 0 && k[2] >= 0; }

// position of the vertex element and a check that what precedes it can be skipped
int locate_vertex(const Header &h, int &vi)
{
    vi = -1;
    for (int e = 0; e < (int)h.elements.size(); ++e)
        if (h.elements[e].name == "vertex")
        {
            vi = e;
            break;
        }
    if (vi < 0)
        return GCA3D_ERR_INVALID_VALUE;
    for (const Prop &p : h.elements[vi].props)
        if (p.list)
            return GCA3D_ERR_NOT_SUPPORTED;
    for (int e = 0; e < vi; ++e)
        for (const Prop &p : h.elements[e].props)
            if (p.list && h.binary)
                return GCA3D_ERR_NOT_SUPPORTED;
    if (!has3(vertex_layout(h.elements[vi]).xyz))
        return GCA3D_ERR_INVALID_VALUE;
    return GCA3D_OK;
}

} // namespace

extern "C" {

int gca3d_ply_info(const char *path, int64_t *n_points, int *has_normals, int *has_colors)
{
    if (!path)
        return GCA3D_ERR_INVALID_VALUE;
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return GCA3D_ERR_INVALID_VALUE;
    Header h;
    int st = read_header(f, h);
    int vi = -1;
    if (!st)
        st = locate_vertex(h, vi);
    if (st)
        return st;
    const Layout L = vertex_layout(h.elements[vi]);
    if (n_points)
        *n_points = h.elements[vi].count;
    if (has_normals)
        *has_normals = has3(L.nrm);
    if (has_colors)
        *has_colors = has3(L.rgb);
    return GCA3D_OK;
}

int gca3d_ply_read(const char *path, float *xyz, float *rgb, float *nrm, int64_t cap, int64_t *n)
{
    if (!path || !xyz)
        return GCA3D_ERR_INVALID_VALUE;
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return GCA3D_ERR_INVALID_VALUE;
    Header h;
    int st = read_header(f, h);
    int vi = -1;
    if (!st)
        st = locate_vertex(h, vi);
    if (st)
        return st;
    const Element &V = h.elements[vi];
    if (V.count > cap)
        return GCA3D_ERR_CAPACITY;
    const Layout L = vertex_layout(V);
    const bool want_n = nrm && has3(L.nrm), want_c = rgb && has3(L.rgb);
    f.seekg(h.data);
    std::vector<double> vals(V.props.size());
    if (!h.binary)
    {
        std::string line;
        for (int e = 0; e < vi; ++e) // preceding elements: one line per item
            for (int64_t i = 0; i < h.elements[e].count; ++i)
                if (!std::getline(f, line))
                    return GCA3D_ERR_INVALID_VALUE;
        for (int64_t i = 0; i < V.count; ++i)
        {
            for (size_t k = 0; k < vals.size(); ++k)
                if (!(f >> vals[k]))
                    return GCA3D_ERR_INVALID_VALUE;
            for (int a = 0; a < 3; ++a)
            {
                xyz[3 * i + a] = (float)vals[L.xyz[a]];
                if (want_n)
                    nrm[3 * i + a] = (float)vals[L.nrm[a]];
                if (want_c)
                    rgb[3 * i + a] = L.rgb8 ? (float)vals[L.rgb[a]] * (1.0f / 255.0f) : (float)vals[L.rgb[a]];
            }
        }
    }
    else
    {
        for (int e = 0; e < vi; ++e)
        {
            int64_t rec = 0;
            for (const Prop &p : h.elements[e].props)
                rec += type_size(p.type);
            f.seekg(rec * h.elements[e].count, std::ios::cur);
        }
        std::vector<int> off(V.props.size());
        int rec = 0;
        for (size_t k = 0; k < V.props.size(); ++k)
        {
            off[k] = rec;
            rec += type_size(V.props[k].type);
        }
        std::vector<unsigned char> buf((size_t)rec * 4096);
        for (int64_t i0 = 0; i0 < V.count; i0 += 4096)
        {
            const int64_t m = std::min<int64_t>(4096, V.count - i0);
            if (!f.read(reinterpret_cast<char *>(buf.data()), (std::streamsize)(rec * m)))
                return GCA3D_ERR_INVALID_VALUE;
            for (int64_t j = 0; j < m; ++j)
            {
                const unsigned char *r = buf.data() + (size_t)rec * j;
                const int64_t i = i0 + j;
                for (int a = 0; a < 3; ++a)
                {
                    xyz[3 * i + a] = (float)load_le(r + off[L.xyz[a]], V.props[L.xyz[a]].type);
                    if (want_n)
                        nrm[3 * i + a] = (float)load_le(r + off[L.nrm[a]], V.props[L.nrm[a]].type);
                    if (want_c)
                    {
                        const float c = (float)load_le(r + off[L.rgb[a]], V.props[L.rgb[a]].type);
                        rgb[3 * i + a] = L.rgb8 ? c * (1.0f / 255.0f) : c;
                    }
                }
            }
        }
    }
    if (n)
        *n = V.count;
    return GCA3D_OK;
}

int gca3d_ply_write(const char *path, const float *xyz, const float *rgb, const float *nrm, int64_t n, int binary)
{
    if (!path || (n > 0 && !xyz) || n < 0)
        return GCA3D_ERR_INVALID_VALUE;
    FILE *f = fopen(path, "wb");
    if (!f)
        return GCA3D_ERR_INVALID_VALUE;
    fprintf(f, "ply\nformat %s 1.0\nelement vertex %lld\n", binary ? "binary_little_endian" : "ascii",
            (long long)n);
    fprintf(f, "property float x\nproperty float y\nproperty float z\n");
    if (nrm)
        fprintf(f, "property float nx\nproperty float ny\nproperty float nz\n");
    if (rgb)
        fprintf(f, "property uchar red\nproperty uchar green\nproperty uchar blue\n");
    fprintf(f, "end_header\n");
    auto c8 = [](float c) {
        const float v = std::nearbyint(c * 255.0f);
        return (unsigned char)(v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v));
    };
    auto put_f32 = [&](float v) {
        uint32_t u;
        memcpy(&u, &v, 4);
        const unsigned char b[4] = {(unsigned char)u, (unsigned char)(u >> 8), (unsigned char)(u >> 16),
                                    (unsigned char)(u >> 24)};
        fwrite(b, 1, 4, f);
    };
    for (int64_t i = 0; i < n; ++i)
    {
        if (binary)
        {
            for (int a = 0; a < 3; ++a)
                put_f32(xyz[3 * i + a]);
            if (nrm)
                for (int a = 0; a < 3; ++a)
                    put_f32(nrm[3 * i + a]);
            if (rgb)
                for (int a = 0; a < 3; ++a)
                {
                    const unsigned char c = c8(rgb[3 * i + a]);
                    fwrite(&c, 1, 1, f);
                }
        }
        else
        {
            fprintf(f, "%.9g %.9g %.9g", xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
            if (nrm)
                fprintf(f, " %.9g %.9g %.9g", nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
            if (rgb)
                fprintf(f, " %d %d %d", c8(rgb[3 * i]), c8(rgb[3 * i + 1]), c8(rgb[3 * i + 2]));
            fprintf(f, "\n");
        }
    }
    const bool ok = ferror(f) == 0;
    fclose(f);
    return ok ? GCA3D_OK : GCA3D_ERR_INVALID_VALUE;
}

} // extern "C"
