// compat_app.cpp -- the registration flow of the reference's apps/test_color_icp.cpp
// (create_from_pcl, voxel_grid_down_sample, estimate_normals, color_icp, transform,
// download), written against the gca:: compatibility headers, plus the front-end
// calls around it (radius_outlier_removal, create_new_by_index, get_abs_residual,
// nn_search).  Input and output are flat binary files so that the Python test can
// replay the same steps through the C ABI and compare.
//
//   compat_app <in.bin> <out.bin>
//   in:  int64 n_src, int64 n_tgt, then per cloud n records {float x, y, z; uint8 r, g, b, pad}
//   out: float T[16], float rmse, int64 n_src_ds, int64 n_tgt_ds, float abs_mean,
//        int64 n_ror, int64 n_sel, int32 nn[n_src_ds], float src_xyz[n_src * 3] (transformed)
#include "geometry/point_cloud.hpp"
#include "registration/color_icp.hpp"

#include <cstdio>
#include <vector>

// a stand-in for pcl::PointCloud<pcl::PointXYZRGB>
struct PointXYZRGB
{
    float x, y, z;
    uint8_t r, g, b, pad;
};
struct HostCloud
{
    std::vector<PointXYZRGB> points;
};

static bool read_cloud(FILE *f, int64_t n, HostCloud &c)
{
    c.points.resize((size_t)n);
    return fread(c.points.data(), sizeof(PointXYZRGB), (size_t)n, f) == (size_t)n;
}

int main(int argc, char **argv)
{
    if (argc != 3)
        return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f)
        return 3;
    int64_t ns = 0, nt = 0;
    HostCloud src, tgt;
    bool ok = fread(&ns, 8, 1, f) == 1 && fread(&nt, 8, 1, f) == 1 && read_cloud(f, ns, src) && read_cloud(f, nt, tgt);
    fclose(f);
    if (!ok)
        return 4;

    auto src_device = gca::point_cloud::create_from_pcl(src);
    auto tgt_device = gca::point_cloud::create_from_pcl(tgt);
    auto down_sample_src = src_device->voxel_grid_down_sample(0.02f);
    auto down_sample_tgt = tgt_device->voxel_grid_down_sample(0.02f);
    if (!down_sample_tgt->estimate_normals(0.05f))
        return 5;

    gca::color_icp color_icp(100, 0.05f, 0.04f);
    color_icp.set_source_point_cloud(down_sample_src);
    color_icp.set_target_point_cloud(down_sample_tgt);
    if (!color_icp.align())
        return 6;
    const gca::mat4x4 T = color_icp.get_final_transformation_matrix();
    const float rmse = color_icp.get_RSME();
    auto res = color_icp.get_abs_residual_host();

    src_device->transform(T);
    auto pc_host = src_device->download();

    auto ror = down_sample_src->radius_outlier_removal(0.05f, 4);
    std::vector<gca::index_t> pick;
    for (int64_t i = 0; i < (int64_t)down_sample_src->points_number(); i += 3)
        pick.push_back((gca::index_t)i);
    auto sel = down_sample_src->create_new_by_index(pick);
    std::vector<gca::index_t> nn;
    gca::point_cloud::nn_search(nn, *down_sample_src, *down_sample_tgt, 0.05f);
    // the AoS view of the reference's point_t must describe the same points
    auto aos = down_sample_src->get_points().download();
    auto ds = down_sample_src->download();
    for (size_t i = 0; i < aos.size(); ++i)
        if (aos[i].coordinates.x != ds[i].coordinates.x || aos[i].color.b != ds[i].color.b)
            return 7;

    FILE *o = fopen(argv[2], "wb");
    if (!o)
        return 8;
    const int64_t n_src_ds = (int64_t)down_sample_src->points_number(),
                  n_tgt_ds = (int64_t)down_sample_tgt->points_number(), n_ror = (int64_t)ror->points_number(),
                  n_sel = (int64_t)sel->points_number();
    fwrite(T.m, sizeof(float), 16, o);
    fwrite(&rmse, sizeof(float), 1, o);
    fwrite(&n_src_ds, 8, 1, o);
    fwrite(&n_tgt_ds, 8, 1, o);
    fwrite(&res.second, sizeof(float), 1, o);
    fwrite(&n_ror, 8, 1, o);
    fwrite(&n_sel, 8, 1, o);
    fwrite(nn.data(), sizeof(gca::index_t), nn.size(), o);
    for (const auto &p : pc_host)
        fwrite(&p.coordinates, sizeof(float), 3, o);
    fclose(o);
    std::printf("compat_app: %lld -> %lld source points, rmse %g\n", (long long)ns, (long long)n_src_ds, rmse);
    return 0;
}
