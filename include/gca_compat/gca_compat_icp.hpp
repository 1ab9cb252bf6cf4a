// gca_compat_icp.hpp -- gca::color_icp over the C ABI (see gca_compat_core.hpp).
#pragma once

#include "gca_compat_cloud.hpp"

namespace gca
{

// registration/color_icp.hpp:16-63 and color_icp.cu:17-234: lambda 0.968, the Euler
// ZYX step map, convergence when cos(step angle) >= 1 - 1e-6 and |step t|^2 <= 1e-6.
// The source is deep-copied and transformed by the result; the target is shared
// and needs normals; its colour gradient is computed with the given radius.
class color_icp
{
public:
    color_icp() = delete;
    color_icp(size_t maximum_iterations, float max_correspondence_distance, float search_radius_color_gradient)
        : m_max_iter(maximum_iterations), m_max_corr_dist(max_correspondence_distance),
          m_search_radius_color_gradient(search_radius_color_gradient)
    {
    }

    void set_source_point_cloud(const std::shared_ptr<const point_cloud> new_pc)
    {
        reset();
        m_source_pc = new_pc ? std::make_shared<point_cloud>(*new_pc) : nullptr;
    }
    void set_target_point_cloud(const std::shared_ptr<const point_cloud> new_pc)
    {
        reset();
        m_target_pc = new_pc;
    }

    bool align()
    {
        if (!m_source_pc || !m_target_pc)
        {
            detail::warn("gca: color_icp needs a source and a target point cloud", nullptr);
            return false;
        }
        if (!m_target_pc->has_normals())
        {
            detail::warn("gca: color_icp needs target normals (estimate_normals)", nullptr);
            return false;
        }
        gca3d_icp_params p;
        std::memset(&p, 0, sizeof p);
        p.n_scales = 1;
        p.scales[0].voxel = 0.0f;
        p.scales[0].max_iter = (int)m_max_iter;
        p.scales[0].max_corr = m_max_corr_dist;
        p.scales[0].normal_radius = 0.0f;
        p.scales[0].grad_radius = m_search_radius_color_gradient;
        p.scales[0].max_nn = 0;
        p.lambda = m_color_icp_lambda;
        p.update_map = GCA3D_UPDATE_EULER_ZYX;
        p.rot_eps = (double)m_translations_thres_square;
        p.trans_eps = (double)m_translations_thres_square;
        p.compensated = 1;
        p.use_graph = 0;
        p.keep_target_normals = 1;
        gca3d_icp_result r;
        const int st = gca3d_color_icp(detail::ctx(), m_source_pc->handle(), m_target_pc->handle(), &p, nullptr, &r);
        if (st != GCA3D_OK)
        {
            detail::warn("gca: color_icp failed", detail::ctx());
            m_transformation_matrix.set_identity();
            return false;
        }
        for (int k = 0; k < 16; ++k)
            m_transformation_matrix.m[k] = (float)r.T[k];
        m_RMSE = (float)r.rmse_ref;
        m_source_pc->transform(m_transformation_matrix);
        m_color_icp_done = true;
        return true;
    }

    // color_icp.cu:90-137: per source point |r_g| + |r_c| against its nearest target
    // point within the correspondence distance, and their mean
    std::pair<device_vector<float>, float> get_abs_residual()
    {
        if (!m_source_pc || !m_target_pc || !m_target_pc->has_normals())
        {
            detail::warn("gca: get_abs_residual needs a source and a target with normals", nullptr);
            return std::make_pair(device_vector<float>(), 0.0f);
        }
        gca3d_context *c = detail::ctx();
        if (!m_color_gradient_done)
        {
            if (!detail::ok(gca3d_color_gradient(c, m_target_pc->handle(), m_search_radius_color_gradient),
                            "gca: color gradient"))
                return std::make_pair(device_vector<float>(), 0.0f);
            m_color_gradient_done = true;
        }
        const size_t n = m_source_pc->points_number();
        auto nn = point_cloud::nn_search(*m_source_pc, *m_target_pc, m_max_corr_dist);
        device_vector<float> res(n);
        if (!n || !detail::ok(gca3d_abs_residual(c, m_source_pc->handle(), m_target_pc->handle(), nn.data(),
                                                 m_color_icp_lambda, res.data()),
                              "gca: abs residual"))
            return std::make_pair(device_vector<float>(), 0.0f);
        const auto h = res.download();
        float s = 0.0f;
        for (float v : h)
            s += v;
        return std::make_pair(std::move(res), s / (float)n);
    }
    std::pair<std::vector<float>, float> get_abs_residual_host()
    {
        auto d = get_abs_residual();
        return std::make_pair(d.first.download(), d.second);
    }

    const mat4x4 &get_final_transformation_matrix() const { return m_transformation_matrix; }
    float get_RSME() const { return m_RMSE; }
    std::shared_ptr<const point_cloud> get_transformed_source_point_cloud() const { return m_source_pc; }

private:
    void reset()
    {
        m_color_icp_done = false;
        m_color_gradient_done = false;
        m_transformation_matrix.set_identity();
        m_RMSE = 0.0f;
    }

    static constexpr float m_color_icp_lambda = 0.968f;
    static constexpr float m_translations_thres_square = 0.000001f;
    size_t m_max_iter;
    float m_max_corr_dist;
    float m_search_radius_color_gradient;
    bool m_color_icp_done = false;
    bool m_color_gradient_done = false;
    std::shared_ptr<point_cloud> m_source_pc;
    std::shared_ptr<const point_cloud> m_target_pc;
    mat4x4 m_transformation_matrix;
    float m_RMSE = 0.0f;
};
} // namespace gca
