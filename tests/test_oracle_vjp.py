"""The oracle's adjoint of K unrolled colored-ICP Gauss-Newton steps, checked on the
CPU against central finite differences of its own FP64 forward function.

The function is L(xi0, X, C) = <G, T_K> + g * E_K with the correspondences of every
evaluation frozen (they are piecewise constant in the inputs, so the frozen
function is the smooth one the adjoint differentiates).  Steps: h = 1e-4 on the
pose, 1e-5 m on points, 1e-4 on colours.  This pins the adjoint derivation that the
GPU kernels implement; the GPU is compared against this oracle and against the same
finite differences in test_gpu_vjp.py."""
import numpy as np
import pytest

import oracle as O
from cuda_3d_gb300 import synth

# central differences of an FP64 function with these steps are accurate to about
# 1e-6 relative here (truncation); the tolerance leaves a margin of 10
FD_RTOL = 1e-5
MAX_CORR = 0.05
RADIUS = 0.08


@pytest.fixture(scope="module")
def pair():
    O.set_threads(8)
    pr = synth.room_pair(3, n_points=12000, rot_deg=2.0, trans=0.02)
    sx = pr.src_xyz.astype(np.float32).astype(np.float64)
    sc = pr.src_rgb.astype(np.float32).astype(np.float64)
    tx, tc = pr.tgt_xyz.astype(np.float32), pr.tgt_rgb.astype(np.float32)
    tn = O.normals_f64(tx, RADIUS)
    tg = O.gradient_f64(tx, tc, tn, RADIUS)
    return sx, sc, tx, tc, tn, tg


def _check(g, fd, scale):
    assert abs(g - fd) <= FD_RTOL * max(abs(fd), 1e-3 * scale), (g, fd)


@pytest.mark.parametrize("K", [1, 2, 5])
@pytest.mark.parametrize("umap", [O.UPDATE_SE3_EXP, O.UPDATE_EULER_ZYX])
def test_oracle_adjoint_matches_finite_differences(pair, K, umap):
    sx, sc, tx, tc, tn, tg = pair
    rng = np.random.default_rng(10 * K + umap)
    xi0 = rng.normal(size=6) * 0.01
    T, E, corr = O.icp_unrolled_f64(sx, sc, tx, tc, tn, tg, xi0, K=K, max_corr=MAX_CORR, update_map=umap)
    assert (corr >= 0).mean() > 0.25  # the views overlap by about 60 %
    G = rng.normal(size=(4, 4))
    G[3] = 0.0
    gE = 0.3

    def L(xi, X, Cc):
        T, E, _ = O.icp_unrolled_f64(X, Cc, tx, tc, tn, tg, xi, K=K, max_corr=MAX_CORR, update_map=umap, corr=corr)
        return (G * T).sum() + gE * E

    dxi, dX, dC, st = O.icp_unrolled_vjp_f64(sx, sc, tx, tc, tn, tg, xi0, corr, G, gE, K=K, max_corr=MAX_CORR,
                                             update_map=umap)
    assert st == 0
    # the pose: at K = 5 Gauss-Newton has converged quadratically and T_K no longer
    # depends on xi0 (both sides are ~0: the absolute floor covers it)
    for m in range(6):
        e = np.zeros(6)
        e[m] = 1e-4
        fd = (L(xi0 + e, sx, sc) - L(xi0 - e, sx, sc)) / 2e-4
        if K >= 5:
            assert abs(dxi[m] - fd) <= 1e-9
        else:
            assert abs(dxi[m] - fd) <= 1e-3 * abs(fd) + 1e-9, (m, dxi[m], fd)
    # points and colours of matched source points
    matched = np.flatnonzero((corr >= 0).all(axis=0))
    for i in rng.choice(matched, 6, replace=False):
        a = int(rng.integers(3))
        for X, g, h, which in ((sx, dX, 1e-5, "xyz"), (sc, dC, 1e-4, "rgb")):
            Xp, Xm = X.copy(), X.copy()
            Xp[i, a] += h
            Xm[i, a] -= h
            if which == "xyz":
                fd = (L(xi0, Xp, sc) - L(xi0, Xm, sc)) / (2 * h)
            else:
                fd = (L(xi0, sx, Xp) - L(xi0, sx, Xm)) / (2 * h)
            _check(g[i, a], fd, np.abs(g).max())


@pytest.mark.parametrize("umap", [O.UPDATE_SE3_EXP, O.UPDATE_EULER_ZYX])
@pytest.mark.parametrize("mag", [1e-5, 3e-3, 0.3, 2.0])
def test_pose_jacobian_matches_finite_differences(umap, mag):
    """dU/dx of both pose maps, on both sides of the series switch (theta = 1e-2)"""
    rng = np.random.default_rng(int(mag * 1e5) + umap)
    x = rng.normal(size=6)
    x[:3] *= mag / np.linalg.norm(x[:3])
    J = O.pose_jacobian(x, umap)
    h = 1e-6
    for m in range(6):
        e = np.zeros(6)
        e[m] = h
        fd = (O.pose_from_x(x + e, umap) - O.pose_from_x(x - e, umap))[:3] / (2 * h)
        np.testing.assert_allclose(J[m], fd, rtol=0, atol=2e-8)


def test_frozen_correspondences_reproduce_the_search(pair):
    """the frozen evaluation with the correspondences a search produced gives the
    same result as the search itself"""
    sx, sc, tx, tc, tn, tg = pair
    xi0 = np.array([0.01, -0.02, 0.005, 0.01, 0.0, -0.01])
    T1, E1, corr = O.icp_unrolled_f64(sx, sc, tx, tc, tn, tg, xi0, K=3)
    T2, E2, _ = O.icp_unrolled_f64(sx, sc, tx, tc, tn, tg, xi0, K=3, corr=corr)
    np.testing.assert_array_equal(T1, T2)
    assert E1 == E2
