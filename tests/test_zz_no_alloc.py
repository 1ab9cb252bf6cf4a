"""The allocation-free Gauss-Newton entry point against the regular one.

gca3d_build_gauss_newton_static serves callers that cannot allocate device memory
while they run; it keeps its scratch in a fixed array inside the library.  Here it is
called twice in a row through the C ABI on the same inputs (the second call runs on
the scratch the first one left behind) and each result must match
gca3d_build_gauss_newton within the tolerance the other system tests use (1e-5
relative).  This file sorts last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


@pytest.fixture(scope="module")
def N():
    from cuda_3d_gb300 import build, native

    build.build()
    return native


@pytest.fixture(scope="module")
def ctx(N):
    return N.Context(0)


def _static_call(ctx, src_views, n_src, tgt_views, nn_ptr, lam, out):
    return ctx.L.gca3d_build_gauss_newton_static(ctx.stream, src_views[0], n_src, tgt_views[0], tgt_views[2],
                                                 tgt_views[3], nn_ptr, lam, out["jtj"].ptr, out["jtr"].ptr,
                                                 out["r2"].ptr)


def test_static_entry_point_matches_regular_twice(ctx, N, golden):
    tgt = ctx.cloud_from(golden.patch_xyz, golden.patch_rgb)
    tgt.set_normals(golden["normals"])
    tgt.set_gradients(golden["grad"])
    src = ctx.cloud_from(golden["gn_src_xyz"], golden.gn_src_rgb)
    nn = golden["gn_nn"]
    nn_buf = ctx.alloc(4 * len(nn))
    nn_buf.write(nn)

    jtj, jtr, r2 = np.zeros(36), np.zeros(6), C.c_double()
    ctx.check(ctx.L.gca3d_build_gauss_newton(ctx.h, src.h, tgt.h, nn_buf.ptr, 0.968, jtj.ctypes.data,
                                             jtr.ctypes.data, C.byref(r2)))

    out = {"jtj": ctx.alloc(36 * 8), "jtr": ctx.alloc(6 * 8), "r2": ctx.alloc(8)}
    sv, tv = src.device_views(), tgt.device_views()
    for _ in range(2):
        assert _static_call(ctx, sv, len(nn), tv, nn_buf.ptr, 0.968, out) == N.OK
        ctx.sync()
        got_jtj = out["jtj"].read(np.float64, 36)
        got_jtr = out["jtr"].read(np.float64, 6)
        got_r2 = out["r2"].read(np.float64, 1)[0]
        assert np.abs(got_jtj - jtj).max() <= REL_TOL * np.abs(jtj).max()
        assert np.abs(got_jtr - jtr).max() <= REL_TOL * np.abs(jtr).max()
        assert abs(got_r2 - r2.value) <= REL_TOL * abs(r2.value)
        np.testing.assert_array_equal(got_jtj.reshape(6, 6), got_jtj.reshape(6, 6).T)


def test_static_entry_point_rejects_oversize_and_bad_arguments(ctx, N, golden):
    tgt = ctx.cloud_from(golden.patch_xyz, golden.patch_rgb)
    tgt.set_normals(golden["normals"])
    tgt.set_gradients(golden["grad"])
    tv = tgt.device_views()
    out = {"jtj": ctx.alloc(36 * 8), "jtr": ctx.alloc(6 * 8), "r2": ctx.alloc(8)}
    nn_buf = ctx.alloc(16)
    # sizes beyond the fixed scratch are refused before anything is launched
    assert _static_call(ctx, tv, 8_388_609, tv, nn_buf.ptr, 0.968, out) == N.ERR_CAPACITY
    assert _static_call(ctx, tv, 16, tv, nn_buf.ptr, 1.5, out) == N.ERR_INVALID_VALUE
    assert _static_call(ctx, tv, -1, tv, nn_buf.ptr, 0.968, out) == N.ERR_INVALID_VALUE
