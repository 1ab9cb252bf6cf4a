"""Failure detection on the GPU, without a GPU fault.

* A cross-block wait whose answer never comes: the scan's look-back waits on a tile
  that is never run; after the context's wait limit it gives up, the call reports
  GCA3D_ERR_TIMEOUT in bounded time, and the context stays usable.
* Correspondence indices from the caller that lie beyond the target are reported as
  GCA3D_ERR_INVALID_VALUE; nothing is read out of bounds.
* The checked build (device-side index checks compiled in, each failure an error bit
  of the context) runs the registration path without a failed check and gives the
  regular build's results bit for bit."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEFAULT_WAIT_LIMIT = 1 << 22


@pytest.fixture(scope="module")
def N():
    from cuda_3d_gb300 import build, native

    build.build()
    return native


@pytest.fixture(scope="module")
def ctx(N):
    return N.Context(0)


def test_wait_limit_is_a_runtime_setting(ctx, N):
    assert N.wait_limit(ctx) == DEFAULT_WAIT_LIMIT
    assert N.wait_limit(ctx, 1000) == 1000
    assert ctx.L.gca3d_set_wait_limit(ctx.h, 0) == N.ERR_INVALID_VALUE
    assert N.wait_limit(ctx, DEFAULT_WAIT_LIMIT) == DEFAULT_WAIT_LIMIT


@pytest.mark.parametrize("tiles,polls", [(2, 1000), (8, 1000), (64, 20000)])
def test_look_back_wait_gives_up(ctx, N, orc, golden, tiles, polls):
    status, ms = N.selfcheck_wait(ctx, tiles=tiles, polls=polls)
    assert status == N.ERR_TIMEOUT
    # every wait ends after `polls` polls of at most a few hundred ns each
    assert ms < 200.0, ms
    # the limit of the context is back, and the context still works
    assert N.wait_limit(ctx) == DEFAULT_WAIT_LIMIT
    xyz, rgb = golden["cloud_xyz"], golden["cloud_rgb"]
    src = ctx.cloud_from(xyz, rgb)
    out = ctx.cloud(src.capacity)
    ctx.check(ctx.L.gca3d_voxel_downsample(ctx.h, src.h, 0.05, out.h))
    got = out.download()
    np.testing.assert_array_equal(got["xyz"], golden["voxel_v05_xyz"])
    np.testing.assert_array_equal(got["rgb"], golden["voxel_v05_rgb"])


def test_selfcheck_wait_rejects_bad_arguments(ctx, N):
    st, ms = C.c_int(), C.c_double()
    for tiles, polls in ((1, 10), (65, 10), (4, 0)):
        assert ctx.L.gca3d_selfcheck_wait(ctx.h, tiles, polls, C.byref(st), C.byref(ms)) == N.ERR_INVALID_VALUE


def gn_inputs(ctx, golden):
    tgt = ctx.cloud_from(golden.patch_xyz, golden.patch_rgb)
    ctx.check(ctx.L.gca3d_estimate_normals(ctx.h, tgt.h, 0.09, 0))
    ctx.check(ctx.L.gca3d_color_gradient(ctx.h, tgt.h, 0.09))
    src = ctx.cloud_from(golden["gn_src_xyz"], golden.gn_src_rgb)
    return src, tgt


def build_gn(ctx, src, tgt, nn):
    buf = ctx.alloc(4 * len(nn))
    buf.write(np.ascontiguousarray(nn, np.int32))
    jtj, jtr, r2 = np.zeros(36), np.zeros(6), C.c_double()
    st = ctx.L.gca3d_build_gauss_newton(ctx.h, src.h, tgt.h, buf.ptr, 0.968, jtj.ctypes.data, jtr.ctypes.data,
                                        C.byref(r2))
    res = ctx.alloc(4 * len(nn))
    st2 = ctx.L.gca3d_abs_residual(ctx.h, src.h, tgt.h, buf.ptr, 0.968, res.ptr)
    return st, st2, jtj, res.read(np.float32, len(nn))


def check_bad_index(ctx, N, golden):
    src, tgt = gn_inputs(ctx, golden)
    nn = golden["gn_nn"].copy()
    st, st2, jtj_ok, res_ok = build_gn(ctx, src, tgt, nn)
    assert st == N.OK and st2 == N.OK
    for bad in (len(golden.patch_xyz), 1 << 30):
        nb = nn.copy()
        nb[17] = bad
        st, st2, _, _ = build_gn(ctx, src, tgt, nb)
        assert st == N.ERR_INVALID_VALUE and st2 == N.ERR_INVALID_VALUE
    # the context still works and the valid call is unchanged
    st, st2, jtj, res = build_gn(ctx, src, tgt, nn)
    assert st == N.OK and st2 == N.OK
    np.testing.assert_array_equal(jtj, jtj_ok)
    np.testing.assert_array_equal(res, res_ok)


def test_correspondence_index_beyond_target_is_reported(ctx, N, golden):
    check_bad_index(ctx, N, golden)


def registration_path(ctx, N, golden, synth):
    """voxels, normals, gradients, NN, radius lists, outlier removal, the frame stage
    and a batched coarse-to-fine ICP; every call must succeed"""
    out = {}
    xyz, rgb = golden["cloud_xyz"], golden["cloud_rgb"]
    c = ctx.cloud_from(xyz, rgb)
    v = ctx.cloud(c.capacity)
    ctx.check(ctx.L.gca3d_voxel_downsample(ctx.h, c.h, 0.02, v.h))
    ctx.check(ctx.L.gca3d_estimate_normals(ctx.h, v.h, 0.05, 30))
    ctx.check(ctx.L.gca3d_color_gradient(ctx.h, v.h, 0.05))
    out["voxel"] = v.download(normals=True, grad=True)
    q = ctx.cloud_from(golden["nn_q"])
    r = ctx.cloud_from(golden.nn_r)
    idx = ctx.alloc(4 * len(golden["nn_q"]))
    ctx.check(ctx.L.gca3d_nn_search(ctx.h, q.h, r.h, 0.05, idx.ptr))
    out["nn"] = idx.read(np.int32, len(golden["nn_q"]))
    ror = ctx.cloud(c.capacity)
    ctx.check(ctx.L.gca3d_radius_outlier_removal(ctx.h, c.h, 0.05, 4, ror.h))
    out["ror"] = ror.download()
    depth, bgr = golden["frame_depth"], golden["frame_bgr"]
    d, b = ctx.alloc(depth.nbytes), ctx.alloc(bgr.nbytes)
    d.write(depth)
    b.write(bgr)
    fc = ctx.cloud(depth.size)
    di = N.Intrinsics(*golden.frame_case("adaptive")[0])
    f = N.Filter(N.FILTER_ADAPTIVE, 2, 3.0, 30.0)
    ctx.check(ctx.L.gca3d_frame_to_cloud(ctx.h, d.ptr, b.ptr, depth.shape[1], depth.shape[0], C.byref(di), None, None,
                                         0.001, 0.2, 10.0, C.byref(f), fc.h))
    out["frame"] = fc.download()
    pairs = synth.batch_pairs(4, seed=7, n_min=20_000, n_max=60_000)
    srcs = [ctx.cloud_from(p.src_xyz, p.src_rgb) for p in pairs]
    tgts = [ctx.cloud_from(p.tgt_xyz, p.tgt_rgb) for p in pairs]
    scales = [N.scale(0.04, 30, 0.06, 0.08, 0.08), N.scale(0.02, 20, 0.03, 0.04, 0.04)]
    res = N.IcpPlan(ctx, srcs, tgts, N.icp_params(scales, update_map=N.UPDATE_SE3_EXP, use_graph=True)).execute()
    out["icp"] = [(r["T"], r["iterations"], r["status"]) for r in res]
    ctx.sync()
    return out


def test_checked_build_runs_clean_and_matches(ctx, N, golden):
    from cuda_3d_gb300 import build, synth

    lib = build.build(checked=True)
    cctx = N.Context(0, lib_path=lib)
    a = registration_path(ctx, N, golden, synth)
    b = registration_path(cctx, N, golden, synth)
    for k in ("voxel", "ror", "frame"):
        for f in a[k]:
            np.testing.assert_array_equal(a[k][f], b[k][f])
    np.testing.assert_array_equal(a["nn"], b["nn"])
    for (Ta, ia, sa), (Tb, ib, sb) in zip(a["icp"], b["icp"]):
        np.testing.assert_array_equal(Ta, Tb)
        assert ia == ib and sa == sb == N.OK
    # a caller's bad index is reported by the checked build as by the regular one
    check_bad_index(cctx, N, golden)
    cctx.close()
