"""The oracle's FP32 flavour against the reference's own code (golden fixtures
generated by tests/golden/make_golden.py from the reference built as host C++).
Bit-exact for keys, indices, neighbour lists and the voxel set; the FP32 normal,
gradient and Gauss-Newton steps follow the reference's operation order and are
bit-exact too on the machine that made the fixtures (x86-64 glibc)."""
import platform

import numpy as np
import pytest

X86 = platform.machine() in ("x86_64", "AMD64")


def test_aabb_including_flt_min_bug(golden, orc):
    for name, pts in (("cloud", golden["cloud_xyz"]),
                      ("neg", golden.voxel_input("neg05")[0])):
        mn, mx = orc.aabb(pts, flt_min_bug=True)
        np.testing.assert_array_equal(mn, golden[f"aabb_{name}_min"])
        np.testing.assert_array_equal(mx, golden[f"aabb_{name}_max"])
    # the reference's max starts at FLT_MIN: an all-negative axis reports ~0
    assert golden["aabb_neg_max"][0] == np.finfo(np.float32).tiny


@pytest.mark.parametrize("tag", ["v05", "v02", "neg05", "dup", "one"])
def test_voxel_downsample_bit_exact(golden, orc, tag):
    xyz, rgb = golden.voxel_input(tag)
    ox, oc, cnt, key = orc.voxel_downsample(xyz, rgb, float(golden[f"voxel_{tag}_size"]))
    np.testing.assert_array_equal(ox, golden[f"voxel_{tag}_xyz"])
    np.testing.assert_array_equal(oc, golden[f"voxel_{tag}_rgb"])
    assert cnt.sum() == len(xyz)
    # output in ascending lexicographic key order
    k = key.astype(np.int64)
    lin = (k[:, 0] << 42) | (k[:, 1] << 21) | k[:, 2]
    assert np.all(np.diff(lin) > 0)


def test_voxel_empty(orc):
    ox, oc, cnt, key = orc.voxel_downsample(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), 0.05)
    assert len(ox) == 0


def test_nn_scan_order_bit_exact(golden, orc):
    idx = orc.nn_search(golden["nn_q"], golden.nn_r, float(golden["nn_radius"]), golden["nn_grid_min"],
                        tie=orc.TIE_SCAN_ORDER)
    np.testing.assert_array_equal(idx, golden["nn_idx"])
    # the (distance, index) tie-break agrees except on exact cross-cell ties
    idx2 = orc.nn_search(golden["nn_q"], golden.nn_r, float(golden["nn_radius"]), tie=orc.TIE_MIN_INDEX)
    np.testing.assert_array_equal(idx2, golden["nn_idx"])


def test_nn_exact_ties(golden, orc):
    q, r, rad = golden["nntie_q"], golden["nntie_r"], float(golden["nntie_radius"])
    scan = orc.nn_search(q, r, rad, golden["nntie_grid_min"], tie=orc.TIE_SCAN_ORDER)
    np.testing.assert_array_equal(scan, golden["nntie_idx"])
    mi = orc.nn_search(q, r, rad, tie=orc.TIE_MIN_INDEX)
    # both choose a point at the minimum distance
    d_scan = np.where(scan >= 0, ((r[np.maximum(scan, 0)] - q) ** 2).sum(1), np.inf)
    d_mi = np.where(mi >= 0, ((r[np.maximum(mi, 0)] - q) ** 2).sum(1), np.inf)
    np.testing.assert_array_equal(d_scan, d_mi)
    # ... and the (distance, index) rule picks the smallest index among them
    for i in np.nonzero(mi >= 0)[0]:
        d = ((r - q[i]) ** 2).sum(1)
        cands = np.nonzero(d == d_mi[i])[0]
        assert mi[i] == cands.min()


def test_radius_lists_bit_exact(golden, orc):
    pts = golden.patch_xyz
    c, s, lst = orc.radius_search(pts, pts, float(golden["radius_r"]), golden["radius_grid_min"])
    np.testing.assert_array_equal(c, golden["radius_counts"])
    np.testing.assert_array_equal(s, golden["radius_starts"])
    np.testing.assert_array_equal(lst, golden["radius_list"])
    np.testing.assert_array_equal(orc.normals_grid_min(pts, golden["radius_r"]), golden["radius_grid_min"])


@pytest.mark.skipif(not X86, reason="bit-exact FP32 transcendental parity holds on the fixture machine")
def test_normals_ref32_bit_exact(golden, orc):
    n = orc.normals_ref32(golden.patch_xyz, float(golden["radius_r"]))
    np.testing.assert_array_equal(n, golden["normals"])


def test_normals_ref32_close(golden, orc):
    n = orc.normals_ref32(golden.patch_xyz, float(golden["radius_r"]))
    np.testing.assert_allclose(n, golden["normals"], atol=1e-5)


def test_gradient_ref32(golden, orc):
    g = orc.gradient_ref32(golden.patch_xyz, golden.patch_rgb, golden["normals"], float(golden["radius_r"]))
    np.testing.assert_array_equal(orc.gradient_grid_min(golden.patch_xyz, golden["radius_r"]),
                                  golden["grad_grid_min"])
    np.testing.assert_array_equal(g, golden["grad"])


def test_build_gn_ref32(golden, orc):
    jtj, jtr, r2 = orc.build_gn_ref32(golden["gn_src_xyz"], golden.gn_src_rgb, golden.patch_xyz,
                                      golden.patch_rgb, golden["normals"], golden["grad"], golden["gn_nn"])
    np.testing.assert_array_equal(jtj, golden["gn_jtj"])
    np.testing.assert_array_equal(jtr, golden["gn_jtr"])
    assert np.float32(r2) == golden["gn_r2"]
    ar = orc.abs_residual_ref32(golden["gn_src_xyz"], golden.gn_src_rgb, golden.patch_xyz, golden.patch_rgb,
                                golden["normals"], golden["grad"], golden["gn_nn"])
    np.testing.assert_array_equal(ar, golden["gn_abs_residual"])


def test_nn_of_gn_case(golden, orc):
    idx = orc.nn_search(golden["gn_src_xyz"], golden.patch_xyz, 0.06, tie=orc.TIE_SCAN_ORDER)
    np.testing.assert_array_equal(idx, golden["gn_nn"])


def test_normals_f64_vs_reference(golden, orc):
    """FP64 normals agree in direction with the reference's FP32 normals (the
    reference's raw-moment covariance loses digits; the bound is loose)"""
    n64 = orc.normals_f64(golden.patch_xyz, float(golden["radius_r"]))
    ref = golden["normals"].astype(np.float64)
    ok = (np.linalg.norm(ref, axis=1) > 0) & (np.linalg.norm(n64, axis=1) > 0)
    assert ok.mean() > 0.3
    dots = np.abs((n64[ok] * ref[ok]).sum(1))
    assert np.median(dots) > np.cos(np.radians(0.5))
    # zero normals exactly where fewer than 3 neighbours
    zero64 = np.linalg.norm(n64, axis=1) == 0
    np.testing.assert_array_equal(zero64, golden["radius_counts"] < 3)


def test_filter_exp_error_bound(orc):
    """the depth filter's exp (shared operation sequence with the CUDA kernel) is
    within 2 ulp of exp(x) over the filter's argument range, subnormals included"""
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-110, 90, 20000), rng.uniform(-3, 0.5, 20000)]).astype(np.float32)
    y = orc.exp32(x).astype(np.float64)
    t = np.exp(x.astype(np.float64))
    normal = (t > np.finfo(np.float32).tiny) & (t < np.finfo(np.float32).max)
    ulp = np.abs(y[normal] - t[normal]) / np.spacing(t[normal].astype(np.float32)).astype(np.float64)
    assert ulp.max() <= 2.0
    sub = t <= np.finfo(np.float32).tiny
    assert np.all(np.abs(y[sub] - t[sub]) <= np.finfo(np.float32).smallest_subnormal)
    assert orc.exp32([np.float32(100.0)])[0] == np.inf and orc.exp32([np.float32(-200.0)])[0] == 0.0


def test_radius_outlier_removal(golden, orc):
    """survivors and their order, bit for bit (reference: cuda_nn_search.cu:416-542,725-800)"""
    xyz, rgb = golden["cloud_xyz"][:8000], golden["cloud_rgb"][:8000]
    ox, oc = orc.radius_outlier_removal(xyz, rgb, golden["ror_radius"], int(golden["ror_min_nn"]))
    assert 0 < len(ox) < len(xyz)
    np.testing.assert_array_equal(ox, golden["ror_xyz"])
    np.testing.assert_array_equal(oc, golden["ror_rgb"])


@pytest.mark.parametrize("case", ["raw", "adaptive", "fixed", "adaptive_extrinsic", "adaptive_tmin0"])
def test_frame_stage_vs_reference(orc, golden, case):
    """bilateral filter (adaptive, fixed, none), back-projection with the half-pixel
    shift, depth-to-colour extrinsic, colour lookup and raster-order compaction
    against the reference's own frame helpers (cuda_point_cloud_factory.cu:19-187
    built as host C++, the kernel body :210-266 restated around them)"""
    di, ci, rot, tr, mode, tmin = golden.frame_case(case)
    r, ss, sd = golden.FRAME_FIXED
    xyz, rgb, fd = orc.make_point_cloud(golden["frame_depth"], golden["frame_bgr"], di, ci, (rot, tr), 0.001, tmin,
                                        10.0, mode, r, ss, sd, return_depth=True)
    golden.check_frame(case, xyz, rgb, fd)
