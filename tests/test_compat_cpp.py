"""The C++ compatibility layer (include/gca_compat: gca::point_cloud, gca::color_icp
and friends with the reference's signatures) through a program that follows the
reference app's registration flow (tests/cpp/compat_app.cpp).

CPU: the program compiles with plain g++ against the headers and links libgca3d.so.
GPU: it runs, and every number it prints is replayed through the C ABI with the
same steps and compared bit for bit (pose, RMSE, point counts, correspondences,
transformed points)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
REC = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("r", "u1"), ("g", "u1"), ("b", "u1"), ("pad", "u1")])


def build_app(out_dir):
    from cuda_3d_gb300 import build

    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = os.path.join(out_dir, "compat_app")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT}/include",
           f"-I{ROOT}/include/gca_compat", f"-I{CUDA}/include", os.path.join(ROOT, "tests", "cpp", "compat_app.cpp"),
           f"-L{libdir}", "-lgca3d", f"-Wl,-rpath,{libdir}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_compat_app_compiles(tmp_path):
    exe = build_app(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_compat_app_matches_c_abi(tmp_path):
    from cuda_3d_gb300 import native as N
    from cuda_3d_gb300 import synth

    exe = build_app(str(tmp_path))
    pr = synth.room_pair(seed=8, n_points=60_000, rot_deg=5.0, trans=0.05)
    clouds = []
    for xyz, rgb in ((pr.src_xyz, pr.src_rgb), (pr.tgt_xyz, pr.tgt_rgb)):
        rec = np.zeros(len(xyz), REC)
        rec["x"], rec["y"], rec["z"] = np.asarray(xyz, np.float32).T
        c8 = np.clip(np.round(np.asarray(rgb) * 255), 0, 255).astype(np.uint8)
        rec["r"], rec["g"], rec["b"] = c8.T
        clouds.append((rec, np.ascontiguousarray(np.stack([rec["x"], rec["y"], rec["z"]], 1)),
                       (c8.astype(np.float32) * (np.float32(1.0) / np.float32(255.0))).astype(np.float32)))
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        f.write(np.array([len(clouds[0][0]), len(clouds[1][0])], np.int64).tobytes())
        f.write(clouds[0][0].tobytes())
        f.write(clouds[1][0].tobytes())
    run = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True)
    assert run.returncode == 0, run.stdout + run.stderr
    raw = outp.read_bytes()
    T = np.frombuffer(raw, np.float32, 16, 0).reshape(4, 4)
    rmse = np.frombuffer(raw, np.float32, 1, 64)[0]
    n_src_ds, n_tgt_ds = np.frombuffer(raw, np.int64, 2, 68)
    abs_mean = np.frombuffer(raw, np.float32, 1, 84)[0]
    n_ror, n_sel = np.frombuffer(raw, np.int64, 2, 88)
    nn = np.frombuffer(raw, np.int32, n_src_ds, 104)
    src_t = np.frombuffer(raw, np.float32, 3 * len(clouds[0][0]), 104 + 4 * n_src_ds).reshape(-1, 3)

    # the same steps through the C ABI
    import ctypes as C

    ctx = N.Context(0)
    src = ctx.cloud_from(clouds[0][1], clouds[0][2])
    tgt = ctx.cloud_from(clouds[1][1], clouds[1][2])
    sds, tds = ctx.cloud(len(clouds[0][1])), ctx.cloud(len(clouds[1][1]))
    ctx.check(ctx.L.gca3d_voxel_downsample(ctx.h, src.h, 0.02, sds.h))
    ctx.check(ctx.L.gca3d_voxel_downsample(ctx.h, tgt.h, 0.02, tds.h))
    assert (len(sds), len(tds)) == (n_src_ds, n_tgt_ds)
    ctx.check(ctx.L.gca3d_estimate_normals(ctx.h, tds.h, 0.05, 0))
    eps = float(np.float32(1e-6))
    prm = N.icp_params([N.scale(0.0, 100, 0.05, 0.0, 0.04, 0)], update_map=N.UPDATE_EULER_ZYX, rot_eps=eps,
                       trans_eps=eps, compensated=True, keep_target_normals=True)
    r = N.color_icp(ctx, sds, tds, prm)
    np.testing.assert_array_equal(T, r["T"].astype(np.float32))
    assert rmse == np.float32(r["rmse_ref"])
    ctx.check(ctx.L.gca3d_transform(ctx.h, src.h, T.astype(np.float64).ctypes.data))
    np.testing.assert_array_equal(src_t, src.download()["xyz"])
    out = ctx.cloud(len(clouds[0][1]))  # capacity of the input cloud
    ctx.check(ctx.L.gca3d_radius_outlier_removal(ctx.h, sds.h, 0.05, 4, out.h))
    assert len(out) == n_ror
    assert n_sel == (n_src_ds + 2) // 3
    buf = ctx.alloc(4 * n_src_ds)
    ctx.check(ctx.L.gca3d_nn_search(ctx.h, sds.h, tds.h, 0.05, buf.ptr))
    np.testing.assert_array_equal(nn, buf.read(np.int32, n_src_ds))
    assert np.isfinite(abs_mean) and abs_mean > 0
    del C
