"""Generate the golden fixtures from the reference's own code.

Builds the reference's Thrust sources (XssZuiNB/CUDA_3D) as host C++ on the
serial Thrust backend (``make -C oracle ref``, outputs only in oracle/_ref/), runs
them on small seeded synthetic inputs and stores inputs and outputs in
``tests/golden/golden.npz``.  The fixtures pin the oracle; the GPU tests also
compare against them directly.  Needs the reference sources, so it runs only where
they are mounted:

    python tests/golden/make_golden.py [REF_SRC]
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cuda_3d_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "golden.npz")


REF_SRC = os.environ.get("GCA_REF_SRC", "/root/reference/src")

# the frame fixture: a small RGB-D frame of the frame scene, and the cases run through
# the reference's frame helpers (oracle/ref_frame.inc): (name, filter mode, tmin,
# depth-to-colour rotation (column-major, as gca::extrinsics stores it), translation,
# colour intrinsics or None for the depth intrinsics)
FRAME_CAM = synth.Camera(96, 72, 78.75, 78.75, 47.5, 35.5)
FRAME_CASES = [
    ("raw", 0, 0.2, None, None, None),
    ("adaptive", 1, 0.2, None, None, None),
    ("fixed", 2, 0.2, None, None, None),
    ("adaptive_extrinsic", 1, 0.2, "rot", (0.025, -0.01, 0.004), (78.0, 80.5, 48.1, 34.8)),
    ("adaptive_tmin0", 1, 0.0, None, None, None),
]
FRAME_FIXED = (2, 3.0, 30.0)  # radius, sigma_space (px), sigma_depth (depth units)
# frame_<case>_args: depth intrinsics (4), colour intrinsics (4), rotation (9), translation (3), mode, tmin


def frame_case_args(case):
    name, mode, tmin, rot, tr, ci = case
    di = np.array([FRAME_CAM.fx, FRAME_CAM.fy, FRAME_CAM.cx, FRAME_CAM.cy], np.float32)
    R = np.eye(3, dtype=np.float32)
    if rot == "rot":
        R = f32(synth.axis_angle([0.2, 1.0, -0.3], np.radians(1.0)))
    return (di, np.array(ci, np.float32) if ci else di, f32(R.T.reshape(-1)), f32(tr or (0.0, 0.0, 0.0)), mode,
            np.float32(tmin))


def load_ref(ref_src):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_SRC={ref_src}"], check=True)
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libgca_ref.so"))
    for f in ("ref_voxel_downsample", "ref_radius_search", "ref_radius_outlier_removal", "ref_make_point_cloud",
              "ref_make_point_cloud_detexp"):
        getattr(L, f).restype = C.c_int64
    return L


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def main(ref_src=REF_SRC):
    L = load_ref(ref_src)
    g = {}
    rng = np.random.default_rng(20240601)
    scene = synth.room_scene(1234)

    # --- clouds -----------------------------------------------------------
    xyz, rgb = synth.sample_room(scene, 16000, rng)
    g["cloud_xyz"], g["cloud_rgb"] = xyz, rgb
    # a displaced copy with all-negative coordinates on x (exercises the FLT_MIN max)
    neg = f32(xyz - np.array([10.0, 0.0, 0.0], np.float32))

    # --- aabb -------------------------------------------------------------
    for name, pts in (("cloud", xyz), ("neg", neg)):
        mn, mx = np.zeros(3, np.float32), np.zeros(3, np.float32)
        L.ref_aabb(P(pts), C.c_int64(len(pts)), P(mn), P(mx))
        g[f"aabb_{name}_min"], g[f"aabb_{name}_max"] = mn, mx

    # --- voxel downsample ---------------------------------------------------
    # inputs are rebuilt by the tests from cloud_xyz/cloud_rgb (voxel_inputs in test_oracle_golden.py)
    for tag, v, pts in (("v05", 0.05, xyz), ("v02", 0.02, xyz), ("neg05", 0.05, neg),
                        ("dup", 0.05, f32(np.repeat(xyz[:500], 3, 0))), ("one", 0.05, xyz[:1])):
        col = rgb[: len(pts)] if tag != "dup" else f32(np.repeat(rgb[:500], 3, 0))
        ox, oc = np.zeros((len(pts), 3), np.float32), np.zeros((len(pts), 3), np.float32)
        m = L.ref_voxel_downsample(P(f32(pts)), P(f32(col)), C.c_int64(len(pts)), C.c_float(v), P(ox), P(oc))
        g[f"voxel_{tag}_size"] = np.float32(v)
        g[f"voxel_{tag}_xyz"], g[f"voxel_{tag}_rgb"] = ox[:m], oc[:m]

    # --- nearest neighbour ----------------------------------------------------
    q = f32(xyz[:4000] + rng.normal(scale=0.01, size=(4000, 3)))
    r = xyz[4000:]
    out, gm = np.zeros(len(q), np.int32), np.zeros(3, np.float32)
    L.ref_nn_search(P(q), C.c_int64(len(q)), P(r), C.c_int64(len(r)), C.c_float(0.05), P(out), P(gm))
    g["nn_q"], g["nn_radius"], g["nn_idx"], g["nn_grid_min"] = q, np.float32(0.05), out, gm
    # exact ties across cells: lattice points with queries on cell faces/midpoints
    lat = np.stack(np.meshgrid(np.arange(8), np.arange(8), np.arange(8), indexing="ij"), -1).reshape(-1, 3)
    lat = f32(lat * 0.25)
    lq = f32(lat[::7] + np.array([0.125, 0.0, 0.125], np.float32))
    out2 = np.zeros(len(lq), np.int32)
    L.ref_nn_search(P(lq), C.c_int64(len(lq)), P(lat), C.c_int64(len(lat)), C.c_float(0.25), P(out2), P(gm))
    g["nntie_q"], g["nntie_r"], g["nntie_radius"] = lq, lat, np.float32(0.25)
    g["nntie_idx"], g["nntie_grid_min"] = out2, gm.copy()

    # --- radius lists, normals, gradient ----------------------------------
    pts = xyz[:8000]
    col = rgb[:8000]
    rad = 0.09
    cnt, st = np.zeros(len(pts), np.int32), np.zeros(len(pts), np.int32)
    cap = len(pts) * 256
    lst = np.zeros(cap, np.int32)
    tot = L.ref_radius_search(P(pts), C.c_int64(len(pts)), C.c_float(rad), P(cnt), P(st), P(lst),
                              C.c_int64(cap), P(gm))
    g["radius_r"] = np.float32(rad)
    g["radius_counts"], g["radius_starts"], g["radius_list"] = cnt, st, lst[:tot]
    g["radius_grid_min"] = gm.copy()
    nrm = np.zeros((len(pts), 3), np.float32)
    L.ref_estimate_normals(P(pts), C.c_int64(len(pts)), C.c_float(rad), P(nrm), P(gm))
    g["normals"], g["normals_grid_min"] = nrm, gm.copy()
    grad = np.zeros((len(pts), 3), np.float32)
    L.ref_color_gradient(P(pts), P(col), P(nrm), C.c_int64(len(pts)), C.c_float(rad), P(grad), P(gm))
    g["grad"], g["grad_grid_min"] = grad, gm.copy()

    # --- Gauss-Newton system and residuals --------------------------------
    T = synth.make_T(synth.axis_angle([0.3, -0.5, 0.8], np.radians(2.0)), [0.02, -0.01, 0.015])
    sx = synth.transform(T, xyz[8000:12000] + rng.normal(scale=0.003, size=(4000, 3)))
    srgb = rgb[8000:12000]
    nn = np.zeros(len(sx), np.int32)
    L.ref_nn_search(P(sx), C.c_int64(len(sx)), P(pts), C.c_int64(len(pts)), C.c_float(0.06), P(nn), P(gm))
    jtj, jtr, r2 = np.zeros(36, np.float32), np.zeros(6, np.float32), C.c_float(0)
    L.ref_build_gn(P(sx), P(srgb), C.c_int64(len(sx)), P(pts), P(col), P(nrm), P(grad),
                   C.c_int64(len(pts)), P(nn), C.c_float(0.968), P(jtj), P(jtr), C.byref(r2))
    ares = np.zeros(len(sx), np.float32)
    L.ref_abs_residual(P(sx), P(srgb), C.c_int64(len(sx)), P(pts), P(col), P(nrm), P(grad),
                       C.c_int64(len(pts)), P(nn), C.c_float(0.968), P(ares))
    g["gn_src_xyz"], g["gn_nn"] = sx, nn
    g["gn_jtj"], g["gn_jtr"], g["gn_r2"], g["gn_abs_residual"] = jtj.reshape(6, 6), jtr, np.float32(r2.value), ares

    # --- rigid transform ----------------------------------------------------
    tx = pts[:3000].copy()
    Tf = f32(T)
    L.ref_transform(P(tx), C.c_int64(len(tx)), P(Tf))
    g["transform_T"], g["transform_out"] = Tf, tx

    # --- radius outlier removal (demo front end) ---------------------------
    ro_x, ro_c = np.zeros_like(pts), np.zeros_like(pts)
    m = L.ref_radius_outlier_removal(P(pts), P(col), C.c_int64(len(pts)), C.c_float(0.05), 4, P(ro_x), P(ro_c))
    g["ror_radius"], g["ror_min_nn"] = np.float32(0.05), np.int32(4)
    g["ror_xyz"], g["ror_rgb"] = ro_x[:m], ro_c[:m]

    # --- RGB-D frame -> cloud (cuda_point_cloud_factory.cu helpers) ------------
    depth, bgr = synth.render_rgbd(synth.frame_scene(1234), np.eye(4), 5, FRAME_CAM)[:2]
    g["frame_depth"], g["frame_bgr"] = depth, bgr
    n = depth.size
    for case in FRAME_CASES:
        di, ci, rot, tr, mode, tmin = frame_case_args(case)
        runs = (("ref_make_point_cloud_detexp", "detexp"), ("ref_make_point_cloud", "stock"))
        for fn, tag in runs[:1] if mode == 0 else runs:  # no exp without a filter
            xyz, rgb = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
            fd, cuv = np.zeros(n, np.float32), np.zeros((n, 2), np.float32)
            m = getattr(L, fn)(P(depth), P(bgr), C.c_uint32(FRAME_CAM.width), C.c_uint32(FRAME_CAM.height), P(di),
                               P(ci), P(rot), P(tr), C.c_float(0.001), C.c_float(tmin), C.c_float(10.0), mode,
                               FRAME_FIXED[0], C.c_float(FRAME_FIXED[1]), C.c_float(FRAME_FIXED[2]), P(xyz), P(rgb),
                               P(fd), P(cuv))
            g[f"frame_{case[0]}_args"] = np.concatenate([di, ci, rot, tr, [mode, tmin]]).astype(np.float32)
            k = f"frame_{case[0]}_{tag}"
            g[k + "_xyz"], g[k + "_rgb"], g[k + "_depth"] = xyz[:m], rgb[:m], fd.reshape(depth.shape)
            if tag == "stock":
                g[k + "_cuv"] = cuv[:m]

    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT}: {os.path.getsize(OUT) / 1e6:.2f} MB, {len(g)} arrays")


if __name__ == "__main__":
    main(*sys.argv[1:])
