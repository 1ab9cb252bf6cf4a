"""The frame-to-model accumulation loop (gca3d_model_*, the reference demo's
reconstruction loop, apps/app.cpp:111-128 and 315-349) through the C ABI.

Frames: the procedural frame scene along a smooth camera path.  Settings: the
reference demo's (voxel 0.008, radius outlier removal 0.01 / 4, normals 0.04,
colored ICP 10 / 0.05 / 0.05, re-voxelisation every 5 appends, adaptive bilateral
filter) except t_max = 10 m: the synthetic room reaches 4 m, a real camera in the demo
was cut at 2.5 m.  Checks:
  * the same loop replayed through the individual stage entry points gives the same
    model, bit for bit, and the same append decisions;
  * the loop replayed with the FP64 oracle's stages (frame stage, voxels and outlier
    removal bit-exact, FP64 normals, gradients and colored ICP) gives every
    registration within 1e-5 rad / 1e-5 m and the same append decisions; the replay
    moves its model by the GPU's FP32 pose, so both loops hold the same model, which
    is compared bit for bit at the end;
  * every registration lands near the ground-truth relative motion;
  * the model stays bounded by the re-voxelisation."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_FRAMES = 9


@pytest.fixture(scope="module")
def N():
    from cuda_3d_gb300 import build, native

    build.build()
    return native


@pytest.fixture(scope="module")
def ctx(N):
    return N.Context(0)


@pytest.fixture(scope="module")
def seq():
    from cuda_3d_gb300 import synth

    scene = synth.frame_scene(1234)
    poses = synth.spline_poses(N_FRAMES, seed=7)
    frames = [synth.render_rgbd_torch(scene, P, 2000 + k) for k, P in enumerate(poses)]
    return synth.Camera(), poses, frames


def test_model_loop_matches_stage_replay(ctx, N, seq):
    from cuda_3d_gb300 import synth

    cam, poses, frames = seq
    prm = N.model_params(cam, tmax=10.0)
    model = N.Model(ctx, prm)
    out = [model.push(d, c) for d, c in frames]
    got = model.cloud().download(rgb=True)

    # replay with the stage entry points
    npix = cam.width * cam.height
    intr = N.Intrinsics(cam.fx, cam.fy, cam.cx, cam.cy)
    filt = N.Filter(N.FILTER_ADAPTIVE, 0, 0.0, 0.0)
    ip = N.icp_params([N.scale(0.0, 10, 0.05, 0.0, 0.05, 0)], update_map=N.UPDATE_EULER_ZYX,
                      rot_eps=float(np.float32(1e-6)), trans_eps=float(np.float32(1e-6)), compensated=True,
                      keep_target_normals=True)
    cap = prm.model_capacity
    mdl, mdl2 = ctx.cloud(cap), ctx.cloud(cap)
    prev = None
    counter = 0
    sizes = []
    for k, (d, c) in enumerate(frames):
        raw, ds, cur = ctx.cloud(npix), ctx.cloud(npix), ctx.cloud(npix)
        d = np.ascontiguousarray(d)
        c = np.ascontiguousarray(c)
        ctx.check(ctx.L.gca3d_frame_to_cloud(ctx.h, d.ctypes.data, c.ctypes.data, cam.width, cam.height,
                                             C.byref(intr), C.byref(intr), None, 0.001, 0.2, 10.0, C.byref(filt),
                                             raw.h))
        ctx.check(ctx.L.gca3d_voxel_downsample(ctx.h, raw.h, 0.008, ds.h))
        ctx.check(ctx.L.gca3d_radius_outlier_removal(ctx.h, ds.h, 0.01, 4, cur.h))
        ctx.check(ctx.L.gca3d_estimate_normals(ctx.h, cur.h, 0.04, 0))
        if k == 0:
            ctx.check(ctx.L.gca3d_cloud_copy(ctx.h, cur.h, mdl.h))
            assert out[0][0]["status"] == N.ERR_NO_CORRESPONDENCES
        else:
            r = N.color_icp(ctx, mdl if counter == 0 else prev, cur, ip)
            assert r["status"] == N.OK
            np.testing.assert_array_equal(out[k][0]["T"], r["T"])
            Tf = r["T"].astype(np.float32)
            cth = np.float32(0.5) * (Tf[0, 0] + Tf[1, 1] + Tf[2, 2] - np.float32(1))
            tsq = Tf[0, 3] * Tf[0, 3] + Tf[1, 3] * Tf[1, 3] + Tf[2, 3] * Tf[2, 3]
            app = bool(cth <= np.float32(0.999999) or tsq >= np.float32(1e-6))
            assert out[k][1] == app
            if app:
                ctx.check(ctx.L.gca3d_transform(ctx.h, mdl.h, Tf.astype(np.float64).ctypes.data))
                ctx.check(ctx.L.gca3d_cloud_append(ctx.h, mdl.h, cur.h))
                counter += 1
            if counter == 5:
                ctx.check(ctx.L.gca3d_voxel_downsample(ctx.h, mdl.h, 0.008, mdl2.h))
                mdl, mdl2 = mdl2, mdl
                counter = 0
            # the registration follows the camera: model (previous camera) -> this camera
            T_gt = np.linalg.inv(poses[k]) @ poses[k - 1]
            rot, tr = synth.pose_error(r["T"], T_gt)
            assert rot < 0.02 and tr < 0.03, (k, rot, tr)
        prev = cur
        sizes.append(len(mdl))
    want = mdl.download(rgb=True)
    np.testing.assert_array_equal(got["xyz"], want["xyz"])
    np.testing.assert_array_equal(got["rgb"], want["rgb"])
    # bounded by the re-voxelisation: never more than 5 frames' worth above one frame
    assert max(sizes) < 7 * sizes[0]


def transform_ref32(T, xyz):
    """point_cloud::transform (src/geometry/point_cloud.cu:93-105): FP32, unfused
    ((R0 x + R1 y) + R2 z) + t"""
    T = np.asarray(T, np.float32)
    x, y, z = (np.ascontiguousarray(xyz[:, k], np.float32) for k in range(3))
    return np.stack([((T[r, 0] * x + T[r, 1] * y) + T[r, 2] * z) + T[r, 3] for r in range(3)], 1).astype(np.float32)


def test_model_loop_matches_fp64_oracle_replay(ctx, N, orc, seq):
    """apps/app.cpp:111-128 and 315-349 replayed with the oracle's stages"""
    from cuda_3d_gb300 import synth

    cam, poses, frames = seq
    model = N.Model(ctx, N.model_params(cam, tmax=10.0))
    out = [model.push(d, c) for d, c in frames]
    got = model.cloud().download(rgb=True)
    intr = (cam.fx, cam.fy, cam.cx, cam.cy)
    eps = float(np.float32(1e-6))  # color_icp.hpp:47-48
    mx = mc = px = pc = None
    counter = 0
    for k, (d, c) in enumerate(frames):
        rx, rc = orc.make_point_cloud(d, c, intr, mode=orc.FILTER_ADAPTIVE, tmin=0.2, tmax=10.0)
        vx, vc, _, _ = orc.voxel_downsample(rx, rc, 0.008)
        cx, cc = orc.radius_outlier_removal(vx, vc, 0.01, 4)
        if k == 0:
            mx, mc = cx, cc
        else:
            sx, sc = (mx, mc) if counter == 0 else (px, pc)
            tn = orc.normals_f64(cx, 0.04, 0)
            tg = orc.gradient_f64(cx, cc, tn, 0.05)
            o = orc.color_icp_f64(sx, sc, cx, cc, tn, tg, max_iter=10, max_corr=0.05, update_map=orc.UPDATE_EULER_ZYX,
                                  rot_eps=eps, trans_eps=eps)
            r, appended = out[k]
            assert r["status"] == N.OK
            rot, tr = synth.pose_error(r["T"], o.T)
            assert rot <= 1e-5 and tr <= 1e-5, (k, rot, tr)
            assert r["iterations"] == o.iterations, k
            # the append decision of the oracle's own pose (app.cpp:328-340, FP32)
            Tf = o.T.astype(np.float32)
            cth = np.float32(0.5) * (Tf[0, 0] + Tf[1, 1] + Tf[2, 2] - np.float32(1))
            tsq = Tf[0, 3] * Tf[0, 3] + Tf[1, 3] * Tf[1, 3] + Tf[2, 3] * Tf[2, 3]
            assert appended == bool(cth <= np.float32(0.999999) or tsq >= np.float32(1e-6)), k
            if appended:
                mx = np.concatenate([transform_ref32(r["T"].astype(np.float32), mx), cx])
                mc = np.concatenate([mc, cc])
                counter += 1
            if counter == 5:
                mx, mc, _, _ = orc.voxel_downsample(mx, mc, 0.008)
                counter = 0
        px, pc = cx, cc
    np.testing.assert_array_equal(got["xyz"], mx)
    np.testing.assert_array_equal(got["rgb"], mc)


def test_model_rejects_bad_parameters(ctx, N, seq):
    cam, _, _ = seq
    h = C.c_void_p()
    bad = N.model_params(cam, voxel=0.0)
    assert ctx.L.gca3d_model_create(ctx.h, C.byref(bad), C.byref(h)) == N.ERR_INVALID_VALUE
    bad = N.model_params(cam, model_capacity=10)
    assert ctx.L.gca3d_model_create(ctx.h, C.byref(bad), C.byref(h)) == N.ERR_INVALID_VALUE
