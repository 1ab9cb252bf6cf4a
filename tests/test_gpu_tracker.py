"""Frame-to-frame tracking of an RGB-D stream (gca3d_tracker_*) through the C ABI.

Frames come from the procedural frame scene rendered along a smooth camera path
(~1.5 cm and ~1 deg per frame).  Pipeline per frame, as the 640x480 frame-pair
workload asks: 5x5 bilateral filter (sigma_s 3 px, sigma_d 30 mm), back-projection
with t_min 0.2 m, 0.01 m voxels, normals with radius 0.02 m and at most 30
neighbours, colour gradients with radius 0.02 m, colored ICP with lambda 0.968, at
most 30 iterations, max correspondence distance 0.03 m.  Checks:
  * every registration equals, bit for bit, the same frames run through the
    individual stage entry points (frame_to_cloud, then color_icp);
  * every registration is within 1e-5 rad / 1e-5 m of the FP64 oracle run on the
    oracle's own clouds of the two frames from the same initial pose, with the same
    iteration count;
  * the captured per-frame graph and the plain eager pipeline give identical poses;
  * the composed trajectory stays within DRIFT_ROT / DRIFT_TRANS of ground truth
    (measured on GB300 after 10 frames: 0.010 rad, 0.017 m; with the reference's
    convergence thresholds each registration stops once a step is below 1 mm and
    0.08 deg, and the depth noise of 0.002 z^2 m sets the floor.  A composition in
    the wrong order would be off by about 0.17 rad)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_FRAMES = 10
DRIFT_ROT = 0.03   # rad after N_FRAMES frames
DRIFT_TRANS = 0.05  # m


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
    poses = synth.spline_poses(N_FRAMES, seed=4)
    frames = [synth.render_rgbd_torch(scene, P, 1000 + k) for k, P in enumerate(poses)]
    return synth.Camera(), poses, frames


def c0_scales(N):
    return [N.scale(0.01, 30, 0.03, 0.02, 0.02, 30)]


def run_tracker(ctx, N, seq, use_graph):
    cam, poses, frames = seq
    tr = N.Tracker(ctx, N.tracker_params(cam, c0_scales(N), use_graph=use_graph))
    out = [tr.push(d, c) for d, c in frames]
    return out, tr


def test_tracker_first_frame(ctx, N, seq):
    cam, poses, frames = seq
    tr = N.Tracker(ctx, N.tracker_params(cam, c0_scales(N), use_graph=True))
    r, pose = tr.push(*frames[0])
    assert r["status"] == N.ERR_NO_CORRESPONDENCES
    np.testing.assert_array_equal(pose, np.eye(4))


def test_tracker_matches_stage_entry_points(ctx, N, seq):
    cam, poses, frames = seq
    out, _ = run_tracker(ctx, N, seq, use_graph=True)
    intr = N.Intrinsics(cam.fx, cam.fy, cam.cx, cam.cy)
    filt = N.Filter(N.FILTER_FIXED, 2, 3.0, 30.0)
    clouds = []
    for d, c in frames:
        cl = ctx.cloud(cam.width * cam.height)
        d = np.ascontiguousarray(d)
        c = np.ascontiguousarray(c)
        ctx.check(ctx.L.gca3d_frame_to_cloud(ctx.h, d.ctypes.data, c.ctypes.data, cam.width, cam.height,
                                             C.byref(intr), None, None, 0.001, 0.2, 10.0, C.byref(filt), cl.h))
        clouds.append(cl)
    prm = N.icp_params(c0_scales(N))
    last = np.eye(4)
    for k in range(1, N_FRAMES):
        r = N.color_icp(ctx, clouds[k], clouds[k - 1], prm, T_init=last)
        assert r["status"] == N.OK
        np.testing.assert_array_equal(out[k][0]["T"], r["T"])
        assert out[k][0]["iterations"] == r["iterations"]
        last = r["T"]


def test_tracker_matches_fp64_oracle(ctx, N, orc, seq):
    """per frame: the oracle's frame stage (bit-exact with the kernel's), 0.01 m voxels,
    FP64 normals (at most 30 neighbours) and gradients, and FP64 colored ICP from the
    tracker's initial pose for that frame (the previous frame's motion)"""
    from cuda_3d_gb300 import synth

    cam, poses, frames = seq
    out, _ = run_tracker(ctx, N, seq, use_graph=True)
    intr = (cam.fx, cam.fy, cam.cx, cam.cy)
    clouds = [orc.make_point_cloud(d, c, intr, mode=orc.FILTER_FIXED, radius=2, sigma_space=3.0, sigma_depth=30.0,
                                   tmin=0.2, tmax=10.0) for d, c in frames]
    T_init = np.eye(4)
    for k in range(1, N_FRAMES):
        (sx, sc), (tx, tc) = clouds[k], clouds[k - 1]
        T64, res = orc.multiscale_f64(sx, sc, tx, tc, [orc.Scale(0.01, 30, 0.03, 0.02, 0.02, 30)],
                                      update_map=orc.UPDATE_EULER_ZYX, T_init=T_init)
        r = out[k][0]
        rot, tr = synth.pose_error(r["T"], T64)
        assert rot <= 1e-5 and tr <= 1e-5, (k, rot, tr)
        assert r["iterations"] == res[0].iterations, k
        T_init = r["T"]


def test_tracker_graph_equals_plain_and_follows_ground_truth(ctx, N, seq):
    from cuda_3d_gb300 import synth

    cam, poses, frames = seq
    g, trg = run_tracker(ctx, N, seq, use_graph=True)
    p, _ = run_tracker(ctx, N, seq, use_graph=False)
    for (rg, pg), (rp, pp) in zip(g, p):
        np.testing.assert_array_equal(pg, pp)
        assert rg["iterations"] == rp["iterations"]
    assert trg.kernels() > 0
    for k in range(1, N_FRAMES):
        assert g[k][0]["status"] == N.OK
        assert g[k][0]["fitness"] > 0.5
    rot, tr = synth.pose_error(g[-1][1], poses[-1])
    assert rot <= DRIFT_ROT and tr <= DRIFT_TRANS, (rot, tr)


def test_tracker_rejects_raw_scales(ctx, N, seq):
    cam, _, _ = seq
    prm = N.tracker_params(cam, [N.scale(0.0, 30, 0.03, 0.02, 0.02, 30)])
    h = C.c_void_p()
    assert ctx.L.gca3d_tracker_create(ctx.h, C.byref(prm), C.byref(h)) == N.ERR_INVALID_VALUE
    prm = N.tracker_params(cam, c0_scales(N), depth_scale=0.0)
    assert ctx.L.gca3d_tracker_create(ctx.h, C.byref(prm), C.byref(h)) == N.ERR_INVALID_VALUE
