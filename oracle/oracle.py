"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module.  It is the checker, never the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgca_oracle.so")

FILTER_NONE, FILTER_ADAPTIVE, FILTER_FIXED = 0, 1, 2
TIE_SCAN_ORDER, TIE_MIN_INDEX = 0, 1
UPDATE_EULER_ZYX, UPDATE_SE3_EXP = 0, 1

_lib = None


def build(force=False):
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _bind(_lib)
    return _lib


F32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
F64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
I64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
U16 = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
U8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


class Intrinsics(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float)]


class Extrinsics(C.Structure):
    _fields_ = [("rotation", C.c_float * 9), ("translation", C.c_float * 3)]


class IcpParams(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("max_corr", C.c_float), ("lambda_", C.c_float),
                ("update_map", C.c_int), ("rot_eps", C.c_double), ("trans_eps", C.c_double),
                ("search_f32", C.c_int)]


class UnrollParams(C.Structure):
    _fields_ = [("K", C.c_int), ("max_corr", C.c_float), ("lambda_", C.c_float), ("update_map", C.c_int)]


class IcpResult(C.Structure):
    _fields_ = [("T", C.c_double * 16), ("rmse_ref", C.c_double), ("fitness", C.c_double),
                ("inlier_rmse", C.c_double), ("iterations", C.c_int), ("converged", C.c_int),
                ("status", C.c_int)]


def _bind(L):
    v, i64 = None, C.c_int64
    sig = {
        "orc_set_threads": (v, [C.c_int]),
        "orc_get_threads": (C.c_int, []),
        "orc_intensity": (C.c_float, [C.c_float, C.c_float, C.c_float]),
        "orc_exp32": (C.c_float, [C.c_float]),
        "orc_aabb": (v, [F32, i64, C.c_int, F32, F32]),
        "orc_make_point_cloud": (i64, [U16, U8, C.c_int, C.c_int, C.POINTER(Intrinsics),
                                       C.POINTER(Intrinsics), C.POINTER(Extrinsics), C.c_float,
                                       C.c_float, C.c_float, C.c_int, C.c_int, C.c_float,
                                       C.c_float, F32, F32, C.c_void_p]),
        "orc_voxel_downsample": (i64, [F32, F32, i64, F32, C.c_float, F32, F32, I32, I32]),
        "orc_nn_search": (v, [F32, i64, F32, i64, C.c_float, F32, C.c_int, I32]),
        "orc_radius_search": (i64, [F32, i64, F32, i64, C.c_float, F32, I32, I64, C.c_void_p, i64]),
        "orc_normals_ref32": (v, [F32, i64, C.c_float, F32, F32]),
        "orc_normals_f64": (v, [F32, i64, C.c_float, C.c_int, F64]),
        "orc_gradient_ref32": (v, [F32, F32, F32, i64, C.c_float, F32, F32]),
        "orc_gradient_f64": (v, [F32, F32, F64, i64, C.c_float, F64]),
        "orc_build_gn_ref32": (v, [F32, F32, i64, F32, F32, F32, F32, I32, C.c_float, F32, F32,
                                   C.POINTER(C.c_float)]),
        "orc_abs_residual_ref32": (v, [F32, F32, i64, F32, F32, F32, F32, I32, C.c_float, F32]),
        "orc_solve6": (C.c_int, [F64, F64, F64]),
        "orc_pose_from_x": (v, [F64, C.c_int, F64]),
        "orc_color_icp_f64": (v, [F32, F32, i64, F32, F32, F64, F64, i64, C.POINTER(IcpParams),
                                  F64, C.POINTER(IcpResult)]),
        "orc_color_icp_ref32": (v, [F32, F32, i64, F32, F32, F32, F32, i64, C.c_int, C.c_float,
                                    F32, C.POINTER(IcpResult)]),
        "orc_pose_jacobian": (v, [F64, C.c_int, F64]),
        "orc_apply_pose_f32": (v, [F64, F32, i64, F32]),
        "orc_radius_outlier_removal": (i64, [F32, F32, i64, C.c_float, C.c_int, F32, F32]),
        "orc_icp_unrolled_f64": (C.c_double, [F64, F64, i64, F32, F32, F64, F64, i64,
                                              C.POINTER(UnrollParams), F64, C.c_void_p, C.c_void_p, F64]),
        "orc_icp_unrolled_vjp_f64": (C.c_int, [F64, F64, i64, F32, F32, F64, F64, i64,
                                               C.POINTER(UnrollParams), F64, I32, F64, C.c_double, F64, F64,
                                               F64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _f32(a, cols=3):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(-1, cols) if cols else a


def set_threads(n):
    lib().orc_set_threads(int(n))


def exp32(x):
    f = lib().orc_exp32
    return np.array([f(float(v)) for v in np.asarray(x, np.float32).reshape(-1)], np.float32)


def intensity(rgb):
    rgb = np.asarray(rgb, np.float32).reshape(-1, 3)
    f = lib().orc_intensity
    return np.array([f(*map(float, c)) for c in rgb], np.float32)


def aabb(xyz, flt_min_bug=False):
    xyz = _f32(xyz)
    mn, mx = np.zeros(3, np.float32), np.zeros(3, np.float32)
    lib().orc_aabb(xyz, len(xyz), int(flt_min_bug), mn, mx)
    return mn, mx


def make_point_cloud(depth, bgr, depth_intrin, color_intrin=None, d2c=None, depth_scale=0.001,
                     tmin=0.2, tmax=10.0, mode=FILTER_ADAPTIVE, radius=2, sigma_space=3.0,
                     sigma_depth=30.0, return_depth=False):
    depth = np.ascontiguousarray(depth, np.uint16)
    bgr = np.ascontiguousarray(bgr, np.uint8)
    h, w = depth.shape
    di = Intrinsics(*depth_intrin)
    ci = Intrinsics(*(color_intrin or depth_intrin))
    e = Extrinsics()
    rot = np.eye(3, dtype=np.float32).T.reshape(-1) if d2c is None else np.asarray(d2c[0], np.float32)
    tr = np.zeros(3, np.float32) if d2c is None else np.asarray(d2c[1], np.float32)
    e.rotation[:] = list(map(float, rot))
    e.translation[:] = list(map(float, tr))
    xyz = np.zeros((h * w, 3), np.float32)
    rgb = np.zeros((h * w, 3), np.float32)
    fd = np.zeros(h * w, np.float32)
    m = lib().orc_make_point_cloud(depth.reshape(-1), bgr.reshape(-1), w, h, C.byref(di), C.byref(ci),
                                   C.byref(e), depth_scale, tmin, tmax, mode, radius, sigma_space,
                                   sigma_depth, xyz, rgb, fd.ctypes.data)
    out = (xyz[:m].copy(), rgb[:m].copy())
    return out + (fd.reshape(h, w),) if return_depth else out


def voxel_downsample(xyz, rgb, voxel, mn=None):
    xyz, rgb = _f32(xyz), _f32(rgb)
    n = len(xyz)
    if mn is None:
        mn = aabb(xyz)[0] if n else np.zeros(3, np.float32)
    mn = np.ascontiguousarray(mn, np.float32)
    ox, orgb = np.zeros((max(n, 1), 3), np.float32), np.zeros((max(n, 1), 3), np.float32)
    cnt, key = np.zeros(max(n, 1), np.int32), np.zeros((max(n, 1), 3), np.int32)
    m = lib().orc_voxel_downsample(xyz, rgb, n, mn, voxel, ox, orgb, cnt, key)
    return ox[:m].copy(), orgb[:m].copy(), cnt[:m].copy(), key[:m].copy()


def nn_search(q, r, radius, grid_min=None, tie=TIE_MIN_INDEX):
    q, r = _f32(q), _f32(r)
    if grid_min is None:
        qa, ra = aabb(q, True), aabb(r, True)
        grid_min = np.minimum(qa[0], ra[0]) - np.float32(1.5) * np.float32(radius)
    out = np.zeros(len(q), np.int32)
    lib().orc_nn_search(q, len(q), r, len(r), radius, np.ascontiguousarray(grid_min, np.float32), tie, out)
    return out


def normals_grid_min(xyz, radius):
    """point_cloud::estimate_normals bounds: double padding narrowed to float"""
    mn = aabb(xyz, True)[0].astype(np.float64)
    return (mn - 1.5 * float(np.float32(radius))).astype(np.float32)


def gradient_grid_min(xyz, radius):
    """color_icp::compute_color_gradient_target bounds: float padding"""
    return aabb(xyz, True)[0] - np.float32(1.5) * np.float32(radius)


def radius_search(q, r, radius, grid_min):
    q, r = _f32(q), _f32(r)
    counts = np.zeros(len(q), np.int32)
    starts = np.zeros(len(q), np.int64)
    gm = np.ascontiguousarray(grid_min, np.float32)
    total = lib().orc_radius_search(q, len(q), r, len(r), radius, gm, counts, starts, None, 0)
    lst = np.zeros(max(total, 1), np.int32)
    lib().orc_radius_search(q, len(q), r, len(r), radius, gm, counts, starts, lst.ctypes.data, total)
    return counts, starts, lst[:total]


def radius_outlier_removal(xyz, rgb, radius, min_nn):
    xyz, rgb = _f32(xyz), _f32(rgb)
    ox, oc = np.zeros_like(xyz), np.zeros_like(rgb)
    m = lib().orc_radius_outlier_removal(xyz, rgb, len(xyz), float(radius), int(min_nn), ox, oc)
    return ox[:m], oc[:m]


def normals_ref32(xyz, radius, grid_min=None):
    xyz = _f32(xyz)
    gm = normals_grid_min(xyz, radius) if grid_min is None else np.asarray(grid_min, np.float32)
    out = np.zeros_like(xyz)
    lib().orc_normals_ref32(xyz, len(xyz), radius, gm, out)
    return out


def normals_f64(xyz, radius, max_nn=0):
    xyz = _f32(xyz)
    out = np.zeros(xyz.shape, np.float64)
    lib().orc_normals_f64(xyz, len(xyz), radius, int(max_nn), out)
    return out


def gradient_ref32(xyz, rgb, nrm, radius, grid_min=None):
    xyz, rgb, nrm = _f32(xyz), _f32(rgb), _f32(nrm)
    gm = gradient_grid_min(xyz, radius) if grid_min is None else np.asarray(grid_min, np.float32)
    out = np.zeros_like(xyz)
    lib().orc_gradient_ref32(xyz, rgb, nrm, len(xyz), radius, gm, out)
    return out


def gradient_f64(xyz, rgb, nrm, radius):
    xyz, rgb = _f32(xyz), _f32(rgb)
    nrm = np.ascontiguousarray(nrm, np.float64).reshape(-1, 3)
    out = np.zeros(xyz.shape, np.float64)
    lib().orc_gradient_f64(xyz, rgb, nrm, len(xyz), radius, out)
    return out


def build_gn_ref32(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad, nn, lam=0.968):
    jtj, jtr, r2 = np.zeros(36, np.float32), np.zeros(6, np.float32), C.c_float(0)
    lib().orc_build_gn_ref32(_f32(src_xyz), _f32(src_rgb), len(src_xyz), _f32(tgt_xyz), _f32(tgt_rgb),
                             _f32(tgt_nrm), _f32(tgt_grad), np.ascontiguousarray(nn, np.int32), lam,
                             jtj, jtr, C.byref(r2))
    return jtj.reshape(6, 6), jtr, r2.value


def abs_residual_ref32(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad, nn, lam=0.968):
    out = np.zeros(len(src_xyz), np.float32)
    lib().orc_abs_residual_ref32(_f32(src_xyz), _f32(src_rgb), len(src_xyz), _f32(tgt_xyz),
                                 _f32(tgt_rgb), _f32(tgt_nrm), _f32(tgt_grad),
                                 np.ascontiguousarray(nn, np.int32), lam, out)
    return out


def solve6(jtj, jtr):
    x = np.zeros(6, np.float64)
    st = lib().orc_solve6(np.ascontiguousarray(jtj, np.float64).reshape(-1),
                          np.ascontiguousarray(jtr, np.float64), x)
    return x, st


def pose_from_x(x, update_map=UPDATE_EULER_ZYX):
    T = np.zeros(16, np.float64)
    lib().orc_pose_from_x(np.ascontiguousarray(x, np.float64), update_map, T)
    return T.reshape(4, 4)


@dataclass
class IcpOut:
    T: np.ndarray
    rmse_ref: float
    fitness: float
    inlier_rmse: float
    iterations: int
    converged: bool
    status: int


def _icp_out(r):
    return IcpOut(np.array(r.T[:]).reshape(4, 4), r.rmse_ref, r.fitness, r.inlier_rmse, r.iterations,
                  bool(r.converged), r.status)


def color_icp_f64(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad, max_iter=30, max_corr=0.03,
                  lam=0.968, update_map=UPDATE_EULER_ZYX, rot_eps=1e-6, trans_eps=1e-6, T_init=None,
                  search_f32=False):
    """search_f32: correspondences of the FP32 points that the GPU kernels search
    (pose rounded to float, fused application, FP32 squared distances); residuals,
    Jacobians, sums and the solve stay FP64"""
    p = IcpParams(int(max_iter), float(max_corr), float(lam), int(update_map), float(rot_eps), float(trans_eps),
                  int(bool(search_f32)))
    T0 = np.eye(4) if T_init is None else np.asarray(T_init, np.float64)
    r = IcpResult()
    lib().orc_color_icp_f64(_f32(src_xyz), _f32(src_rgb), len(src_xyz), _f32(tgt_xyz), _f32(tgt_rgb),
                            np.ascontiguousarray(tgt_nrm, np.float64).reshape(-1, 3),
                            np.ascontiguousarray(tgt_grad, np.float64).reshape(-1, 3), len(tgt_xyz),
                            C.byref(p), np.ascontiguousarray(T0, np.float64).reshape(-1), C.byref(r))
    return _icp_out(r)


def color_icp_ref32(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad, max_iter=30, max_corr=0.03,
                    T_init=None):
    T0 = np.eye(4, dtype=np.float32) if T_init is None else np.asarray(T_init, np.float32)
    r = IcpResult()
    lib().orc_color_icp_ref32(_f32(src_xyz), _f32(src_rgb), len(src_xyz), _f32(tgt_xyz), _f32(tgt_rgb),
                              _f32(tgt_nrm), _f32(tgt_grad), len(tgt_xyz), int(max_iter), float(max_corr),
                              np.ascontiguousarray(T0, np.float32).reshape(-1), C.byref(r))
    return _icp_out(r)


# --------------------------------------------------------------------------- #
# multi-scale schedule (no reference counterpart beyond the commented example in
# apps/test_color_icp.cpp:378-400): per scale, downsample both clouds from the
# originals, estimate target normals and colour gradients, run ICP from the pose
# of the previous scale.
# --------------------------------------------------------------------------- #
@dataclass
class Scale:
    voxel: float
    iters: int
    max_corr: float
    normal_radius: float
    grad_radius: float
    max_nn: int = 0


def multiscale_f64(src_xyz, src_rgb, tgt_xyz, tgt_rgb, scales, lam=0.968, update_map=UPDATE_SE3_EXP,
                   rot_eps=1e-6, trans_eps=1e-6, T_init=None, search_f32=False):
    T = np.eye(4) if T_init is None else np.asarray(T_init, np.float64)
    results = []
    for s in scales:
        sx, sc, _, _ = voxel_downsample(src_xyz, src_rgb, s.voxel)
        tx, tc, _, _ = voxel_downsample(tgt_xyz, tgt_rgb, s.voxel)
        tn = normals_f64(tx, s.normal_radius, s.max_nn)
        tg = gradient_f64(tx, tc, tn, s.grad_radius)
        r = color_icp_f64(sx, sc, tx, tc, tn, tg, s.iters, s.max_corr, lam, update_map, rot_eps, trans_eps, T,
                          search_f32)
        T = r.T
        results.append(r)
    return T, results


def multiscale_ref32(src_xyz, src_rgb, tgt_xyz, tgt_rgb, scales, T_init=None):
    """the reference's FP32 algorithm chained over the scales (the CPU port that the
    CPU baseline times)"""
    T = np.eye(4, dtype=np.float32) if T_init is None else np.asarray(T_init, np.float32)
    results = []
    for s in scales:
        sx, sc, _, _ = voxel_downsample(src_xyz, src_rgb, s.voxel)
        tx, tc, _, _ = voxel_downsample(tgt_xyz, tgt_rgb, s.voxel)
        tn = normals_ref32(tx, s.normal_radius)
        tg = gradient_ref32(tx, tc, tn, s.grad_radius)
        r = color_icp_ref32(sx, sc, tx, tc, tn, tg, s.iters, s.max_corr, T)
        T = r.T.astype(np.float32)
        results.append(r)
    return T.astype(np.float64), results


# --------------------------------------------------------------------------- #
# K unrolled Gauss-Newton steps and their adjoint (FP64; no reference
# counterpart).  T_0 = Exp(xi0); corr is (K + 1) x ns target indices.
# --------------------------------------------------------------------------- #
def apply_pose_f32(T, xyz):
    """the GPU ICP kernels' FP32 transform of points (fused, in a fixed order)"""
    xyz = _f32(xyz)
    out = np.empty_like(xyz)
    lib().orc_apply_pose_f32(np.ascontiguousarray(T, np.float64).reshape(-1), xyz, len(xyz), out)
    return out


def pose_jacobian(x, update_map=UPDATE_SE3_EXP):
    d = np.zeros(72, np.float64)
    lib().orc_pose_jacobian(np.ascontiguousarray(x, np.float64), int(update_map), d)
    return d.reshape(6, 3, 4)


def _unroll_args(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad):
    return (np.ascontiguousarray(src_xyz, np.float64).reshape(-1, 3),
            np.ascontiguousarray(src_rgb, np.float64).reshape(-1, 3), len(src_xyz), _f32(tgt_xyz), _f32(tgt_rgb),
            np.ascontiguousarray(tgt_nrm, np.float64).reshape(-1, 3),
            np.ascontiguousarray(tgt_grad, np.float64).reshape(-1, 3), len(tgt_xyz))


def icp_unrolled_f64(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad, xi0, K=5, max_corr=0.05, lam=0.968,
                     update_map=UPDATE_SE3_EXP, corr=None):
    """Returns (T_K, E, corr); corr is searched when not given (then returned)."""
    a = _unroll_args(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad)
    p = UnrollParams(int(K), float(max_corr), float(lam), int(update_map))
    T = np.zeros(16, np.float64)
    cout = None
    if corr is None:
        cout = np.zeros((K + 1, len(src_xyz)), np.int32)
        cin_p, cout_p = None, cout.ctypes.data
    else:
        corr = np.ascontiguousarray(corr, np.int32)
        cin_p, cout_p = corr.ctypes.data, None
    E = lib().orc_icp_unrolled_f64(*a, C.byref(p), np.ascontiguousarray(xi0, np.float64), cin_p, cout_p, T)
    return T.reshape(4, 4), E, (corr if cout is None else cout)


def icp_unrolled_vjp_f64(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad, xi0, corr, dT, dE, K=5,
                         max_corr=0.05, lam=0.968, update_map=UPDATE_SE3_EXP):
    """Gradient of <dT, T_K> + dE * E: returns (dxi0, dxyz, drgb, status)."""
    a = _unroll_args(src_xyz, src_rgb, tgt_xyz, tgt_rgb, tgt_nrm, tgt_grad)
    p = UnrollParams(int(K), float(max_corr), float(lam), int(update_map))
    n = len(src_xyz)
    dxi, dxyz, drgb = np.zeros(6), np.zeros((n, 3)), np.zeros((n, 3))
    st = lib().orc_icp_unrolled_vjp_f64(*a, C.byref(p), np.ascontiguousarray(xi0, np.float64),
                                        np.ascontiguousarray(corr, np.int32).reshape(-1),
                                        np.ascontiguousarray(dT, np.float64).reshape(-1), float(dE), dxi, dxyz, drgb)
    return dxi, dxyz, drgb, st
