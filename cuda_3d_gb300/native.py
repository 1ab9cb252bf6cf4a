"""ctypes binding of the gca3d C ABI (include/gca3d.h).

This module is how Python (tests, bench) reaches the CUDA path: every call goes
through the same extern "C" entry points a C or C++ caller uses.  There is no
fallback: if libgca3d.so is missing or no CUDA device is present, loading fails
loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgca3d.so")

OK = 0
ERR_INVALID_VALUE = 1
ERR_OUT_OF_MEMORY = 2
ERR_NO_CORRESPONDENCES = 3
ERR_SINGULAR = 4
ERR_TIMEOUT = 5
ERR_CUDA = 6
ERR_CAPACITY = 7
ERR_NOT_SUPPORTED = 8

FILTER_NONE, FILTER_ADAPTIVE, FILTER_FIXED = 0, 1, 2
UPLOAD_IN_PLACE, UPLOAD_COPY_ENGINE = 0, 1
UPDATE_EULER_ZYX, UPDATE_SE3_EXP = 0, 1
MAX_SCALES = 8


class Intrinsics(C.Structure):
    _fields_ = [("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float)]


class Extrinsics(C.Structure):
    _fields_ = [("rotation", C.c_float * 9), ("translation", C.c_float * 3)]


class Filter(C.Structure):
    _fields_ = [("mode", C.c_int), ("radius", C.c_int), ("sigma_space", C.c_float), ("sigma_depth", C.c_float)]


class ScaleParams(C.Structure):
    _fields_ = [("voxel", C.c_float), ("max_iter", C.c_int), ("max_corr", C.c_float),
                ("normal_radius", C.c_float), ("grad_radius", C.c_float), ("max_nn", C.c_int)]


class Tuning(C.Structure):
    _fields_ = [("nn_item_points", C.c_int), ("nn_blocks_per_sm", C.c_int), ("accum_blocks_per_sm", C.c_int),
                ("voxel_resort", C.c_int), ("fused_finalize", C.c_int),
                ("serial_prep", C.c_int)]


class IcpParams(C.Structure):
    _fields_ = [("n_scales", C.c_int), ("scales", ScaleParams * MAX_SCALES), ("lambda_", C.c_float),
                ("update_map", C.c_int), ("rot_eps", C.c_double), ("trans_eps", C.c_double),
                ("compensated", C.c_int), ("use_graph", C.c_int), ("keep_target_normals", C.c_int),
                ("tuning", Tuning)]


class IcpResult(C.Structure):
    _fields_ = [("T", C.c_double * 16), ("rmse_ref", C.c_double), ("fitness", C.c_double),
                ("inlier_rmse", C.c_double), ("iterations", C.c_int), ("converged", C.c_int),
                ("status", C.c_int), ("n_src", C.c_int), ("n_tgt", C.c_int),
                ("scale_iterations", C.c_int * MAX_SCALES), ("scale_n_src", C.c_int * MAX_SCALES),
                ("scale_n_tgt", C.c_int * MAX_SCALES)]


class TrackerParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("depth_intrin", Intrinsics), ("color_intrin", Intrinsics),
                ("depth_to_color", Extrinsics), ("depth_scale", C.c_float), ("tmin", C.c_float), ("tmax", C.c_float),
                ("filter", Filter), ("icp", IcpParams), ("constant_velocity", C.c_int)]


class ModelParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("depth_intrin", Intrinsics), ("color_intrin", Intrinsics),
                ("depth_to_color", Extrinsics), ("depth_scale", C.c_float), ("tmin", C.c_float), ("tmax", C.c_float),
                ("filter", Filter), ("voxel", C.c_float), ("ror_radius", C.c_float), ("ror_min_neighbors", C.c_int),
                ("normal_radius", C.c_float), ("max_iter", C.c_int), ("max_corr", C.c_float),
                ("grad_radius", C.c_float), ("revoxel_every", C.c_int), ("model_capacity", C.c_int64)]


class VjpParams(C.Structure):
    _fields_ = [("K", C.c_int), ("max_corr", C.c_float), ("lambda_", C.c_float), ("update_map", C.c_int)]


_P = C.c_void_p
_I64 = C.c_int64
_F = C.c_float
_SIGS = {
    "gca3d_create": [C.c_int, _P, C.POINTER(_P)],
    "gca3d_destroy": [_P],
    "gca3d_synchronize": [_P],
    "gca3d_status_string": [C.c_int],
    "gca3d_last_error": [_P],
    "gca3d_kernel_launches": [_P],
    "gca3d_stream": [_P],
    "gca3d_profile_begin": [_P, C.c_char_p],
    "gca3d_profile_read": [_P, C.POINTER(C.c_double), C.POINTER(_I64)],
    "gca3d_device_alloc": [_P, _I64, C.POINTER(_P)],
    "gca3d_device_free": [_P, _P],
    "gca3d_copy": [_P, _P, _P, _I64],
    "gca3d_cloud_create": [_P, _I64, C.POINTER(_P)],
    "gca3d_cloud_destroy": [_P],
    "gca3d_cloud_upload": [_P, _P, _P, _P, _I64],
    "gca3d_cloud_upload_many": [_P, C.c_int, _P, _P, _P, _P],
    "gca3d_set_upload_mode": [_P, C.c_int],
    "gca3d_cloud_set_normals": [_P, _P, _P, _I64],
    "gca3d_cloud_set_gradients": [_P, _P, _P, _I64],
    "gca3d_cloud_capacity": [_P, C.POINTER(_I64)],
    "gca3d_cloud_size": [_P, _P, C.POINTER(_I64)],
    "gca3d_cloud_has_normals": [_P, C.POINTER(C.c_int)],
    "gca3d_cloud_download": [_P, _P, _P, _P, _P, _P, _I64, C.POINTER(_I64)],
    "gca3d_cloud_device_views": [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)],
    "gca3d_cloud_copy": [_P, _P, _P],
    "gca3d_cloud_append": [_P, _P, _P],
    "gca3d_bounds": [_P, _P, _P, _P],
    "gca3d_transform": [_P, _P, _P],
    "gca3d_frame_to_cloud": [_P, _P, _P, C.c_int, C.c_int, C.POINTER(Intrinsics), C.POINTER(Intrinsics),
                             C.POINTER(Extrinsics), _F, _F, _F, C.POINTER(Filter), _P],
    "gca3d_voxel_downsample": [_P, _P, _F, _P],
    "gca3d_estimate_normals": [_P, _P, _F, C.c_int],
    "gca3d_color_gradient": [_P, _P, _F],
    "gca3d_nn_search": [_P, _P, _P, _F, _P],
    "gca3d_radius_search": [_P, _P, _P, _F, _P, _P, _P, _P, _I64, C.POINTER(_I64)],
    "gca3d_build_gauss_newton": [_P, _P, _P, _P, _F, _P, _P, C.POINTER(C.c_double)],
    "gca3d_build_gauss_newton_static": [_P, _P, C.c_int32, _P, _P, _P, _P, _F, _P, _P, _P],
    "gca3d_abs_residual": [_P, _P, _P, _P, _F, _P],
    "gca3d_color_icp": [_P, _P, _P, C.POINTER(IcpParams), _P, C.POINTER(IcpResult)],
    "gca3d_color_icp_batched": [_P, C.c_int, _P, _P, C.POINTER(IcpParams), _P, _P],
    "gca3d_icp_plan_create": [_P, C.c_int, _P, _P, C.POINTER(IcpParams), C.POINTER(_P)],
    "gca3d_icp_plan_execute": [_P, _P, _P],
    "gca3d_icp_plan_results": [_P, _P],
    "gca3d_icp_plan_destroy": [_P],
    "gca3d_icp_plan_kernels": [_P, C.POINTER(_I64)],
    "gca3d_icp_plan_readback_bytes": [_P, C.POINTER(_I64)],
    "gca3d_icp_autotune": [_P, C.c_int, _P, _P, C.POINTER(IcpParams), C.c_int, C.POINTER(Tuning),
                           C.POINTER(C.c_double)],
    "gca3d_radius_outlier_removal": [_P, _P, _F, C.c_int, _P],
    "gca3d_cloud_select": [_P, _P, _P, _I64, _P],
    "gca3d_cloud_to_aos": [_P, _P, _P, _P],
    "gca3d_ply_info": [C.c_char_p, C.POINTER(_I64), C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "gca3d_ply_read": [C.c_char_p, _P, _P, _P, _I64, C.POINTER(_I64)],
    "gca3d_ply_write": [C.c_char_p, _P, _P, _P, _I64, C.c_int],
    "gca3d_model_create": [_P, C.POINTER(ModelParams), C.POINTER(_P)],
    "gca3d_model_destroy": [_P],
    "gca3d_model_push": [_P, _P, _P, C.POINTER(IcpResult), C.POINTER(C.c_int)],
    "gca3d_model_cloud": [_P, C.POINTER(_P)],
    "gca3d_tracker_create": [_P, C.POINTER(TrackerParams), C.POINTER(_P)],
    "gca3d_tracker_destroy": [_P],
    "gca3d_tracker_frame_buffers": [_P, C.POINTER(_P), C.POINTER(_P)],
    "gca3d_tracker_push": [_P, _P, _P, C.POINTER(IcpResult), _P],
    "gca3d_tracker_kernels": [_P, C.POINTER(_I64)],
    "gca3d_color_icp_vjp": [_P, _P, _P, C.POINTER(VjpParams), _P, _P, C.c_double, _P, C.POINTER(C.c_double), _P,
                            _P, _P, _P],
    "gca3d_selfcheck_fp64": [_P, C.c_int, _P],
    "gca3d_set_wait_limit": [_P, C.c_int],
    "gca3d_get_wait_limit": [_P, C.POINTER(C.c_int)],
    "gca3d_selfcheck_wait": [_P, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)],
}
_RESTYPES = {"gca3d_status_string": C.c_char_p, "gca3d_last_error": C.c_char_p,
             "gca3d_kernel_launches": C.c_int64, "gca3d_stream": C.c_void_p}

_lib = {}


def exported_symbols():
    """the entry points include/gca3d.h declares"""
    return sorted(_SIGS)


def load(path=LIB_PATH):
    """load libgca3d.so, or another build of it such as libgca3d_checked.so (raises if
    it was not built)"""
    if path in _lib:
        return _lib[path]
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    for name, args in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = _RESTYPES.get(name, C.c_int)
    _lib[path] = L
    return L


class GcaError(RuntimeError):
    def __init__(self, status, detail):
        super().__init__(f"gca3d status {status}: {detail}")
        self.status = status


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Context:
    """owns a gca3d_context; stream=None creates a private non-blocking stream;
    lib_path selects another build of the library (the checked build)"""

    def __init__(self, device=0, stream=None, lib_path=LIB_PATH):
        self.L = load(lib_path)
        h = C.c_void_p()
        st = self.L.gca3d_create(device, stream, C.byref(h))
        if st != OK:
            raise GcaError(st, self.L.gca3d_status_string(st).decode())
        self.h = h

    def check(self, st):
        if st != OK:
            raise GcaError(st, self.L.gca3d_last_error(self.h).decode())
        return st

    def close(self):
        if getattr(self, "h", None):
            self.L.gca3d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        return self.check(self.L.gca3d_synchronize(self.h))

    @property
    def stream(self):
        return self.L.gca3d_stream(self.h)

    def launches(self):
        return self.L.gca3d_kernel_launches(self.h)

    def profile_begin(self, kernel):
        self.check(self.L.gca3d_profile_begin(self.h, kernel.encode()))

    def profile_read(self):
        ms, n = C.c_double(), C.c_int64()
        self.check(self.L.gca3d_profile_read(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    # -- buffers ---------------------------------------------------------
    def alloc(self, nbytes):
        p = C.c_void_p()
        self.check(self.L.gca3d_device_alloc(self.h, int(nbytes), C.byref(p)))
        return DeviceBuffer(self, p, int(nbytes))

    def cloud(self, capacity):
        return Cloud(self, capacity)

    def cloud_from(self, xyz, rgb=None, capacity=None):
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        c = Cloud(self, max(len(xyz), capacity or 0, 1))
        c.upload(xyz, rgb)
        return c


class DeviceBuffer:
    def __init__(self, ctx, ptr, nbytes):
        self.ctx, self.ptr, self.nbytes = ctx, ptr, nbytes

    def __del__(self):
        try:
            if self.ptr and self.ctx.h:
                self.ctx.L.gca3d_device_free(self.ctx.h, self.ptr)
        except Exception:
            pass

    def read(self, dtype, count):
        out = np.empty(count, dtype)
        if count:
            self.ctx.check(self.ctx.L.gca3d_copy(self.ctx.h, _ptr(out), self.ptr, out.nbytes))
        return out

    def write(self, arr):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        self.ctx.check(self.ctx.L.gca3d_copy(self.ctx.h, self.ptr, _ptr(arr), arr.nbytes))


class Cloud:
    def __init__(self, ctx, capacity):
        self.ctx = ctx
        self.h = C.c_void_p()
        ctx.check(ctx.L.gca3d_cloud_create(ctx.h, int(capacity), C.byref(self.h)))
        self.capacity = int(capacity)

    def __del__(self):
        try:
            if self.h:
                self.ctx.L.gca3d_cloud_destroy(self.h)
        except Exception:
            pass

    def upload(self, xyz, rgb=None):
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        rgb = None if rgb is None else np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
        self.ctx.check(self.ctx.L.gca3d_cloud_upload(self.ctx.h, self.h, _ptr(xyz), _ptr(rgb), len(xyz)))
        return self

    def set_normals(self, nrm):
        nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
        self.ctx.check(self.ctx.L.gca3d_cloud_set_normals(self.ctx.h, self.h, _ptr(nrm), len(nrm)))

    def set_gradients(self, grd):
        grd = np.ascontiguousarray(grd, np.float32).reshape(-1, 3)
        self.ctx.check(self.ctx.L.gca3d_cloud_set_gradients(self.ctx.h, self.h, _ptr(grd), len(grd)))

    def __len__(self):
        n = C.c_int64()
        self.ctx.check(self.ctx.L.gca3d_cloud_size(self.ctx.h, self.h, C.byref(n)))
        return n.value

    def download(self, xyz=True, rgb=True, normals=False, grad=False):
        n = len(self)
        out = {k: np.empty((n, 3), np.float32) for k, w in (("xyz", xyz), ("rgb", rgb), ("normals", normals),
                                                            ("grad", grad)) if w}
        cnt = C.c_int64()
        self.ctx.check(self.ctx.L.gca3d_cloud_download(
            self.ctx.h, self.h, _ptr(out.get("xyz")), _ptr(out.get("rgb")), _ptr(out.get("normals")),
            _ptr(out.get("grad")), n, C.byref(cnt)))
        return out

    def device_views(self):
        v = [C.c_void_p() for _ in range(5)]
        self.ctx.check(self.ctx.L.gca3d_cloud_device_views(self.h, *[C.byref(x) for x in v]))
        return [x.value for x in v]


def scale(voxel, max_iter, max_corr, normal_radius, grad_radius, max_nn=0):
    return ScaleParams(voxel, max_iter, max_corr, normal_radius, grad_radius, max_nn)


def icp_params(scales, lam=0.968, update_map=UPDATE_EULER_ZYX, rot_eps=1e-6, trans_eps=1e-6, compensated=True,
               use_graph=False, keep_target_normals=False, tuning=None):
    p = IcpParams()
    p.n_scales = len(scales)
    for i, s in enumerate(scales):
        p.scales[i] = s if isinstance(s, ScaleParams) else ScaleParams(*s)
    p.lambda_ = lam
    p.update_map = update_map
    p.rot_eps = rot_eps
    p.trans_eps = trans_eps
    p.compensated = int(compensated)
    p.use_graph = int(use_graph)
    p.keep_target_normals = int(keep_target_normals)
    if tuning is not None:
        p.tuning = tuning if isinstance(tuning, Tuning) else Tuning(*tuning)
    return p


def icp_autotune(ctx, srcs, tgts, params, reps=3):
    """the fastest launch shape for this workload: (Tuning, ms per execute)"""
    best, ms = Tuning(), C.c_double()
    ctx.check(ctx.L.gca3d_icp_autotune(ctx.h, len(srcs), cloud_array(srcs), cloud_array(tgts), C.byref(params),
                                       int(reps), C.byref(best), C.byref(ms)))
    return best, ms.value


def result_dict(r):
    return dict(T=np.array(r.T[:]).reshape(4, 4), rmse_ref=r.rmse_ref, fitness=r.fitness,
                inlier_rmse=r.inlier_rmse, iterations=r.iterations, converged=bool(r.converged),
                status=r.status, n_src=r.n_src, n_tgt=r.n_tgt, scale_iterations=list(r.scale_iterations),
                scale_n_src=list(r.scale_n_src), scale_n_tgt=list(r.scale_n_tgt))


def cloud_array(clouds):
    arr = (C.c_void_p * len(clouds))(*[c.h.value for c in clouds])
    return arr


def upload_many(ctx, clouds, xyz_ptrs, rgb_ptrs, counts):
    """gca3d_cloud_upload_many: raw buffer addresses (pinned host or device memory is
    read in place), one call for all clouds"""
    k = len(clouds)
    xa = (C.c_void_p * k)(*[int(p) for p in xyz_ptrs])
    ra = (C.c_void_p * k)(*[int(p) if p else None for p in rgb_ptrs])
    na = (C.c_int64 * k)(*[int(v) for v in counts])
    ctx.check(ctx.L.gca3d_cloud_upload_many(ctx.h, k, cloud_array(clouds), xa, ra, na))


class IcpPlan:
    """a reusable (optionally graph-captured) schedule over fixed clouds"""

    def __init__(self, ctx, src, tgt, params):
        self.ctx = ctx
        self.src, self.tgt = list(src), list(tgt)
        self.h = C.c_void_p()
        self._sa, self._ta = cloud_array(self.src), cloud_array(self.tgt)
        ctx.check(ctx.L.gca3d_icp_plan_create(ctx.h, len(self.src), self._sa, self._ta, C.byref(params),
                                              C.byref(self.h)))
        self.P = len(self.src)
        self._res = (IcpResult * self.P)()

    def execute(self, T_init=None, results=True):
        Ti = None
        if T_init is not None:
            Ti = np.ascontiguousarray(np.asarray(T_init, np.float64).reshape(self.P, 16))
        self.ctx.check(self.ctx.L.gca3d_icp_plan_execute(self.h, _ptr(Ti), self._res if results else None))
        return [result_dict(r) for r in self._res] if results else None

    def results(self):
        """the results of the last execute (waits for it)"""
        self.ctx.check(self.ctx.L.gca3d_icp_plan_results(self.h, self._res))
        return [result_dict(r) for r in self._res]

    def kernels(self):
        n = C.c_int64()
        self.ctx.check(self.ctx.L.gca3d_icp_plan_kernels(self.h, C.byref(n)))
        return n.value

    def readback_bytes(self):
        """bytes an execute copies back to the host"""
        n = C.c_int64()
        self.ctx.check(self.ctx.L.gca3d_icp_plan_readback_bytes(self.h, C.byref(n)))
        return n.value

    def __del__(self):
        try:
            if self.h:
                self.ctx.L.gca3d_icp_plan_destroy(self.h)
        except Exception:
            pass


def color_icp(ctx, src, tgt, params, T_init=None):
    r = IcpResult()
    Ti = None if T_init is None else np.ascontiguousarray(np.asarray(T_init, np.float64).reshape(16))
    ctx.check(ctx.L.gca3d_color_icp(ctx.h, src.h, tgt.h, C.byref(params), _ptr(Ti), C.byref(r)))
    return result_dict(r)


def color_icp_batched(ctx, srcs, tgts, params, T_init=None):
    P = len(srcs)
    res = (IcpResult * P)()
    Ti = None if T_init is None else np.ascontiguousarray(np.asarray(T_init, np.float64).reshape(P, 16))
    ctx.check(ctx.L.gca3d_color_icp_batched(ctx.h, P, cloud_array(srcs), cloud_array(tgts), C.byref(params),
                                            _ptr(Ti), res))
    return [result_dict(r) for r in res]


def selfcheck_fp64(ctx, n=1 << 20):
    """largest errors of the pose update's short FP64 routines on this device: Newton
    reciprocal and small-angle sine / cosine in ulps against IEEE division and sincos,
    and the exponential-map series' relative difference from the closed forms in units of
    the closed forms' rounding bound"""
    out = np.zeros(4, np.float64)
    ctx.check(ctx.L.gca3d_selfcheck_fp64(ctx.h, int(n), out.ctypes.data_as(C.c_void_p)))
    return {"rcp_ulp": float(out[0]), "sin_ulp": float(out[1]), "cos_ulp": float(out[2]),
            "exp_coeff_vs_bound": float(out[3])}


def selfcheck_wait(ctx, tiles=8, polls=1000):
    """run a look-back whose predecessor never publishes: (status the scan reported,
    its duration in ms)"""
    st, ms = C.c_int(), C.c_double()
    ctx.check(ctx.L.gca3d_selfcheck_wait(ctx.h, int(tiles), int(polls), C.byref(st), C.byref(ms)))
    return st.value, ms.value


def wait_limit(ctx, polls=None):
    """the context's wait limit in polls; sets it first when polls is given"""
    if polls is not None:
        ctx.check(ctx.L.gca3d_set_wait_limit(ctx.h, int(polls)))
    v = C.c_int()
    ctx.check(ctx.L.gca3d_get_wait_limit(ctx.h, C.byref(v)))
    return v.value


def color_icp_vjp(ctx, src, tgt, xi0, K=5, max_corr=0.05, lam=0.968, update_map=UPDATE_SE3_EXP, dT=None, dE=0.0,
                  n_src=None, want_corr=False, out=None):
    """K unrolled Gauss-Newton steps from Exp(xi0) and, when dT is given, the gradient of
    <dT, T_K> + dE * E.  Returns a dict with T (4x4), E and, with dT, dxi0 (6),
    dxyz / drgb (n_src x 3, host arrays unless `out` supplies device buffers
    {"dxyz", "drgb"}), plus corr ((K + 1) x n_src) when want_corr."""
    p = VjpParams(int(K), float(max_corr), float(lam), int(update_map))
    n = len(src) if n_src is None else int(n_src)
    x0 = np.ascontiguousarray(np.asarray(xi0, np.float64).reshape(6))
    T = np.zeros(16, np.float64)
    E = C.c_double()
    res = {}
    dxi = np.zeros(6, np.float64)
    gT = None if dT is None else np.ascontiguousarray(np.asarray(dT, np.float64).reshape(16))
    own = out is None and dT is not None
    bx = by = None
    if dT is not None:
        bx = ctx.alloc(12 * max(n, 1)) if own else out["dxyz"]
        by = ctx.alloc(12 * max(n, 1)) if own else out["drgb"]
    bc = ctx.alloc(4 * (K + 1) * max(n, 1)) if want_corr else None
    st = ctx.L.gca3d_color_icp_vjp(ctx.h, src.h, tgt.h, C.byref(p), _ptr(x0), _ptr(gT), float(dE), _ptr(T),
                                   C.byref(E), _ptr(dxi) if dT is not None else None, bx.ptr if bx else None,
                                   by.ptr if by else None, bc.ptr if bc else None)
    res["status"] = st
    if st not in (OK, ERR_SINGULAR):
        ctx.check(st)
    res["T"] = T.reshape(4, 4)
    res["E"] = E.value
    if dT is not None:
        res["dxi0"] = dxi
        if own:
            res["dxyz"] = bx.read(np.float32, 3 * n).reshape(n, 3)
            res["drgb"] = by.read(np.float32, 3 * n).reshape(n, 3)
    if want_corr:
        res["corr"] = bc.read(np.int32, (K + 1) * n).reshape(K + 1, n)
    return res


def tracker_params(cam, scales, depth_scale=0.001, tmin=0.2, tmax=10.0, filter=(FILTER_FIXED, 2, 3.0, 30.0),
                   constant_velocity=True, **icp_kw):
    """cam: width, height, fx, fy, cx, cy (identity depth -> colour extrinsic, equal
    intrinsics); filter: (mode, radius, sigma_space px, sigma_depth in depth units)"""
    p = TrackerParams()
    p.width, p.height = cam.width, cam.height
    p.depth_intrin = Intrinsics(cam.fx, cam.fy, cam.cx, cam.cy)
    p.color_intrin = Intrinsics(cam.fx, cam.fy, cam.cx, cam.cy)
    p.depth_to_color = Extrinsics((C.c_float * 9)(1, 0, 0, 0, 1, 0, 0, 0, 1), (C.c_float * 3)(0, 0, 0))
    p.depth_scale, p.tmin, p.tmax = depth_scale, tmin, tmax
    p.filter = Filter(*filter)
    p.icp = icp_params(scales, **icp_kw)
    p.constant_velocity = int(constant_velocity)
    return p


class Tracker:
    """frame-to-frame colored-ICP tracking of an RGB-D stream"""

    def __init__(self, ctx, params):
        self.ctx = ctx
        self.h = C.c_void_p()
        ctx.check(ctx.L.gca3d_tracker_create(ctx.h, C.byref(params), C.byref(self.h)))
        self.shape = (params.height, params.width)
        self._res = IcpResult()
        self._pose = np.zeros(16, np.float64)

    def frame_buffers(self):
        """numpy views of the pinned staging (depth H x W uint16, BGR H x W x 3 uint8)"""
        d, c = C.c_void_p(), C.c_void_p()
        self.ctx.check(self.ctx.L.gca3d_tracker_frame_buffers(self.h, C.byref(d), C.byref(c)))
        H, W = self.shape
        depth = np.ctypeslib.as_array(C.cast(d, C.POINTER(C.c_uint16)), shape=(H, W))
        bgr = np.ctypeslib.as_array(C.cast(c, C.POINTER(C.c_uint8)), shape=(H, W, 3))
        return depth, bgr

    def push(self, depth=None, bgr=None):
        """returns (result dict, camera pose relative to the first frame)"""
        d = None if depth is None else np.ascontiguousarray(depth, np.uint16)
        c = None if bgr is None else np.ascontiguousarray(bgr, np.uint8)
        self.ctx.check(self.ctx.L.gca3d_tracker_push(self.h, _ptr(d), _ptr(c), C.byref(self._res),
                                                     self._pose.ctypes.data))
        return result_dict(self._res), self._pose.reshape(4, 4).copy()

    def kernels(self):
        n = C.c_int64()
        self.ctx.check(self.ctx.L.gca3d_tracker_kernels(self.h, C.byref(n)))
        return n.value

    def __del__(self):
        try:
            if self.h:
                self.ctx.L.gca3d_tracker_destroy(self.h)
        except Exception:
            pass


def ply_read(path):
    """(xyz, rgb or None, normals or None) from a PLY file (host only)"""
    L = load()
    n, hn, hc = C.c_int64(), C.c_int(), C.c_int()
    st = L.gca3d_ply_info(str(path).encode(), C.byref(n), C.byref(hn), C.byref(hc))
    if st != OK:
        raise GcaError(st, f"ply_info {path}")
    xyz = np.empty((n.value, 3), np.float32)
    rgb = np.empty((n.value, 3), np.float32) if hc.value else None
    nrm = np.empty((n.value, 3), np.float32) if hn.value else None
    got = C.c_int64()
    st = L.gca3d_ply_read(str(path).encode(), _ptr(xyz), _ptr(rgb), _ptr(nrm), n.value, C.byref(got))
    if st != OK:
        raise GcaError(st, f"ply_read {path}")
    return xyz, rgb, nrm


def ply_write(path, xyz, rgb=None, nrm=None, binary=True):
    L = load()
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    rgb = None if rgb is None else np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
    nrm = None if nrm is None else np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    st = L.gca3d_ply_write(str(path).encode(), _ptr(xyz), _ptr(rgb), _ptr(nrm), len(xyz), int(binary))
    if st != OK:
        raise GcaError(st, f"ply_write {path}")


def model_params(cam, tmin=0.2, tmax=2.5, voxel=0.008, ror_radius=0.01, ror_min_neighbors=4, normal_radius=0.04,
                 max_iter=10, max_corr=0.05, grad_radius=0.05, revoxel_every=5, model_capacity=None,
                 filter=(FILTER_ADAPTIVE, 0, 0.0, 0.0), depth_scale=0.001):
    """the reference demo's reconstruction settings (apps/app.cpp:91, 121-128, 315-349)"""
    p = ModelParams()
    p.width, p.height = cam.width, cam.height
    p.depth_intrin = Intrinsics(cam.fx, cam.fy, cam.cx, cam.cy)
    p.color_intrin = Intrinsics(cam.fx, cam.fy, cam.cx, cam.cy)
    p.depth_to_color = Extrinsics((C.c_float * 9)(1, 0, 0, 0, 1, 0, 0, 0, 1), (C.c_float * 3)(0, 0, 0))
    p.depth_scale, p.tmin, p.tmax = depth_scale, tmin, tmax
    p.filter = Filter(*filter)
    p.voxel, p.ror_radius, p.ror_min_neighbors = voxel, ror_radius, ror_min_neighbors
    p.normal_radius, p.max_iter, p.max_corr, p.grad_radius = normal_radius, max_iter, max_corr, grad_radius
    p.revoxel_every = revoxel_every
    p.model_capacity = model_capacity or 16 * cam.width * cam.height
    return p


class CloudView(Cloud):
    """a cloud owned by another object (no destroy)"""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.h = handle
        c = C.c_int64()
        ctx.check(ctx.L.gca3d_cloud_capacity(handle, C.byref(c)))
        self.capacity = c.value

    def __del__(self):
        pass


class Model:
    """the frame-to-model accumulation loop of the reference demo"""

    def __init__(self, ctx, params):
        self.ctx = ctx
        self.h = C.c_void_p()
        ctx.check(ctx.L.gca3d_model_create(ctx.h, C.byref(params), C.byref(self.h)))
        self._res = IcpResult()

    def push(self, depth, bgr):
        """returns (registration result dict, appended)"""
        d = np.ascontiguousarray(depth, np.uint16)
        c = np.ascontiguousarray(bgr, np.uint8)
        app = C.c_int()
        self.ctx.check(self.ctx.L.gca3d_model_push(self.h, _ptr(d), _ptr(c), C.byref(self._res), C.byref(app)))
        return result_dict(self._res), bool(app.value)

    def cloud(self):
        h = C.c_void_p()
        self.ctx.check(self.ctx.L.gca3d_model_cloud(self.h, C.byref(h)))
        return CloudView(self.ctx, h)

    def __del__(self):
        try:
            if self.h:
                self.ctx.L.gca3d_model_destroy(self.h)
        except Exception:
            pass
