"""Seeded synthetic inputs for the RGB-D registration path.

The reference measures on a RealSense stream and on a pair of fragment files that
are not available, so every workload here is generated:

* ``room_scene`` / ``sample_room`` -- a 4 x 5 x 2.7 m room with 8 boxes and 4
  cylinders, sampled uniformly by area, coloured by a 3-octave value-noise texture
  (fragment-scale clouds, the precision and batching workloads).
* ``render_rgbd`` -- a procedural room (floor, 3 walls, 5 boxes, 3 spheres) ray-cast
  to a 640 x 480 uint16 depth image in millimetres and a BGR8 colour image with a
  per-surface sinusoidal colour field (the frame-pair and streaming workloads).

Everything is plain arithmetic with numpy; no graphics API is involved.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# --------------------------------------------------------------------------- #
# rigid transforms
# --------------------------------------------------------------------------- #


def axis_angle(axis, angle):
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * (K @ K)


def random_rotation(rng, angle_deg):
    axis = rng.normal(size=3)
    return axis_angle(axis, math.radians(angle_deg))


def make_T(R, t):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def transform(T, xyz):
    return (np.asarray(xyz, np.float64) @ T[:3, :3].T + T[:3, 3]).astype(np.float32)


def pose_error(Ta, Tb):
    """rotation error (rad) and translation error (m) between two 4x4 poses"""
    R = Ta[:3, :3] @ Tb[:3, :3].T
    c = max(-1.0, min(1.0, (np.trace(R) - 1.0) / 2.0))
    return math.acos(c), float(np.linalg.norm(Ta[:3, 3] - Tb[:3, 3]))


# --------------------------------------------------------------------------- #
# value-noise colour texture
# --------------------------------------------------------------------------- #


class ValueNoise:
    """3-octave lattice value noise with smoothstep trilinear interpolation."""

    def __init__(self, seed, base_freq=1.5, octaves=3):
        rng = np.random.default_rng(seed)
        self.perm = rng.permutation(256).astype(np.int64)
        self.vals = rng.random(256)
        self.base = base_freq
        self.octaves = octaves

    def _lattice(self, ix, iy, iz):
        p = self.perm
        return self.vals[p[(p[(p[ix & 255] + iy) & 255] + iz) & 255]]

    def _octave(self, x):
        f = np.floor(x)
        i = f.astype(np.int64)
        t = x - f
        s = t * t * (3 - 2 * t)
        out = 0.0
        for dx in (0, 1):
            wx = s[:, 0] if dx else 1 - s[:, 0]
            for dy in (0, 1):
                wy = s[:, 1] if dy else 1 - s[:, 1]
                for dz in (0, 1):
                    wz = s[:, 2] if dz else 1 - s[:, 2]
                    out = out + wx * wy * wz * self._lattice(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz)
        return out

    def __call__(self, xyz):
        xyz = np.asarray(xyz, np.float64) + 17.0
        total, amp, norm, freq = 0.0, 1.0, 0.0, self.base
        for _ in range(self.octaves):
            total = total + amp * self._octave(xyz * freq)
            norm += amp
            amp *= 0.5
            freq *= 2.0
        return total / norm


# --------------------------------------------------------------------------- #
# fragment-scale room clouds
# --------------------------------------------------------------------------- #

ROOM = (4.0, 5.0, 2.7)


@dataclass
class RoomScene:
    boxes: list = field(default_factory=list)      # (min xyz, max xyz)
    cylinders: list = field(default_factory=list)  # (cx, cy, r, h)
    noise: tuple = ()


def room_scene(seed=1234):
    rng = np.random.default_rng(seed)
    W, D, H = ROOM
    boxes = []
    for _ in range(8):
        sx, sy, sz = rng.uniform(0.3, 1.0), rng.uniform(0.3, 1.0), rng.uniform(0.3, 1.4)
        x0, y0 = rng.uniform(0.1, W - sx - 0.1), rng.uniform(0.1, D - sy - 0.1)
        boxes.append((np.array([x0, y0, 0.0]), np.array([x0 + sx, y0 + sy, sz])))
    cyls = []
    for _ in range(4):
        r, h = rng.uniform(0.1, 0.3), rng.uniform(0.5, 2.5)
        cyls.append((rng.uniform(r + 0.1, W - r - 0.1), rng.uniform(r + 0.1, D - r - 0.1), r, h))
    return RoomScene(boxes, cyls, (seed * 3 + 1, seed * 3 + 2, seed * 3 + 3))


def _surfaces(scene):
    """list of (area, sampler(rng, k) -> k x 3 points)"""
    W, D, H = ROOM
    surf = []

    def rect(o, u, v):
        o, u, v = (np.asarray(a, np.float64) for a in (o, u, v))
        area = float(np.linalg.norm(np.cross(u, v)))
        return area, lambda rng, k: o + rng.random((k, 1)) * u + rng.random((k, 1)) * v

    surf += [rect((0, 0, 0), (W, 0, 0), (0, D, 0)), rect((0, 0, H), (W, 0, 0), (0, D, 0)),
             rect((0, 0, 0), (W, 0, 0), (0, 0, H)), rect((0, D, 0), (W, 0, 0), (0, 0, H)),
             rect((0, 0, 0), (0, D, 0), (0, 0, H)), rect((W, 0, 0), (0, D, 0), (0, 0, H))]
    for lo, hi in scene.boxes:
        s = hi - lo
        surf += [rect((lo[0], lo[1], hi[2]), (s[0], 0, 0), (0, s[1], 0)),
                 rect(lo, (s[0], 0, 0), (0, 0, s[2])), rect((lo[0], hi[1], lo[2]), (s[0], 0, 0), (0, 0, s[2])),
                 rect(lo, (0, s[1], 0), (0, 0, s[2])), rect((hi[0], lo[1], lo[2]), (0, s[1], 0), (0, 0, s[2]))]
    for cx, cy, r, h in scene.cylinders:
        def side(rng, k, cx=cx, cy=cy, r=r, h=h):
            a = rng.random(k) * 2 * math.pi
            return np.stack([cx + r * np.cos(a), cy + r * np.sin(a), rng.random(k) * h], 1)

        def top(rng, k, cx=cx, cy=cy, r=r, h=h):
            a = rng.random(k) * 2 * math.pi
            rr = r * np.sqrt(rng.random(k))
            return np.stack([cx + rr * np.cos(a), cy + rr * np.sin(a), np.full(k, h)], 1)

        surf += [(2 * math.pi * r * h, side), (math.pi * r * r, top)]
    return surf


def room_colors(scene, xyz):
    return np.stack([ValueNoise(s)(xyz) for s in scene.noise], 1).astype(np.float32)


def sample_room(scene, n, rng, noise_sigma=0.003):
    """n points uniformly by area, with N(0, noise_sigma) position noise"""
    surf = _surfaces(scene)
    areas = np.array([a for a, _ in surf])
    counts = rng.multinomial(n, areas / areas.sum())
    pts = np.concatenate([f(rng, int(k)) for (_, f), k in zip(surf, counts) if k > 0], 0)
    pts = pts[rng.permutation(len(pts))]
    col = room_colors(scene, pts)
    pts = pts + rng.normal(scale=noise_sigma, size=pts.shape)
    return pts.astype(np.float32), col


def _crop(pts, col, direction, lo, hi):
    c = np.array([ROOM[0] / 2, ROOM[1] / 2, 0.0])
    s = (pts[:, :2] - c[:2]) @ direction
    keep = (s >= lo) & (s <= hi)
    return pts[keep], col[keep]


@dataclass
class Pair:
    src_xyz: np.ndarray
    src_rgb: np.ndarray
    tgt_xyz: np.ndarray
    tgt_rgb: np.ndarray
    T_gt: np.ndarray   # maps source coordinates onto target coordinates


def room_pair(seed, n_points=250_000, overlap=0.6, rot_deg=10.0, trans=0.10, scene_seed=1234):
    """Two independently sampled, cropped views of the room.  The source is
    expressed in a frame displaced by T_gt^-1 (rotation about the room centre), so
    registration has to recover T_gt."""
    rng = np.random.default_rng(seed)
    scene = room_scene(scene_seed)
    # crop extents along a random horizontal direction so that the shared part is
    # `overlap` of each view
    ang = rng.uniform(0, 2 * math.pi)
    d = np.array([math.cos(ang), math.sin(ang)])
    half = 0.5 * (abs(d[0]) * ROOM[0] + abs(d[1]) * ROOM[1])
    L = 2 * half
    s = L / (2 - overlap)           # view length so that shared/view = overlap
    n_view = int(n_points)
    # oversample so that each view keeps about n_points after cropping
    frac = s / L
    tgt, tcol = sample_room(scene, int(n_view / frac) + 1, rng)
    src, scol = sample_room(scene, int(n_view / frac) + 1, rng)
    tgt, tcol = _crop(tgt, tcol, d, half - s, half)
    src, scol = _crop(src, scol, d, -half, -half + s)
    tgt, tcol = tgt[:n_view], tcol[:n_view]
    src, scol = src[:n_view], scol[:n_view]
    R = random_rotation(rng, rot_deg)
    tdir = rng.normal(size=3)
    t = tdir / np.linalg.norm(tdir) * trans
    c = np.array([ROOM[0] / 2, ROOM[1] / 2, ROOM[2] / 2])
    T_gt = make_T(R, c + t - R @ c)
    src = transform(np.linalg.inv(T_gt), src)
    return Pair(src, scol, tgt.astype(np.float32), tcol, T_gt)


class RoomSampler:
    """a large clean area-uniform sample of the room (with colours) that many pairs
    draw from; each draw adds fresh position noise"""

    def __init__(self, scene_seed=1234, n_master=2_000_000, seed=99):
        rng = np.random.default_rng(seed)
        self.scene = room_scene(scene_seed)
        self.xyz, self.rgb = sample_room(self.scene, n_master, rng, noise_sigma=0.0)

    def draw(self, rng, n, noise_sigma=0.003):
        idx = rng.integers(0, len(self.xyz), n)
        return (self.xyz[idx] + rng.normal(scale=noise_sigma, size=(n, 3))).astype(np.float32), self.rgb[idx]


def room_pair_from(sampler, seed, n_points, overlap=0.6, rot_deg=10.0, trans=0.10):
    """room_pair with both views drawn from a shared RoomSampler"""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, 2 * math.pi)
    d = np.array([math.cos(ang), math.sin(ang)])
    half = 0.5 * (abs(d[0]) * ROOM[0] + abs(d[1]) * ROOM[1])
    s = 2 * half / (2 - overlap)
    m = int(n_points * 2 * half / s) + 1
    tgt, tcol = _crop(*sampler.draw(rng, m), d, half - s, half)
    src, scol = _crop(*sampler.draw(rng, m), d, -half, -half + s)
    tgt, tcol, src, scol = tgt[:n_points], tcol[:n_points], src[:n_points], scol[:n_points]
    R = random_rotation(rng, rot_deg)
    tdir = rng.normal(size=3)
    t = tdir / np.linalg.norm(tdir) * trans
    c = np.array([ROOM[0] / 2, ROOM[1] / 2, ROOM[2] / 2])
    T_gt = make_T(R, c + t - R @ c)
    return Pair(transform(np.linalg.inv(T_gt), src), scol, tgt.astype(np.float32), tcol, T_gt)


def batch_pairs(n_pairs=64, seed=0, n_min=20_000, n_max=300_000, max_rot=15.0, max_trans=0.15, sampler=None):
    """the multi-pair workload: sizes log-uniform in [n_min, n_max] per cloud, a
    random transform per pair (rotation uniform in [0, max_rot] deg about a random
    axis, translation uniform in [0, max_trans] m) and overlap uniform in [0.4, 0.9]"""
    sampler = sampler or RoomSampler()
    out = []
    for k in range(n_pairs):
        rng = np.random.default_rng(10_000 + seed * 1000 + k)
        n = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
        out.append(room_pair_from(sampler, 7 * k + 1 + seed * 100_003, n, overlap=rng.uniform(0.4, 0.9),
                                  rot_deg=rng.uniform(0, max_rot), trans=rng.uniform(0, max_trans)))
    return out


# --------------------------------------------------------------------------- #
# RGB-D frames
# --------------------------------------------------------------------------- #

DEFAULT_INTRIN = (525.0, 525.0, 319.5, 239.5)


@dataclass
class Camera:
    width: int = 640
    height: int = 480
    fx: float = 525.0
    fy: float = 525.0
    cx: float = 319.5
    cy: float = 239.5


def frame_scene(seed=1234):
    """camera-1 frame: x right, y down, z forward.  Floor at y = +1.2, back wall
    z = 4.0, side walls x = +-2.0, 5 boxes on the floor, 3 spheres."""
    rng = np.random.default_rng(seed)
    planes = [  # (normal, offset) with n . p = offset, surface id
        (np.array([0.0, 1.0, 0.0]), 1.2), (np.array([0.0, 0.0, 1.0]), 4.0),
        (np.array([1.0, 0.0, 0.0]), -2.0), (np.array([1.0, 0.0, 0.0]), 2.0)]
    boxes = []
    for _ in range(5):
        sx, sy, sz = rng.uniform(0.2, 0.7), rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.7)
        x0, z0 = rng.uniform(-1.6, 1.6 - sx), rng.uniform(1.4, 3.6 - sz)
        boxes.append((np.array([x0, 1.2 - sy, z0]), np.array([x0 + sx, 1.2, z0 + sz])))
    spheres = []
    for _ in range(3):
        r = rng.uniform(0.15, 0.35)
        spheres.append((np.array([rng.uniform(-1.4, 1.4), rng.uniform(-0.6, 1.2 - r), rng.uniform(1.5, 3.5)]), r))
    n_surf = len(planes) + len(boxes) + len(spheres)
    colp = rng.uniform(0, 2 * math.pi, size=(n_surf, 3))
    colk = rng.normal(size=(n_surf, 3, 3)) * 6.0
    return dict(planes=planes, boxes=boxes, spheres=spheres, colp=colp, colk=colk)


def _raycast(scene, o, d):
    """nearest hit distance t (inf if none) and surface id for rays o + t d"""
    n = d.shape[0]
    best = np.full(n, np.inf)
    sid = np.full(n, -1)
    k = 0
    for nrm, off in scene["planes"]:
        den = d @ nrm
        with np.errstate(divide="ignore", invalid="ignore"):
            t = (off - o @ nrm) / den
        ok = (t > 1e-6) & (t < best)
        best = np.where(ok, t, best)
        sid = np.where(ok, k, sid)
        k += 1
    for lo, hi in scene["boxes"]:
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1.0 / d
            t0 = (lo - o) * inv
            t1 = (hi - o) * inv
        tmin = np.nanmax(np.minimum(t0, t1), axis=1)
        tmax = np.nanmin(np.maximum(t0, t1), axis=1)
        ok = (tmax >= tmin) & (tmin > 1e-6) & (tmin < best)
        best = np.where(ok, tmin, best)
        sid = np.where(ok, k, sid)
        k += 1
    dd = (d * d).sum(1)
    for c, r in scene["spheres"]:
        oc = o - c
        b = (oc * d).sum(1)
        cc = (oc * oc).sum(1) - r * r
        disc = b * b - dd * cc
        with np.errstate(invalid="ignore"):
            t = (-b - np.sqrt(disc)) / dd
        ok = (disc >= 0) & (t > 1e-6) & (t < best)
        best = np.where(ok, t, best)
        sid = np.where(ok, k, sid)
        k += 1
    return best, sid


def render_rgbd(scene, T_cam, seed, cam=Camera(), zero_frac=0.05, color_noise=4.0, depth_noise=True):
    """depth (uint16 mm, H x W) and BGR8 (H x W x 3) seen from camera pose T_cam
    (camera -> scene frame).  Depth noise N(0, (0.002 z^2)^2) m."""
    rng = np.random.default_rng(seed)
    # pixel (x, y) looks along (x - 0.5, y - 0.5): the reference back-projects with
    # that half-pixel shift (cuda_point_cloud_factory.cu:232)
    u, v = np.meshgrid(np.arange(cam.width, dtype=np.float64) - 0.5, np.arange(cam.height, dtype=np.float64) - 0.5)
    dcam = np.stack([(u - cam.cx) / cam.fx, (v - cam.cy) / cam.fy, np.ones_like(u)], -1).reshape(-1, 3)
    R, t = T_cam[:3, :3], T_cam[:3, 3]
    dw = dcam @ R.T
    o = np.broadcast_to(t, dw.shape)
    tt, sid = _raycast(scene, o, dw)
    z = tt  # dcam has unit z, so the ray parameter is the camera-frame depth
    hit = o + dw * tt[:, None]
    if depth_noise:
        z = z + rng.normal(size=z.shape) * (0.002 * z * z)
    depth = np.where(np.isfinite(z) & (z > 0), np.round(z * 1000.0), 0)
    depth = np.clip(depth, 0, 65535).astype(np.uint16)
    zero = rng.random(depth.shape) < zero_frac
    depth[zero] = 0
    # per-surface sinusoidal colour field
    col = np.zeros((hit.shape[0], 3))
    ok = sid >= 0
    hp = np.where(ok[:, None], hit, 0.0)
    for ch in range(3):
        ph = scene["colp"][np.maximum(sid, 0), ch]
        kv = scene["colk"][np.maximum(sid, 0), ch]
        col[:, ch] = 128 + 90 * np.sin((hp * kv).sum(1) + ph)
    col = col + rng.normal(scale=color_noise, size=col.shape)
    col = np.clip(np.round(col), 0, 255).astype(np.uint8)
    bgr = col[:, ::-1].reshape(cam.height, cam.width, 3).copy()
    return depth.reshape(cam.height, cam.width), bgr


@dataclass
class FramePair:
    depth0: np.ndarray
    bgr0: np.ndarray
    depth1: np.ndarray
    bgr1: np.ndarray
    T_gt: np.ndarray   # camera-1 coordinates -> camera-0 coordinates
    cam: Camera


def frame_pair(seed=0, scene_seed=1234, rot_deg=2.0, trans=0.03, cam=Camera()):
    rng = np.random.default_rng(seed)
    scene = frame_scene(scene_seed)
    R = random_rotation(rng, rot_deg)
    tdir = rng.normal(size=3)
    T1 = make_T(R, tdir / np.linalg.norm(tdir) * trans)
    d0, c0 = render_rgbd(scene, np.eye(4), 1000 + 2 * seed, cam)
    d1, c1 = render_rgbd(scene, T1, 1001 + 2 * seed, cam)
    return FramePair(d0, c0, d1, c1, T1, cam)


def spline_poses(n_frames, seed=0, step_m=0.015, step_deg=1.0):
    """camera poses along a smooth path: a Catmull-Rom spline through random
    knots, moving about step_m and step_deg per frame"""
    rng = np.random.default_rng(seed)
    n_knots = max(4, n_frames // 25 + 4)
    knots_t = np.cumsum(rng.normal(size=(n_knots, 3)) * 0.6 * step_m * 25 / math.sqrt(3), 0)
    knots_t[:, 2] *= 0.3
    knots_r = np.cumsum(rng.normal(size=(n_knots, 3)) * math.radians(step_deg) * 25 / math.sqrt(3) * 0.6, 0)
    poses = []
    for f in range(n_frames):
        s = f / 25.0 + 1.0
        i = int(s)
        u = s - i

        def cr(P):
            p0, p1, p2, p3 = P[i - 1], P[i], P[i + 1], P[i + 2]
            return 0.5 * ((2 * p1) + (-p0 + p2) * u + (2 * p0 - 5 * p1 + 4 * p2 - p3) * u * u
                          + (-p0 + 3 * p1 - 3 * p2 + p3) * u ** 3)
        tr = cr(knots_t)
        rv = cr(knots_r)
        ang = float(np.linalg.norm(rv))
        R = axis_angle(rv, ang) if ang > 0 else np.eye(3)
        poses.append(make_T(R, tr))
    p0inv = np.linalg.inv(poses[0])
    return [p0inv @ p for p in poses]


# --------------------------------------------------------------------------- #
# the same frame renderer in torch, for long synthetic sequences on the GPU
# (data generation only: identical geometry and colour field; the noise comes from
# a torch generator seeded with the frame seed)
# --------------------------------------------------------------------------- #
def _raycast_torch(scene, o, d):
    import torch

    n = d.shape[0]
    best = torch.full((n,), math.inf, dtype=d.dtype, device=d.device)
    sid = torch.full((n,), -1, dtype=torch.int64, device=d.device)
    k = 0

    def take(t, ok, k, best, sid):
        return torch.where(ok, t, best), torch.where(ok, torch.full_like(sid, k), sid)

    for nrm, off in scene["planes"]:
        nv = torch.as_tensor(nrm, dtype=d.dtype, device=d.device)
        t = (off - o @ nv) / (d @ nv)
        best, sid = take(t, (t > 1e-6) & (t < best), k, best, sid)
        k += 1
    inv = 1.0 / d
    for lo, hi in scene["boxes"]:
        lo_t = torch.as_tensor(lo, dtype=d.dtype, device=d.device)
        hi_t = torch.as_tensor(hi, dtype=d.dtype, device=d.device)
        t0, t1 = (lo_t - o) * inv, (hi_t - o) * inv
        a, b = torch.minimum(t0, t1), torch.maximum(t0, t1)
        tmin = torch.where(torch.isnan(a), -math.inf, a).max(1).values
        tmax = torch.where(torch.isnan(b), math.inf, b).min(1).values
        best, sid = take(tmin, (tmax >= tmin) & (tmin > 1e-6) & (tmin < best), k, best, sid)
        k += 1
    dd = (d * d).sum(1)
    for c, r in scene["spheres"]:
        oc = o - torch.as_tensor(c, dtype=d.dtype, device=d.device)
        b = (oc * d).sum(1)
        cc = (oc * oc).sum(1) - r * r
        disc = b * b - dd * cc
        t = (-b - torch.sqrt(disc)) / dd
        best, sid = take(t, (disc >= 0) & (t > 1e-6) & (t < best), k, best, sid)
        k += 1
    return best, sid


def render_rgbd_torch(scene, T_cam, seed, cam=Camera(), device="cuda", zero_frac=0.05, color_noise=4.0,
                      depth_noise=True):
    """render_rgbd on a torch device; returns host numpy depth (H x W uint16) and
    BGR (H x W x 3 uint8)"""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    f64 = torch.float64
    u = torch.arange(cam.width, dtype=f64, device=device) - 0.5
    v = torch.arange(cam.height, dtype=f64, device=device) - 0.5
    vv, uu = torch.meshgrid(v, u, indexing="ij")
    dcam = torch.stack([(uu - cam.cx) / cam.fx, (vv - cam.cy) / cam.fy, torch.ones_like(uu)], -1).reshape(-1, 3)
    T = torch.as_tensor(np.asarray(T_cam), dtype=f64, device=device)
    dw = dcam @ T[:3, :3].T
    o = T[:3, 3].expand_as(dw)
    tt, sid = _raycast_torch(scene, o, dw)
    hit = o + dw * tt[:, None]
    z = tt + torch.randn(tt.shape, generator=g, dtype=f64, device=device) * (0.002 * tt * tt) * float(depth_noise)
    depth = torch.where(torch.isfinite(z) & (z > 0), torch.round(z * 1000.0), torch.zeros_like(z))
    depth = depth.clamp(0, 65535).to(torch.int32)
    zero = torch.rand(depth.shape, generator=g, dtype=f64, device=device) < zero_frac
    depth = torch.where(zero, torch.zeros_like(depth), depth)
    ok = sid >= 0
    hp = torch.where(ok[:, None], hit, torch.zeros_like(hit))
    s = sid.clamp(min=0)
    colp = torch.as_tensor(scene["colp"], dtype=f64, device=device)[s]
    colk = torch.as_tensor(scene["colk"], dtype=f64, device=device)[s]
    col = 128 + 90 * torch.sin((hp[:, None, :] * colk).sum(-1) + colp)
    col = col + torch.randn(col.shape, generator=g, dtype=f64, device=device) * color_noise
    col = torch.round(col).clamp(0, 255).to(torch.uint8)
    bgr = col.flip(1).reshape(cam.height, cam.width, 3)
    return (depth.reshape(cam.height, cam.width).to(torch.int32).cpu().numpy().astype(np.uint16),
            bgr.cpu().numpy())
