"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


class Golden(dict):
    """golden.npz plus the inputs the generator derived from the stored cloud"""

    def voxel_input(self, tag):
        xyz, rgb = self["cloud_xyz"], self["cloud_rgb"]
        if tag == "neg05":
            return _f32(xyz - np.array([10.0, 0.0, 0.0], np.float32)), rgb
        if tag == "dup":
            return _f32(np.repeat(xyz[:500], 3, 0)), _f32(np.repeat(rgb[:500], 3, 0))
        if tag == "one":
            return xyz[:1], rgb[:1]
        return xyz, rgb

    @property
    def nn_r(self):
        return self["cloud_xyz"][4000:]

    @property
    def patch_xyz(self):
        return self["cloud_xyz"][:8000]

    @property
    def patch_rgb(self):
        return self["cloud_rgb"][:8000]

    @property
    def gn_src_rgb(self):
        return self["cloud_rgb"][8000:12000]

    # --- the RGB-D frame fixture (the reference's cuda_point_cloud_factory.cu helpers) ---
    FRAME_CASES = ("raw", "adaptive", "fixed", "adaptive_extrinsic", "adaptive_tmin0")
    FRAME_FIXED = (2, 3.0, 30.0)  # radius, sigma_space (px), sigma_depth (depth units)

    def frame_case(self, name):
        """(depth intrinsics, colour intrinsics, rotation (9, column-major), translation,
        filter mode, tmin) of a frame case"""
        a = self[f"frame_{name}_args"]
        return (tuple(map(float, a[0:4])), tuple(map(float, a[4:8])), a[8:17].copy(), a[17:20].copy(), int(a[20]),
                float(a[21]))

    def check_frame(self, name, xyz, rgb, depth=None):
        """Against the frame helpers built with the Cody-Waite exp of the frame kernel:
        bit for bit.  Against the helpers with the host's expf: the filtered depth and
        the points within 8 ulp (the two exps differ by up to about 2 ulp per weight),
        the same points in the same raster order, and the same colours except where the
        colour-image coordinate + 0.5 lies within 1e-4 of an integer, where an ulp of
        depth moves the colour lookup to the next pixel (at most 3 % of the points)."""
        k = f"frame_{name}"
        np.testing.assert_array_equal(xyz, self[k + "_detexp_xyz"])
        np.testing.assert_array_equal(rgb, self[k + "_detexp_rgb"])
        if depth is not None:
            np.testing.assert_array_equal(depth, self[k + "_detexp_depth"])
        if k + "_stock_xyz" not in self:
            return
        sx, sc, scuv = self[k + "_stock_xyz"], self[k + "_stock_rgb"], self[k + "_stock_cuv"]
        assert len(xyz) == len(sx)

        def ulp(a, b):
            nan = np.isnan(a) | np.isnan(b)
            assert (np.isnan(a) == np.isnan(b)).all()
            d = np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))
            return np.where(nan, 0, d).max() if d.size else 0

        assert ulp(xyz, sx) <= 8
        if depth is not None:
            assert ulp(depth, self[k + "_stock_depth"]) <= 8
        differ = (rgb != sc).any(1)
        finite = np.isfinite(scuv).all(1)
        edge = np.zeros(len(scuv), bool)
        edge[finite] = (np.abs(scuv[finite] - np.round(scuv[finite])) < 1e-4).any(1)
        assert not (differ & ~edge).any()
        assert differ.sum() <= 0.03 * len(rgb)


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as g:
        return Golden({k: g[k] for k in g.files})


@pytest.fixture(scope="session")
def orc():
    import oracle as O

    O.set_threads(1)
    return O
