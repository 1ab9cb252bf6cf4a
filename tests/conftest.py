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


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as g:
        return Golden({k: g[k] for k in g.files})


@pytest.fixture(scope="session")
def orc():
    import oracle as O

    O.set_threads(1)
    return O
