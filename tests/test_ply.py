"""PLY point files (host side of the library; no GPU needed).

Round trips in both encodings are exact for float coordinates and normals and for
colours that are multiples of 1/255 (the 8-bit scaling of point_cloud::create_from_pcl,
src/geometry/point_cloud.cu:481-504).  When the reference tree is present, its real
fragment file (data/frag_115.ply: 64,365 points with normals and 8-bit colours) is
read as a real-data check."""
import os

import numpy as np
import pytest

# the reference tree's data/ sits beside its src/ (GCA_REF_SRC)
FRAG = os.path.join(os.path.dirname(os.environ.get("GCA_REF_SRC", "/root/reference/src").rstrip("/")), "data",
                    "frag_115.ply")


@pytest.fixture(scope="module")
def N():
    from cuda_3d_gb300 import build, native

    build.build()
    return native


def _cloud(n=5000, seed=0):
    rng = np.random.default_rng(seed)
    xyz = rng.normal(size=(n, 3)).astype(np.float32) * np.float32(3.0)
    rgb = (rng.integers(0, 256, size=(n, 3)).astype(np.float32) * (np.float32(1.0) / np.float32(255.0)))
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    return xyz, rgb.astype(np.float32), nrm


@pytest.mark.parametrize("binary", [True, False])
def test_ply_round_trip(N, tmp_path, binary):
    xyz, rgb, nrm = _cloud()
    path = tmp_path / "c.ply"
    N.ply_write(path, xyz, rgb, nrm, binary=binary)
    x2, c2, n2 = N.ply_read(path)
    np.testing.assert_array_equal(x2, xyz)
    np.testing.assert_array_equal(c2, rgb)
    np.testing.assert_array_equal(n2, nrm)


def test_ply_optional_attributes_and_errors(N, tmp_path):
    xyz, _, _ = _cloud(100)
    path = tmp_path / "xyz.ply"
    N.ply_write(path, xyz)
    x2, c2, n2 = N.ply_read(path)
    np.testing.assert_array_equal(x2, xyz)
    assert c2 is None and n2 is None
    # a vertex element after another element, float colours, extra properties (ascii)
    p2 = tmp_path / "mixed.ply"
    p2.write_text("ply\nformat ascii 1.0\ncomment made by a test\nelement camera 1\nproperty float f\n"
                  "element vertex 2\nproperty double x\nproperty double y\nproperty double z\n"
                  "property float red\nproperty float green\nproperty float blue\nproperty int label\n"
                  "end_header\n7.5\n1 2 3 0.25 0.5 0.75 9\n-1 -2 -3 1 0 0 8\n")
    x3, c3, n3 = N.ply_read(p2)
    np.testing.assert_array_equal(x3, np.array([[1, 2, 3], [-1, -2, -3]], np.float32))
    np.testing.assert_array_equal(c3, np.array([[0.25, 0.5, 0.75], [1, 0, 0]], np.float32))
    # big-endian and list properties in the vertex element are refused
    p3 = tmp_path / "be.ply"
    p3.write_bytes(b"ply\nformat binary_big_endian 1.0\nelement vertex 1\nproperty float x\nproperty float y\n"
                   b"property float z\nend_header\n" + b"\0" * 12)
    with pytest.raises(N.GcaError):
        N.ply_read(p3)
    p4 = tmp_path / "notply.ply"
    p4.write_text("hello\n")
    with pytest.raises(N.GcaError):
        N.ply_read(p4)


@pytest.mark.skipif(not os.path.exists(FRAG), reason="the reference tree is not present")
def test_reads_the_reference_fragment(N):
    xyz, rgb, nrm = N.ply_read(FRAG)
    assert len(xyz) == 64365
    assert rgb is not None and nrm is not None
    assert np.isfinite(xyz).all()
    assert rgb.min() >= 0 and rgb.max() <= 1
    # 8-bit colours: every value is a multiple of 1/255
    k = rgb * 255
    assert np.abs(k - np.round(k)).max() < 1e-4
    np.testing.assert_allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-3)
