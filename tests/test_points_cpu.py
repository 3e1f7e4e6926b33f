"""Point clouds on the CPU: the oracle's restatement of cudaPointCloud
(cuda_point_cloud.cu) on known answers and edge cases, and the argument
checks of the gbt_points_* entry points (no device work)."""
import ctypes as C

import numpy as np
import pytest

# column-major 3x3 (the reference's Eigen-backed callers): cx at [6], cy at [7]
K_COL = np.array([100.0, 0, 0, 0, 100.0, 0, 31.5, 23.5, 1.0])
# row-major (point_cloud_dataset.cpp:30): cx at [2], cy at [5]
K_ROW = np.array([100.0, 0, 31.5, 0, 100.0, 23.5, 0, 0, 1.0])
IDENTITY = np.array([1.0, 0, 0, 0, 0, 0, 0])


def test_extract_known_answers(oracle):
    d = np.zeros((48, 64), np.float32)
    d[23, 31] = 2.0       # half a pixel left of cx and above cy
    d[10, 5] = 1.5
    d[0, 1] = -1.0        # negative depth: slot untouched
    d[0, 2] = np.nan      # NaN passes "depth <= 0" and is written
    rgb = np.zeros((48, 64, 3), np.uint8)
    rgb[10, 5] = (1, 2, 3)
    pts = np.full((64 * 48, 33), 7, np.uint8)
    oracle.points_extract(K_COL, d, rgb, IDENTITY, pts)
    v = pts.reshape(-1).view(oracle.POINT_DTYPE)
    p = v[23 * 64 + 31]
    assert p["pos"].tolist() == [np.float32(-0.01), np.float32(-0.01), 2.0]
    assert p["normal"].tolist() == [0, 0, 0, 0] and p["class_id"] == 0
    assert p["color"].tolist() == [0, 0, 0]
    q = v[10 * 64 + 5]
    assert q["pos"].tolist() == [np.float32((5 - 31.5) * 1.5 / 100), np.float32((10 - 23.5) * 1.5 / 100), 1.5]
    assert q["color"].tolist() == [1, 2, 3]
    assert (pts[1] == 7).all() and (pts[0] == 7).all()          # depth <= 0 leaves the slot
    assert np.isnan(v[2]["pos"]).all()
    # no colour image: white points; start index offsets the frame
    pts2 = np.zeros((2 * 64 * 48, 33), np.uint8)
    oracle.points_extract(K_COL, d, None, IDENTITY, pts2, start=64 * 48)
    v2 = pts2.reshape(-1).view(oracle.POINT_DTYPE)
    assert (pts2[:64 * 48] == 0).all()
    assert v2[64 * 48 + 23 * 64 + 31]["color"].tolist() == [255, 255, 255]


def test_transform_matches_rotation(oracle):
    rng = np.random.default_rng(0)
    n = 100
    pts = np.zeros((n, 33), np.uint8)
    v = pts.reshape(-1).view(oracle.POINT_DTYPE)
    v["pos"] = rng.normal(size=(n, 3)).astype(np.float32)
    P0 = v["pos"].astype(np.float64).copy()
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    pose = np.concatenate([q, [0.3, -0.2, 1.0]])
    oracle.points_transform(pts, pose)
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    np.testing.assert_allclose(v["pos"], P0 @ R.T + pose[4:], atol=1e-5)


def _cloud(oracle, positions, colors):
    pts = np.zeros((len(positions), 33), np.uint8)
    v = pts.reshape(-1).view(oracle.POINT_DTYPE)
    v["pos"] = np.asarray(positions, np.float32)
    v["color"] = np.asarray(colors, np.uint8)
    return pts


def test_project_zbuffer_rules(oracle):
    """Nearest z wins; equal z: the first point; z == 0 dropped; negative z is
    kept (as in the reference); untouched pixels are 0."""
    # pixel of (x, y, z): ((x*100)/z + 31.5, (y*100)/z + 23.5) truncated
    pos = [(0.0, 0.0, 2.0),      # pixel (31, 23), z 2
           (0.0, 0.0, 1.0),      # same pixel, nearer: wins
           (0.0, 0.0, 1.0),      # same z as the previous one: the first keeps the pixel
           (0.1, 0.0, 0.0),      # z == 0: dropped
           (0.2, 0.1, -1.0),     # negative z: pixel (11, 13), kept
           (100.0, 0.0, 1.0)]    # off the image
    col = [(1, 1, 1), (2, 2, 2), (3, 3, 3), (4, 4, 4), (5, 5, 5), (6, 6, 6)]
    pts = _cloud(oracle, pos, col)
    depth, rgb = oracle.points_project(pts, K_ROW, IDENTITY, 64, 48)
    assert depth[23, 31] == 1.0 and rgb[23, 31].tolist() == [2, 2, 2]
    assert depth[13, 11] == -1.0 and rgb[13, 11].tolist() == [5, 5, 5]
    assert np.count_nonzero(depth) == 2 and np.count_nonzero(rgb.any(-1)) == 2
    # project_to_depth: no colour
    d2, none = oracle.points_project(pts, K_ROW, IDENTITY, 64, 48, color=False)
    assert none is None and np.array_equal(d2, depth)


def test_extract_project_round_trip(oracle):
    """A frame back-projected with the column-major reading and projected with
    the row-major reading of the same intrinsics lands on its own pixels."""
    rng = np.random.default_rng(1)
    d = rng.uniform(0.5, 3.0, (48, 64)).astype(np.float32)
    d[rng.random((48, 64)) < 0.1] = 0
    pts = np.zeros((64 * 48, 33), np.uint8)
    oracle.points_extract(K_COL, d, None, IDENTITY, pts)
    depth, _ = oracle.points_project(pts, K_ROW, IDENTITY, 64, 48)
    # back-projected x/z*fx + cx returns the pixel index up to rounding; where it
    # truncates to the pixel itself the depth comes back exactly
    same = depth == d
    assert same[d > 0].mean() > 0.4


def test_filter_if(oracle):
    img = np.array([0.0, 1.0, np.float32(3.4028235e38), 5e-11, -5e-11, 2.0], np.float32)
    out = oracle.filter_if(img, np.float32(3.4028235e38), 0.0)
    assert out.tolist() == [0.0, 1.0, 0.0, np.float32(5e-11), np.float32(-5e-11), 2.0]
    out = oracle.filter_if(img, 0.0, 9.0)   # |v - 0| < 1e-10
    assert out.tolist() == [9.0, 1.0, np.float32(3.4028235e38), 9.0, 9.0, 2.0]


def test_points_entry_points_reject_bad_arguments(engine_lib):
    """Argument checks run before any device work (no GPU needed)."""
    L = engine_lib
    lib = L.lib()
    K = (C.c_double * 9)(*K_COL)
    P = (C.c_double * 7)(*IDENTITY)
    dev = C.c_void_p(4096)   # never dereferenced: every call below fails its checks first
    st = lib.gbt_points_extract(None, dev, 256, L.DEPTH_F32_M, 0.001, None, 0, 64, 48, C.byref(P), 0, dev, 3072,
                                None)
    assert st == L.GBT_ERR_INVALID_ARG
    st = lib.gbt_points_extract(C.byref(K), dev, 256, L.DEPTH_F32_M, 0.001, None, 0, 64, 48, C.byref(P), 1, dev,
                                3072, None)
    assert st == L.GBT_ERR_CAPACITY and b"capacity" in lib.gbt_last_error()
    st = lib.gbt_points_extract(C.byref(K), dev, 200, L.DEPTH_F32_M, 0.001, None, 0, 64, 48, C.byref(P), 0, dev,
                                3072, None)
    assert st == L.GBT_ERR_INVALID_ARG   # pitch below the row
    st = lib.gbt_points_extract(C.byref(K), C.c_void_p(4098), 256, L.DEPTH_F32_M, 0.001, None, 0, 64, 48, C.byref(P),
                                0, dev, 3072, None)
    assert st == L.GBT_ERR_INVALID_ARG and b"aligned" in lib.gbt_last_error()
    st = lib.gbt_points_extract(C.byref(K), dev, 256, 7, 0.001, None, 0, 64, 48, C.byref(P), 0, dev, 3072, None)
    assert st == L.GBT_ERR_INVALID_ARG
    assert lib.gbt_points_transform(dev, 0, C.byref(P), None) == L.GBT_ERR_INVALID_ARG
    # counts that one launch's 32-bit block numbering does not cover
    assert lib.gbt_points_transform(dev, 1 << 33, C.byref(P), None) == L.GBT_ERR_INVALID_ARG
    st = lib.gbt_points_extract(C.byref(K), dev, 1 << 20, L.DEPTH_F32_M, 0.001, None, 0, 1 << 18, 1 << 15, C.byref(P),
                                0, dev, 1 << 40, None)
    assert st == L.GBT_ERR_INVALID_ARG and b"2^32" in lib.gbt_last_error()
    st = lib.gbt_points_project(dev, 10, C.byref(K), C.byref(P), dev, 256, None, 0, 64, 48, None, None)
    assert st == L.GBT_ERR_INVALID_ARG   # no scratch
    st = lib.gbt_points_project(dev, 1 << 33, C.byref(K), C.byref(P), dev, 256, None, 0, 64, 48, dev, None)
    assert st == L.GBT_ERR_INVALID_ARG   # more points than a 32-bit index
    assert lib.gbt_image_filter_if(None, 256, 64, 48, 0.0, 0.0, None) == L.GBT_ERR_INVALID_ARG
    assert lib.gbt_image_filter_if(dev, 100, 64, 48, 0.0, 0.0, None) == L.GBT_ERR_INVALID_ARG


@pytest.mark.parametrize("case", ["scene", "edges"])
def test_project_oracle_against_reference_host_loop(oracle, case):
    """The oracle's restatement of project_to_color_depth against the
    reference's own host loop (golden vectors made by
    tests/golden/make_golden_project.py from the reference's sources): depth
    bits and colours identical."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "points_project_ref.npz"))
    w, h = (int(x) for x in g[case + "_size"])
    d, c = oracle.points_project(g[case + "_points"], g[case + "_camera_matrix"], g[case + "_pose"], w, h)
    assert np.array_equal(d.view(np.uint32), g[case + "_depth"].view(np.uint32))
    assert np.array_equal(c, g[case + "_color"])
