"""Point clouds on the GPU: the engine's gbt_points_* kernels against the
oracle (bit-exact) and against the reference's own point_cloud_extract,
transform_points and filter_image_if kernels (bit-exact), the z-buffer
against the reference's host loop as the oracle restates it, and the
PointCloud mirror end to end (cloud -> colour + depth -> TSDF -> mesh)."""
import ctypes as C
import os

import numpy as np
import pytest

from cuphoto import synthetic as S

pytestmark = pytest.mark.gpu

K_COL = np.array([262.5, 0, 0, 0, 262.5, 0, 159.5, 119.5, 1.0])
K_ROW = np.array([262.5, 0, 159.5, 0, 262.5, 119.5, 0, 0, 1.0])


@pytest.fixture(scope="module")
def ref(oracle, gpu):
    if not oracle.RefHarness.available():
        pytest.skip("reference kernels were not built here (no oracle/_ref/ref_tsdf.cubin)")
    oracle.RefHarness.lib()
    return oracle.RefHarness


def frame(seed=0, w=320, h=240):
    """A ray-cast depth frame (float32 metres, some zeros, one negative and
    one NaN pixel), a colour image and a pose."""
    cam = S.Camera.half()
    scene = S.make_scene(seed)
    pose = S.circle_poses(8)[seed % 8]
    d = S.render_depth_m(scene, pose, cam).astype(np.float32)
    d = np.where(np.isfinite(d) & (d < 8.0), d, 0.0).astype(np.float32)
    rng = np.random.default_rng(seed)
    d[rng.random(d.shape) < 0.05] = 0
    d[3, 4] = -1.0
    d[5, 6] = np.nan
    rgb = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    return d, rgb, pose


def inverse(pose):
    R = S.matrix_from_quat(pose[:4])
    return S.pose7(R.T, -R.T @ pose[4:])


def pitched(torch, a, pad_bytes):
    """A (H, W[, C]) CUDA view of a with rows pad_bytes longer than needed."""
    h = a.shape[0]
    row = a[0].nbytes
    buf = torch.zeros((h, row + pad_bytes), dtype=torch.uint8, device="cuda")
    buf[:, :row] = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(h, row)).cuda()
    return buf


def same_points(a, b, dtype):
    """Byte equality, except that a position holding NaN in both matches
    whatever the NaN's payload (the GPU writes the canonical NaN, the CPU
    oracle propagates numpy's)."""
    va, vb = a.reshape(-1).view(dtype), b.reshape(-1).view(dtype)
    pa, pb = va["pos"], vb["pos"]
    both_nan = np.isnan(pa) & np.isnan(pb)
    bits_a = np.where(both_nan, 0, pa.view(np.uint32))
    bits_b = np.where(both_nan, 0, pb.view(np.uint32))
    rest = [n for n in dtype.names if n != "pos"]
    return np.array_equal(bits_a, bits_b) and all(np.array_equal(va[n], vb[n]) for n in rest)


def engine_extract(L, torch, K, d_buf, pitch, fmt, scale, w, h, rgb_buf, rgb_pitch, pose, start, pts):
    st = L.lib().gbt_points_extract(C.byref((C.c_double * 9)(*K)), C.c_void_p(d_buf.data_ptr()), pitch, fmt, scale,
                                    C.c_void_p(rgb_buf.data_ptr()) if rgb_buf is not None else None, rgb_pitch, w, h,
                                    C.byref((C.c_double * 7)(*pose)), start, C.c_void_p(pts.data_ptr()),
                                    pts.shape[0], None)
    L.check(st)
    torch.cuda.synchronize()


@pytest.mark.parametrize("with_color", [False, True])
def test_extract_bitexact_vs_oracle(gpu, engine_lib, oracle, with_color):
    d, rgb, pose = frame(1)
    h, w = d.shape
    pad = 192
    d_buf = pitched(gpu, d, pad)
    rgb_buf = pitched(gpu, rgb, 64) if with_color else None
    n = 2 * w * h
    pts = gpu.full((n, 33), 0xAB, dtype=gpu.uint8, device="cuda")
    engine_extract(engine_lib, gpu, K_COL, d_buf, w * 4 + pad, engine_lib.DEPTH_F32_M, 0.001, w, h, rgb_buf,
                   w * 3 + 64, pose, w * h, pts)
    exp = np.full((n, 33), 0xAB, np.uint8)
    oracle.points_extract(K_COL, d, rgb if with_color else None, pose, exp, start=w * h)
    assert same_points(pts.cpu().numpy(), exp, oracle.POINT_DTYPE)
    assert (exp[: w * h] == 0xAB).all() and (exp[w * h:] != 0xAB).any()


def test_extract_uint16_depth(gpu, engine_lib, oracle):
    d, _, pose = frame(2)
    h, w = d.shape
    raw = np.where(np.isfinite(d) & (d > 0), np.round(d * 1000), 0).astype(np.uint16)
    metres = raw.astype(np.float32) * np.float32(0.001)
    pts = gpu.zeros((w * h, 33), dtype=gpu.uint8, device="cuda")
    engine_extract(engine_lib, gpu, K_COL, pitched(gpu, raw, 0), w * 2, engine_lib.DEPTH_U16, 0.001, w, h, None, 0,
                   pose, 0, pts)
    exp = np.zeros((w * h, 33), np.uint8)
    oracle.points_extract(K_COL, metres, None, pose, exp)
    assert same_points(pts.cpu().numpy(), exp, oracle.POINT_DTYPE)


@pytest.mark.parametrize("with_color", [False, True])
def test_extract_bitexact_vs_reference_kernel(gpu, engine_lib, ref, with_color):
    """The engine's extraction against the reference's point_cloud_extract
    (its __device__ double K, 8x8 blocks), byte for byte."""
    d, rgb, pose = frame(3)
    h, w = d.shape
    d_t = gpu.from_numpy(d).cuda()
    rgb_t = gpu.from_numpy(rgb).cuda() if with_color else None
    ours = gpu.full((w * h, 33), 0x5A, dtype=gpu.uint8, device="cuda")
    theirs = ours.clone()
    engine_extract(engine_lib, gpu, K_COL, d_t, w * 4, engine_lib.DEPTH_F32_M, 1.0, w, h, rgb_t, w * 3, pose, 0, ours)
    ref.points_extract(K_COL, d_t.data_ptr(), w * 4, w, h, rgb_t.data_ptr() if with_color else 0, w * 3, pose, 0,
                       theirs.data_ptr())
    gpu.cuda.synchronize()
    a, b = ours.cpu().numpy(), theirs.cpu().numpy()
    assert (a != 0x5A).any()
    assert np.array_equal(a, b), np.argwhere((a != b).any(1))[:5]


def test_transform_bitexact_vs_reference_and_oracle(gpu, engine_lib, oracle, ref):
    rng = np.random.default_rng(4)
    n = 5000
    base = np.zeros((n, 33), np.uint8)
    v = base.reshape(-1).view(oracle.POINT_DTYPE)
    v["pos"] = rng.normal(scale=2.0, size=(n, 3)).astype(np.float32)
    v["color"] = rng.integers(0, 256, (n, 3))
    q = rng.normal(size=4)
    pose = np.concatenate([q / np.linalg.norm(q), rng.normal(size=3)])
    ours = gpu.from_numpy(base.copy()).cuda()
    theirs = ours.clone()
    engine_lib.check(engine_lib.lib().gbt_points_transform(C.c_void_p(ours.data_ptr()), n,
                                                           C.byref((C.c_double * 7)(*pose)), None))
    ref.points_transform(theirs.data_ptr(), n, pose)
    gpu.cuda.synchronize()
    exp = base.copy()
    oracle.points_transform(exp, pose)
    assert np.array_equal(ours.cpu().numpy(), theirs.cpu().numpy())
    assert np.array_equal(ours.cpu().numpy(), exp)


def engine_project(L, torch, pts, n, K, pose, w, h, color=True, pad=0):
    depth = torch.full((h, w + pad // 4), 7.0, dtype=torch.float32, device="cuda")
    rgb = torch.full((h, w * 3 + pad), 9, dtype=torch.uint8, device="cuda") if color else None
    scratch = torch.empty(w * h, dtype=torch.int64, device="cuda")
    st = L.lib().gbt_points_project(C.c_void_p(pts.data_ptr()), n, C.byref((C.c_double * 9)(*K)),
                                    C.byref((C.c_double * 7)(*pose)), C.c_void_p(depth.data_ptr()), (w * 4 + pad),
                                    C.c_void_p(rgb.data_ptr()) if color else None, w * 3 + pad, w, h,
                                    C.c_void_p(scratch.data_ptr()), None)
    L.check(st)
    torch.cuda.synchronize()
    d = depth.cpu().numpy()[:, :w]
    c = rgb.cpu().numpy()[:, :w * 3].reshape(h, w, 3) if color else None
    return d, c


def test_project_bitexact_vs_oracle(gpu, engine_lib, oracle):
    """A cloud from two frames plus exact duplicates (ties), points at z = 0
    and behind the camera, seen from a third pose: depth and colour as the
    reference's first-wins host loop produces them."""
    d1, rgb1, p1 = frame(5)
    d2, rgb2, p2 = frame(6)
    h, w = d1.shape
    cloud = np.zeros((2 * w * h, 33), np.uint8)
    # camera-to-world poses take each frame's points to the world
    oracle.points_extract(K_COL, d1, rgb1, inverse(p1), cloud, start=0)
    oracle.points_extract(K_COL, d2, rgb2, inverse(p2), cloud, start=w * h)
    rng = np.random.default_rng(7)
    dup = cloud[rng.integers(0, 2 * w * h, 20000)].copy()
    dup[:, 28:31] = rng.integers(0, 256, (len(dup), 3))        # same position, other colour: ties
    cloud = np.concatenate([cloud, dup])
    v = cloud.reshape(-1).view(oracle.POINT_DTYPE)
    v["pos"][:50, 2] = -v["pos"][:50, 2]
    n = len(cloud)
    pts = gpu.from_numpy(cloud).cuda()
    # world-to-camera of a pose between the two frames; both readings of K
    pose = S.circle_poses(16)[11]
    for K in (K_COL, K_ROW):
        d, c = engine_project(engine_lib, gpu, pts, n, K, pose, w, h, pad=32)
        ed, ec = oracle.points_project(cloud, K, pose, w, h)
        assert np.array_equal(d.view(np.uint32), ed.view(np.uint32))
        assert np.array_equal(c, ec)
    assert (ed > 0).mean() > 0.3   # the row-major reading puts the principal point in the image
    d, c = engine_project(engine_lib, gpu, pts, n, K_ROW, pose, w, h, color=False)
    ed, _ = oracle.points_project(cloud, K_ROW, pose, w, h, color=False)
    assert c is None and np.array_equal(d.view(np.uint32), ed.view(np.uint32))


@pytest.mark.parametrize("case", ["scene", "edges"])
def test_project_bitexact_vs_reference_host_loop(gpu, engine_lib, case):
    """gbt_points_project against the reference's own z-buffer loop,
    project_to_color_depth (cuda_point_cloud.cu:292-353) compiled from its
    sources and run on the host (tests/golden/make_golden_project.py): depth
    bits and colours identical, for a synthetic scene seen from another
    camera and for the loop's corner cases (z = 0, points behind the camera,
    ties, border pixels, NaN and infinite positions)."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "points_project_ref.npz"))
    cloud = g[case + "_points"]
    w, h = (int(x) for x in g[case + "_size"])
    pts = gpu.from_numpy(np.ascontiguousarray(cloud)).cuda()
    d, c = engine_project(engine_lib, gpu, pts, len(cloud), g[case + "_camera_matrix"], g[case + "_pose"], w, h,
                          pad=16)
    assert (g[case + "_depth"] != 0).sum() > 1000
    assert np.array_equal(d.view(np.uint32), g[case + "_depth"].view(np.uint32))
    assert np.array_equal(c, g[case + "_color"])


def test_filter_bitexact_vs_reference(gpu, engine_lib, oracle, ref):
    rng = np.random.default_rng(8)
    img = rng.normal(size=(60, 70)).astype(np.float32)
    img[rng.random(img.shape) < 0.2] = np.float32(3.4028235e38)
    img[0, :5] = [0.0, 5e-11, -5e-11, 1e-9, np.nan]
    for fv, sv in ((np.float32(3.4028235e38), 0.0), (0.0, 4.0)):
        ours = gpu.from_numpy(img.copy()).cuda()
        theirs = ours.clone()
        engine_lib.check(engine_lib.lib().gbt_image_filter_if(C.c_void_p(ours.data_ptr()), 70 * 4, 70, 60, fv, sv,
                                                              None))
        ref.filter_if(theirs.data_ptr(), 70 * 4, 70, 60, fv, sv)
        gpu.cuda.synchronize()
        a = ours.cpu().numpy()
        assert np.array_equal(a.view(np.uint32), theirs.cpu().numpy().view(np.uint32))
        assert np.array_equal(a.view(np.uint32), oracle.filter_if(img, fv, sv).view(np.uint32))


def test_point_cloud_to_surface(gpu, engine_lib):
    """The PointCloud mirror end to end, as TSDFSurface::reconstruct_surface(
    cudaPointCloud) is meant to run: frames back-projected into one cloud,
    the cloud projected to colour + depth at a pose, integrated, meshed."""
    from cuphoto import PointCloud, TSDFVolume, TSDFVolumeConfig, extract_mesh_device
    cam = S.Camera.half()
    scene = S.make_scene(0)
    poses = S.circle_poses(8)
    pc = PointCloud.create(list(K_COL), 3 * cam.width * cam.height)
    for k in range(3):
        d = S.render_depth_m(scene, poses[k], cam).astype(np.float32)
        d = np.where(np.isfinite(d) & (d < 8.0), d, 0.0).astype(np.float32)
        # a camera-space cloud of frame k, taken to world by the inverse pose
        assert pc.extract_points(gpu.from_numpy(d).cuda(), None, inverse(poses[k]), k)
    assert pc.get_num_points() == 3 * cam.width * cam.height
    depth = gpu.zeros((cam.height, cam.width), dtype=gpu.float32, device="cuda")
    color = gpu.zeros((cam.height, cam.width, 3), dtype=gpu.uint8, device="cuda")
    pc.camera_matrix = list(K_ROW)   # projection reads cx, cy from m[2], m[5]
    assert pc.project_to_color_depth(color, depth, poses[1])
    seen = (depth > 0).float().mean().item()
    assert seen > 0.5
    assert (color.sum(-1) > 0).float().mean().item() > 0.5    # white points
    tc = TSDFVolumeConfig(**S.grid_for(128, 2.56), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy,
                          camera_width=cam.width, camera_height=cam.height, mode="fixed")
    vol = TSDFVolume(tc)
    assert vol.integrate(color, depth, poses[1])
    V, T = extract_mesh_device(vol)
    assert len(T) > 1000
    # filter_depth keeps what lies outside (min, max), as the reference does
    n0 = pc.get_num_points()
    z = pc.to_numpy()["pos"][:, 2]
    pc.filter_depth(-0.5, 0.5)
    assert pc.get_num_points() == int(((z <= -0.5) | (z >= 0.5)).sum()) < n0
