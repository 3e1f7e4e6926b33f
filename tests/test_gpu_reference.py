"""The engine's compat mode against the reference's own kernels, compiled from
the reference's sources (oracle/build.py) and run on the same GPU, and
against the golden vectors those kernels produced."""
import glob
import os

import numpy as np
import pytest

from cuphoto import TSDFVolume, TSDFVolumeConfig
from cuphoto import synthetic as S

from helpers import circle_case, dev_depth, engine_run, frontal_case, mesh, set_distances

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ref(oracle, gpu):
    if not oracle.RefHarness.available():
        pytest.skip("reference kernels were not built here (no oracle/_ref/ref_tsdf.cubin)")
    oracle.RefHarness.lib()
    return oracle.RefHarness


def run_reference(gpu, ref, tc, depths_m, poses):
    r = ref(tc)
    ms = 0.0
    for d, p in zip(depths_m, poses):
        t = dev_depth(gpu, d)
        ms += r.integrate(t.data_ptr(), t.stride(0) * 4, t.shape[1], t.shape[0], p)
    D, W = r.read()
    return r, D, W, ms


@pytest.mark.parametrize("k", [1, 4])
@pytest.mark.parametrize("case", ["frontal", "circle"])
def test_integrate_bitexact_vs_reference_kernels(gpu, ref, case, k):
    seq, tc = frontal_case(64, 48, 64, frames=4) if case == "frontal" else circle_case(64, frames=4)
    depths = list(seq.depth_m())
    r, Dr, Wr, _ = run_reference(gpu, ref, tc, depths, seq.poses)
    assert abs(r.truncation - TSDFVolume(tc).truncation) == 0
    _, D, W = engine_run(gpu, tc, depths, seq.poses, k=k)
    assert (Wr > 0).mean() > 0.05
    assert np.array_equal(W, Wr)
    assert np.array_equal(D.view(np.uint32), Dr.view(np.uint32))


def zero_z_case():
    """Voxel layer 16 has world z exactly 0 and, under the identity rotation
    with t = (., ., -0.25), layer 20 has camera z exactly 0: both map to pixel
    (0, 0) in the reference (camera_util.cu:9,46), whose depth is 1 m."""
    vs = 0.0625
    n = (64, 48, 32)
    tc = TSDFVolumeConfig(voxel_grid_size=n, physical_size=tuple(vs * k for k in n),
                          global_offset=(-2.0, -1.5, -16.5 * vs), focal_x=100.0, focal_y=100.0, cx=31.5, cy=23.5,
                          camera_width=64, camera_height=48)
    rng = np.random.default_rng(7)
    depths = []
    for _ in range(3):
        d = rng.uniform(0.05, 2.5, (48, 64)).astype(np.float32)
        d[0, 0] = 1.0
        depths.append(d)
    poses = [np.array([1.0, 0, 0, 0, 0.0, 0.0, -0.25]), np.array([1.0, 0, 0, 0, 0.1, -0.05, -0.25]),
             np.array([1.0, 0, 0, 0, -0.2, 0.15, -0.25])]
    return tc, depths, poses


@pytest.mark.parametrize("k", [1, 3])
def test_zero_z_voxels_bitexact_vs_reference_kernels(gpu, ref, k):
    tc, depths, poses = zero_z_case()
    r, Dr, Wr, _ = run_reference(gpu, ref, tc, depths, poses)
    _, D, W = engine_run(gpu, tc, depths, poses, k=k)
    # both quirk layers were updated by every frame, through pixel (0, 0)
    assert (Wr[16] == 3).all() and (Wr[20] == 3).all()
    assert np.array_equal(W, Wr)
    assert np.array_equal(D.view(np.uint32), Dr.view(np.uint32))


def test_mesh_bitexact_vs_reference_kernels(gpu, ref):
    seq, tc = frontal_case(96, 64, 64, frames=4)
    depths = list(seq.depth_m())
    r, Dr, Wr, _ = run_reference(gpu, ref, tc, depths, seq.poses)
    Vr, Tr, _ = r.extract()
    vol = TSDFVolume(tc)
    set_distances(gpu, vol, Dr, Wr)
    V, T = mesh(vol)
    assert len(Vr) > 100 and len(V) == len(Vr)
    assert np.array_equal(T, Tr)
    assert np.array_equal(V.view(np.uint32), Vr.view(np.uint32))


def test_full_size_c1_vs_reference_kernels(gpu, ref):
    """256^3, 20 frames of 640x480: integrate bit-exact, mesh bit-exact."""
    seq = S.make_sequence(20, scene_id=0, camera=S.Camera(), trajectory="circle")
    tc = TSDFVolumeConfig(**S.grid_for(256))
    depths = list(seq.depth_m())
    r, Dr, Wr, _ = run_reference(gpu, ref, tc, depths, seq.poses)
    vol, D, W = engine_run(gpu, tc, depths, seq.poses, k=20)
    assert np.array_equal(W, Wr)
    assert np.array_equal(D.view(np.uint32), Dr.view(np.uint32))
    Vr, Tr, _ = r.extract()
    V, T = mesh(vol)
    assert len(V) == len(Vr)
    assert np.array_equal(V.view(np.uint32), Vr.view(np.uint32)) and np.array_equal(T, Tr)


def test_full_size_c2_batched_vs_reference_kernels(gpu, ref):
    """The benchmark's default workload: 512^3 voxels of 0.5 cm, 300 frames
    640x480 uint16 along the helix, integrated by the batched kernel with the
    bench's launch shape (brick 2, 64-frame windows, resident CTAs) and by
    the reference's kernel one frame per call: bit-exact."""
    from cuphoto.batch import BatchIntegrator
    cam = S.Camera()
    scene = S.make_scene(scene_id=0, n_spheres=6)
    poses = S.helix_poses(300, seed=0)
    frames = S.render_sequence_torch(scene, poses, cam, seed=0)            # (300, H, W) uint16 bits in int16
    tc = TSDFVolumeConfig(**S.grid_for(512, 2.56), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy,
                          camera_width=cam.width, camera_height=cam.height, max_weight=128.0)
    # the reference reads float metres: float(u16) * 0.001 rounded once, as the engine converts
    metres = (frames.to(gpu.int32) & 0xFFFF).to(gpu.float32) * gpu.tensor(0.001, dtype=gpu.float32, device="cuda")
    r = ref(tc)
    for k in range(len(poses)):
        r.integrate(metres[k].data_ptr(), metres.stride(1) * 4, metres.shape[2], metres.shape[1], poses[k])
    Dr, Wr = r.read()
    del metres
    vol = TSDFVolume(tc)
    BatchIntegrator(max_scenes=1, max_frames=300).integrate([vol], [[frames[k] for k in range(300)]], [poses],
                                                             brick=2, ctas_per_sm=0, frames_per_launch=64)
    gpu.cuda.synchronize()
    W = vol.voxel_weights_data().cpu().numpy()
    assert (Wr > 0).mean() > 0.05
    assert np.array_equal(W, Wr)
    assert np.array_equal(vol.voxel_distances_data().cpu().numpy().view(np.uint32), Dr.view(np.uint32))


GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "ref_*.npz")))


@pytest.mark.skipif(not GOLDEN, reason="no golden vectors")
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_engine_against_reference_golden(gpu, path):
    g = np.load(path)
    tc = TSDFVolumeConfig(voxel_grid_size=tuple(int(x) for x in g["grid"]), physical_size=tuple(g["phys"]),
                          global_offset=tuple(g["offset"]), focal_x=float(g["K"][0]), focal_y=float(g["K"][1]),
                          cx=float(g["K"][2]), cy=float(g["K"][3]), max_weight=float(g["max_weight"]))
    depth = g["depth_u16"].astype(np.float32) * np.float32(g["depth_scale"])
    vol, D, W = engine_run(gpu, tc, list(depth), g["poses"], k=len(depth))
    assert np.array_equal(W, g["W"])
    assert np.array_equal(D.view(np.uint32), g["D"].view(np.uint32))
    V, T = mesh(vol)
    assert len(V) == int(g["ntri"])
    assert np.array_equal(V.view(np.uint32), g["verts"].view(np.uint32)) and np.array_equal(T, g["tris"])


def test_pixel_indices_match_reference_kernels(gpu, ref):
    """Every voxel picks the same depth pixel as the reference's kernel.

    The depth image codes (u mod 16, v mod 16) in the metre value, within the
    truncation band of a thin 256x256x8 slab; after one frame each updated
    voxel's distance gives back the pixel it read.  16 generic poses, about
    5 million decoded projections, no differing pixel allowed."""
    W_, H_ = 640, 480
    u = np.arange(W_)[None, :] % 16
    v = np.arange(H_)[:, None] % 16
    base, delta = 0.480, 0.008 / 256
    depth = (base + (u + 16 * v) * delta).astype(np.float32)
    tc = TSDFVolumeConfig(voxel_grid_size=(256, 256, 8), physical_size=(2.56, 2.56, 0.008),
                          global_offset=(-1.28, -1.28, 0.48))
    vs = np.float32(2.56) / np.float32(256), np.float32(2.56) / np.float32(256), np.float32(0.008) / np.float32(8)
    trunc = TSDFVolume(tc).truncation
    pz = (np.arange(8, dtype=np.float32) + np.float32(0.5)) * vs[2] + np.float32(0.48)
    rng = np.random.default_rng(5)
    decoded = 0
    for trial in range(16):
        ang = rng.uniform(0, 2 * np.pi)
        c = np.array([1.2 * np.cos(ang), 1.2 * np.sin(ang), -0.8 + 0.2 * rng.normal()])
        R, t = S.look_at(c, target=(0.1 * rng.normal(), 0.1 * rng.normal(), 0.5),
                         up=(0, 0, 1.0) if trial % 2 else (0, 1.0, 0))
        pose = S.pose7(R, t)
        _, Dr, Wr, _ = run_reference(gpu, ref, tc, [depth], [pose])
        _, D, W = engine_run(gpu, tc, [depth], [pose])
        m = (Wr > 0) & (np.abs(Dr) < trunc * 0.999)
        code_r = np.rint((Dr.astype(np.float64) + pz[:, None, None] - base) / delta)
        code_e = np.rint((D.astype(np.float64) + pz[:, None, None] - base) / delta)
        assert np.array_equal(W, Wr)
        assert np.array_equal(code_e[m], code_r[m])
        assert np.array_equal(D.view(np.uint32), Dr.view(np.uint32))
        decoded += int(m.sum())
    assert decoded > 4_000_000
