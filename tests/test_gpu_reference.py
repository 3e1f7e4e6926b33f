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
