"""Marching cubes on the GPU against the CPU oracle (through the C ABI)."""
import ctypes as C

import numpy as np
import pytest

from cuphoto import TSDFVolume, TSDFVolumeConfig, extract_mesh_device, generate_triangular_surface
from cuphoto import _lib as L

from helpers import circle_case, engine_run, frontal_case, mesh, oracle_run, set_distances

pytestmark = pytest.mark.gpu


def smooth_field(shape, seed, scale=0.05):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    f = np.zeros(shape)
    for _ in range(5):
        k = rng.uniform(2, 9, size=3)
        ph = rng.uniform(0, 6.3, size=3)
        f += np.sin(k[0] * x + ph[0]) * np.sin(k[1] * y + ph[1]) * np.sin(k[2] * z + ph[2])
    return (scale * f / 5).astype(np.float32)


# (64, 130, 5): 63 cubes per row (two segments of 31 and one of 1), 129 rows
# per layer (two runs of 64 rows and one of 1)
@pytest.mark.parametrize("grid", [(64, 48, 40), (77, 50, 37), (2, 2, 2), (130, 3, 9), (64, 130, 5)])
def test_compat_ieee_mesh_bitexact(gpu, oracle, grid):
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=tuple(0.01 * g for g in grid),
                          global_offset=(-0.3, 0.2, 0.5), arith="ieee")
    vol = TSDFVolume(tc)
    D = smooth_field(grid[::-1], sum(grid))
    set_distances(gpu, vol, D)
    V, T = mesh(vol)
    Vo, To = oracle.mc_compat(oracle.cfg_from(tc), D.ravel())
    assert len(V) == len(Vo)
    assert np.array_equal(T, To)
    assert np.array_equal(V.view(np.uint32), Vo.view(np.uint32))


@pytest.mark.parametrize("grid", [(64, 48, 40), (77, 50, 37), (33, 65, 17), (129, 66, 6)])
def test_fixed_mesh_bitexact(gpu, oracle, grid):
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=tuple(0.01 * g for g in grid),
                          global_offset=(-0.3, 0.2, 0.5), mode="fixed", max_weight=16)
    vol = TSDFVolume(tc)
    D = smooth_field(grid[::-1], 7 + sum(grid))
    W = (np.random.default_rng(1).random(D.shape) > 0.02).astype(np.float32)
    set_distances(gpu, vol, D, W)
    V, T = mesh(vol)
    Vo, To = oracle.mc_fixed(oracle.cfg_from(tc), D.ravel(), W.ravel())
    assert len(V) > 100 and len(V) == len(Vo)
    assert np.array_equal(T, To)
    assert np.array_equal(V.view(np.uint32), Vo.view(np.uint32))


def test_compat_reference_mesh_vs_oracle(gpu, oracle):
    """Reference arithmetic: same triangles and indices; vertices within the
    approximate divide's error (1e-5 voxel)."""
    grid = (96, 64, 48)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.96, 0.64, 0.48), global_offset=(0.0, 0.0, 0.3))
    vol = TSDFVolume(tc)
    D = smooth_field(grid[::-1], 3)
    set_distances(gpu, vol, D)
    V, T = mesh(vol)
    Vo, To = oracle.mc_compat(oracle.cfg_from(tc), D.ravel())
    assert len(V) == len(Vo) > 100
    assert np.array_equal(T, To)
    # 1e-5 voxel, or two float ulps of the coordinate where that is coarser
    tol = max(1e-5 * 0.01, 2 * float(np.spacing(np.float32(np.abs(Vo).max()))))
    np.testing.assert_allclose(V, Vo, rtol=0, atol=tol)


def test_integrated_frontal_scene_meshes(gpu, oracle):
    """End to end: compat (IEEE) integrate + mesh equals the oracle's."""
    seq, tc = frontal_case(128, 96, 96, frames=6, arith="ieee")
    vol, D, W = engine_run(gpu, tc, list(seq.depth_m()), seq.poses, k=6)
    V, T = mesh(vol)
    Do, Wo = oracle_run(oracle, tc, list(seq.depth_m()), seq.poses)
    Vo, To = oracle.mc_compat(oracle.cfg_from(tc), Do.ravel())
    assert len(V) == len(Vo) > 1000
    assert np.array_equal(V.view(np.uint32), Vo.view(np.uint32)) and np.array_equal(T, To)


def test_capacity_and_count_only(gpu, oracle):
    grid = (64, 48, 40)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.64, 0.48, 0.4), arith="ieee")
    vol = TSDFVolume(tc)
    D = smooth_field(grid[::-1], 11)
    set_distances(gpu, vol, D)
    lib = L.lib()
    n = C.c_int64()
    assert lib.gbt_extract_mesh(vol.handle, None, None, 0, 0, C.byref(n), None) == L.GBT_OK
    total = n.value
    assert total > 100
    cap = total // 3
    Vb = gpu.zeros((cap, 3, 3), dtype=gpu.float32, device="cuda")
    Tb = gpu.zeros((cap, 3), dtype=gpu.int32, device="cuda")
    st = lib.gbt_extract_mesh(vol.handle, C.c_void_p(Vb.data_ptr()), C.c_void_p(Tb.data_ptr()), cap, 0,
                              C.byref(n), None)
    assert st == L.GBT_ERR_CAPACITY and n.value == total
    Vo, To = oracle.mc_compat(oracle.cfg_from(tc), D.ravel())
    assert np.array_equal(Vb.cpu().numpy(), Vo[:cap]) and np.array_equal(Tb.cpu().numpy(), To[:cap])
    # int32 indices: one triangle from 2^31 - 3 ends at INT32_MAX; from 2^31 - 2
    # it would pass it, and nothing is written
    st = lib.gbt_extract_mesh(vol.handle, C.c_void_p(Vb.data_ptr()), C.c_void_p(Tb.data_ptr()), 1, 2 ** 31 - 3,
                              C.byref(n), None)
    assert st == L.GBT_ERR_CAPACITY and n.value == total
    assert Tb[0].tolist() == [2 ** 31 - 3, 2 ** 31 - 2, 2 ** 31 - 1]
    Tb.zero_()
    st = lib.gbt_extract_mesh(vol.handle, C.c_void_p(Vb.data_ptr()), C.c_void_p(Tb.data_ptr()), 1, 2 ** 31 - 2,
                              C.byref(n), None)
    assert st == L.GBT_ERR_INVALID_ARG and b"int32" in lib.gbt_last_error()
    assert int(Tb.abs().sum().item()) == 0


def test_async_count_and_index_base(gpu, oracle):
    grid = (40, 40, 40)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.4, 0.4, 0.4), mode="fixed", max_weight=4)
    vol = TSDFVolume(tc)
    D = smooth_field(grid, 5)
    set_distances(gpu, vol, D, np.ones_like(D))
    V, T = extract_mesh_device(vol, index_base=1000)
    assert T.min().item() == 1000
    lib = L.lib()
    cnt = gpu.zeros(1, dtype=gpu.int64, device="cuda")
    cap = len(V)
    Vb = gpu.empty((cap, 3, 3), dtype=gpu.float32, device="cuda")
    Tb = gpu.empty((cap, 3), dtype=gpu.int32, device="cuda")
    L.check(lib.gbt_extract_mesh_async(vol.handle, C.c_void_p(Vb.data_ptr()), C.c_void_p(Tb.data_ptr()), cap, 0,
                                       C.c_void_p(cnt.data_ptr()), C.c_void_p(gpu.cuda.current_stream().cuda_stream)))
    gpu.cuda.synchronize()
    assert cnt.item() == cap
    assert np.array_equal(Vb.cpu().numpy(), V.cpu().numpy())


@pytest.mark.parametrize("grid", [(1, 1, 1), (2, 1, 5), (1, 7, 7)])
def test_degenerate_grids_have_no_cubes(gpu, grid):
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.1, 0.1, 0.1))
    vol = TSDFVolume(tc)
    V, T = mesh(vol)
    assert len(V) == 0 and len(T) == 0


@pytest.mark.parametrize("value", [1.0, -1.0])
def test_uniform_fields_have_no_surface(gpu, value):
    grid = (33, 20, 12)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.3, 0.2, 0.1))
    vol = TSDFVolume(tc)
    set_distances(gpu, vol, np.full(grid[::-1], value, np.float32))
    assert len(mesh(vol)[0]) == 0


def test_generate_triangular_surface_appends(gpu, oracle):
    grid = (24, 24, 24)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.24, 0.24, 0.24), arith="ieee")
    vol = TSDFVolume(tc)
    D = smooth_field(grid, 9)
    set_distances(gpu, vol, D)
    verts, tris = [(0.0, 0.0, 0.0)] * 5, []
    v, t = generate_triangular_surface(vol, verts, tris)
    assert len(verts) == 5 + len(v) and len(tris) == len(t)
    assert tris[0] == (5, 6, 7)
    Vo, To = oracle.mc_compat(oracle.cfg_from(tc), D.ravel(), index_base=5)
    assert np.array_equal(t, To)


def test_large_field_mesh_tiles_chain(gpu, oracle):
    """A 256^3 field (about 16k tiles: counts, the tile scan, emission of the listed tiles) against the oracle."""
    grid = (256, 256, 256)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(2.56,) * 3, mode="fixed", max_weight=4)
    vol = TSDFVolume(tc)
    D = smooth_field(grid, 21)
    W = np.ones_like(D)
    set_distances(gpu, vol, D, W)
    V, T = mesh(vol)
    Vo, To = oracle.mc_fixed(oracle.cfg_from(tc), D.ravel(), W.ravel())
    assert len(V) == len(Vo) > 10000
    assert np.array_equal(V.view(np.uint32), Vo.view(np.uint32))


# ---------------------------------------------------------------------------
# Fixed-mode mesh with shared vertices (gbt_extract_mesh_indexed)
def _scene_normals(scene, P):
    """Unit gradient of the scene's analytic SDF (plane + spheres) at P (n, 3)."""
    P = np.asarray(P, np.float64)
    d = scene.plane_up * (P[:, 1] - scene.plane_y)
    g = np.tile([0.0, scene.plane_up, 0.0], (len(P), 1))
    for c, r in zip(scene.centres, scene.radii):
        v = P - c
        n = np.linalg.norm(v, axis=1)
        ds = n - r
        nearer = ds < d
        d = np.where(nearer, ds, d)
        g = np.where(nearer[:, None], v / np.maximum(n, 1e-12)[:, None], g)
    return g


@pytest.mark.parametrize("grid", [(64, 48, 40), (33, 65, 17)])
def test_indexed_mesh_is_the_soup_with_shared_vertices(gpu, grid):
    """The shared-vertex mesh gathers back to the triangle soup bit for bit,
    in the same triangle order; every vertex is used and none repeats."""
    from cuphoto import extract_mesh_indexed
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=tuple(0.01 * g for g in grid),
                          global_offset=(-0.3, 0.2, 0.5), mode="fixed", max_weight=16)
    vol = TSDFVolume(tc)
    D = smooth_field(grid[::-1], 7 + sum(grid))
    W = (np.random.default_rng(1).random(D.shape) > 0.02).astype(np.float32)
    set_distances(gpu, vol, D, W)
    V, T = mesh(vol)
    Vi, Ni, Ti = (x.cpu().numpy() for x in extract_mesh_indexed(vol))
    assert len(Ti) == len(T) > 100
    assert np.array_equal(Vi[Ti].view(np.uint32), V.view(np.uint32))
    assert np.unique(Ti).size == len(Vi)                 # no orphan vertices
    assert len(Vi) < 0.6 * 3 * len(Ti)                   # each vertex shared by several triangles
    assert len(np.unique(Vi, axis=0)) >= 0.999 * len(Vi)
    n = np.linalg.norm(Ni, axis=1)
    assert np.all(np.abs(n - 1) < 1e-5)


def test_indexed_mesh_normals_point_to_free_space(gpu):
    """On an integrated scene the normals agree with the analytic surface
    normals, and the triangle winding is consistent with them."""
    from cuphoto import extract_mesh_indexed
    seq, tc = circle_case(n=96, frames=8, mode="fixed")
    vol, _, _ = engine_run(gpu, tc, seq.depth_u16, seq.poses, k=8)
    Vi, Ni, Ti = (x.cpu().numpy() for x in extract_mesh_indexed(vol))
    assert len(Ti) > 1000
    g = _scene_normals(seq.scene, Vi)
    assert (np.sum(Ni * g, axis=1) > 0.7).mean() > 0.9
    tri = Vi[Ti]
    face = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    s = np.sign(np.sum(face * Ni[Ti].mean(axis=1), axis=1))
    assert max((s > 0).mean(), (s < 0).mean()) > 0.95


def test_indexed_mesh_capacity_counts_and_mode(gpu):
    from cuphoto import extract_mesh_indexed
    grid = (40, 36, 32)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.4, 0.36, 0.32), mode="fixed")
    vol = TSDFVolume(tc)
    D = smooth_field(grid[::-1], 3)
    set_distances(gpu, vol, D, np.ones_like(D))
    Vi, _, Ti = extract_mesh_indexed(vol, normals=False)
    lib = L.lib()
    nv, nt = C.c_int64(), C.c_int64()
    small = gpu.empty((10, 3), dtype=gpu.float32, device="cuda")
    tris = gpu.empty((len(Ti), 3), dtype=gpu.int32, device="cuda")
    st = lib.gbt_extract_mesh_indexed(vol.handle, C.c_void_p(small.data_ptr()), None, C.c_void_p(tris.data_ptr()),
                                      10, len(Ti), 0, C.byref(nv), C.byref(nt), None)
    assert st == L.GBT_ERR_CAPACITY and nv.value == len(Vi) and nt.value == len(Ti)
    compat = TSDFVolume(TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.4, 0.36, 0.32)))
    with pytest.raises(L.GbtError):
        extract_mesh_indexed(compat)
