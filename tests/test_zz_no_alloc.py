"""gbt_extract_mesh_noalloc: mesh extraction for callers that must not
allocate device memory (work recorded during global-mode graph capture,
applications whose device memory belongs to their own pool or budget).

Checked through the C ABI against gbt_extract_mesh, the entry point that may
allocate, on two calls in a row: both must give the same triangles, vertices
and count (bit for bit, the tolerance of the other mesh tests), and the
second call must not change the device's free memory.  This file is
collected last so a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

from cuphoto import TSDFVolume, TSDFVolumeConfig, extract_mesh_device
from cuphoto import _lib as L

pytestmark = pytest.mark.gpu


def smooth_field(shape, seed):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    f = np.zeros(shape)
    for _ in range(4):
        k = rng.uniform(2, 8, size=3)
        ph = rng.uniform(0, 6.3, size=3)
        f += np.sin(k[0] * x + ph[0]) * np.sin(k[1] * y + ph[1]) * np.sin(k[2] * z + ph[2])
    return (0.02 * f).astype(np.float32)


@pytest.mark.parametrize("mode,arith", [("fixed", "ieee"), ("compat", "reference"), ("compat", "ieee")])
def test_noalloc_mesh_matches_allocating_entry_point(gpu, mode, arith):
    grid = (96, 80, 72)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.96, 0.8, 0.72), global_offset=(-0.4, 0.1, 0.5),
                          mode=mode, arith=arith, max_weight=8)
    vol = TSDFVolume(tc)
    D = smooth_field(grid[::-1], 17)
    vol.voxel_distances_data().copy_(gpu.from_numpy(D).cuda())
    vol.voxel_weights_data().fill_(1.0)
    gpu.cuda.synchronize()
    V0, T0 = extract_mesh_device(vol, index_base=7)
    V0, T0 = V0.cpu().numpy(), T0.cpu().numpy()
    assert len(V0) > 1000

    lib = L.lib()
    cap = len(V0) + 16
    verts = gpu.full((cap, 3, 3), -1.0, dtype=gpu.float32, device="cuda")
    tris = gpu.full((cap, 3), -1, dtype=gpu.int32, device="cuda")
    count = gpu.zeros(1, dtype=gpu.int64, device="cuda")
    stream = C.c_void_p(gpu.cuda.current_stream().cuda_stream)
    free_after = []
    for call in range(2):
        verts.fill_(-1.0)
        tris.fill_(-1)
        count.fill_(-2)
        gpu.cuda.synchronize()
        st = lib.gbt_extract_mesh_noalloc(vol.handle, C.c_void_p(verts.data_ptr()), C.c_void_p(tris.data_ptr()),
                                          cap, 7, C.c_void_p(count.data_ptr()), stream)
        assert st == L.GBT_OK, lib.gbt_last_error().decode()
        gpu.cuda.synchronize()
        free_after.append(gpu.cuda.mem_get_info()[0])
        n = int(count.item())
        assert n == len(V0), (call, n, len(V0))
        assert np.array_equal(verts[:n].cpu().numpy().view(np.uint32), V0.view(np.uint32))
        assert np.array_equal(tris[:n].cpu().numpy(), T0)
        assert np.all(tris[n:].cpu().numpy() == -1)
    assert free_after[1] == free_after[0]


def test_noalloc_rejects_volumes_beyond_its_scratch(gpu):
    # 600^3 voxels = 599^3 cubes, above GBT_NOALLOC_MAX_CUBES (196348 tiles of 1024 cubes)
    tc = TSDFVolumeConfig(voxel_grid_size=(600, 600, 600), physical_size=(3.0, 3.0, 3.0))
    vol = TSDFVolume(tc)
    lib = L.lib()
    count = gpu.zeros(1, dtype=gpu.int64, device="cuda")
    st = lib.gbt_extract_mesh_noalloc(vol.handle, None, None, 0, 0, C.c_void_p(count.data_ptr()), None)
    assert st == L.GBT_ERR_INVALID_ARG
    msg = lib.gbt_last_error().decode()
    assert "static scratch" in msg and "201060352" in msg


def test_noalloc_mesh_recorded_in_global_mode_graph_capture(gpu):
    """The use the entry point exists for: recording mesh extraction into a
    CUDA graph captured in the global mode, where any cudaMalloc would fail
    the capture.  One call first (it resolves the scratch address), then the
    capture; two replays give gbt_extract_mesh's triangles and count."""
    grid = (64, 72, 80)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=(0.64, 0.72, 0.8), mode="fixed", arith="ieee",
                          max_weight=8)
    vol = TSDFVolume(tc)
    vol.voxel_distances_data().copy_(gpu.from_numpy(smooth_field(grid[::-1], 5)).cuda())
    vol.voxel_weights_data().fill_(1.0)
    gpu.cuda.synchronize()
    V0, T0 = extract_mesh_device(vol)
    V0, T0 = V0.cpu().numpy(), T0.cpu().numpy()
    assert len(V0) > 500
    lib = L.lib()
    cap = len(V0) + 8
    verts = gpu.zeros((cap, 3, 3), dtype=gpu.float32, device="cuda")
    tris = gpu.zeros((cap, 3), dtype=gpu.int32, device="cuda")
    count = gpu.zeros(1, dtype=gpu.int64, device="cuda")

    def call():
        st = lib.gbt_extract_mesh_noalloc(vol.handle, C.c_void_p(verts.data_ptr()), C.c_void_p(tris.data_ptr()),
                                          cap, 0, C.c_void_p(count.data_ptr()),
                                          C.c_void_p(gpu.cuda.current_stream().cuda_stream))
        assert st == L.GBT_OK, lib.gbt_last_error().decode()

    call()
    gpu.cuda.synchronize()
    g = gpu.cuda.CUDAGraph()
    with gpu.cuda.graph(g, capture_error_mode="global"):
        call()
    for _ in range(2):
        verts.zero_()
        tris.zero_()
        count.fill_(-2)
        g.replay()
        gpu.cuda.synchronize()
        n = int(count.item())
        assert n == len(V0)
        assert np.array_equal(verts[:n].cpu().numpy().view(np.uint32), V0.view(np.uint32))
        assert np.array_equal(tris[:n].cpu().numpy(), T0)
