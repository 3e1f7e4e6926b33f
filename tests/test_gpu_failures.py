"""Failure paths of the C ABI on a GPU, caused on the host side only (no
kernel is made to fault, trap or hang).

* Device allocations made to fail through gbt_debug_inject: each call
  reports GBT_ERR_ALLOC with its message, hands out no handle, frees what it
  had already allocated, and the engine works again afterwards.  The
  reference's constructor swallows these failures (tsdf_volume.cu:203-209).
* A launch error left pending by earlier work: the next entry point reports
  only its own result.
* A synchronising call issued while the stream is being captured into a CUDA
  graph: the call fails with the runtime's capture error in gbt_last_error,
  and the volume is usable after the capture is abandoned.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from cuphoto import TSDFVolume, TSDFVolumeConfig, extract_mesh_device
from cuphoto import _lib as L

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _cfg(n=256, managed=False):
    tc = TSDFVolumeConfig(voxel_grid_size=(n, n, n), physical_size=(2.56, 2.56, 2.56),
                          global_offset=(-1.28, -1.28, -1.28), memory="managed" if managed else "device")
    return tc


def _free(gpu):
    gpu.cuda.synchronize()
    return gpu.cuda.mem_get_info()[0]


@pytest.fixture(autouse=True)
def _no_injection_left(engine_lib):
    yield
    engine_lib.lib().gbt_debug_inject(L.INJECT_NONE, 0, 0)


@pytest.mark.parametrize("managed", [False, True])
@pytest.mark.parametrize("skip", [0, 1])
def test_volume_allocation_failure_leaks_nothing(gpu, managed, skip):
    lib = L.lib()
    probe = TSDFVolume(_cfg(64))   # context, module and allocator set up before measuring
    del probe
    free0 = _free(gpu)
    assert lib.gbt_debug_inject(L.INJECT_ALLOC, skip, 1) == L.GBT_OK
    out = C.c_void_p(0)
    c = _cfg(256, managed).to_c()
    st = lib.gbt_volume_create(C.byref(c), None, C.byref(out))
    assert st == L.GBT_ERR_ALLOC
    assert out.value is None
    assert "allocating 134217728 bytes for the volume" in lib.gbt_last_error().decode()
    # the 64 MiB distance grid of the skip=1 case was freed again
    assert abs(_free(gpu) - free0) < (16 << 20)
    # the injection is used up: the same configuration now builds a volume
    vol = TSDFVolume(_cfg(256, managed))
    assert vol.voxel_weights_data().sum().item() == 0.0


def _surface_volume(gpu, n=96):
    tc = TSDFVolumeConfig(voxel_grid_size=(n, n, n), physical_size=(0.96, 0.96, 0.96), mode="fixed", arith="ieee",
                          max_weight=8)
    vol = TSDFVolume(tc)
    z, y, x = np.meshgrid(*[np.linspace(-1, 1, n)] * 3, indexing="ij")
    D = (0.05 * (np.sqrt(x * x + y * y + z * z) - 0.6)).astype(np.float32)
    vol.voxel_distances_data().copy_(gpu.from_numpy(D).cuda())
    vol.voxel_weights_data().fill_(1.0)
    gpu.cuda.synchronize()
    return vol


def test_mesh_scratch_allocation_failure_then_recovery(gpu):
    lib = L.lib()
    vol = _surface_volume(gpu)
    n = C.c_int64(-1)
    assert lib.gbt_debug_inject(L.INJECT_ALLOC, 0, 1) == L.GBT_OK
    st = lib.gbt_extract_mesh(vol.handle, None, None, 0, 0, C.byref(n), None)
    assert st == L.GBT_ERR_ALLOC
    assert "mesh scratch" in lib.gbt_last_error().decode()
    assert n.value == 0
    V, T = extract_mesh_device(vol)
    assert len(V) > 1000 and len(T) == len(V)
    # the voxel-transform records of the accessor fail alike and leave no buffer behind
    assert lib.gbt_debug_inject(L.INJECT_ALLOC, 0, 1) == L.GBT_OK
    p = C.c_void_p(0)
    assert lib.gbt_volume_transformation_voxels(vol.handle, None, C.byref(p)) == L.GBT_ERR_ALLOC
    assert p.value is None
    assert lib.gbt_volume_transformation_voxels(vol.handle, None, C.byref(p)) == L.GBT_OK and p.value


@pytest.mark.parametrize("skip", [0, 1])
def test_batch_table_allocation_failure(gpu, skip):
    lib = L.lib()
    assert lib.gbt_debug_inject(L.INJECT_ALLOC, skip, 1) == L.GBT_OK
    b = C.c_void_p(0)
    assert lib.gbt_batch_create(16, 1024, C.byref(b)) == L.GBT_ERR_ALLOC
    assert b.value is None and "batch tables" in lib.gbt_last_error().decode()
    assert lib.gbt_batch_create(16, 1024, C.byref(b)) == L.GBT_OK and b.value
    assert lib.gbt_batch_destroy(b) == L.GBT_OK


def test_pending_launch_error_is_not_reported_by_the_next_call(gpu):
    lib = L.lib()
    vol = _surface_volume(gpu)
    V0, T0 = extract_mesh_device(vol)
    n0 = len(V0)
    verts = gpu.empty((n0, 3, 3), dtype=gpu.float32, device="cuda")
    tris = gpu.empty((n0, 3), dtype=gpu.int32, device="cuda")
    count = gpu.zeros(1, dtype=gpu.int64, device="cuda")
    stream = C.c_void_p(gpu.cuda.current_stream().cuda_stream)
    calls = {
        "noalloc": lambda: lib.gbt_extract_mesh_noalloc(vol.handle, C.c_void_p(verts.data_ptr()),
                                                        C.c_void_p(tris.data_ptr()), n0, 0,
                                                        C.c_void_p(count.data_ptr()), stream),
        "async": lambda: lib.gbt_extract_mesh_async(vol.handle, C.c_void_p(verts.data_ptr()),
                                                    C.c_void_p(tris.data_ptr()), n0, 0,
                                                    C.c_void_p(count.data_ptr()), stream),
        "reset": lambda: lib.gbt_volume_reset(vol.handle, stream),
    }
    for name, call in calls.items():
        assert lib.gbt_debug_inject(L.INJECT_LAUNCH_ERROR, 0, 0) == L.GBT_OK
        st = call()
        assert st == L.GBT_OK, (name, lib.gbt_last_error().decode())
        gpu.cuda.synchronize()
        if name != "reset":
            assert int(count.item()) == n0
            assert np.array_equal(verts.cpu().numpy().view(np.uint32), V0.cpu().numpy().view(np.uint32))
            assert np.array_equal(tris.cpu().numpy(), T0.cpu().numpy())


def test_synchronising_call_inside_graph_capture_is_reported(gpu):
    """Runs in a child process: an abandoned capture leaves the capturing
    stream and torch's graph pool in a state the rest of the suite should
    not inherit."""
    code = r'''
import ctypes as C, sys
sys.path[:0] = [%r, %r]
import torch
import numpy as np
from cuphoto import TSDFVolume, TSDFVolumeConfig, extract_mesh_device
from cuphoto import _lib as L
n = 64
tc = TSDFVolumeConfig(voxel_grid_size=(n, n, n), physical_size=(0.64, 0.64, 0.64), mode="fixed", arith="ieee",
                      max_weight=8)
vol = TSDFVolume(tc)
z, y, x = np.meshgrid(*[np.linspace(-1, 1, n)] * 3, indexing="ij")
vol.voxel_distances_data().copy_(torch.from_numpy((0.05 * (np.sqrt(x*x + y*y + z*z) - 0.6)).astype(np.float32)).cuda())
vol.voxel_weights_data().fill_(1.0)
V0, _ = extract_mesh_device(vol)     # the tile scratch exists before the capture
torch.cuda.synchronize()
lib = L.lib()
s = torch.cuda.Stream()
g = torch.cuda.CUDAGraph()
n_tris = C.c_int64(-1)
with torch.cuda.stream(s):
    g.capture_begin(capture_error_mode="thread_local")
    st = lib.gbt_extract_mesh(vol.handle, None, None, 0, 0, C.byref(n_tris), C.c_void_p(s.cuda_stream))
    msg = lib.gbt_last_error().decode()
    try:
        g.capture_end()
        ended = "ok"
    except RuntimeError as e:
        ended = "refused"
print("STATUS", st, "ENDED", ended)
print("MSG", msg)
torch.cuda.synchronize()
V1, _ = extract_mesh_device(vol)
print("AFTER", len(V0), len(V1))
''' % (os.path.join(HERE, ".."), os.path.join(HERE, "..", "cu-reconstruction_gb300"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    out = r.stdout
    assert r.returncode == 0, out + r.stderr[-3000:]
    line = [l for l in out.splitlines() if l.startswith("STATUS")][0].split()
    assert int(line[1]) == L.GBT_ERR_CUDA, out
    assert line[3] == "refused", out
    msg = [l for l in out.splitlines() if l.startswith("MSG")][0]
    assert "mesh extraction" in msg and "captur" in msg.lower(), msg
    after = [l for l in out.splitlines() if l.startswith("AFTER")][0].split()
    assert int(after[1]) == int(after[2]) > 0, out
