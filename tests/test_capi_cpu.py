"""The C-ABI library without a GPU: it loads, exports every entry point the
header declares, its structs have the header's layout, and argument errors
are reported before any CUDA call."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "..", "include", "gbt_tsdf.h")


def declared_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:gbt_status|const char\*)\s+(gbt_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_declared_symbol(engine_lib):
    lib = engine_lib.lib()
    names = declared_functions()
    assert len(names) >= 11
    sig_names = {n for n, _, _ in engine_lib.SIGNATURES}
    for n in names:
        assert hasattr(lib, n), n
        assert n in sig_names, n
    assert lib.gbt_version().decode().startswith("gbt-tsdf")


def test_struct_layout_matches_header(engine_lib):
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "gbt_tsdf.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(gbt_volume_cfg), offsetof(gbt_volume_cfg, mode),
         offsetof(gbt_volume_cfg, memory), sizeof(gbt_volume_info), offsetof(gbt_volume_info, tsdf),
         sizeof(gbt_frame), offsetof(gbt_frame, pose));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "l")
        subprocess.check_call(["gcc", "-I" + os.path.dirname(HEADER), c, "-o", exe])
        got = [int(x) for x in subprocess.check_output([exe]).split()]
    L = engine_lib
    want = [C.sizeof(L.VolumeCfg), L.VolumeCfg.mode.offset, L.VolumeCfg.memory.offset, C.sizeof(L.VolumeInfo),
            L.VolumeInfo.tsdf.offset, C.sizeof(L.Frame), L.Frame.pose.offset]
    assert got == want


def _cfg(L, **kw):
    c = L.VolumeCfg()
    for i in range(3):
        c.voxel_grid_size[i] = 8
        c.physical_size[i] = 1.0
    c.max_weight = 16
    c.focal_x = c.focal_y = 100.0
    for k, v in kw.items():
        if isinstance(v, tuple):
            arr = getattr(c, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(c, k, v)
    return c


@pytest.mark.parametrize("kw,msg", [
    (dict(voxel_grid_size=(0, 8, 8)), "voxel_grid_size[0] is 0"),
    (dict(physical_size=(1.0, -1.0, 1.0)), "physical_size[1]"),
    (dict(mode=7), "unknown mode"),
    (dict(arith=3), "unknown arith"),
    (dict(memory=2), "unknown memory"),
    (dict(mode=1, max_weight=0.0), "max_weight"),
    (dict(voxel_grid_size=(2048, 2048, 1024)), "limit is 2^32-1"),
    # a product of 2^72: rejected without an overflowing multiplication
    (dict(voxel_grid_size=(1 << 24, 1 << 24, 1 << 24)), "limit is 2^32-1"),
])
def test_volume_create_rejects_bad_config(engine_lib, kw, msg):
    L = engine_lib
    lib = L.lib()
    h = C.c_void_p()
    st = lib.gbt_volume_create(C.byref(_cfg(L, **kw)), None, C.byref(h))
    assert st == L.GBT_ERR_INVALID_ARG
    assert msg in lib.gbt_last_error().decode()
    assert not h.value


def test_null_arguments_are_rejected(engine_lib):
    L = engine_lib
    lib = L.lib()
    assert lib.gbt_volume_create(None, None, None) == L.GBT_ERR_INVALID_ARG
    f = L.Frame()
    assert lib.gbt_integrate(None, C.byref(f), 1, None) == L.GBT_ERR_INVALID_ARG
    n = C.c_int64()
    assert lib.gbt_extract_mesh(None, None, None, 0, 0, C.byref(n), None) == L.GBT_ERR_INVALID_ARG
    assert lib.gbt_volume_get_info(None, None) == L.GBT_ERR_INVALID_ARG
    cfg = L.VolumeCfg()
    assert lib.gbt_volume_get_cfg(None, C.byref(cfg)) == L.GBT_ERR_INVALID_ARG
    assert b"gbt_volume_get_cfg" in lib.gbt_last_error()
    assert lib.gbt_volume_check(None, None) == L.GBT_ERR_INVALID_ARG
    assert lib.gbt_debug_inject(L.INJECT_HOLD_COPY, 0, -1) == L.GBT_ERR_INVALID_ARG
    assert lib.gbt_debug_inject(L.INJECT_NONE, 0, 0) == L.GBT_OK
    assert lib.gbt_volume_destroy(None) == L.GBT_OK


def test_mesh_index_range_is_checked_first(engine_lib):
    """A capacity whose int32 triangle indices would pass INT32_MAX, or a
    negative index base, is refused before the volume handle is used (the
    handle here is a placeholder the library never reads)."""
    L = engine_lib
    lib = L.lib()
    fake = C.create_string_buffer(4096)
    buf = C.create_string_buffer(64)
    n = C.c_int64()
    # (2^29 triangles from 2^29 end exactly at INT32_MAX; one more passes it)
    for cap, base in [(1, 2 ** 31 - 2), (2, -1), (2 ** 29 + 1, 2 ** 29)]:
        st = lib.gbt_extract_mesh(C.cast(fake, C.c_void_p), buf, buf, cap, base, C.byref(n), None)
        assert st == L.GBT_ERR_INVALID_ARG and b"int32" in lib.gbt_last_error()
        st = lib.gbt_extract_mesh_noalloc(C.cast(fake, C.c_void_p), buf, buf, cap, base, buf, None)
        assert st == L.GBT_ERR_INVALID_ARG and b"int32" in lib.gbt_last_error()


def test_diff_rejects_bad_arguments(engine_lib):
    """Argument checks of the differentiable entry points run before any
    device work (no GPU needed)."""
    from cuphoto import _lib as L
    lib = L.lib()
    c = L.DiffCfg()
    for i in range(3):
        c.voxel_grid_size[i] = 8
        c.voxel_size[i] = 0.01
    c.focal_x = c.focal_y = 50.0
    c.truncation, c.max_weight, c.max_depth = 0.03, 8.0, 4.0
    c.width, c.height, c.dtype = 16, 12, 0
    p = C.c_void_p(16)
    # NULL tensors
    assert lib.gbt_diff_forward(C.byref(c), None, p, None, None, p, 1, p, p, None) == L.GBT_ERR_INVALID_ARG
    # more than one chunk of frames and no checkpoints for the adjoint
    assert lib.gbt_diff_backward(C.byref(c), p, None, p, p, None, p, 9, p, p, p, p, None, None,
                                 None) == L.GBT_ERR_INVALID_ARG
    assert b"checkpoints" in lib.gbt_last_error()
    c.dtype = 2
    assert lib.gbt_diff_forward(C.byref(c), p, p, None, None, p, 1, p, p, None) == L.GBT_ERR_INVALID_ARG
    c.dtype = 0
    c.truncation = 0.0
    assert lib.gbt_diff_forward(C.byref(c), p, p, None, None, p, 1, p, p, None) == L.GBT_ERR_INVALID_ARG
    c.truncation = 0.03
    # one axis of 2^31 + 5 voxels: fewer than 2^32 in all, but not a 32-bit signed extent
    c.voxel_grid_size[0], c.voxel_grid_size[1], c.voxel_grid_size[2] = (1 << 31) + 5, 1, 1
    assert lib.gbt_diff_forward(C.byref(c), p, p, None, None, p, 1, p, p, None) == L.GBT_ERR_INVALID_ARG
    assert b"above 2^24" in lib.gbt_last_error()


def test_se3_helpers():
    """so3_exp against Rodrigues in numpy; se3_gradient against a central
    difference of a smooth function of (R, t) under the left update."""
    import numpy as np
    import torch
    import diffcase
    from cuphoto.diff import checkpoint_shape, se3_gradient, se3_left_update, so3_exp
    rng = np.random.default_rng(0)
    phi = rng.normal(size=(5, 3))
    phi[0] = 0
    E = so3_exp(torch.as_tensor(phi)).numpy()
    for k in range(5):
        np.testing.assert_allclose(E[k], diffcase.rot_exp(phi[k]), atol=1e-14)
    R = so3_exp(torch.as_tensor(rng.normal(size=(3, 3))))
    t = torch.as_tensor(rng.normal(size=(3, 3)))
    P = torch.as_tensor(rng.normal(size=(7, 3)))

    def f(R, t):   # any smooth function of the world-to-camera poses
        c = torch.einsum("fij,pj->fpi", R, P) + t[:, None, :]
        return (torch.sin(c) * c).sum()

    Rv, tv = R.clone().requires_grad_(True), t.clone().requires_grad_(True)
    f(Rv, tv).backward()
    g = se3_gradient(Rv.grad, tv.grad, R, t)
    xi = torch.as_tensor(rng.normal(size=(3, 6)))
    h = 1e-6
    fd = (f(*se3_left_update(R, t, h * xi)) - f(*se3_left_update(R, t, -h * xi))) / (2 * h)
    assert abs(float(fd) - float((g * xi).sum())) <= 1e-7 * abs(float(fd))
    # the camera centre stays put under a pure rotation update
    xi[:, :3] = 0
    R2, t2 = se3_left_update(R, t, xi)
    c1 = -(R.transpose(1, 2) @ t[..., None])
    c2 = -(R2.transpose(1, 2) @ t2[..., None])
    np.testing.assert_allclose(c1.numpy(), c2.numpy(), atol=1e-12)
    assert checkpoint_shape(16, (2, 3, 4)) == (1, 2, 2, 3, 4)
    assert checkpoint_shape(8, (2, 3, 4))[0] == 0 and checkpoint_shape(17, (1, 1, 1))[0] == 2


def test_volume_files_rejected_before_any_device_work(engine_lib, tmp_path):
    """gbt_volume_save / gbt_volume_load argument and format checks."""
    L = engine_lib
    lib = L.lib()
    out = C.c_void_p()
    assert lib.gbt_volume_save(None, b"/nonexistent/x", None) == L.GBT_ERR_INVALID_ARG
    assert lib.gbt_volume_load(None, None, C.byref(out)) == L.GBT_ERR_INVALID_ARG
    missing = str(tmp_path / "missing.gbtv").encode()
    assert lib.gbt_volume_load(missing, None, C.byref(out)) == L.GBT_ERR_IO
    assert b"cannot open" in lib.gbt_last_error()
    bad = tmp_path / "bad.gbtv"
    bad.write_bytes(b"NOTAVOLUME" + bytes(300))
    assert lib.gbt_volume_load(str(bad).encode(), None, C.byref(out)) == L.GBT_ERR_IO
    assert b"not a volume file" in lib.gbt_last_error()
    short = tmp_path / "short.gbtv"
    short.write_bytes(L.VOLUME_FILE_MAGIC + bytes(10))
    assert lib.gbt_volume_load(str(short).encode(), None, C.byref(out)) == L.GBT_ERR_IO
    # a header whose voxel count disagrees with its grid
    cfg = L.VolumeCfg()
    cfg.voxel_grid_size[0] = cfg.voxel_grid_size[1] = cfg.voxel_grid_size[2] = 4
    head = bytearray(L.VOLUME_FILE_HEADER_BYTES)
    head[0:8] = L.VOLUME_FILE_MAGIC
    head[8:12] = L.VOLUME_FILE_HEADER_BYTES.to_bytes(4, "little")
    head[12:16] = C.sizeof(L.VolumeCfg).to_bytes(4, "little")
    head[16:24] = (65).to_bytes(8, "little")
    head[24:24 + C.sizeof(cfg)] = bytes(cfg)
    mism = tmp_path / "mismatch.gbtv"
    mism.write_bytes(bytes(head))
    assert lib.gbt_volume_load(str(mism).encode(), None, C.byref(out)) == L.GBT_ERR_IO
    assert b"voxel count" in lib.gbt_last_error()
    # a grid of 2^64 voxels, whose count wraps to the header's 0 in 64 bits
    cfg.voxel_grid_size[0] = cfg.voxel_grid_size[1] = 1 << 22
    cfg.voxel_grid_size[2] = 1 << 20
    head[16:24] = (0).to_bytes(8, "little")
    head[24:24 + C.sizeof(cfg)] = bytes(cfg)
    huge = tmp_path / "huge.gbtv"
    huge.write_bytes(bytes(head))
    assert lib.gbt_volume_load(str(huge).encode(), None, C.byref(out)) == L.GBT_ERR_IO
    assert b"voxel count" in lib.gbt_last_error()
    assert not out.value


def test_bulk_frame_records_match_single_frames(engine_lib, monkeypatch):
    """The batch API's numpy frame records are byte-identical to the ctypes
    gbt_frame of each frame, for a list of images and for one 3-D tensor
    (CPU tensors, whose pointers and strides alone are read: the device check
    is lifted here, where nothing is launched)."""
    torch = pytest.importorskip("torch")
    import numpy as np
    from cuphoto.batch import _frame_records
    from cuphoto.tsdf import make_frame
    L = engine_lib
    frames = torch.zeros((5, 48, 64), dtype=torch.int16)
    with pytest.raises(ValueError, match="CUDA tensor"):
        make_frame(frames[0], np.zeros(7), 0.001)
    with pytest.raises(ValueError, match="CUDA tensor"):
        _frame_records(frames, np.zeros((5, 7)), 0.001)
    monkeypatch.setattr(L, "device_tensor", lambda t, name: t)
    poses = np.random.default_rng(0).normal(size=(5, 7))
    single = b"".join(bytes(make_frame(frames[k], poses[k], 0.001)) for k in range(5))
    assert _frame_records(frames, poses, 0.001).tobytes() == single
    assert _frame_records([frames[k] for k in range(5)], list(poses), 0.001).tobytes() == single
    # pitched rows and a float image among uint16 ones
    wide = torch.zeros((48, 80), dtype=torch.float32)[:, :64]
    mixed = _frame_records([frames[0], wide], list(poses[:2]), 0.002)
    assert mixed["format"].tolist() == [L.DEPTH_U16, L.DEPTH_F32_M]
    assert mixed["pitch_bytes"].tolist() == [128, 320]
    with pytest.raises(ValueError):
        _frame_records(frames, poses[:4], 0.001)


def test_autotune_cache_round_trip(engine_lib, tmp_path, monkeypatch):
    """The tuner's JSON cache: stored through a per-process temporary file,
    read back, and an unreadable cache counts as empty (tuning again)."""
    from cuphoto import autotune as A
    monkeypatch.setattr(A, "CACHE", str(tmp_path / "tune" / "autotune.json"))
    assert A._load() == {}
    A._store("k", {"brick": 2, "frames": 64, "ctas": 0})
    assert A._load() == {"k": {"brick": 2, "frames": 64, "ctas": 0}}
    A._store("k2", {"brick": 1, "frames": 32, "ctas": 16})
    assert sorted(A._load()) == ["k", "k2"]
    assert sorted(p.name for p in (tmp_path / "tune").iterdir()) == ["autotune.json", "autotune.json.lock"]
    (tmp_path / "tune" / "autotune.json").write_text("{not json")
    assert A._load() == {}


def _store_keys(cache, rank, n):
    from cuphoto import autotune as A
    A.CACHE = cache
    for i in range(n):
        A._store("rank%d-%d" % (rank, i), {"brick": rank, "frames": i, "ctas": 0})


def test_autotune_cache_keeps_every_process_entries(engine_lib, tmp_path):
    """Processes that tune at once (ranks of one job) all keep their entries:
    each store reloads the file under a lock and merges its key in."""
    import multiprocessing as mp
    cache = str(tmp_path / "autotune.json")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_store_keys, args=(cache, r, 8)) for r in range(3)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    import json
    with open(cache) as f:
        d = json.load(f)
    assert sorted(d) == sorted("rank%d-%d" % (r, i) for r in range(3) for i in range(8))


def test_injected_allocation_failure_before_any_device_work(engine_lib):
    """gbt_debug_inject: the volume's first allocation fails on the host side;
    the call reports GBT_ERR_ALLOC with the size in gbt_last_error and leaves
    no handle (the reference's constructor logs such a failure and carries
    on, tsdf_volume.cu:203-209)."""
    L = engine_lib
    lib = L.lib()
    assert lib.gbt_debug_inject(L.INJECT_ALLOC, 0, 1) == L.GBT_OK
    c = _cfg(L)
    out = C.c_void_p(12345)
    st = lib.gbt_volume_create(C.byref(c), None, C.byref(out))
    assert st == L.GBT_ERR_ALLOC
    assert out.value is None
    msg = lib.gbt_last_error().decode()
    assert "allocating 4096 bytes for the volume" in msg and "out of memory" in msg
    # the same for the batch tables' pinned staging copy
    assert lib.gbt_debug_inject(L.INJECT_ALLOC, 0, 1) == L.GBT_OK
    b = C.c_void_p(1)
    assert lib.gbt_batch_create(4, 16, C.byref(b)) == L.GBT_ERR_ALLOC
    assert b.value is None and "batch tables" in lib.gbt_last_error().decode()
    assert lib.gbt_debug_inject(L.INJECT_NONE, 0, 0) == L.GBT_OK
    assert lib.gbt_debug_inject(L.INJECT_ALLOC, -1, 1) == L.GBT_ERR_INVALID_ARG
    assert lib.gbt_debug_inject(7, 0, 0) == L.GBT_ERR_INVALID_ARG
