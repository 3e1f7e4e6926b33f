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
    assert lib.gbt_volume_destroy(None) == L.GBT_OK
