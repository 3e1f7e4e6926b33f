"""Autotuner for the integrate pass: brick shape x frames per pass x CTAs per SM.

Each candidate integrates the same frames into the volume (which is reset
before and after), timed with CUDA events on the launching stream; the
fastest is kept.  Results are cached per (GPU, grid, image size, mode,
arithmetic, build of the engine library, candidate sets) in a JSON file next
to the library.
"""
import json
import os

from . import _lib as L

BRICKS = (0, 1, 2, 3)
FRAMES = (8, 16, 32)
CTAS = (0, 4, 8, 16)   # 0: as many as the kernel keeps resident
CACHE = os.path.join(L.PKG_ROOT, "_build", "autotune.json")


def _key(vol, width, height):
    import torch
    c = vol.cfg
    try:
        st = os.stat(L.LIB_PATH)
        build = "%d-%d" % (st.st_size, st.st_mtime_ns)
    except OSError:
        build = "?"
    return "%s|%s|%dx%d|%s|%s|%s" % (torch.cuda.get_device_name(), "x".join(map(str, c.voxel_grid_size)), width,
                                     height, c.mode, c.arith, build)


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(key, value):
    """Adds one entry to the cache file.  The file is reloaded under an
    exclusive lock and the entry merged in, so ranks that tune at once keep
    each other's entries; each process writes through its own temporary file
    and renames it over the cache (readers never see a torn file)."""
    try:
        import fcntl
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        with open(CACHE + ".lock", "a") as lk:
            fcntl.flock(lk, fcntl.LOCK_EX)
            try:
                d = _load()
                d[key] = value
                tmp = "%s.%d.tmp" % (CACHE, os.getpid())
                with open(tmp, "w") as f:
                    json.dump(d, f, indent=1, sort_keys=True)
                os.replace(tmp, CACHE)
            finally:
                fcntl.flock(lk, fcntl.LOCK_UN)
    except OSError:
        pass


def tune_integrate(vol, depths, poses, depth_scale=0.001, bricks=BRICKS, frames=FRAMES, ctas=CTAS, repeats=2,
                   use_cache=True):
    """Returns {"brick", "frames", "ctas", "ns_per_update", "table"} for this volume and frame size."""
    import torch
    h, w = int(depths[0].shape[0]), int(depths[0].shape[1])
    key = _key(vol, w, h) + "|pass|%s|%s|%s" % (tuple(bricks), tuple(frames), tuple(ctas))
    cache = _load() if use_cache else {}
    if key in cache:
        return cache[key]
    nvox = 1
    for g in vol.voxel_grid_size():
        nvox *= g
    table = []
    best = None
    stream = torch.cuda.current_stream()
    for k in frames:
        n = min(len(depths), 2 * k)
        for b in bricks:
            for c in ctas:
                vol.reset()
                vol.integrate_sequence(depths[:n], poses[:n], frames_per_pass=k, depth_scale=depth_scale, brick=b,
                                       ctas_per_sm=c)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(repeats):
                    vol.integrate_sequence(depths[:n], poses[:n], frames_per_pass=k, depth_scale=depth_scale,
                                           brick=b, ctas_per_sm=c)
                e1.record(stream)
                e1.synchronize()
                ns = e0.elapsed_time(e1) * 1e6 / (repeats * n * nvox)
                table.append((b, k, c, ns))
                if best is None or ns < best[3]:
                    best = (b, k, c, ns)
    vol.reset()
    torch.cuda.synchronize()
    res = {"brick": best[0], "frames": best[1], "ctas": best[2], "ns_per_update": best[3], "table": table}
    if use_cache:
        _store(key, res)
    return res


WINDOWS = (32, 64, 128)


def tune_batched(vol, depths, poses, batch, depth_scale=0.001, bricks=(0, 1, 2, 3), windows=WINDOWS, ctas=(0, 16),
                 repeats=2, use_cache=True):
    """The same search for the batched path (gbt_integrate_batch with this one
    volume): brick shape x frames per launch window x CTAs per SM, timed on
    the whole sequence.  Returns {"brick", "frames", "ctas", "ns_per_update",
    "table"}; "frames" is the window."""
    import torch
    h, w = int(depths[0].shape[0]), int(depths[0].shape[1])
    key = _key(vol, w, h) + "|batched|%d|%s|%s|%s" % (len(depths), tuple(bricks), tuple(windows), tuple(ctas))
    cache = _load() if use_cache else {}
    if key in cache:
        return cache[key]
    nvox = 1
    for g in vol.voxel_grid_size():
        nvox *= g
    table = []
    best = None
    stream = torch.cuda.current_stream()
    for k in windows:
        for b in bricks:
            for c in ctas:
                def run():
                    vol.reset()
                    batch.integrate([vol], [depths], [poses], depth_scale=depth_scale, brick=b, ctas_per_sm=c,
                                    frames_per_launch=k)
                run()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(repeats):
                    run()
                e1.record(stream)
                e1.synchronize()
                ns = e0.elapsed_time(e1) * 1e6 / (repeats * len(depths) * nvox)
                table.append((b, k, c, ns))
                if best is None or ns < best[3]:
                    best = (b, k, c, ns)
    vol.reset()
    torch.cuda.synchronize()
    res = {"brick": best[0], "frames": best[1], "ctas": best[2], "ns_per_update": best[3], "table": table}
    if use_cache:
        _store(key, res)
    return res
