"""Many volumes integrated by persistent launches that cover all scenes
(gbt_integrate_batch).

Each scene has its own volume (any grid size), depth frames and poses.  One
launch applies the next `frames_per_launch` (<= 128) frames of every scene.
A call records into a CUDA graph unchanged (the batch object owns its device
tables); a graph should hold one call per BatchIntegrator.
"""
import ctypes as C

from . import _lib as L
from .tsdf import _stream_handle, make_frame


class BatchIntegrator:
    def __init__(self, max_scenes=64, max_frames=4096):
        self._lib = L.lib()
        self._h = C.c_void_p()
        L.check(self._lib.gbt_batch_create(int(max_scenes), int(max_frames), C.byref(self._h)))
        self.max_scenes = max_scenes
        self.max_frames = max_frames
        self._keep = None

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.gbt_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def integrate(self, volumes, depth_lists, pose_lists, depth_scale=0.001, brick=0, ctas_per_sm=0,
                  frames_per_launch=L.MAX_FRAMES_PER_SCENE_PASS, stream=None):
        items, frames = [], []
        for vol, ds, ps in zip(volumes, depth_lists, pose_lists):
            items.append(L.BatchItem(vol.handle.value, len(frames), len(ds)))
            frames.extend(make_frame(d, p, depth_scale) for d, p in zip(ds, ps))
        it = (L.BatchItem * len(items))(*items)
        fr = (L.Frame * len(frames))(*frames)
        self._keep = (it, fr)
        L.check(self._lib.gbt_integrate_batch(self._h, it, len(items), fr, len(frames), int(frames_per_launch),
                                              int(brick), int(ctas_per_sm), _stream_handle(stream)))
