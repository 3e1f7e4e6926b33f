"""Many volumes integrated by persistent launches that cover all scenes
(gbt_integrate_batch).

Each scene has its own volume (any grid size), depth frames and poses.  One
launch applies the next `frames_per_launch` (<= 128) frames of every scene.
A call records into a CUDA graph unchanged (the batch object owns its device
tables); a graph should hold one call per BatchIntegrator.
"""
import ctypes as C

from . import _lib as L
from .tsdf import _stream_handle, _torch, make_frame


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

    def integrate_streamed(self, volumes, host_frames, device_frames, pose_lists, depth_scale=0.001, brick=0,
                           ctas_per_sm=0, frames_per_launch=L.MAX_FRAMES_PER_SCENE_PASS, stream=None,
                           copy_stream=None):
        """integrate() from host memory, the copies overlapped with the launches.

        host_frames[i]: scene i's depth frames as one pinned host tensor
        (frames, height, width); device_frames[i]: a device tensor of the same
        shape and dtype that receives them.  The frames of launch window w + 1
        are copied on `copy_stream` while window w is integrated on `stream`
        (one gbt_integrate_batch call per window; the volumes see the same
        frames in the same order, so the result equals integrate()).  The
        first window takes the remainder of the longest sequence modulo
        frames_per_launch, so the copy that nothing overlaps is the shortest.
        The work is queued and the call returns; it is done when `stream` is."""
        torch = _torch()
        cur = stream if stream is not None else torch.cuda.current_stream()
        if copy_stream is None:
            if getattr(self, "_copy_stream", None) is None:
                self._copy_stream = torch.cuda.Stream()
            copy_stream = self._copy_stream
        k = int(frames_per_launch)
        longest = max((int(h.shape[0]) for h in host_frames), default=0)
        starts = list(range(longest % k, longest, k))
        if longest % k:
            starts.insert(0, 0)
        # the device buffers may still be read by earlier work on `cur`
        copy_stream.wait_stream(cur)
        for w, w0 in enumerate(starts):
            k_w = (starts[w + 1] if w + 1 < len(starts) else longest) - w0
            with torch.cuda.stream(copy_stream):
                for h, d in zip(host_frames, device_frames):
                    if h.shape[0] > w0:
                        d[w0:w0 + k_w].copy_(h[w0:w0 + k_w], non_blocking=True)
                done = torch.cuda.Event()
                done.record(copy_stream)
            cur.wait_event(done)
            sel = [i for i, h in enumerate(host_frames) if h.shape[0] > w0]
            frames = [[device_frames[i][f] for f in range(w0, min(w0 + k_w, host_frames[i].shape[0]))] for i in sel]
            self.integrate([volumes[i] for i in sel], frames, [pose_lists[i][w0:w0 + k_w] for i in sel],
                           depth_scale=depth_scale, brick=brick, ctas_per_sm=ctas_per_sm, frames_per_launch=k_w,
                           stream=cur)
        # the device buffers are also used on the copy stream
        for d in device_frames:
            d.record_stream(copy_stream)
