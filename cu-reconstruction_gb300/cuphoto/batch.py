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


def _frame_records(depths, poses, depth_scale):
    """gbt_frame records (numpy) for a list of (height, width) CUDA depth
    tensors or one (frames, height, width) tensor, with one pose per frame."""
    import numpy as np
    torch = _torch()
    rec = np.zeros(len(poses), L.frame_dtype())
    if len(poses) == 0:
        return rec
    if torch.is_tensor(depths) and depths.dim() == 3:
        if depths.shape[0] != len(poses):
            raise ValueError("%d frames but %d poses" % (depths.shape[0], len(poses)))
        L.device_tensor(depths, "depths")
        first = depths[0]
        rec["depth"] = first.data_ptr() + np.arange(len(poses), dtype=np.uint64) * (depths.stride(0) *
                                                                                     depths.element_size())
    else:
        if len(depths) != len(poses):
            raise ValueError("%d frames but %d poses" % (len(depths), len(poses)))
        first = depths[0]
        for d in depths:
            L.device_tensor(d, "depth")
            if d.shape != first.shape or d.dtype != first.dtype or d.stride() != first.stride():
                return np.concatenate([np.frombuffer(bytes(make_frame(d, p, depth_scale)), L.frame_dtype())
                                       for d, p in zip(depths, poses)])
        rec["depth"] = [d.data_ptr() for d in depths]
    # one frame describes them all: format, size and pitch checks as make_frame does them
    f = make_frame(first, poses[0], depth_scale)
    rec["pitch_bytes"] = f.pitch_bytes
    rec["width"], rec["height"] = f.width, f.height
    rec["format"] = f.format
    rec["depth_scale"] = f.depth_scale
    rec["pose"] = np.asarray(poses, dtype=np.float64).reshape(len(poses), 7)
    return rec


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
        """depth_lists[i]: scene i's frames, a list of (height, width) CUDA
        tensors (float32 metres or uint16 bits) or one (frames, height, width)
        tensor; pose_lists[i]: one pose per frame."""
        import numpy as np
        items = (L.BatchItem * len(volumes))()
        parts = []
        n = 0
        for k, (vol, ds, ps) in enumerate(zip(volumes, depth_lists, pose_lists)):
            rec = _frame_records(ds, ps, depth_scale)
            items[k] = L.BatchItem(vol.handle.value, n, len(rec))
            parts.append(rec)
            n += len(rec)
        fr = np.concatenate(parts) if parts else np.zeros(0, L.frame_dtype())
        self._keep = (items, fr)
        L.check(self._lib.gbt_integrate_batch(self._h, items, len(volumes), fr.ctypes.data_as(C.POINTER(L.Frame)), n,
                                              int(frames_per_launch), int(brick), int(ctas_per_sm),
                                              _stream_handle(stream)))

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
            self.integrate([volumes[i] for i in sel], [device_frames[i][w0:w0 + k_w] for i in sel],
                           [pose_lists[i][w0:w0 + k_w] for i in sel], depth_scale=depth_scale, brick=brick,
                           ctas_per_sm=ctas_per_sm, frames_per_launch=k_w, stream=cur)
        # the device buffers are also used on the copy stream
        for d in device_frames:
            d.record_stream(copy_stream)
