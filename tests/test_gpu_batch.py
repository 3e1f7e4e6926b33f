"""Batched integrate (many volumes, one persistent launch) against the
single-volume path, through the C ABI."""
import numpy as np
import pytest

from cuphoto import TSDFVolume, TSDFVolumeConfig
from cuphoto import synthetic as S
from cuphoto.batch import BatchIntegrator

from helpers import dev_depth

pytestmark = pytest.mark.gpu

SCENES = [((64, 64, 64), 10), ((40, 56, 72), 37), ((96, 80, 48), 140), ((20, 20, 20), 1), ((33, 17, 9), 5)]


def scene_data(gpu, mode, arith="reference", scenes=SCENES):
    cam = S.Camera.half()
    vols, depths, poses, cfgs = [], [], [], []
    for i, (grid, nf) in enumerate(scenes):
        seq = S.make_sequence(nf, scene_id=10 + i, camera=cam, trajectory="circle")
        tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=tuple(2.56 * g / max(grid) for g in grid),
                              global_offset=(-1.28, -1.0, -1.28), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx,
                              cy=cam.cy, mode=mode, arith=arith, max_weight=20)
        cfgs.append(tc)
        vols.append(TSDFVolume(tc))
        d = seq.depth_u16 if mode == "fixed" or i % 2 else seq.depth_m()
        depths.append([dev_depth(gpu, x) for x in d])
        poses.append(seq.poses)
    return cfgs, vols, depths, poses


@pytest.mark.parametrize("mode,arith", [("fixed", "ieee"), ("compat", "reference"), ("compat", "ieee")])
@pytest.mark.parametrize("brick", [0, 1])
def test_batch_equals_per_volume_integrate(gpu, mode, arith, brick):
    cfgs, vols, depths, poses = scene_data(gpu, mode, arith)
    BatchIntegrator(max_scenes=8, max_frames=512).integrate(vols, depths, poses, brick=brick, ctas_per_sm=4)
    gpu.cuda.synchronize()
    for tc, vol, ds, ps in zip(cfgs, vols, depths, poses):
        ref = TSDFVolume(tc)
        ref.integrate_sequence(ds, ps, frames_per_pass=32)
        gpu.cuda.synchronize()
        W0, W1 = ref.voxel_weights_data().cpu().numpy(), vol.voxel_weights_data().cpu().numpy()
        D0, D1 = ref.voxel_distances_data().cpu().numpy(), vol.voxel_distances_data().cpu().numpy()
        assert np.array_equal(W0, W1)
        assert np.array_equal(D0.view(np.uint32), D1.view(np.uint32))
    assert (vols[2].voxel_weights_data() > 0).float().mean().item() > 0.05


@pytest.mark.parametrize("mode,arith", [("fixed", "ieee"), ("compat", "reference")])
def test_batch_of_rows_of_4_equals_per_volume_integrate(gpu, mode, arith):
    """Every scene's x extent a multiple of 4: the batched kernel's instance
    without per-voxel count checks."""
    scenes = [s for s in SCENES if s[0][0] % 4 == 0]
    assert len(scenes) == 4
    cfgs, vols, depths, poses = scene_data(gpu, mode, arith, scenes)
    BatchIntegrator(max_scenes=8, max_frames=512).integrate(vols, depths, poses, brick=2, frames_per_launch=64)
    gpu.cuda.synchronize()
    for tc, vol, ds, ps in zip(cfgs, vols, depths, poses):
        ref = TSDFVolume(tc)
        ref.integrate_sequence(ds, ps, frames_per_pass=32)
        gpu.cuda.synchronize()
        assert np.array_equal(ref.voxel_weights_data().cpu().numpy(), vol.voxel_weights_data().cpu().numpy())
        assert np.array_equal(ref.voxel_distances_data().cpu().numpy().view(np.uint32),
                              vol.voxel_distances_data().cpu().numpy().view(np.uint32))


def test_batch_chunks_and_graph_replay(gpu):
    """Frames split over launches of 16 per scene, recorded in a CUDA graph and
    replayed: the same volumes as one direct call."""
    cfgs, vols, depths, poses = scene_data(gpu, "fixed", "ieee")
    b = BatchIntegrator(max_scenes=8, max_frames=512)
    stream = gpu.cuda.Stream()
    with gpu.cuda.stream(stream):
        for v in vols:
            v.reset()
        b.integrate(vols, depths, poses, frames_per_launch=16)
        gpu.cuda.synchronize()
        g = gpu.cuda.CUDAGraph()
        with gpu.cuda.graph(g, stream=stream):
            for v in vols:
                v.reset()
            b.integrate(vols, depths, poses, frames_per_launch=16)
    gpu.cuda.synchronize()
    for v in vols:
        v.voxel_weights_data().fill_(-7.0)
    gpu.cuda.synchronize()
    with gpu.cuda.stream(stream):
        g.replay()
    gpu.cuda.synchronize()
    for tc, vol, ds, ps in zip(cfgs, vols, depths, poses):
        ref = TSDFVolume(tc)
        ref.integrate_sequence(ds, ps, frames_per_pass=32)
        gpu.cuda.synchronize()
        assert np.array_equal(ref.voxel_weights_data().cpu().numpy(), vol.voxel_weights_data().cpu().numpy())
        assert np.array_equal(ref.voxel_distances_data().cpu().numpy().view(np.uint32),
                              vol.voxel_distances_data().cpu().numpy().view(np.uint32))


def test_batch_rejects_mixed_modes(gpu):
    from cuphoto import _lib as L
    import ctypes as C
    a = TSDFVolume(TSDFVolumeConfig(voxel_grid_size=(8, 8, 8), physical_size=(1, 1, 1)))
    b = TSDFVolume(TSDFVolumeConfig(voxel_grid_size=(8, 8, 8), physical_size=(1, 1, 1), mode="fixed"))
    d = gpu.zeros((4, 4), dtype=gpu.float32, device="cuda")
    bi = BatchIntegrator(4, 8)
    with pytest.raises(L.GbtError, match="same mode"):
        bi.integrate([a, b], [[d], [d]], [[np.array([1.0, 0, 0, 0, 0, 0, 0])]] * 2)


@pytest.mark.parametrize("mode,fmt", [("compat", "u16"), ("fixed", "u16"), ("compat", "f32")])
def test_streamed_from_host_equals_device_integrate(gpu, mode, fmt):
    """integrate_streamed copies window w + 1 from pinned host memory while
    window w integrates; the volumes equal a plain batched call on frames
    already on the device."""
    cfgs, vols, depths, poses = scene_data(gpu, mode)
    cam = S.Camera.half()
    host, dev = [], []
    for i, (grid, nf) in enumerate(SCENES):
        seq = S.make_sequence(nf, scene_id=10 + i, camera=cam, trajectory="circle")
        d = np.ascontiguousarray(seq.depth_u16 if fmt == "u16" else seq.depth_m())
        host.append(gpu.from_numpy(d.view(np.int16) if fmt == "u16" else d).pin_memory())
        dev.append(gpu.empty(host[-1].shape, dtype=host[-1].dtype, device="cuda"))
        depths[i] = [dev_depth(gpu, x) for x in d]
    b = BatchIntegrator(max_scenes=8, max_frames=512)
    b.integrate(vols, depths, poses, frames_per_launch=16)
    gpu.cuda.synchronize()
    expect = [(v.voxel_weights_data().cpu().numpy(), v.voxel_distances_data().cpu().numpy()) for v in vols]
    for v in vols:
        v.reset()
    b.integrate_streamed(vols, host, dev, poses, frames_per_launch=16)
    gpu.cuda.synchronize()
    for (W0, D0), v, h, d in zip(expect, vols, host, dev):
        assert np.array_equal(d.cpu().numpy(), h.numpy())
        assert np.array_equal(v.voxel_weights_data().cpu().numpy(), W0)
        assert np.array_equal(v.voxel_distances_data().cpu().numpy().view(np.uint32), D0.view(np.uint32))
    assert (expect[2][0] > 0).mean() > 0.05
