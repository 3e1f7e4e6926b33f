"""The streamed pass kernel (brick 8 of gbt_integrate_tuned): bricks' distances
and weights copied into shared memory by the Tensor Memory Accelerator, a few
bricks ahead of the one being updated.  Its volumes must be those of the
gathering pass kernel (brick 0, the same 32x4x4 bricks) bit for bit, and of
the oracle in IEEE arithmetic; its bounded wait is exercised by holding back
one copy (host-side failure injection), which must mark the volume, not hang
or fault the GPU."""
import numpy as np
import pytest

from cuphoto import TSDFVolume
from cuphoto import _lib as L

from helpers import circle_case, dev_depth, engine_run, frontal_case, oracle_run

pytestmark = pytest.mark.gpu

STREAMED = 8


def _volumes(gpu, tc, depths, poses, k, brick, ctas_per_sm=0):
    _, D, W = engine_run(gpu, tc, depths, poses, k=k, brick=brick, ctas_per_sm=ctas_per_sm)
    return D, W


def _same(a, b):
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))


@pytest.mark.parametrize("k", [1, 5, 16])
@pytest.mark.parametrize("mode,arith,fmt", [("compat", "reference", "u16"), ("compat", "ieee", "f32"),
                                           ("fixed", "ieee", "u16"), ("fixed", "ieee", "f32")])
def test_streamed_pass_is_bit_identical(gpu, mode, arith, fmt, k):
    """Brick 8 = brick 0, bit for bit, for both sample formats and the three
    arithmetics, one to 16 frames per pass."""
    seq, tc = circle_case(n=96, frames=16, mode=mode, max_weight=8)
    tc.arith = arith
    imgs = list(seq.depth_u16) if fmt == "u16" else list(seq.depth_m())
    ref = _volumes(gpu, tc, imgs, seq.poses, k, 0)
    out = _volumes(gpu, tc, imgs, seq.poses, k, STREAMED)
    assert (ref[1] > 0).mean() > 0.05
    _same(out, ref)


@pytest.mark.parametrize("grid", [(84, 50, 37), (4, 9, 5), (132, 3, 70)])
def test_streamed_pass_ragged_grids_vs_oracle(gpu, oracle, grid):
    """Grids whose extents are not multiples of the 32x4x4 brick (the copies of
    the last bricks read zeros past the volume's end, which are never
    stored): bit-exact against the oracle (compat, IEEE arithmetic)."""
    seq, tc = frontal_case(*grid, frames=6, arith="ieee")
    depths = list(seq.depth_m())
    D, W = _volumes(gpu, tc, depths, seq.poses, 3, STREAMED)
    Do, Wo = oracle_run(oracle, tc, depths, seq.poses)
    assert (Wo > 0).any()
    assert np.array_equal(W, Wo)
    assert np.array_equal(D.view(np.uint32), Do.view(np.uint32))


@pytest.mark.parametrize("ctas", [1, 2])
def test_streamed_pass_many_bricks_per_cta(gpu, ctas):
    """Few CTAs over a 512x512x384 volume (196,608 bricks: 1293 per CTA at one
    CTA per SM): each CTA culls its bricks in many rounds of 128, and the
    indices of its 256-entry ring of queued bricks wrap around (more live
    bricks per CTA than the ring holds) while copies are in flight; the
    volume is that of brick 0."""
    seq, tc = circle_case(n=256, frames=4, physical=2.56)
    tc.voxel_grid_size = (512, 512, 384)
    tc.physical_size = (5.12, 5.12, 3.84)
    tc.global_offset = (-2.56, -2.56, -1.92)
    imgs = list(seq.depth_u16)
    ref = _volumes(gpu, tc, imgs, seq.poses, 1, 0)
    out = _volumes(gpu, tc, imgs, seq.poses, 1, STREAMED, ctas_per_sm=ctas)
    assert (ref[1] > 0).mean() > 0.05
    _same(out, ref)


@pytest.mark.parametrize("fmt", ["u16", "f32"])
def test_streamed_pass_pitched_images(gpu, fmt):
    """Depth images with 3 unused elements after each row (the samples are
    read through the pitch): brick 8 = brick 0, bit for bit."""
    from test_gpu_integrate import _pitched
    seq, tc = circle_case(n=96, frames=8, max_weight=8)
    imgs = list(seq.depth_u16) if fmt == "u16" else list(seq.depth_m())
    dd = [_pitched(gpu, d, 3) for d in imgs]
    out = {}
    for brick in (0, STREAMED):
        vol = TSDFVolume(tc)
        vol.integrate_frames(dd, seq.poses, depth_scale=0.001, brick=brick)
        gpu.cuda.synchronize()
        out[brick] = (vol.voxel_distances_data().cpu().numpy(), vol.voxel_weights_data().cpu().numpy())
    assert (out[0][1] > 0).mean() > 0.05
    _same(out[STREAMED], out[0])


def test_streamed_pass_rejects_what_it_cannot_run(gpu):
    seq, tc = frontal_case(77, 40, 32, frames=17)
    vol = TSDFVolume(tc)
    dd = [dev_depth(gpu, d) for d in seq.depth_u16]
    with pytest.raises(L.GbtError, match="multiple of 4"):
        vol.integrate_frames(dd[:1], seq.poses[:1], brick=STREAMED)
    seq, tc = frontal_case(80, 40, 32, frames=17)
    vol = TSDFVolume(tc)
    dd = [dev_depth(gpu, d) for d in seq.depth_u16]
    with pytest.raises(L.GbtError, match="up to 16 frames"):
        vol.integrate_frames(dd, seq.poses, brick=STREAMED)
    with pytest.raises(L.GbtError, match="outside 0..8"):
        vol.integrate_frames(dd[:1], seq.poses[:1], brick=9)


def test_held_copy_expires_and_marks_the_volume(gpu):
    """Failure injection: the first copy of the first CTA is never issued, so
    that CTA's bounded wait gives up after about a second.  The pass returns,
    the GPU stays usable, gbt_volume_check reports GBT_ERR_TIMEOUT once (the
    mark is cleared), and after a reset the same pass gives brick 0's volume.
    One CTA per SM: the first CTA's bricks (0, 152, 304, ... of the 960)
    include some in view of the camera, so it has a first copy to hold."""
    seq, tc = frontal_case(96, 80, 64, frames=4)
    dd = [dev_depth(gpu, d) for d in seq.depth_u16]
    vol = TSDFVolume(tc)
    vol.check()
    L.check(L.lib().gbt_debug_inject(L.INJECT_HOLD_COPY, 0, 1))
    try:
        vol.integrate_frames(dd, seq.poses, brick=STREAMED, ctas_per_sm=1)
        with pytest.raises(L.GbtError, match="gave up waiting"):
            vol.check()
    finally:
        L.lib().gbt_debug_inject(L.INJECT_NONE, 0, 0)
    vol.check()   # the mark was cleared
    vol.reset()
    vol.integrate_frames(dd, seq.poses, brick=STREAMED)
    vol.check()
    gpu.cuda.synchronize()
    out = (vol.voxel_distances_data().cpu().numpy(), vol.voxel_weights_data().cpu().numpy())
    ref = _volumes(gpu, tc, list(seq.depth_u16), seq.poses, 4, 0)
    assert (ref[1] > 0).mean() > 0.05
    _same(out, ref)
