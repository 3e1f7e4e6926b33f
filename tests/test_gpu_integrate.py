"""Integrate on the GPU against the CPU oracle (through the C ABI)."""
import os

import numpy as np
import pytest

from cuphoto import TSDFVolumeConfig
from cuphoto import synthetic as S

from helpers import circle_case, dev_depth, engine_run, frontal_case, oracle_run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [1, 3, 32])
@pytest.mark.parametrize("case", ["frontal", "circle", "odd"])
def test_compat_ieee_bitexact_vs_oracle(gpu, oracle, case, k):
    """Compat mode in IEEE arithmetic = the oracle's operations: bit-exact,
    whatever the number of frames fused per pass."""
    if case == "frontal":
        seq, tc = frontal_case(frames=7, arith="ieee")
    elif case == "circle":
        seq, tc = circle_case(frames=7, arith="ieee")
    else:  # x not a multiple of 4 (scalar tail path), y/z not multiples of 8
        seq, tc = frontal_case(77, 50, 37, frames=7, arith="ieee")
    depths = list(seq.depth_m())
    _, D, W = engine_run(gpu, tc, depths, seq.poses, k=k)
    Do, Wo = oracle_run(oracle, tc, depths, seq.poses)
    assert (Wo > 0).mean() > 0.05
    assert np.array_equal(W, Wo)
    assert np.array_equal(D.view(np.uint32), Do.view(np.uint32))


@pytest.mark.parametrize("k", [1, 3])
def test_compat_ieee_zero_z_voxels_vs_oracle(gpu, oracle, k):
    """Voxels with world z == 0 or camera z == 0 read pixel (0, 0)."""
    from test_gpu_reference import zero_z_case
    tc, depths, poses = zero_z_case()
    tc.arith = "ieee"
    _, D, W = engine_run(gpu, tc, depths, poses, k=k)
    Do, Wo = oracle_run(oracle, tc, depths, poses)
    assert (Wo[16] == 3).all() and (Wo[20] == 3).all()
    assert np.array_equal(W, Wo)
    assert np.array_equal(D.view(np.uint32), Do.view(np.uint32))


def tiny_depth_case():
    """A 32x24x32 grid of 1/64 m voxels (every size and offset exact in
    float) whose every voxel projects into the 64x48 image of a camera
    1.9-2.1 m away (identity rotation); voxel centres reach from world
    z = -0.4375 up to 0.0469, layer 28 at exactly 0, so samples of any size
    update most of the volume (compat distances are measured from world z).
    Layer 28 reads pixel (0, 0) (world z == 0), whose raw values 2, 5, 7 make
    the layer's distances, the samples' running average, subnormal at a
    subnormal scale."""
    vs = 1.0 / 64
    n = (32, 24, 32)
    tc = TSDFVolumeConfig(voxel_grid_size=n, physical_size=tuple(vs * k for k in n),
                          global_offset=(-0.25, -0.1875, -28.5 * vs), focal_x=100.0, focal_y=100.0, cx=31.5,
                          cy=23.5, camera_width=64, camera_height=48, arith="ieee")
    rng = np.random.default_rng(11)
    d16 = []
    for raw00 in (2, 5, 7):
        d = rng.integers(1, 2000, (48, 64)).astype(np.uint16)
        d[rng.random(d.shape) < 0.05] = 0
        d[0, 0] = raw00
        d16.append(d)
    poses = [np.array([1.0, 0, 0, 0, 0.0, 0.0, 2.0]), np.array([1.0, 0, 0, 0, 0.02, -0.01, 1.9]),
             np.array([1.0, 0, 0, 0, -0.03, 0.02, 2.1])]
    return tc, d16, poses


@pytest.mark.parametrize("scale", [1e-39, 2.0 ** -126, 0.0125])
@pytest.mark.parametrize("k", [1, 3])
def test_uint16_depth_scales_vs_oracle(gpu, oracle, scale, k):
    """uint16 depth at depth scales that take either form of the sample
    conversion: a subnormal scale (the conversion and multiply), the smallest
    normal scale and an ordinary one (the fused form): bit-exact against the
    oracle's float32 products, subnormal distances included."""
    tc, d16, poses = tiny_depth_case()
    _, D, W = engine_run(gpu, tc, d16, poses, k=k, depth_scale=scale)
    Do, Wo = oracle_run(oracle, tc, d16, poses, depth_scale=scale)
    assert (Wo > 0).mean() > 0.5
    assert np.array_equal(W, Wo)
    assert np.array_equal(D.view(np.uint32), Do.view(np.uint32))
    if scale < 2.0 ** -126:
        # a subnormal scale: layer 28 averages subnormal samples
        tiny = (Do != 0) & (np.abs(Do) < np.finfo(np.float32).tiny)
        assert tiny.any()


@pytest.mark.parametrize("fmt", ["u16", "f32"])
@pytest.mark.parametrize("k", [1, 5, 32])
@pytest.mark.parametrize("case", ["circle", "odd"])
def test_fixed_bitexact_vs_oracle(gpu, oracle, case, fmt, k):
    if case == "circle":
        seq, tc = circle_case(frames=9, mode="fixed", max_weight=6)
    else:
        seq, tc = frontal_case(77, 50, 37, frames=9, mode="fixed", max_weight=6)
    depths = list(seq.depth_u16) if fmt == "u16" else list(seq.depth_m())
    _, D, W = engine_run(gpu, tc, depths, seq.poses, k=k)
    Do, Wo = oracle_run(oracle, tc, depths, seq.poses)
    assert (Wo > 0).mean() > 0.05 and Wo.max() == 6
    assert np.array_equal(W, Wo)
    assert np.array_equal(D.view(np.uint32), Do.view(np.uint32))


@pytest.mark.parametrize("case", ["frontal", "circle"])
def test_compat_reference_arith_vs_oracle(gpu, oracle, case):
    """Compat mode in the reference's arithmetic: weights and distances equal
    the oracle's except where a pixel index sits within 8 ulp of a truncation
    boundary; distances elsewhere agree to the approximate divide's error."""
    seq, tc = (frontal_case if case == "frontal" else circle_case)(frames=7)
    depths = list(seq.depth_m())
    _, D, W = engine_run(gpu, tc, depths, seq.poses, k=4)
    flags = np.zeros(D.shape, np.uint8)
    Do, Wo = oracle_run(oracle, tc, depths, seq.poses, flags=flags)
    ok = flags == 0
    # voxels behind the camera (projected through negative z, a reference
    # quirk) land near pixel boundaries more often; most are still unflagged
    assert ok.mean() > 0.8
    assert np.array_equal(W[ok], Wo[ok])
    trunc = oracle.derive(oracle.cfg_from(tc))[1]
    np.testing.assert_allclose(D[ok], Do[ok], rtol=0, atol=1e-6 * trunc * len(depths))
    n_flip = int(((W != Wo) | (np.abs(D - Do) > 1e-6 * trunc * len(depths))).sum())
    assert n_flip <= max(20, 2e-3 * D.size)


@pytest.mark.parametrize("k", [16, 24])
@pytest.mark.parametrize("mode", ["compat", "fixed"])
@pytest.mark.parametrize("brick", [0, 1, 2, 3])
def test_fused_pass_equals_per_frame_passes(gpu, mode, brick, k):
    """Frames fused in one pass give bit-identical volumes to one pass per
    frame, for every brick shape and both forms of the pass kernel (16
    frames: a lane per brick culls, frame by frame; 24: a lane per frame
    culls, the next frame's samples gathered during the current update)."""
    seq, tc = circle_case(n=96, frames=k, mode=mode, max_weight=8)
    depths = list(seq.depth_u16) if mode == "fixed" else list(seq.depth_m())
    _, D1, W1 = engine_run(gpu, tc, depths, seq.poses, k=1, brick=brick)
    _, D2, W2 = engine_run(gpu, tc, depths, seq.poses, k=k, brick=brick, ctas_per_sm=3)
    assert np.array_equal(W1, W2) and np.array_equal(D1.view(np.uint32), D2.view(np.uint32))


def test_edge_cases_invalid_depth(gpu, oracle):
    """Zero, NaN, negative and beyond-range depth are skipped; a pitched
    image (row stride above width) is read through its pitch."""
    seq, tc = frontal_case(64, 48, 32, frames=2, arith="ieee")
    d = seq.depth_m()[0].copy()
    h, w = d.shape
    d[:, : w // 4] = 0.0
    d[: h // 4, :] = np.nan
    d[h // 2:, w // 2:] = 30.0      # beyond the reference's 24 m limit
    d[h // 3: h // 2, :] = -1.0
    pitched = np.zeros((h, w + 13), np.float32)
    pitched[:, :w] = d
    t = gpu.from_numpy(pitched).cuda()[:, :w]
    from cuphoto import TSDFVolume
    vol = TSDFVolume(tc)
    assert vol.integrate(t, t, seq.poses[0])
    gpu.cuda.synchronize()
    Do, Wo = oracle_run(oracle, tc, [d], seq.poses[:1])
    assert np.array_equal(vol.voxel_weights_data().cpu().numpy(), Wo)
    assert np.array_equal(vol.voxel_distances_data().cpu().numpy(), Do)


def test_reference_error_behaviour(gpu):
    """integrate() returns False for missing or empty images, as the reference does."""
    from cuphoto import TSDFVolume
    seq, tc = frontal_case(16, 16, 16, frames=1)
    vol = TSDFVolume(tc)
    d = dev_depth(gpu, seq.depth_m()[0])
    assert vol.integrate(None, d, seq.poses[0]) is False
    assert vol.integrate(d, None, seq.poses[0]) is False
    assert vol.integrate(d, d[:0], seq.poses[0]) is False
    bad_pose = np.array(seq.poses[0]).copy()
    bad_pose[4] = np.nan
    assert vol.integrate(d, d, bad_pose) is False
    W = vol.voxel_weights_data().cpu().numpy()
    assert np.all(W == 0)


def test_camera_facing_away_leaves_volume_untouched(gpu):
    seq, tc = circle_case(n=48, frames=1, mode="fixed")
    pose = S.pose7(*S.look_at((0.0, 0.5, 5.0), target=(0.0, 0.5, 10.0)))
    _, D, W = engine_run(gpu, tc, [seq.depth_u16[0]], [pose])
    assert np.all(W == 0)


@pytest.mark.parametrize("mode", ["compat", "fixed"])
def test_full_size_c1_against_oracle(gpu, oracle, mode):
    """256^3 grid, 20 frames of 640x480 (the 1 cm configuration), fused 20 per
    pass, against the oracle: bit-exact in IEEE/fixed arithmetic."""
    cam = S.Camera()
    seq = S.make_sequence(20, scene_id=0, camera=cam, trajectory="circle")
    kw = dict(arith="ieee") if mode == "compat" else dict(mode="fixed", max_weight=128)
    tc = TSDFVolumeConfig(**S.grid_for(256), **kw)
    depths = list(seq.depth_m()) if mode == "compat" else list(seq.depth_u16)
    _, D, W = engine_run(gpu, tc, depths, seq.poses, k=20)
    Do, Wo = oracle_run(oracle, tc, depths, seq.poses)
    assert np.array_equal(W, Wo)
    assert np.array_equal(D.view(np.uint32), Do.view(np.uint32))


@pytest.mark.parametrize("mode", ["compat", "fixed"])
def test_checkpoint_and_resume_is_bit_identical(gpu, tmp_path, mode):
    """Integrate 5 frames, save, load into a new volume, integrate 4 more:
    the same bits as 9 frames into one volume; the loaded volume's
    configuration is the saved one."""
    from cuphoto import TSDFVolume
    seq, tc = circle_case(n=64, frames=9, mode=mode, max_weight=6)
    depths = [dev_depth(gpu, d) for d in (seq.depth_u16 if mode == "fixed" else seq.depth_m())]
    whole = TSDFVolume(tc)
    whole.integrate_frames(depths, seq.poses)
    first = TSDFVolume(tc)
    first.integrate_frames(depths[:5], seq.poses[:5])
    path = str(tmp_path / "vol.gbtv")
    first.save(path)
    assert os.path.getsize(path) == 256 + 8 * 64 ** 3
    resumed = TSDFVolume.load(path)
    # (the file holds the float32 configuration the volume was created from)
    assert bytes(resumed.cfg.to_c()) == bytes(tc.to_c()) and resumed.truncation == whole.truncation
    assert np.array_equal(resumed.voxel_weights_data().cpu().numpy(), first.voxel_weights_data().cpu().numpy())
    resumed.integrate_frames(depths[5:], seq.poses[5:])
    gpu.cuda.synchronize()
    assert (whole.voxel_weights_data() > 0).float().mean().item() > 0.05
    assert np.array_equal(resumed.voxel_weights_data().cpu().numpy(), whole.voxel_weights_data().cpu().numpy())
    assert np.array_equal(resumed.voxel_distances_data().cpu().numpy().view(np.uint32),
                          whole.voxel_distances_data().cpu().numpy().view(np.uint32))
    # a file cut short is refused
    with open(path, "rb") as f:
        data = f.read()
    cut = tmp_path / "cut.gbtv"
    cut.write_bytes(data[:len(data) - 4])
    from cuphoto import _lib as L
    with pytest.raises(L.GbtError):
        TSDFVolume.load(str(cut))


def _pitched(gpu, arr, extra):
    """A device copy of the (H, W) image with `extra` unused elements after
    each row (the kernels read it through its pitch)."""
    h, w = arr.shape
    host = np.zeros((h, w + extra), arr.dtype)
    host[:, :w] = arr
    return dev_depth(gpu, host)[:, :w]


@pytest.mark.parametrize("k", [1, 16])
@pytest.mark.parametrize("mode,arith,fmt", [("compat", "reference", "u16"), ("compat", "ieee", "f32"),
                                           ("fixed", "ieee", "u16"), ("fixed", "ieee", "f32")])
@pytest.mark.parametrize("pitch_extra", [0, 3])
def test_depth_staged_in_shared_memory_is_bit_identical(gpu, mode, arith, fmt, k, pitch_extra):
    """Bricks 4-7 (each warp's depth staged in shared memory) give the same
    bits as bricks 0-3 (gathered from the image), for both sample formats,
    rows copied in 8-byte chunks (pitch 0 extra) or element by element (a
    pitch of 3 extra elements breaks the 8-byte row alignment), one frame and
    16 frames per pass."""
    from cuphoto import TSDFVolume
    seq, tc = circle_case(n=96, frames=k, mode=mode, max_weight=8)
    tc.arith = arith
    imgs = list(seq.depth_u16) if fmt == "u16" else list(seq.depth_m())
    dd = [_pitched(gpu, d, pitch_extra) for d in imgs]
    out = {}
    for brick in (0, 1, 2, 3, 4, 5, 6, 7):
        vol = TSDFVolume(tc)
        vol.integrate_frames(dd, seq.poses, depth_scale=0.001, brick=brick)
        gpu.cuda.synchronize()
        out[brick] = (vol.voxel_distances_data().cpu().numpy(), vol.voxel_weights_data().cpu().numpy())
    assert (out[0][1] > 0).mean() > 0.05
    for b in range(1, 8):
        assert np.array_equal(out[b][1], out[0][1]), b
        assert np.array_equal(out[b][0].view(np.uint32), out[0][0].view(np.uint32)), b


def test_depth_staged_rejects_long_passes(gpu):
    from cuphoto import TSDFVolume
    from cuphoto import _lib as L
    seq, tc = circle_case(n=32, frames=17)
    vol = TSDFVolume(tc)
    dd = [dev_depth(gpu, d) for d in seq.depth_u16]
    with pytest.raises(L.GbtError, match="up to 16 frames"):
        vol.integrate_frames(dd, seq.poses, brick=4)
