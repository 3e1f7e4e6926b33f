"""Differentiable integrate on the GPU: forward against the oracle, the
adjoint against the oracle's FP64 gradient and against FP64 central finite
differences (step 1e-4, Richardson-extrapolated) computed on the GPU,
chaining, autograd, pose refinement."""
import numpy as np
import pytest

from cuphoto import synthetic as S
from cuphoto.diff import DiffConfig, backward_raw, checkpoint_shape, forward_raw, integrate, se3_gradient

import diffcase

pytestmark = pytest.mark.gpu


def cfg_of(case):
    return DiffConfig(case["grid"], tuple(float(v) for v in case["vs"]), tuple(float(v) for v in case["off"]),
                      *case["K"], truncation=case["trunc"], max_weight=case["max_weight"],
                      max_depth=case["max_depth"], min_z=case["min_z"])


def gpu_forward(torch, case, R, t, depth, dtype, D0=None, W0=None, sig=False):
    dt = torch.float64 if dtype == np.float64 else torch.float32
    shape = case["grid"][::-1]
    D = torch.full(shape, case["trunc"], dtype=dt, device="cuda") if D0 is None else D0.clone()
    W = torch.zeros(shape, dtype=dt, device="cuda") if W0 is None else W0.clone()
    Din, Win = D.clone(), W.clone()
    ck = torch.empty(checkpoint_shape(len(depth), shape), dtype=dt, device="cuda")
    s = torch.empty(shape, dtype=torch.int32, device="cuda") if sig else None
    args = [torch.as_tensor(np.ascontiguousarray(x, dtype), device="cuda") for x in (depth, R.reshape(-1, 9), t)]
    forward_raw(cfg_of(case), D, W, args[0], args[1], args[2], ck if ck.numel() else None, s)
    torch.cuda.synchronize()
    return D, W, (Din, Win, ck if ck.numel() else None), s, args


def gpu_backward(torch, case, gD, gW, state, args, want_start=False):
    dep, R, t = args
    D0, W0, ck = state
    gdep = torch.zeros_like(dep)
    gpose = torch.zeros((dep.shape[0], 12), dtype=torch.float64, device="cuda")
    gD0 = torch.empty_like(D0) if want_start else None
    gW0 = torch.empty_like(W0) if want_start else None
    backward_raw(cfg_of(case), gD.contiguous(), None if gW is None else gW.contiguous(), D0, W0, ck, dep, R, t,
                 gdep, gpose, gD0, gW0)
    torch.cuda.synchronize()
    out = (gdep.double().cpu().numpy(), gpose.cpu().numpy())
    if want_start:
        out += (gD0.double().cpu().numpy(), gW0.double().cpu().numpy())
    return out


def c3_case(smooth=False):
    """The 128^3, 16-frame, 320x240 configuration: seeded plane + spheres
    scene, circle cameras, uint16 depth with noise and dropped pixels (float64
    copies of its metres for the check), the analytic truncated SDF of the
    scene as the target.  smooth=True: the ground plane alone with exact
    depth, so no depth edge lies in the grid's view."""
    return S.diff_case_c3(128, 16, smooth=smooth)


def _oracle_cfg(oracle, case, dtype):
    return oracle.diff_cfg(case["grid"], case["vs"], case["off"], case["K"], case["trunc"], case["max_weight"],
                           case["max_depth"], case["min_z"], case["width"], case["height"],
                           1 if dtype == np.float64 else 0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("frames", [5, 19])
def test_diff_forward_bitexact_vs_oracle(gpu, oracle, dtype, frames):
    case = diffcase.make_case(grid=(40, 36, 32), frames=frames, seed=4)
    D, W, (_, _, ck), sig, _ = gpu_forward(gpu, case, case["R"], case["t"], case["depth"], dtype, sig=True)
    shape = case["grid"][::-1]
    Do = np.full(shape, case["trunc"], dtype)
    Wo = np.zeros(shape, dtype)
    so = oracle.diff_forward(_oracle_cfg(oracle, case, dtype), Do, Wo, case["depth"].astype(dtype),
                             case["R"].reshape(-1, 9).astype(dtype), case["t"].astype(dtype))
    assert (Wo > 0).mean() > 0.05
    assert np.array_equal(W.cpu().numpy(), Wo)
    assert np.array_equal(D.cpu().numpy(), Do)
    assert np.array_equal(sig.cpu().numpy().view(np.uint32), so)
    # each checkpoint is the volume after the frames before its chunk
    for c in range(0 if ck is None else ck.shape[0]):
        nf = 8 * (c + 1)
        Dc = np.full(shape, case["trunc"], dtype)
        Wc = np.zeros(shape, dtype)
        oracle.diff_forward(_oracle_cfg(oracle, case, dtype), Dc, Wc, case["depth"][:nf].astype(dtype),
                            case["R"][:nf].reshape(-1, 9).astype(dtype), case["t"][:nf].astype(dtype))
        assert np.array_equal(ck[c, 0].cpu().numpy(), Dc) and np.array_equal(ck[c, 1].cpu().numpy(), Wc)


@pytest.mark.parametrize("frames", [5, 19])
def test_diff_gradient_fp64_vs_oracle(gpu, oracle, frames):
    """FP64 adjoint (chunks of 8 recomputed from checkpoints, saturating
    weights) against the oracle's full-history FP64 reverse mode, for a loss
    of both outputs and with gradients to the starting volume."""
    case = diffcase.make_case(grid=(40, 36, 32), frames=frames, seed=6)
    case["max_weight"] = 6.0
    shape = case["grid"][::-1]
    rng = np.random.default_rng(2)
    D0 = gpu.as_tensor(rng.uniform(-case["trunc"], case["trunc"], shape), device="cuda")
    W0 = gpu.as_tensor(rng.uniform(0, 2, shape), device="cuda")
    D, W, state, _, args = gpu_forward(gpu, case, case["R"], case["t"], case["depth"], np.float64, D0, W0)
    gt = gpu.as_tensor(case["gt"], device="cuda")
    gD = 2 * W * (D - gt)
    gW = (D - gt) ** 2
    gdep, gpose, gD0, gW0 = gpu_backward(gpu, case, gD, gW, state, args, want_start=True)
    odep, opose, oD0, oW0 = oracle.diff_backward(_oracle_cfg(oracle, case, np.float64), gD.cpu().numpy(),
                                                 gW.cpu().numpy(), D0.cpu().numpy(), W0.cpu().numpy(),
                                                 case["depth"], case["R"].reshape(-1, 9), case["t"])
    assert np.abs(opose).max() > 0 and (W.cpu().numpy() == 6.0).any()
    for a, b in ((gpose, opose), (gdep, odep), (gD0, oD0), (gW0, oW0)):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12 * np.abs(b).max())


def _masked_loss(torch, case, R, t, depth, mask):
    D, W, _, _, _ = gpu_forward(torch, case, R, t, depth, np.float64)
    gt = torch.as_tensor(case["gt"], device="cuda", dtype=torch.float64)
    return float(((W * (D - gt) ** 2)[mask]).sum().item())


def c3_fd_check(torch, case, dphi, dtr, ddep, h=1e-4):
    """(Richardson-extrapolated FP64 central difference from steps h and h/2,
    FP64 adjoint) of the directional derivative of L = sum W (D - gt)^2 over
    the voxels whose decisions are the same at all four perturbed inputs."""
    runs = {k: diffcase.perturbed(case, k * h, dphi, dtr, ddep) for k in (1, 0.5, -0.5, -1)}
    sigs = {k: gpu_forward(torch, case, *runs[k], np.float64, sig=True)[3] for k in runs}
    D, W, state, s0, args = gpu_forward(torch, case, case["R"], case["t"], case["depth"], np.float64, sig=True)
    mask = s0 == s0
    for s in sigs.values():
        mask &= s == s0
    L = {k: _masked_loss(torch, case, *runs[k], mask) for k in runs}
    d1 = (L[1] - L[-1]) / (2 * h)
    d2 = (L[0.5] - L[-0.5]) / h
    gt = torch.as_tensor(case["gt"], device="cuda", dtype=torch.float64)
    gdep, gpose = gpu_backward(torch, case, 2 * W * (D - gt) * mask, (D - gt) ** 2 * mask, state, args)
    an64 = diffcase.directional(gpose[:, :9].reshape(-1, 3, 3), gpose[:, 9:], gdep, case, dphi, dtr, ddep)
    return (4 * d2 - d1) / 3, an64, mask


@pytest.mark.parametrize("smooth,which,h,tol", [
    (False, "pose", 1e-4, 1e-4),
    (False, "depth", 1e-4, 1e-5),
    (False, "pose", 1e-5, 1e-6),
    (True, "pose", 1e-4, 1e-4),
    (True, "pose", 1e-5, 1e-5),
    (True, "depth", 1e-4, 1e-5),
])
def test_c3_adjoint_against_fp64_central_differences(gpu, smooth, which, h, tol):
    """128^3 grid, 16 frames 320x240: the directional derivative along a random
    unit direction (all 16 poses, or every valid depth pixel) from FP64
    central differences on the GPU (steps h and h/2, Richardson-
    extrapolated) against the FP64 adjoint, on the voxels whose discrete
    decisions are the same at every perturbed input.

    The configured scene meets the 1e-4 target at the configured step 1e-4
    (measured 2.9e-6 along the poses, 6.9e-7 along the depths) and agrees to
    5e-9 at step 1e-5.  The ground plane alone, seen at grazing angles, is
    the harder case for the difference: its depth is a rational function of
    the pixel row with a pole at the horizon, and at step 1e-4 the
    difference is off by ~1e-4 (measured 9.6e-5, inside the 1e-4 target);
    at step 1e-5 it agrees to 7e-10."""
    case = c3_case(smooth)
    dphi, dtr, ddep = diffcase.perturbation(case, seed=3)
    if which == "pose":
        ddep = ddep * 0
    else:
        dphi, dtr = dphi * 0, dtr * 0
    nrm = np.sqrt((dphi ** 2).sum() + (dtr ** 2).sum() + (ddep ** 2).sum())
    dphi, dtr, ddep = dphi / nrm, dtr / nrm, ddep / nrm
    fd, an64, mask = c3_fd_check(gpu, case, dphi, dtr, ddep, h)
    assert mask.float().mean().item() > 0.5
    assert fd != 0.0
    assert abs(an64 - fd) <= tol * abs(fd), (an64, fd, abs(an64 - fd) / abs(fd))


def test_c3_fp32_adjoint_against_fp64(gpu):
    """The FP32 forward + adjoint against FP64 at 128^3 x 16 frames, on the
    voxels where both precisions take the same discrete decisions (a few
    dozen voxels near a footprint or band boundary differ): relative L2
    error of dL/ddepth and dL/dpose below 1e-3.  (On the voxels that differ
    the two precisions follow different branches; there FP32 rounding of the
    pixel coordinate, ~2e-5 px at u ~ 300, meets depth edges of ~1 m/px.)"""
    case = c3_case()
    D, W, st, s64, a = gpu_forward(gpu, case, case["R"], case["t"], case["depth"], np.float64, sig=True)
    D32, W32, st32, s32, a32 = gpu_forward(gpu, case, case["R"], case["t"], case["depth"], np.float32, sig=True)
    m = s32 == s64
    assert m.float().mean().item() > 0.999
    gt = gpu.as_tensor(case["gt"], device="cuda", dtype=gpu.float64)
    g64 = gpu_backward(gpu, case, 2 * W * (D - gt) * m, (D - gt) ** 2 * m, st, a)
    g32 = gpu_backward(gpu, case, (2 * W32 * (D32 - gt.float()) * m).float(), ((D32 - gt.float()) ** 2 * m).float(),
                       st32, a32)
    for x, y in zip(g32, g64):
        assert np.abs(y).max() > 0
        assert np.linalg.norm(x - y) <= 1e-3 * np.linalg.norm(y), np.linalg.norm(x - y) / np.linalg.norm(y)


def test_chained_calls_match_one_call(gpu):
    """Integrating frames 0..2 then 3..5 (gradient passed back through the
    distances in between) gives the one-call gradient."""
    case = diffcase.make_case(grid=(32, 28, 24), frames=6, seed=8)
    dt = gpu.float64
    dep = gpu.as_tensor(case["depth"], device="cuda", dtype=dt).requires_grad_(True)
    R = gpu.as_tensor(case["R"], device="cuda", dtype=dt).requires_grad_(True)
    t = gpu.as_tensor(case["t"], device="cuda", dtype=dt).requires_grad_(True)
    shape = case["grid"][::-1]
    D0 = gpu.full(shape, case["trunc"], dtype=dt, device="cuda")
    W0 = gpu.zeros(shape, dtype=dt, device="cuda")
    gt = gpu.as_tensor(case["gt"], device="cuda", dtype=dt)
    cfg = cfg_of(case)
    D, W = integrate(dep, R, t, D0, W0, cfg)
    (W * (D - gt) ** 2).sum().backward()
    g1 = [x.grad.clone() for x in (dep, R, t)]
    for x in (dep, R, t):
        x.grad = None
    D1, W1 = integrate(dep[:3], R[:3], t[:3], D0, W0, cfg)
    D2, W2 = integrate(dep[3:], R[3:], t[3:], D1, W1, cfg)
    assert gpu.equal(D2, D) and gpu.equal(W2, W)
    (W2 * (D2 - gt) ** 2).sum().backward()
    for a, b in zip(g1, (dep.grad, R.grad, t.grad)):
        np.testing.assert_allclose(b.cpu().numpy(), a.cpu().numpy(), rtol=1e-9, atol=1e-12 * a.abs().max().item())


def test_autograd_pose_refinement_reduces_error(gpu):
    """Adam on the se(3) left updates of four jittered frames (1 deg / 5 mm),
    gradients from autograd through the FP32 adjoint, the volume integrated
    with the true poses as the target: the loss and the frames' surface
    registration error fall."""
    from cuphoto.diff import se3_left_update, surface_alignment_error
    case = S.diff_case_circle(128, 16)
    dt = gpu.float32
    dev = "cuda"
    dep = gpu.as_tensor(case["depth"], device=dev, dtype=dt)
    R_true = gpu.as_tensor(case["R"], device=dev, dtype=dt)
    t_true = gpu.as_tensor(case["t"], device=dev, dtype=dt)
    moved = [1, 5, 9, 13]
    Rj, tj = S.jitter_poses(case["R"], case["t"], moved, 1.0, 0.005, seed=11)
    R = gpu.as_tensor(Rj, device=dev, dtype=dt)
    t = gpu.as_tensor(tj, device=dev, dtype=dt)
    shape = case["grid"][::-1]
    cfg = cfg_of(case)
    D0 = gpu.full(shape, case["trunc"], dtype=dt, device=dev)
    W0 = gpu.zeros(shape, dtype=dt, device=dev)
    with gpu.no_grad():
        D_true, W_true = integrate(dep, R_true, t_true, D0, W0, cfg)
    seen = (W_true > 0).to(dt)

    def loss_and_grad(R, t):
        Rv = R.clone().requires_grad_(True)
        tv = t.clone().requires_grad_(True)
        D, W = integrate(dep, Rv, tv, D0, W0, cfg)
        L = (seen * W * (D - D_true) ** 2).sum()
        L.backward()
        return L.item(), se3_gradient(Rv.grad.double(), tv.grad.double(), R.double(), t.double())

    def align(R, t):
        return surface_alignment_error(dep[moved], R[moved], t[moved], R_true[moved], t_true[moved],
                                       *case["K"]).mean().item()

    mask = gpu.zeros(len(case["R"]), 1, dtype=gpu.float64, device=dev)
    mask[moved] = 1
    L0, g = loss_and_grad(R, t)
    e0 = align(R, t)
    m = gpu.zeros_like(g)
    v = gpu.zeros_like(g)
    for it in range(1, 41):
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        xi = -3e-4 * (m / (1 - 0.9 ** it)) / ((v / (1 - 0.999 ** it)).sqrt() + 1e-12) * mask
        R, t = se3_left_update(R, t, xi)
        L, g = loss_and_grad(R, t)
    assert L < 0.5 * L0, (L, L0)
    assert align(R, t) < 0.7 * e0, (align(R, t), e0)


def test_gauss_newton_refinement_reduces_every_pose_error(gpu):
    """cuphoto.diff.refine_poses on six jittered frames (1 deg / 5 mm) of a
    48-frame 1280x720 circle around 20 spheres, against the engine's
    fixed-mode volume of the other 42 frames (512^3, 0.5 cm voxels, 4 cm
    truncation): after 30 steps the loss, the rotation error, the
    camera-centre error and the surface registration error have all fallen
    (the Gauss-Newton blocks separate a rotation from the lateral
    translation that moves the surface almost alike; with Adam on the same
    gradients the centre error grows).  The centre is the weakest direction
    of the loss: it must fall by a fifth, the others by half."""
    from cuphoto import TSDFVolume, TSDFVolumeConfig
    from cuphoto.diff import DiffConfig, refine_poses, surface_alignment_error
    cam = S.Camera.hd()
    scene = S.make_scene(7, n_spheres=20)
    nf = 48
    poses = S.circle_poses(nf)
    frames = S.render_sequence_torch(scene, poses, cam, seed=3)
    R_true = np.stack([S.matrix_from_quat(p[:4]) for p in poses])
    t_true = np.stack([p[4:] for p in poses])
    moved = [2, 10, 18, 26, 34, 42]
    fixed = [k for k in range(nf) if k not in moved]
    Rj, tj = S.jitter_poses(R_true, t_true, moved, 1.0, 0.005, seed=5)
    tr = 0.04
    n = 512
    tc = TSDFVolumeConfig(**S.grid_for(n, 2.56), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy,
                          camera_width=cam.width, camera_height=cam.height, max_weight=128.0, mode="fixed",
                          truncation=tr, max_depth=8.0, min_z=0.05)
    model = TSDFVolume(tc)
    model.integrate_sequence([frames[k] for k in fixed], poses[fixed], frames_per_pass=16)
    dj = (frames[moved].to(gpu.int32) & 0xFFFF).to(gpu.float32) * np.float32(0.001)
    cfg = DiffConfig((n, n, n), tuple(float(v) for v in model.scale_voxel_size()), tuple(model.global_offset()),
                     cam.fx, cam.fy, cam.cx, cam.cy, truncation=tr, max_weight=128.0, max_depth=8.0, min_z=0.05)
    dev = "cuda"
    R = gpu.as_tensor(Rj[moved], dtype=gpu.float32, device=dev)
    t = gpu.as_tensor(tj[moved], dtype=gpu.float32, device=dev)
    Rt = gpu.as_tensor(R_true[moved], dtype=gpu.float32, device=dev)
    tt = gpu.as_tensor(t_true[moved], dtype=gpu.float32, device=dev)

    def errors(R, t):
        Rd, td = R.double().cpu().numpy(), t.double().cpu().numpy()
        rot = np.degrees(np.arccos(np.clip((np.einsum("kij,kij->k", Rd, R_true[moved]) - 1) / 2, -1, 1))).mean()
        C = np.einsum("kji,kj->ki", Rd, td)
        Ct = np.einsum("kji,kj->ki", R_true[moved], t_true[moved])
        cen = 1e3 * np.linalg.norm(C - Ct, axis=1).mean()
        surf = 1e3 * surface_alignment_error(dj, R, t, Rt, tt, cam.fx, cam.fy, cam.cx, cam.cy).mean().item()
        return rot, cen, surf

    e0 = errors(R, t)
    r = refine_poses(dj, R, t, model.voxel_distances_data(), model.voxel_weights_data(), cfg, steps=30)
    e1 = errors(r["R"], r["t"])
    print("rotation deg, centre mm, surface mm:", e0, "->", e1, "loss", r["losses"][0], "->", r["losses"][-1])
    assert r["losses"][-1] < 0.5 * r["losses"][0], r["losses"]
    for before, after, bar in zip(e0, e1, (0.5, 0.8, 0.5)):
        assert after < bar * before, (e0, e1)
