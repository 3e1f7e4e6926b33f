"""Differentiable integrate on the GPU: forward against the oracle, the
adjoint against the oracle's FP64 gradient and against FP64 central finite
differences (step 1e-4) computed on the GPU, chaining, autograd."""
import numpy as np
import pytest

from cuphoto import synthetic as S
from cuphoto.diff import DiffConfig, backward_raw, forward_raw, integrate, se3_gradient

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
    cnt = torch.empty(shape, dtype=torch.int16, device="cuda")
    s = torch.empty(shape, dtype=torch.int32, device="cuda") if sig else None
    args = [torch.as_tensor(np.ascontiguousarray(x, dtype), device="cuda") for x in (depth, R.reshape(-1, 9), t)]
    forward_raw(cfg_of(case), D, W, args[0], args[1], args[2], cnt, s)
    torch.cuda.synchronize()
    return D, W, cnt, s, args


def gpu_backward(torch, case, gD, W0, cnt, args):
    dep, R, t = args
    gdep = torch.zeros_like(dep)
    gpose = torch.zeros((dep.shape[0], 12), dtype=torch.float64, device="cuda")
    backward_raw(cfg_of(case), gD.contiguous(), W0, cnt, dep, R, t, gdep, gpose)
    torch.cuda.synchronize()
    return gdep.double().cpu().numpy(), gpose.cpu().numpy()


def c3_case():
    """The 128^3, 16-frame, 320x240 configuration (float64 inputs for the
    check, the analytic truncated SDF of the scene as the target)."""
    cam = S.Camera.half()
    scene = S.make_frontal_scene(5)
    poses = S.frontal_poses(16, seed=5, jitter_deg=3.0, jitter_m=0.05)
    depth = np.stack([S.render_depth_m(scene, p, cam) for p in poses])
    depth = np.where(np.isfinite(depth) & (depth < 8.0), depth, 0.0)
    grid = (128, 128, 128)
    phys = np.array([2.0, 1.6, 2.4])
    vs = (phys / 128).astype(np.float32)
    off = np.array([-1.0, -0.8, 0.4], np.float32)
    trunc = float(np.float32(4 * vs.max()))
    gt = S.sdf_gt(scene, grid, vs, off, trunc)
    R = np.stack([S.matrix_from_quat(p[:4]) for p in poses])
    t = np.stack([p[4:] for p in poses])
    return dict(grid=grid, vs=vs, off=off, K=(cam.fx, cam.fy, cam.cx, cam.cy), trunc=trunc, max_weight=128.0,
                max_depth=8.0, min_z=0.05, width=cam.width, height=cam.height, depth=depth, R=R, t=t, gt=gt)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_diff_forward_bitexact_vs_oracle(gpu, oracle, dtype):
    case = diffcase.make_case(grid=(40, 36, 32), frames=5, seed=4)
    D, W, cnt, sig, _ = gpu_forward(gpu, case, case["R"], case["t"], case["depth"], dtype, sig=True)
    cfg = oracle.diff_cfg(case["grid"], case["vs"], case["off"], case["K"], case["trunc"], case["max_weight"],
                          case["max_depth"], case["min_z"], case["width"], case["height"],
                          1 if dtype == np.float64 else 0)
    shape = case["grid"][::-1]
    Do = np.full(shape, case["trunc"], dtype)
    Wo = np.zeros(shape, dtype)
    co, so = oracle.diff_forward(cfg, Do, Wo, case["depth"].astype(dtype), case["R"].reshape(-1, 9).astype(dtype),
                                 case["t"].astype(dtype))
    assert (Wo > 0).mean() > 0.05
    assert np.array_equal(W.cpu().numpy(), Wo)
    assert np.array_equal(D.cpu().numpy(), Do)
    assert np.array_equal(cnt.cpu().numpy().view(np.uint16), co)
    assert np.array_equal(sig.cpu().numpy().view(np.uint32), so)


def test_diff_gradient_fp64_vs_oracle(gpu, oracle):
    case = diffcase.make_case(grid=(40, 36, 32), frames=5, seed=6)
    D, W, cnt, _, args = gpu_forward(gpu, case, case["R"], case["t"], case["depth"], np.float64)
    gD = 2 * W * (D - gpu.as_tensor(case["gt"], device="cuda"))
    W0 = gpu.zeros_like(W)
    gdep, gpose = gpu_backward(gpu, case, gD, W0, cnt, args)
    cfg = oracle.diff_cfg(case["grid"], case["vs"], case["off"], case["K"], case["trunc"], case["max_weight"],
                          case["max_depth"], case["min_z"], case["width"], case["height"], 1)
    odep, opose = oracle.diff_backward(cfg, gD.cpu().numpy(), np.zeros(W.shape), case["depth"],
                                       case["R"].reshape(-1, 9), case["t"])
    assert np.abs(opose).max() > 0
    np.testing.assert_allclose(gpose, opose, rtol=1e-9, atol=1e-12 * np.abs(opose).max())
    np.testing.assert_allclose(gdep, odep, rtol=1e-9, atol=1e-12 * np.abs(odep).max())


def _masked_loss(torch, case, R, t, depth, mask):
    D, W, _, _, _ = gpu_forward(torch, case, R, t, depth, np.float64)
    gt = torch.as_tensor(case["gt"], device="cuda", dtype=torch.float64)
    return float(((W * (D - gt) ** 2)[mask]).sum().item())


@pytest.mark.parametrize("which", ["pose", "depth"])
def test_c3_adjoint_against_fp64_central_differences(gpu, which):
    """128^3 grid, 16 frames 320x240: the directional derivative along a random
    unit direction (all 16 poses, or every depth pixel), FP64 central
    differences with step 1e-4 on the GPU against the FP64 and the FP32
    adjoint, on the voxels whose discrete decisions are the same at both
    ends of the step.  Error bound 1e-4 relative."""
    case = c3_case()
    dphi, dtr, ddep = diffcase.perturbation(case, seed=3)
    if which == "pose":
        ddep = ddep * 0
    else:
        dphi, dtr = dphi * 0, dtr * 0
    nrm = np.sqrt((dphi ** 2).sum() + (dtr ** 2).sum() + (ddep ** 2).sum())
    dphi, dtr, ddep = dphi / nrm, dtr / nrm, ddep / nrm
    h = 1e-4
    Rp, tp, dp = diffcase.perturbed(case, h, dphi, dtr, ddep)
    Rm, tm, dm = diffcase.perturbed(case, -h, dphi, dtr, ddep)
    _, _, _, sp, _ = gpu_forward(gpu, case, Rp, tp, dp, np.float64, sig=True)
    _, _, _, sm, _ = gpu_forward(gpu, case, Rm, tm, dm, np.float64, sig=True)
    D, W, cnt, s0, args = gpu_forward(gpu, case, case["R"], case["t"], case["depth"], np.float64, sig=True)
    mask = (sp == s0) & (sm == s0)
    assert mask.float().mean().item() > 0.5 and (W[mask] > 0).sum().item() > 20000
    fd = (_masked_loss(gpu, case, Rp, tp, dp, mask) - _masked_loss(gpu, case, Rm, tm, dm, mask)) / (2 * h)
    gt = gpu.as_tensor(case["gt"], device="cuda", dtype=gpu.float64)
    gD = 2 * W * (D - gt) * mask
    gdep, gpose = gpu_backward(gpu, case, gD, gpu.zeros_like(W), cnt, args)
    an64 = diffcase.directional(gpose[:, :9].reshape(-1, 3, 3), gpose[:, 9:], gdep, case, dphi, dtr, ddep)
    # the FP32 adjoint on the FP32 forward of the same inputs
    D32, W32, c32, _, a32 = gpu_forward(gpu, case, case["R"], case["t"], case["depth"], np.float32)
    gD32 = (2 * W32 * (D32 - gt.float()) * mask).float()
    gdep32, gpose32 = gpu_backward(gpu, case, gD32, gpu.zeros_like(W32), c32, a32)
    an32 = diffcase.directional(gpose32[:, :9].reshape(-1, 3, 3), gpose32[:, 9:], gdep32, case, dphi, dtr, ddep)
    assert fd != 0.0
    assert abs(an64 - fd) <= 1e-4 * abs(fd), (an64, fd)
    assert abs(an32 - fd) <= 1e-4 * abs(fd), (an32, fd)


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
    """A few gradient steps on jittered frame poses (se(3) left updates from
    the autograd gradient) lower the loss and the pose error."""
    case = c3_case()
    dt = gpu.float32
    dep = gpu.as_tensor(case["depth"], device="cuda", dtype=dt)
    R_true = gpu.as_tensor(case["R"], device="cuda", dtype=dt)
    t_true = gpu.as_tensor(case["t"], device="cuda", dtype=dt)
    shape = case["grid"][::-1]
    gt = gpu.as_tensor(case["gt"], device="cuda", dtype=dt)
    cfg = cfg_of(case)
    rng = np.random.default_rng(11)
    R = R_true.clone()
    t = t_true.clone()
    for k in range(4, 16, 3):   # jitter a few frames by ~0.5 deg / 5 mm
        R[k] = gpu.as_tensor(diffcase.rot_exp(np.deg2rad(0.5) * rng.normal(size=3)), device="cuda", dtype=dt) @ R[k]
        t[k] = t[k] + gpu.as_tensor(0.005 * rng.normal(size=3), device="cuda", dtype=dt)

    # target: the volume integrated with the true poses (its own minimiser)
    D_true, W_true = integrate(dep, R_true, t_true, gpu.full(shape, case["trunc"], dtype=dt, device="cuda"),
                               gpu.zeros(shape, dtype=dt, device="cuda"), cfg)
    target = D_true.detach()
    seen = (W_true > 0).to(dt)

    def loss_and_grad(R, t):
        Rv = R.clone().requires_grad_(True)
        tv = t.clone().requires_grad_(True)
        D, W = integrate(dep, Rv, tv, gpu.full(shape, case["trunc"], dtype=dt, device="cuda"),
                         gpu.zeros(shape, dtype=dt, device="cuda"), cfg)
        L = (seen * W * (D - target) ** 2).sum()
        L.backward()
        return L.item(), se3_gradient(Rv.grad.double(), tv.grad.double(), R.double(), t.double())

    moved = list(range(4, 16, 3))

    def pose_err(R, t):
        return float((t[moved] - t_true[moved]).norm(dim=1).mean().item())

    def apply(R, t, xi):
        R2, t2 = R.clone(), t.clone()
        for k in range(R.shape[0]):
            dR = gpu.as_tensor(diffcase.rot_exp(xi[k, 3:].cpu().numpy()), device="cuda", dtype=dt)
            R2[k] = dR @ R[k]
            t2[k] = dR @ t[k] + xi[k, :3].to(dt)
        return R2, t2

    L0, g = loss_and_grad(R, t)
    e0 = pose_err(R, t)
    L = L0
    step = 2e-3 / max(g.abs().max().item(), 1e-30)
    for it in range(10):   # gradient steps with backtracking on the loss
        while step * g.abs().max().item() > 1e-7:
            R2, t2 = apply(R, t, -step * g)
            L2, g2 = loss_and_grad(R2, t2)
            if L2 < L:
                R, t, L, g = R2, t2, L2, g2
                step *= 1.5
                break
            step *= 0.5
    assert L < 0.9 * L0
    assert pose_err(R, t) < e0
