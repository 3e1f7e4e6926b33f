"""Small differentiable-integrate cases shared by the CPU and GPU tests."""
import numpy as np

from cuphoto import synthetic as S


def rot_exp(w):
    """Rotation matrix of the axis-angle vector w (Rodrigues)."""
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        return np.eye(3) + K
    return np.eye(3) + np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K


def hat(w):
    return np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])


def make_case(grid=(24, 20, 16), frames=3, width=64, height=48, seed=0, scene_id=2):
    """A frontal scene seen from jittered poses at low resolution, float64
    depth without dropped pixels; a smooth target field; the cfg fields."""
    f = 0.9 * width
    cam = S.Camera(width, height, f, f, (width - 1) / 2, (height - 1) / 2)
    scene = S.make_frontal_scene(scene_id)
    poses = S.frontal_poses(frames, seed=seed, jitter_deg=2.0, jitter_m=0.03)
    depth = np.stack([S.render_depth_m(scene, p, cam) for p in poses])
    depth = np.where(np.isfinite(depth) & (depth < 8.0), depth, 0.0)
    rng = np.random.default_rng(seed)
    depth = depth + 0.002 * rng.normal(size=depth.shape) * (depth > 0)
    R = np.stack([S.matrix_from_quat(p[:4]) for p in poses])
    t = np.stack([p[4:] for p in poses])
    phys = np.array([1.6, 1.2, 1.0])
    vs = (phys / np.array(grid)).astype(np.float32)
    off = np.array([-0.8, -0.6, 0.45], np.float32)
    trunc = np.float32(3.0 * vs.max())
    z = (np.arange(grid[2]) + 0.5) * vs[2] + off[2]
    y = (np.arange(grid[1]) + 0.5) * vs[1] + off[1]
    x = (np.arange(grid[0]) + 0.5) * vs[0] + off[0]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    gt = np.clip(0.05 * np.sin(3 * X) + 0.04 * np.cos(4 * Y) - 0.03 * (Z - 1.0), -trunc, trunc)
    return dict(grid=grid, vs=vs, off=off, K=(cam.fx, cam.fy, cam.cx, cam.cy), trunc=float(trunc), max_weight=8.0,
                max_depth=8.0, min_z=0.05, width=width, height=height, depth=depth, R=R, t=t, gt=gt)


def perturbation(case, seed=1, scale_rot=1.0, scale_t=1.0, scale_depth=1.0):
    rng = np.random.default_rng(seed)
    F = len(case["R"])
    dphi = scale_rot * rng.normal(size=(F, 3))
    dt = scale_t * rng.normal(size=(F, 3))
    ddep = scale_depth * rng.normal(size=case["depth"].shape) * (case["depth"] > 0)
    return dphi, dt, ddep


def perturbed(case, h, dphi, dt, ddep):
    R = np.stack([rot_exp(h * dphi[k]) @ case["R"][k] for k in range(len(case["R"]))])
    return R, case["t"] + h * dt, case["depth"] + h * ddep


def directional(grad_R, grad_t, grad_depth, case, dphi, dt, ddep):
    """Directional derivative of the loss along (dphi, dt, ddep) from the gradients."""
    s = float(np.sum(grad_depth * ddep))
    for k in range(len(case["R"])):
        dR = hat(dphi[k]) @ case["R"][k]
        s += float(np.sum(grad_R[k] * dR) + np.dot(grad_t[k], dt[k]))
    return s
