"""Seeded synthetic RGB-D scenes: a ground plane plus spheres, ray-cast depth.

This stands in for the reference's RGB-D dataset reader
(examples/common/rgbd_dataset.cpp:17-32), which loads colour/depth PNG pairs
from disk and converts depth with ``convertTo(CV_32F, depth_scale)``.  No
dataset is shipped with the reference, so every workload here is generated
from a seed:

* scene: plane y = plane_y and ``n_spheres`` spheres, radii U[0.1, 0.5] m,
  centres uniform in a 2.5 m cube, spheres that would swallow the camera path
  re-drawn; seed = 1000 + scene_id.
* cameras: on a circle (or helix) of radius 1.5 m around the centre, looking
  at it; OpenCV convention (x right, y down, z forward); poses are
  world-to-camera (qw, qx, qy, qz, tx, ty, tz).
* depth: ray-cast, + N(0, sigma) noise, a fraction of pixels zeroed,
  quantised to uint16 millimetres (0 = no depth).  Float metres are
  float32(u16) * float32(depth_scale), the value the engine computes from the
  uint16 image.
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class Scene:
    scene_id: int
    plane_y: float
    centres: np.ndarray
    radii: np.ndarray
    plane_up: float = 1.0   # +1: free space at y > plane_y; -1: at y < plane_y


@dataclass
class Camera:
    width: int = 640
    height: int = 480
    fx: float = 525.0
    fy: float = 525.0
    cx: float = 319.5
    cy: float = 239.5

    @staticmethod
    def half():
        """320x240 with the intrinsics scaled by 1/2 about pixel centres."""
        return Camera(320, 240, 262.5, 262.5, 159.5, 119.5)

    @staticmethod
    def hd():
        return Camera(1280, 720, 920.0, 920.0, 639.5, 359.5)


CIRCLE_RADIUS = 1.5
CIRCLE_HEIGHT = 0.5


def make_scene(scene_id=0, n_spheres=6, cube=2.5, plane_y=-0.9):
    rng = np.random.default_rng(1000 + scene_id)
    centres, radii = [], []
    while len(centres) < n_spheres:
        r = rng.uniform(0.1, 0.5)
        c = rng.uniform(-cube / 2, cube / 2, size=3)
        # keep the camera path (radius 1.5 m, heights 0.1..1.0 m) outside every sphere
        ring = np.hypot(c[0], c[2])
        d_ring = np.hypot(ring - CIRCLE_RADIUS, max(0.0, max(0.1 - c[1], c[1] - 1.0)))
        if d_ring < r + 0.25:
            continue
        centres.append(c)
        radii.append(r)
    return Scene(scene_id, plane_y, np.array(centres, np.float64), np.array(radii, np.float64))


def quat_from_matrix(R):
    """(w, x, y, z) of a rotation matrix (Shepperd's method)."""
    t = np.trace(R)
    if t > 0:
        s = np.sqrt(t + 1.0) * 2
        w, x, y, z = 0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s
    elif R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = np.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        w, x, y, z = (R[2, 1] - R[1, 2]) / s, 0.25 * s, (R[0, 1] + R[1, 0]) / s, (R[0, 2] + R[2, 0]) / s
    elif R[1, 1] > R[2, 2]:
        s = np.sqrt(1.0 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        w, x, y, z = (R[0, 2] - R[2, 0]) / s, (R[0, 1] + R[1, 0]) / s, 0.25 * s, (R[1, 2] + R[2, 1]) / s
    else:
        s = np.sqrt(1.0 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
        w, x, y, z = (R[1, 0] - R[0, 1]) / s, (R[0, 2] + R[2, 0]) / s, (R[1, 2] + R[2, 1]) / s, 0.25 * s
    q = np.array([w, x, y, z])
    return q / np.linalg.norm(q)


def matrix_from_quat(q):
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def look_at(centre, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)):
    """World-to-camera (R, t) for a camera at `centre` looking at `target`."""
    centre = np.asarray(centre, np.float64)
    f = np.asarray(target, np.float64) - centre
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    R = np.stack([r, d, f])
    return R, -R @ centre


def pose7(R, t):
    q = quat_from_matrix(R)
    return np.array([q[0], q[1], q[2], q[3], t[0], t[1], t[2]], np.float64)


def circle_poses(n, radius=CIRCLE_RADIUS, height=CIRCLE_HEIGHT, arc=2 * np.pi, phase=0.0):
    out = []
    for k in range(n):
        a = phase + arc * k / n
        out.append(pose7(*look_at((radius * np.cos(a), height, radius * np.sin(a)))))
    return np.array(out)


def helix_poses(n, seed=0, radius=CIRCLE_RADIUS, turns=2.0, h0=0.2, h1=0.9, jitter_deg=0.5, jitter_m=0.002):
    rng = np.random.default_rng(2000 + seed)
    out = []
    for k in range(n):
        s = k / max(1, n - 1)
        a = 2 * np.pi * turns * s
        R, t = look_at((radius * np.cos(a), h0 + (h1 - h0) * s, radius * np.sin(a)))
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        ang = np.deg2rad(jitter_deg) * rng.normal()
        K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
        dR = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
        out.append(pose7(dR @ R, t + jitter_m * rng.normal(size=3)))
    return np.array(out)


def render_depth_m(scene, pose, cam):
    """Exact ray-cast camera-z depth in metres (inf where nothing is hit)."""
    R = matrix_from_quat(pose[:4])
    t = pose[4:]
    C = -R.T @ t
    u = np.arange(cam.width, dtype=np.float64)
    v = np.arange(cam.height, dtype=np.float64)
    uu, vv = np.meshgrid(u, v)
    dc = np.stack([(uu - cam.cx) / cam.fx, (vv - cam.cy) / cam.fy, np.ones_like(uu)], -1)
    dw = dc @ R  # R^T d for row vectors
    best = np.full(uu.shape, np.inf)
    with np.errstate(divide="ignore", invalid="ignore"):
        tp = (scene.plane_y - C[1]) / dw[..., 1]
    best = np.where((tp > 1e-6) & (tp < best), tp, best)
    for c, r in zip(scene.centres, scene.radii):
        oc = C - c
        a = np.einsum("hwk,hwk->hw", dw, dw)
        b = dw @ oc
        cc = oc @ oc - r * r
        disc = b * b - a * cc
        ok = disc >= 0
        sq = np.sqrt(np.where(ok, disc, 0.0))
        t0 = (-b - sq) / a
        t1 = (-b + sq) / a
        tt = np.where(t0 > 1e-6, t0, t1)
        best = np.where(ok & (tt > 1e-6) & (tt < best), tt, best)
    return best


def render_depth_u16(scene, pose, cam, frame_seed, sigma=0.001, drop=0.02, depth_scale=0.001, max_range=8.0):
    z = render_depth_m(scene, pose, cam)
    rng = np.random.default_rng(frame_seed)
    z = z + sigma * rng.normal(size=z.shape)
    raw = np.where(np.isfinite(z) & (z < max_range), np.rint(z / depth_scale), 0.0)
    raw = np.clip(raw, 0, 65535).astype(np.uint16)
    raw[rng.random(size=z.shape) < drop] = 0
    return raw


def u16_to_metres(raw, depth_scale=0.001):
    return raw.astype(np.float32) * np.float32(depth_scale)


def sdf_gt(scene, grid, voxel_size, offset, trunc):
    """Analytic truncated SDF of the scene at voxel centres, (z, y, x) float32."""
    ax = [(np.arange(grid[i], dtype=np.float64) + 0.5) * voxel_size[i] + offset[i] for i in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    d = scene.plane_up * (Y - scene.plane_y)
    for c, r in zip(scene.centres, scene.radii):
        d = np.minimum(d, np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - r)
    return np.clip(d, -trunc, trunc).astype(np.float32)


@dataclass
class Sequence:
    scene: Scene
    camera: Camera
    poses: np.ndarray       # (n, 7)
    depth_u16: np.ndarray   # (n, H, W)
    depth_scale: float = 0.001

    def depth_m(self):
        return u16_to_metres(self.depth_u16, self.depth_scale)


def make_frontal_scene(scene_id=0, n_spheres=6):
    """Scene in front of a camera at the identity pose (the reference example's
    set-up: world frame = first camera frame, +z forward, +y down), with one
    sphere close to the camera so the first z-layers of a grid placed at
    z = 0.5 m cross a surface."""
    rng = np.random.default_rng(1000 + scene_id)
    centres = [np.array([rng.uniform(-0.1, 0.1), rng.uniform(-0.1, 0.1), 0.62])]
    radii = [0.15]
    while len(centres) < n_spheres:
        r = rng.uniform(0.1, 0.5)
        c = np.array([rng.uniform(-1.0, 1.0), rng.uniform(-0.6, 0.4), rng.uniform(1.2, 2.8)])
        centres.append(c)
        radii.append(r)
    return Scene(scene_id, 0.6, np.array(centres, np.float64), np.array(radii, np.float64), plane_up=-1.0)


def frontal_poses(n, seed=0, jitter_deg=2.0, jitter_m=0.05):
    """Poses jittered around the identity (world-to-camera)."""
    rng = np.random.default_rng(3000 + seed)
    out = [np.array([1.0, 0, 0, 0, 0, 0, 0])]
    for _ in range(1, n):
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        ang = np.deg2rad(jitter_deg) * rng.uniform(-1, 1)
        K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
        R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
        out.append(pose7(R, jitter_m * rng.uniform(-1, 1, size=3)))
    return np.array(out)


def axis_angle_matrix(w):
    """Rotation matrix of the axis-angle vector w (Rodrigues)."""
    w = np.asarray(w, np.float64)
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        return np.eye(3) + K
    return np.eye(3) + np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K


def jitter_poses(R, t, frames, deg, metres, seed):
    """Left-perturb the listed frames of world-to-camera (R [F,3,3], t [F,3]):
    a rotation of `deg` about a random axis through the camera centre, then a
    translation of `metres` in a random direction."""
    rng = np.random.default_rng(seed)
    R, t = np.array(R, np.float64), np.array(t, np.float64)
    for k in frames:
        ax = rng.normal(size=3)
        dR = axis_angle_matrix(np.deg2rad(deg) * ax / np.linalg.norm(ax))
        d = rng.normal(size=3)
        R[k] = dR @ R[k]
        t[k] = dR @ t[k] + metres * d / np.linalg.norm(d)
    return R, t


def diff_case_frontal(n=128, frames=16, camera=None, scene_id=5):
    """The differentiable-integrate check configuration: the frontal scene
    seen from `frames` poses jittered by up to 3 deg / 5 cm, float64 depth
    metres without noise, an n^3 grid over 2.0 x 1.6 x 2.4 m starting 0.4 m in
    front of the first camera, truncation 4 voxels, and the analytic
    truncated SDF of the scene as the loss target.  Returns a dict of arrays
    (R [F,3,3], t [F,3], depth [F,H,W], gt [nz,ny,nx]) and the cfg fields."""
    cam = camera or Camera.half()
    scene = make_frontal_scene(scene_id)
    poses = frontal_poses(frames, seed=scene_id, jitter_deg=3.0, jitter_m=0.05)
    depth = np.stack([render_depth_m(scene, p, cam) for p in poses])
    depth = np.where(np.isfinite(depth) & (depth < 8.0), depth, 0.0)
    grid = (n, n, n)
    vs = (np.array([2.0, 1.6, 2.4]) / n).astype(np.float32)
    off = np.array([-1.0, -0.8, 0.4], np.float32)
    trunc = float(np.float32(4 * vs.max()))
    R = np.stack([matrix_from_quat(p[:4]) for p in poses])
    t = np.stack([p[4:] for p in poses])
    return dict(grid=grid, vs=vs, off=off, K=(cam.fx, cam.fy, cam.cx, cam.cy), trunc=trunc, max_weight=128.0,
                max_depth=8.0, min_z=0.05, width=cam.width, height=cam.height, depth=depth, R=R, t=t,
                gt=sdf_gt(scene, grid, vs, off, trunc))


def diff_case_circle(n=128, frames=16, camera=None, scene_id=5, n_spheres=12):
    """The pose-refinement setting: spheres on a ground plane seen from a
    circle of cameras, float64 depth metres without noise, an n^3 grid over
    the 2.56 m cube, truncation 4 voxels."""
    cam = camera or Camera(320, 240, 262.5, 262.5, 159.5, 119.5)
    scene = make_scene(scene_id, n_spheres=n_spheres)
    poses = circle_poses(frames)
    depth = np.stack([render_depth_m(scene, p, cam) for p in poses])
    depth = np.where(np.isfinite(depth) & (depth < 8.0), depth, 0.0)
    vs = np.full(3, 2.56 / n, np.float32)
    R = np.stack([matrix_from_quat(p[:4]) for p in poses])
    t = np.stack([p[4:] for p in poses])
    return dict(grid=(n, n, n), vs=vs, off=np.full(3, -1.28, np.float32), K=(cam.fx, cam.fy, cam.cx, cam.cy),
                trunc=float(np.float32(4 * vs[0])), max_weight=128.0, max_depth=8.0, min_z=0.05, width=cam.width,
                height=cam.height, depth=depth, R=R, t=t, scene=scene)


def diff_case_c3(n=128, frames=16, scene_id=3, smooth=False):
    """The differentiable-integrate configuration (128^3, 16 frames 320x240):
    the seeded plane + 6 spheres scene seen from `frames` cameras on the
    1.5 m circle (fx = fy = 262.5, cx = 159.5, cy = 119.5), uint16 millimetre
    depth with N(0, 1 mm) noise and 2 % dropped pixels, converted to metres
    as the engine converts it (float32(raw) * float32(0.001)); an n^3 grid
    over the 2.56 m cube centred on the scene, truncation 4 voxels; the
    analytic truncated SDF of the scene as the loss target.

    smooth=True gives the same cameras and grid over the ground plane alone,
    with exact depth (no noise, no dropped pixels): a depth image without
    edges inside the grid's view."""
    cam = Camera.half()
    scene = make_scene(scene_id, n_spheres=0 if smooth else 6)
    poses = circle_poses(frames)
    if smooth:
        depth = np.stack([render_depth_m(scene, p, cam) for p in poses])
        depth = np.where(np.isfinite(depth) & (depth < 8.0), depth, 0.0)
    else:
        depth = np.stack([u16_to_metres(render_depth_u16(scene, p, cam, frame_seed=100 * scene_id + k))
                          for k, p in enumerate(poses)]).astype(np.float64)
    vs = np.full(3, 2.56 / n, np.float32)
    off = np.full(3, -1.28, np.float32)
    trunc = float(np.float32(4 * vs[0]))
    R = np.stack([matrix_from_quat(p[:4]) for p in poses])
    t = np.stack([p[4:] for p in poses])
    return dict(grid=(n, n, n), vs=vs, off=off, K=(cam.fx, cam.fy, cam.cx, cam.cy), trunc=trunc, max_weight=128.0,
                max_depth=8.0, min_z=0.05, width=cam.width, height=cam.height, depth=depth, R=R, t=t,
                gt=sdf_gt(scene, (n, n, n), vs, off, trunc), scene=scene)


def make_sequence(n_frames, scene_id=0, camera=None, n_spheres=6, trajectory="circle", **kw):
    camera = camera or Camera()
    if trajectory == "frontal":
        scene = make_frontal_scene(scene_id, n_spheres)
    else:
        scene = make_scene(scene_id, n_spheres)
    if trajectory == "helix":
        poses = helix_poses(n_frames, seed=scene_id)
    elif trajectory == "frontal":
        poses = frontal_poses(n_frames, seed=scene_id)
    else:
        poses = circle_poses(n_frames, **kw)
    depth = np.stack([render_depth_u16(scene, p, camera, frame_seed=100000 * (scene_id + 1) + k)
                      for k, p in enumerate(poses)])
    return Sequence(scene, camera, poses, depth)


def grid_for(n, physical=2.56):
    """Cubic grid of n^3 voxels of side `physical`, centred on the origin."""
    return dict(voxel_grid_size=(n, n, n), physical_size=(physical,) * 3, global_offset=(-physical / 2,) * 3)


def frontal_grid(nx, ny, nz, physical=(2.0, 1.6, 2.56), z0=0.5):
    """Grid in front of the identity camera, starting at depth z0."""
    return dict(voxel_grid_size=(nx, ny, nz), physical_size=tuple(physical),
                global_offset=(-physical[0] / 2, -physical[1] / 2, z0))


def render_sequence_torch(scene, poses, cam, seed=0, sigma=0.001, drop=0.02, depth_scale=0.001, max_range=8.0,
                          device="cuda"):
    """The same ray-cast as render_depth_u16, batched on the GPU with torch
    (float64 geometry, noise from a seeded torch generator).  Returns an
    (n, H, W) int16 tensor holding the uint16 depth bits, on `device`."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    u = torch.arange(cam.width, dtype=torch.float64, device=device)
    v = torch.arange(cam.height, dtype=torch.float64, device=device)
    vv, uu = torch.meshgrid(v, u, indexing="ij")
    dc = torch.stack([(uu - cam.cx) / cam.fx, (vv - cam.cy) / cam.fy, torch.ones_like(uu)], -1)
    centres = torch.tensor(scene.centres, dtype=torch.float64, device=device)
    radii = torch.tensor(scene.radii, dtype=torch.float64, device=device)
    out = torch.empty((len(poses), cam.height, cam.width), dtype=torch.int16, device=device)
    for k, pose in enumerate(poses):
        R = torch.tensor(matrix_from_quat(np.asarray(pose[:4], np.float64)), dtype=torch.float64, device=device)
        t = torch.tensor(np.asarray(pose[4:], np.float64), dtype=torch.float64, device=device)
        C = -R.T @ t
        dw = dc @ R
        best = torch.full(uu.shape, float("inf"), dtype=torch.float64, device=device)
        tp = (scene.plane_y - C[1]) / dw[..., 1]
        best = torch.where((tp > 1e-6) & (tp < best), tp, best)
        a = (dw * dw).sum(-1)
        for c, r in zip(centres, radii):
            oc = C - c
            b = dw @ oc
            cc = oc @ oc - r * r
            disc = b * b - a * cc
            ok = disc >= 0
            sq = torch.sqrt(torch.clamp(disc, min=0.0))
            t0 = (-b - sq) / a
            t1 = (-b + sq) / a
            tt = torch.where(t0 > 1e-6, t0, t1)
            best = torch.where(ok & (tt > 1e-6) & (tt < best), tt, best)
        z = best + sigma * torch.randn(best.shape, generator=gen, dtype=torch.float64, device=device)
        raw = torch.where(torch.isfinite(z) & (z < max_range), torch.round(z / depth_scale), torch.zeros_like(z))
        raw = torch.clamp(raw, 0, 65535)
        raw = torch.where(torch.rand(raw.shape, generator=gen, device=device) < drop, torch.zeros_like(raw), raw)
        out[k] = (raw.to(torch.int32) - (raw >= 32768).to(torch.int32) * 65536).to(torch.int16)
    return out
