"""Differentiable TSDF integrate as a torch.autograd.Function.

    D, W = integrate(depth, R, t, D0, W0, cfg)

depth [F, H, W] metres, R [F, 3, 3] world-to-camera rotations, t [F, 3]
(float32 or float64 CUDA tensors of one dtype); D0, W0 the starting
distances and weights [nz, ny, nx].  Gradients flow to depth, R, t and D0
(W is piecewise constant).  The adjoint is the engine's gbt_diff_backward:
one recomputation of each voxel-frame, no per-frame volumes kept.  Sequences
longer than 128 frames are integrated in chunks, chained through D.
"""
import ctypes as C
from dataclasses import dataclass

from . import _lib as L
from .tsdf import _stream_handle

MAX_FRAMES = L.MAX_FRAMES_PER_SCENE_PASS


@dataclass
class DiffConfig:
    voxel_grid_size: tuple
    voxel_size: tuple
    global_offset: tuple
    focal_x: float
    focal_y: float
    cx: float
    cy: float
    truncation: float
    max_weight: float = 128.0
    max_depth: float = 24.0
    min_z: float = 0.0

    @staticmethod
    def from_volume_config(tc, truncation=None):
        vs = tuple(float(p) / float(g) for p, g in zip(tc.physical_size, tc.voxel_grid_size))
        tr = truncation if truncation else 1.1 * sum(v * v for v in vs) ** 0.5
        return DiffConfig(tuple(tc.voxel_grid_size), vs, tuple(tc.global_offset), tc.focal_x, tc.focal_y, tc.cx,
                          tc.cy, tr, float(tc.max_weight), float(tc.max_depth or 24.0), float(tc.min_z))

    def to_c(self, width, height, dtype):
        import torch
        c = L.DiffCfg()
        for i in range(3):
            c.voxel_grid_size[i] = int(self.voxel_grid_size[i])
            c.voxel_size[i] = float(self.voxel_size[i])
            c.global_offset[i] = float(self.global_offset[i])
        c.focal_x, c.focal_y, c.cx, c.cy = float(self.focal_x), float(self.focal_y), float(self.cx), float(self.cy)
        c.truncation, c.max_weight = float(self.truncation), float(self.max_weight)
        c.max_depth, c.min_z = float(self.max_depth), float(self.min_z)
        c.width, c.height = int(width), int(height)
        c.dtype = 1 if dtype == torch.float64 else 0
        return c


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def forward_raw(cfg, D, W, depth, R, t, counts, signature=None, stream=None):
    """In place on D, W; fills counts (int16 storage of the uint16 counts)."""
    c = cfg.to_c(depth.shape[2], depth.shape[1], depth.dtype)
    L.check(L.lib().gbt_diff_forward(C.byref(c), _ptr(D), _ptr(W), _ptr(counts), _ptr(depth), int(depth.shape[0]),
                                     _ptr(R), _ptr(t), _ptr(signature) if signature is not None else None,
                                     _stream_handle(stream)))


def backward_raw(cfg, grad_D, W0, counts, depth, R, t, grad_depth, grad_pose, grad_D0=None, stream=None):
    c = cfg.to_c(depth.shape[2], depth.shape[1], depth.dtype)
    L.check(L.lib().gbt_diff_backward(C.byref(c), _ptr(grad_D), _ptr(W0), _ptr(counts), _ptr(depth),
                                      int(depth.shape[0]), _ptr(R), _ptr(t), _ptr(grad_depth), _ptr(grad_pose),
                                      _ptr(grad_D0) if grad_D0 is not None else None, _stream_handle(stream)))


def _function():
    import torch

    class IntegrateFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, depth, R, t, D0, W0, cfg):
            depth, R, t = depth.contiguous(), R.contiguous(), t.contiguous()
            if not (depth.dtype == R.dtype == t.dtype == D0.dtype == W0.dtype):
                raise TypeError("depth, R, t, D0 and W0 need one dtype")
            if depth.shape[0] > MAX_FRAMES:
                raise ValueError("at most %d frames per call" % MAX_FRAMES)
            D = D0.detach().clone()
            W = W0.detach().clone()
            counts = torch.empty(D.shape, dtype=torch.int16, device=D.device)
            forward_raw(cfg, D, W, depth, R, t, counts)
            ctx.save_for_backward(depth, R, t, W0.detach(), counts)
            ctx.cfg = cfg
            ctx.mark_non_differentiable(W)
            return D, W

        @staticmethod
        def backward(ctx, gD, gW):
            depth, R, t, W0, counts = ctx.saved_tensors
            gdep = torch.zeros_like(depth)
            gpose = torch.zeros((depth.shape[0], 12), dtype=torch.float64, device=depth.device)
            gD0 = torch.empty_like(W0) if ctx.needs_input_grad[3] else None
            if gD is None:
                gD = torch.zeros_like(W0)
            backward_raw(ctx.cfg, gD.contiguous(), W0, counts, depth, R, t, gdep, gpose, gD0)
            gR = gpose[:, :9].reshape(-1, 3, 3).to(R.dtype)
            gt = gpose[:, 9:].to(t.dtype)
            return (gdep if ctx.needs_input_grad[0] else None, gR if ctx.needs_input_grad[1] else None,
                    gt if ctx.needs_input_grad[2] else None, gD0, None, None)

    return IntegrateFn


_FN = None


def integrate(depth, R, t, D0, W0, cfg):
    """Differentiable integrate of F frames (chunks of 128 chained through D)."""
    global _FN
    if _FN is None:
        _FN = _function()
    D, W = D0, W0
    for s in range(0, depth.shape[0], MAX_FRAMES):
        D, W = _FN.apply(depth[s:s + MAX_FRAMES], R[s:s + MAX_FRAMES], t[s:s + MAX_FRAMES], D, W, cfg)
    return D, W


def se3_gradient(grad_R, grad_t, R, t):
    """dL/d(rho, phi) per frame for the left perturbation exp(xi^) T from
    dL/dR, dL/dt: rho = dL/dt, phi = vee(G R^T - R G^T)/... written out."""
    import torch
    A = grad_R @ R.transpose(1, 2)
    phi = torch.stack([A[:, 2, 1] - A[:, 1, 2], A[:, 0, 2] - A[:, 2, 0], A[:, 1, 0] - A[:, 0, 1]], -1)
    phi = phi + torch.linalg.cross(t, grad_t, dim=-1)
    return torch.cat([grad_t, phi], -1)
