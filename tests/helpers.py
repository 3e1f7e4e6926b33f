"""Shared helpers of the GPU parity tests."""
import numpy as np

from cuphoto import TSDFVolume, TSDFVolumeConfig, extract_mesh_device
from cuphoto import synthetic as S


def dev_depth(torch, arr):
    """numpy uint16 / float32 image (H, W) -> CUDA tensor (uint16 travels as int16)."""
    if arr.dtype == np.uint16:
        return torch.from_numpy(np.ascontiguousarray(arr).view(np.int16)).cuda()
    return torch.from_numpy(np.ascontiguousarray(arr, np.float32)).cuda()


def engine_run(torch, tc, depths, poses, k=1, depth_scale=0.001, brick=0, ctas_per_sm=0):
    vol = TSDFVolume(tc)
    dd = [dev_depth(torch, d) for d in depths]
    for s in range(0, len(dd), k):
        vol.integrate_frames(dd[s:s + k], poses[s:s + k], depth_scale=depth_scale, brick=brick,
                             ctas_per_sm=ctas_per_sm)
    torch.cuda.synchronize()
    D = vol.voxel_distances_data().cpu().numpy()
    W = vol.voxel_weights_data().cpu().numpy()
    return vol, D, W


def oracle_run(oracle, tc, depths, poses, depth_scale=0.001, flags=None):
    c = oracle.cfg_from(tc)
    D, W = oracle.init_volume(c)
    for d, p in zip(depths, poses):
        if tc.mode == "compat":
            dm = d.astype(np.float32) * np.float32(depth_scale) if d.dtype == np.uint16 else d
            oracle.integrate_compat(c, D, W, dm, p)
            if flags is not None:
                oracle.compat_ambiguous(c, p, d.shape[1], d.shape[0], 8.0, flags)
        else:
            oracle.integrate_fixed(c, D, W, d, p, depth_scale)
    return D, W


def frontal_case(nx=96, ny=80, nz=64, frames=6, cam=None, scene_id=1, **kw):
    cam = cam or S.Camera.half()
    seq = S.make_sequence(frames, scene_id=scene_id, camera=cam, trajectory="frontal")
    tc = TSDFVolumeConfig(**S.frontal_grid(nx, ny, nz), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy,
                          camera_width=cam.width, camera_height=cam.height, **kw)
    return seq, tc


def circle_case(n=64, frames=6, cam=None, scene_id=0, physical=2.56, **kw):
    cam = cam or S.Camera.half()
    seq = S.make_sequence(frames, scene_id=scene_id, camera=cam, trajectory="circle")
    tc = TSDFVolumeConfig(**S.grid_for(n, physical), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy,
                          camera_width=cam.width, camera_height=cam.height, **kw)
    return seq, tc


def mesh(vol):
    V, T = extract_mesh_device(vol)
    return V.cpu().numpy(), T.cpu().numpy()


def set_distances(torch, vol, D, W=None):
    vol.voxel_distances_data().copy_(torch.from_numpy(np.ascontiguousarray(D, np.float32)).cuda())
    if W is not None:
        vol.voxel_weights_data().copy_(torch.from_numpy(np.ascontiguousarray(W, np.float32)).cuda())
    torch.cuda.synchronize()
