"""Generate golden vectors from the reference's own kernels.

Runs on a machine with a GPU and the reference kernels built by
oracle/build.py (oracle/_ref/ref_tsdf.cubin).  For each case it stores the
inputs (uint16 depth frames, poses, volume configuration) and the reference's
outputs (distance and weight grids after integrate, and the mesh that
generate_triangular_surface extracts from them) in ref_<case>.npz.

    python tests/golden/make_golden.py [out_dir]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cu-reconstruction_gb300"))

import oracle  # noqa: E402
from cuphoto import TSDFVolumeConfig  # noqa: E402
from cuphoto import synthetic as S  # noqa: E402

CASES = {
    "frontal": dict(traj="frontal", grid=(48, 40, 48), frames=3, scene=2),
    "circle": dict(traj="circle", grid=(40, 40, 40), frames=3, scene=4),
}


def main(out_dir):
    import torch
    oracle.ensure_built()
    os.makedirs(out_dir, exist_ok=True)
    cam = S.Camera.half()
    for name, c in CASES.items():
        seq = S.make_sequence(c["frames"], scene_id=c["scene"], camera=cam, trajectory=c["traj"])
        g = S.frontal_grid(*c["grid"]) if c["traj"] == "frontal" else S.grid_for(c["grid"][0])
        tc = TSDFVolumeConfig(**g, focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy, max_weight=64)
        r = oracle.RefHarness(tc)
        for d, p in zip(seq.depth_m(), seq.poses):
            t = torch.from_numpy(np.ascontiguousarray(d)).cuda()
            r.integrate(t.data_ptr(), t.stride(0) * 4, t.shape[1], t.shape[0], p)
        D, W = r.read()
        V, T, _ = r.extract()
        path = os.path.join(out_dir, "ref_%s.npz" % name)
        np.savez_compressed(path, grid=np.array(tc.voxel_grid_size), phys=np.array(tc.physical_size, np.float32),
                            offset=np.array(tc.global_offset, np.float32),
                            K=np.array([cam.fx, cam.fy, cam.cx, cam.cy], np.float32), max_weight=np.float32(64),
                            depth_scale=np.float32(seq.depth_scale), depth_u16=seq.depth_u16, poses=seq.poses,
                            D=D, W=W, ntri=np.int64(len(V)), verts=V, tris=T)
        print(name, path, "updated voxels", int((W > 0).sum()), "triangles", len(V))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
