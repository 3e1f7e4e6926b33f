"""Golden vectors for the z-buffer projection from the reference's own host
loop, cudaPointCloud::project_to_color_depth (cuda_point_cloud.cu:292-353).

The loop runs in oracle/_ref/ref_project, built by oracle/build.py from the
reference's sources as its Release build compiles them (host code -O3 for
x86-64: single-precision operations, no fused multiply-adds).  This script
makes seeded point clouds, runs the program on each and stores the inputs
and both output images in tests/golden/points_project_ref.npz.  It needs the
reference checkout; the tests read only the .npz.

Cases:
  scene  -- points back-projected from a synthetic 320x240 depth frame of a
            seeded plane + spheres scene (circle camera), with random colours,
            projected into the view of another camera on the circle;
  edges  -- the loop's corner cases under the identity pose: a point at
            camera z = 0 (skipped), points behind the camera (negative z is
            not rejected), a cloud of exact duplicates with different colours
            (equal z: the first point in the cloud keeps the pixel), points on
            integer pixel coordinates and on the image border, points off the
            image, and NaN and infinite positions.

Run: python tests/golden/make_golden_project.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "cu-reconstruction_gb300")]

POINT = np.dtype([("pos", "<f4", 3), ("normal", "<f4", 4), ("color", "u1", 3), ("class_id", "<u2")])
assert POINT.itemsize == 33


def run_reference(exe, pts, m, pose, W, H):
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(np.int64(len(pts)).tobytes())
            f.write(np.int32(W).tobytes())
            f.write(np.int32(H).tobytes())
            f.write(np.asarray(m, np.float64).tobytes())
            f.write(np.asarray(pose, np.float64).tobytes())
            f.write(pts.tobytes())
        r = subprocess.run([exe, fin, fout], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference harness failed (%d): %s" % (r.returncode, r.stderr[-2000:]))
        raw = np.fromfile(fout, np.uint8)
    depth = raw[: W * H * 4].view(np.float32).reshape(H, W).copy()
    color = raw[W * H * 4:].reshape(H, W, 3).copy()
    return depth, color


def scene_case(rng):
    from cuphoto import synthetic as S
    cam = S.Camera.half()
    scene = S.make_scene(scene_id=4)
    poses = S.circle_poses(8)
    z = S.render_depth_m(scene, poses[0], cam)
    v, u = np.nonzero(np.isfinite(z) & (z < 8.0))
    keep = rng.random(len(v)) < 0.35          # a sparser cloud keeps the fixture small
    v, u = v[keep], u[keep]
    zz = z[v, u]
    pc = np.stack([(u - cam.cx) * zz / cam.fx, (v - cam.cy) * zz / cam.fy, zz], 1)
    R = S.matrix_from_quat(poses[0][:4])
    t = poses[0][4:]
    world = (pc - t) @ R           # R^T (p - t), row vectors
    pts = np.zeros(len(world), POINT)
    pts["pos"] = world.astype(np.float32)
    pts["color"] = rng.integers(0, 256, size=(len(world), 3), dtype=np.uint8)
    m = np.array([cam.fx, 0, cam.cx, 0, cam.fy, cam.cy, 0, 0, 1.0])   # row-major, as the projection reads it
    return pts, m, poses[1], cam.width, cam.height


def edge_case(rng):
    W, H = 64, 48
    m = np.array([100.0, 0, 31.5, 0, 100.0, 23.5, 0, 0, 1.0])
    pose = np.array([1.0, 0, 0, 0, 0, 0, 0])
    rows = []
    rows.append((0.1, 0.1, 0.0))                        # camera z == 0: skipped
    rows += [(-0.2, 0.1, -1.0), (0.3, -0.2, -2.5)]      # behind the camera: not rejected
    for k in range(5):                                 # exact duplicates, equal z: the first keeps the pixel
        rows.append((0.05, 0.05, 1.25))
    for uu in range(0, W, 7):                          # integer pixel coordinates and the border
        for vv in (0, 11, H - 1):
            zc = 2.0
            rows.append(((uu - 31.5) * zc / 100.0, (vv - 23.5) * zc / 100.0, zc))
    rows += [(5.0, 0.0, 1.0), (0.0, -5.0, 1.0), (1e30, 0.0, 1.0)]   # off the image
    rows += [(np.nan, 0.0, 1.0), (0.0, np.inf, 1.0), (0.0, 0.0, np.nan)]
    # a random cloud in front of the camera, many points per pixel
    n = 4000
    xyz = np.stack([rng.uniform(-0.7, 0.7, n), rng.uniform(-0.5, 0.5, n), rng.uniform(0.8, 3.0, n)], 1)
    pts = np.zeros(len(rows) + n, POINT)
    pts["pos"][: len(rows)] = np.array(rows, np.float64).astype(np.float32)
    pts["pos"][len(rows):] = xyz.astype(np.float32)
    pts["color"] = rng.integers(0, 256, size=(len(pts), 3), dtype=np.uint8)
    return pts, m, pose, W, H


def main():
    import oracle.build as B
    exe = B.build_ref_project()
    if exe is None:
        sys.exit("the reference checkout is needed (REFERENCE_ROOT)")
    rng = np.random.default_rng(2024)
    out = {}
    for name, maker in (("scene", scene_case), ("edges", edge_case)):
        pts, m, pose, W, H = maker(rng)
        depth, color = run_reference(exe, pts, m, pose, W, H)
        out[name + "_points"] = pts.view(np.uint8).reshape(-1, 33)
        out[name + "_camera_matrix"] = m
        out[name + "_pose"] = np.asarray(pose, np.float64)
        out[name + "_size"] = np.array([W, H], np.int32)
        out[name + "_depth"] = depth
        out[name + "_color"] = color
        print(name, len(pts), "points,", int((depth != 0).sum()), "pixels hit")
    np.savez_compressed(os.path.join(HERE, "points_project_ref.npz"), **out)


if __name__ == "__main__":
    main()
