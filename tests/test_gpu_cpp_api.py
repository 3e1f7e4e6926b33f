"""The C++ layer (cuphoto::TSDFSurface / TSDFVolume / generate_triangular_surface /
Mesh / Config) through the headless driver that mirrors the reference's
tsdf_surface example, against the Python binding of the same C ABI."""
import os
import subprocess

import numpy as np
import pytest

from cuphoto import TSDFVolume, TSDFVolumeConfig, generate_triangular_surface
from cuphoto import synthetic as S

from helpers import dev_depth

HERE = os.path.dirname(os.path.abspath(__file__))
EXAMPLE = os.path.join(HERE, "..", "cu-reconstruction_gb300", "_build", "tsdf_surface_headless")


def read_ply(path):
    with open(path) as f:
        lines = f.read().splitlines()
    assert lines[0] == "ply" and lines[1] == "format ascii 1.0"
    nv = int(lines[2].split()[-1])
    nf = int(lines[6].split()[-1])
    assert lines[3:6] == ["property float x", "property float y", "property float z"]
    assert lines[7:9] == ["property list uchar int vertex_indices", "end_header"]
    V = np.array([[float(x) for x in l.split()] for l in lines[9:9 + nv]], np.float64).reshape(-1, 3)
    F = np.array([[int(x) for x in l.split()] for l in lines[9 + nv:9 + nv + nf]], np.int64).reshape(-1, 4)
    assert np.all(F[:, 0] == 3)
    return V, F[:, 1:]


def write_config(path, grid, phys, offset, cam, ply, extra=""):
    text = """%%YAML:1.0
mesh_store.path: "%s"
camera.fx: %r
camera.fy: %r
camera.cx: %r
camera.cy: %r
camera.width: %d
camera.height: %d
depth_scale: 0.001  # metres per unit
tsdf.volume.voxel_grid_size.x: %d
tsdf.volume.voxel_grid_size.y: %d
tsdf.volume.voxel_grid_size.z: %d
tsdf.volume.physical_size.x: %r
tsdf.volume.physical_size.y: %r
tsdf.volume.physical_size.z: %r
tsdf.volume.max_weight: 15.0
tsdf.volume.global_offset.x: %r
tsdf.volume.global_offset.y: %r
tsdf.volume.global_offset.z: %r
%s
""" % (ply, cam.fx, cam.fy, cam.cx, cam.cy, cam.width, cam.height, grid[0], grid[1], grid[2], phys[0], phys[1],
       phys[2], offset[0], offset[1], offset[2], extra)
    with open(path, "w") as f:
        f.write(text)


def euler_pose(roll, yaw, pitch, t):
    """Pose the reference builds from the config's Euler angles
    (tsdf_surface_reconstruction.cpp:66-81, 127-130), in double."""
    def aa(angle, axis):
        s = np.sin(angle / 2)
        return np.array([np.cos(angle / 2), axis[0] * s, axis[1] * s, axis[2] * s])

    def qmul(a, b):
        w1, x1, y1, z1 = a
        w2, x2, y2, z2 = b
        return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                         w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])
    c = np.float32(np.pi / 180.0)
    # degrees * (pi/180) is a float product (the factor is a float constant), the rest is double
    ang = [float(np.float32(x) * c) for x in (roll, yaw, pitch)]
    q = qmul(qmul(aa(ang[0], (0, 0, 1)), aa(ang[1], (0, 1, 0))), aa(ang[2], (1, 0, 0)))
    q /= np.linalg.norm(q)
    R = S.matrix_from_quat(q)
    q2 = S.quat_from_matrix(R)
    return np.array([q2[0], q2[1], q2[2], q2[3], t[0], t[1], t[2]])


@pytest.mark.gpu
@pytest.mark.parametrize("euler", [None, (4.0, -6.0, 3.0)])
def test_headless_example_matches_python_api(gpu, tmp_path, euler):
    cam = S.Camera.half()
    seq = S.make_sequence(1, scene_id=3, camera=cam, trajectory="frontal")
    grid, phys, off = (96, 80, 64), (1.6, 1.2, 1.28), (-0.8, -0.6, 0.5)
    extra = ""
    t = (0.02, -0.01, 0.03)
    if euler:
        extra = ("tsdf.volume.camera.pose.euler.roll: %r\ntsdf.volume.camera.pose.euler.yaw: %r\n"
                 "tsdf.volume.camera.pose.euler.pitch: %r\ntsdf.volume.camera.pose.translation.x: %r\n"
                 "tsdf.volume.camera.pose.translation.y: %r\ntsdf.volume.camera.pose.translation.z: %r\n"
                 % (euler + t))
        pose = euler_pose(*euler, t=[float(np.float32(x)) for x in t])
    else:
        pose = np.array([1.0, 0, 0, 0, 0, 0, 0])
    ply = str(tmp_path / "mesh.ply")
    cfgp = str(tmp_path / "cfg.yaml")
    write_config(cfgp, grid, phys, off, cam, ply, extra)
    (tmp_path / "depth.u16").write_bytes(seq.depth_u16[0].astype("<u2").tobytes())
    r = subprocess.run([EXAMPLE, "--config_path", cfgp, "--depth", str(tmp_path / "depth.u16")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    V, F = read_ply(ply)
    # the pose the C++ layer derived from the configuration (printed in full)
    used = np.array([float(x) for x in r.stdout.split("pose")[1].split()[:7]])
    np.testing.assert_allclose(used, pose, rtol=0, atol=1e-12)
    pose = used

    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=phys, global_offset=off, max_weight=15.0,
                          focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy)
    vol = TSDFVolume(tc)
    d = dev_depth(gpu, seq.depth_m()[0])
    assert vol.integrate(d, d, pose)
    v, tri = generate_triangular_surface(vol)
    assert len(v) > 1000 and len(V) == len(v) and len(F) == len(tri)
    assert np.array_equal(F, tri)
    np.testing.assert_allclose(V, v, rtol=1e-5, atol=1e-6)   # ASCII PLY keeps 6 significant digits


@pytest.mark.gpu
def test_headless_multi_frame_driver(gpu, tmp_path):
    """reconstruct_sequence: uint16 frames with their own poses, fixed mode,
    several frames per pass, equal to the Python binding's result."""
    cam = S.Camera.half()
    seq = S.make_sequence(12, scene_id=0, camera=cam, trajectory="circle")
    grid, phys, off = (96, 96, 96), (2.56,) * 3, (-1.28,) * 3
    ply = str(tmp_path / "seq.ply")
    cfgp = str(tmp_path / "cfg.yaml")
    write_config(cfgp, grid, phys, off, cam, ply, "tsdf.engine.mode: fixed\n")
    (tmp_path / "frames.u16").write_bytes(seq.depth_u16.astype("<u2").tobytes())
    (tmp_path / "poses.f64").write_bytes(seq.poses.astype("<f8").tobytes())
    r = subprocess.run([EXAMPLE, "--config_path", cfgp, "--sequence", str(tmp_path / "frames.u16"), "--poses",
                        str(tmp_path / "poses.f64"), "--frames", "12", "--per_pass", "5"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    V, F = read_ply(ply)
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=phys, global_offset=off, max_weight=15.0,
                          focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy, mode="fixed")
    vol = TSDFVolume(tc)
    vol.integrate_sequence([dev_depth(gpu, d) for d in seq.depth_u16], seq.poses, frames_per_pass=5)
    v, tri = generate_triangular_surface(vol)
    assert len(v) > 1000 and len(V) == len(v)
    assert np.array_equal(F, tri)
    np.testing.assert_allclose(V, v, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_headless_checkpoint_and_resume(gpu, tmp_path):
    """TSDFVolume::save / load through reconstruct_sequence: 7 frames, save,
    then the other 5 into the loaded volume give the same mesh file as all 12
    in one run; a missing checkpoint is reported, not integrated."""
    cam = S.Camera.half()
    seq = S.make_sequence(12, scene_id=0, camera=cam, trajectory="circle")
    grid, phys, off = (96, 96, 96), (2.56,) * 3, (-1.28,) * 3
    cfgp = str(tmp_path / "cfg.yaml")
    whole, part = str(tmp_path / "whole.ply"), str(tmp_path / "resumed.ply")
    frames, poses = seq.depth_u16.astype("<u2"), seq.poses.astype("<f8")

    def run(ply, first, n, *extra):
        write_config(cfgp, grid, phys, off, cam, ply)
        (tmp_path / "f.u16").write_bytes(frames[first:first + n].tobytes())
        (tmp_path / "p.f64").write_bytes(poses[first:first + n].tobytes())
        return subprocess.run([EXAMPLE, "--config_path", cfgp, "--sequence", str(tmp_path / "f.u16"), "--poses",
                               str(tmp_path / "p.f64"), "--frames", str(n), "--per_pass", "4", *extra],
                              capture_output=True, text=True, timeout=120)

    r = run(whole, 0, 12)
    assert r.returncode == 0, r.stderr
    ckpt = str(tmp_path / "vol.gbtv")
    r = run(str(tmp_path / "first.ply"), 0, 7, "--save_volume", ckpt)
    assert r.returncode == 0, r.stderr
    assert os.path.getsize(ckpt) == 256 + 8 * 96 ** 3
    r = run(part, 7, 5, "--resume_volume", ckpt)
    assert r.returncode == 0, r.stderr
    with open(whole, "rb") as a, open(part, "rb") as b:
        assert a.read() == b.read()
    r = run(str(tmp_path / "none.ply"), 7, 5, "--resume_volume", str(tmp_path / "missing.gbtv"))
    assert r.returncode != 0 and "missing.gbtv" in r.stderr


def test_headless_example_reports_missing_config(engine_lib, tmp_path):
    """Same failure behaviour as the reference example: a missing parameter
    file is reported and the program exits with EXIT_FAILURE (no GPU needed)."""
    r = subprocess.run([EXAMPLE, "--config_path", str(tmp_path / "missing.yaml")], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1
    assert "does not exist" in r.stderr


@pytest.mark.gpu
def test_headless_point_cloud_path(gpu, tmp_path):
    """reconstruct_surface(cudaPointCloud) through the C++ layer: the frame is
    back-projected into a cloud at the inverse of the configured pose, stored
    with save_ply, projected back and integrated.  The depth image it gets
    back is the frame up to pixels whose round trip truncates to a neighbour
    (the reference's pixel rule), which leaves holes, so its mesh is a large
    part of the depth-image path's; both in the fixed mode.  Each step's
    arithmetic is checked bit for bit in test_gpu_points."""
    cam = S.Camera.half()
    seq = S.make_sequence(1, scene_id=3, camera=cam, trajectory="frontal")
    grid, phys, off = (96, 80, 64), (1.6, 1.2, 1.28), (-0.8, -0.6, 0.3)
    (tmp_path / "depth.u16").write_bytes(seq.depth_u16[0].astype("<u2").tobytes())
    extra = ("tsdf.engine.mode: fixed\ntsdf.volume.camera.pose.euler.yaw: 4.0\n"
             "tsdf.volume.camera.pose.translation.x: 0.03\n")
    counts = {}
    for mode in ("depth", "points"):
        ply = str(tmp_path / ("%s.ply" % mode))
        cfgp = str(tmp_path / ("%s.yaml" % mode))
        write_config(cfgp, grid, phys, off, cam, ply, extra)
        cmd = [EXAMPLE, "--config_path", cfgp, "--depth", str(tmp_path / "depth.u16")]
        if mode == "points":
            cmd += ["--points", "--points_ply", str(tmp_path / "cloud.ply")]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
        V, F = read_ply(ply)
        counts[mode] = len(F)
        if mode == "points":
            assert "points %d" % (cam.width * cam.height) in r.stdout
    lines = (tmp_path / "cloud.ply").read_text().splitlines()
    assert lines[:3] == ["ply", "format ascii 1.0", "element vertex %d" % (cam.width * cam.height)]
    assert lines[9] == "end_header" and len(lines) == 10 + cam.width * cam.height
    assert counts["depth"] > 300, counts
    assert 0.5 * counts["depth"] <= counts["points"] <= 1.1 * counts["depth"], counts


def read_binary_ply(path):
    data = open(path, "rb").read()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    header = data[:end].decode().splitlines()
    nv = int([l for l in header if l.startswith("element vertex")][0].split()[-1])
    nf = int([l for l in header if l.startswith("element face")][0].split()[-1])
    vdt = np.dtype([("p", "<f4", 3), ("c", "u1", 3), ("n", "<f4", 4)])
    V = np.frombuffer(data, vdt, nv, end)
    F = np.frombuffer(data, np.dtype([("k", "u1"), ("i", "<i4", 3)]), nf, end + nv * vdt.itemsize)
    assert np.all(F["k"] == 3)
    return V, F["i"]


@pytest.mark.gpu
def test_headless_shared_vertex_mesh(gpu, tmp_path):
    """tsdf.engine.shared_vertices: the fixed-mode mesh through
    generate_indexed_surface, stored as a binary PLY with normals: the same
    triangles as the three-vertices-per-triangle mesh, fewer vertices."""
    cam = S.Camera.half()
    seq = S.make_sequence(1, scene_id=3, camera=cam, trajectory="frontal")
    grid, phys, off = (96, 80, 64), (1.6, 1.2, 1.28), (-0.8, -0.6, 0.3)
    (tmp_path / "depth.u16").write_bytes(seq.depth_u16[0].astype("<u2").tobytes())
    out = {}
    for shared in ("false", "true"):
        ply = str(tmp_path / ("m_%s.ply" % shared))
        cfgp = str(tmp_path / ("c_%s.yaml" % shared))
        write_config(cfgp, grid, phys, off, cam, ply, "tsdf.engine.mode: fixed\ntsdf.engine.shared_vertices: %s\n"
                     % shared)
        r = subprocess.run([EXAMPLE, "--config_path", cfgp, "--depth", str(tmp_path / "depth.u16")],
                           capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
        out[shared] = ply
    Vs, Fs = read_ply(out["false"])
    V, F = read_binary_ply(out["true"])
    assert len(F) == len(Fs) > 300
    assert len(V) < 0.6 * len(Vs)
    # the same triangles: gather the shared vertices back (PLY text has 6 digits)
    np.testing.assert_allclose(V["p"][F].reshape(-1, 3), Vs[Fs.reshape(-1)], rtol=0, atol=1e-5)
    n = np.linalg.norm(V["n"][:, :3], axis=1)
    assert np.all(np.abs(n - 1) < 1e-5)
