"""Benchmark of the TSDF engine: batched integrate + marching cubes.

Workload (the batched plain-forward configuration): a 512^3 grid of 0.5 cm
voxels (2.56 m cube, FP32 distance + FP32 weight = 1 GiB), 300 synthetic
640x480 uint16 depth frames along a helix around a seeded plane+spheres scene,
fx=fy=525, cx=319.5, cy=239.5, integrated K frames per pass (K, brick shape
and CTAs/SM chosen by the autotuner) inside a captured CUDA graph, then the
iso-0 mesh extracted.  One step = reset the volume, integrate all 300 frames,
extract the mesh.  Metric: voxel-updates/s = 512^3 * 300 per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--mode compat|fixed]

With torchrun (N > 1) every rank runs its own scene (seed = rank) on its own
GPU: independent volumes, weak scaling, no collective on the data path.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cu-reconstruction_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "TSDF voxel-updates/s & %HBM peak; fwd+adjoint vs plain fwd time, 1 GB300"
UNIT = "voxel-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="compat", choices=["compat", "fixed"])
    ap.add_argument("--grid", type=int, default=None, help="default 512 (batched), 1024 (refine)")
    ap.add_argument("--frames", type=int, default=None, help="default 300 (batched), 1000 (refine)")
    ap.add_argument("--split-scenes", action="store_true",
                    help="multiscene under torchrun: split one set of 16 scenes over the ranks (strong scaling)")
    ap.add_argument("--refine-steps", type=int, default=50)
    ap.add_argument("--refine-frames", type=int, default=64)
    ap.add_argument("--refine-trunc", type=float, default=0.04, help="truncation (m) of the refinement volumes")
    ap.add_argument("--refine-lr", type=float, default=3e-4, help="Adam step (--refine-method adam)")
    ap.add_argument("--refine-method", default="gn", choices=["gn", "adam"],
                    help="gn: adjoint gradients preconditioned by per-frame 6x6 Gauss-Newton blocks, backtracking "
                         "line search; adam: Adam on the se(3) left updates")
    ap.add_argument("--no-extras", action="store_true", help="skip the CPU baseline and reference-CUDA legs")
    ap.add_argument("--config", default="", help="brick,frames,ctas: skip the autotuner (e.g. 0,32,8)")
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "multiscene", "diff", "refine", "points", "onepass"],
                    help="batched: one 512^3 volume, 300 frames; multiscene: 16 volumes 64^3..384^3, 10..120 frames; "
                         "diff: forward + adjoint timing and finite-difference check at 128^3 x 16 frames; "
                         "refine: 1024^3 x 1000 frames 1280x720, then pose refinement of 64 jittered frames; "
                         "points: 30 frames 640x480 to a cloud, projected to a view; "
                         "onepass: the 512^3 volume, one frame per pass (the reference's calling pattern), "
                         "every brick shape with the depth gathered and staged in shared memory")
    a = ap.parse_args()
    if a.grid is None:
        a.grid = 1024 if a.workload == "refine" else 512
    if a.frames is None:
        a.frames = 1000 if a.workload == "refine" else 300
    return a


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def workload(args, rank):
    from cuphoto import synthetic as S
    cam = S.Camera()
    scene = S.make_scene(scene_id=rank, n_spheres=6)
    poses = S.helix_poses(args.frames, seed=rank)
    return S, cam, scene, poses


def volume_cfg(args, cam, mode):
    from cuphoto import TSDFVolumeConfig
    from cuphoto import synthetic as S
    return TSDFVolumeConfig(**S.grid_for(args.grid, 2.56), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy,
                            camera_width=cam.width, camera_height=cam.height, max_weight=128.0, mode=mode)


class ClockSampler:
    """nvidia-smi samples (every 100 ms) of SM clock and throttle reasons
    while running.  Entering waits for nvidia-smi's first sample, so that the
    region timed inside the block is sampled from its start; the summary
    keeps the samples taken inside the block."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.start = 0
        self.first = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=5.0)
        except OSError:
            self.proc = None
        self.start = len(self.lines)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self.first.set()
        self.first.set()

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # a region shorter than the sampling interval keeps the sample taken
        # just before it
        for ln in self.lines[self.start:] if len(self.lines) > self.start else self.lines[-1:]:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx = max(mx, float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline(args, cam, scene, poses, budget_s=12.0):
    """The oracle's OpenMP restatement of the reference integrate on the host
    cores, on the full grid, for as many frames as fit in `budget_s`."""
    import oracle
    from cuphoto import synthetic as S
    oracle.ensure_built()
    tc = volume_cfg(args, cam, "compat")
    c = oracle.cfg_from(tc)
    D, W = oracle.init_volume(c)
    cores = os.cpu_count() or 1
    nvox = args.grid ** 3
    done, spent = 0, 0.0
    for k, p in enumerate(poses):
        dm = S.u16_to_metres(S.render_depth_u16(scene, p, cam, frame_seed=k))   # rendering is not timed
        a = time.perf_counter()
        oracle.integrate_compat(c, D, W, dm, p, threads=cores)
        spent += time.perf_counter() - a
        done += 1
        if spent > budget_s:
            break
    return {"value": nvox * done / spent, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d of %d frames integrated into the full %d^3 grid (compat arithmetic, OpenMP over rows)"
                      % (done, len(poses), args.grid), "seconds": spent}


def reference_cuda(args, cam, scene, poses, torch, nframes=8):
    """The reference's own integrate kernel (built from its sources) on this GPU."""
    import oracle
    if not oracle.RefHarness.available():
        return {"unavailable": "reference kernels not built (oracle/_ref/ref_tsdf.cubin missing)"}
    from cuphoto import synthetic as S
    tc = volume_cfg(args, cam, "compat")
    r = oracle.RefHarness(tc)
    ms = []
    for k in range(nframes):
        d = torch.from_numpy(S.u16_to_metres(S.render_depth_u16(scene, poses[k], cam, frame_seed=k))).cuda()
        t0 = time.perf_counter()
        kms = r.integrate(d.data_ptr(), d.stride(0) * 4, d.shape[1], d.shape[0], poses[k])
        wall = time.perf_counter() - t0
        if k > 0:  # first frame warms up
            ms.append((kms, wall * 1e3))
    r.close()
    nvox = args.grid ** 3
    kern = float(np.median([m[0] for m in ms]))
    wall = float(np.median([m[1] for m in ms]))
    return {"value": nvox / (kern * 1e-3), "unit": UNIT, "kernel_ms_per_frame": kern, "call_ms_per_frame": wall,
            "frames_timed": len(ms), "what": "TSDFVolume::integrate of the reference, one launch + sync per frame"}


def fixed_mode_mesh(args, torch, cam, depths, poses, K, brick, ctas, reps=10):
    """The same frames in the fixed mode (camera-space SDF, a real surface;
    the compat field of a camera circling the scene has no zero crossing, so
    the compat mesh is empty as it is for the reference), then meshes of
    that field: the engine's fixed-mode marching cubes, the engine's compat
    marching cubes (the reference's quirks) and the reference's own
    generate_triangular_surface path (per-layer kernel + host copy loop),
    all on the same distances."""
    import ctypes as C
    from cuphoto import TSDFVolume
    from cuphoto import _lib as L
    lib = L.lib()
    nvox = args.grid ** 3
    vf = TSDFVolume(volume_cfg(args, cam, "fixed"))

    def integ():
        vf.reset()
        vf.integrate_sequence(depths, poses, frames_per_pass=min(K, 32), brick=brick, ctas_per_sm=ctas)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    peak, peak_kind = peaks()

    def mesh_timer(vol, mode):
        """The mesh as the timed step runs it: gbt_extract_mesh_async captured
        in a CUDA graph, replayed `reps` times between CUDA events after three
        warm-up replays; the distances (and weights) are 1 GiB, above L2."""
        n = C.c_int64()
        L.check(lib.gbt_extract_mesh(vol.handle, None, None, 0, 0, C.byref(n),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        cap = max(n.value, 1)
        verts = torch.empty((cap, 3, 3), dtype=torch.float32, device="cuda")
        tris = torch.empty((cap, 3), dtype=torch.int32, device="cuda")
        count = torch.zeros(1, dtype=torch.int64, device="cuda")
        stream = torch.cuda.Stream()

        def run():
            L.check(lib.gbt_extract_mesh_async(vol.handle, C.c_void_p(verts.data_ptr()), C.c_void_p(tris.data_ptr()),
                                               cap, 0, C.c_void_p(count.data_ptr()),
                                               C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        with torch.cuda.stream(stream):
            run()
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                run()
            for _ in range(3):
                g.replay()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                g.replay()
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        assert int(count.item()) == n.value
        # algorithmic bytes: distances read once (and weights in the fixed
        # mode), 36 B of vertices + 12 B of indices per triangle, the count
        alg = (8.0 if mode == "fixed" else 4.0) * nvox + 48.0 * n.value + 8
        gbs = alg / (ms * 1e-3) / 1e9
        return {"ms": ms, "triangles": int(n.value), "triangles_per_s": n.value / (ms * 1e-3),
                "roofline": {"bound": "hbm", "algorithmic_bytes": alg, "achieved": gbs, "peak": peak,
                             "unit": "GB/s", "frac": gbs / peak, "peak_kind": peak_kind},
                "timing": "graph replay x %d, CUDA events" % reps}

    t_int = timed(integ)
    out = {"integrate_voxel_updates_per_s": nvox * len(depths) / (t_int * 1e-3), "integrate_ms": t_int,
           "mesh_fixed": mesh_timer(vf, "fixed")}
    vc = TSDFVolume(volume_cfg(args, cam, "compat"))
    vc.voxel_distances_data().copy_(vf.voxel_distances_data())
    out["mesh_compat_same_field"] = mesh_timer(vc, "compat")
    import oracle
    if oracle.RefHarness.available():
        r = oracle.RefHarness(volume_cfg(args, cam, "compat"))
        r.write_distances(vf.voxel_distances_data().cpu().numpy())
        V, T, ms = r.extract()
        r.close()
        out["reference_mesh_same_field"] = {"ms": ms, "triangles": int(len(T)), "triangles_per_s": len(T) / (ms * 1e-3),
                                            "what": "generate_triangular_surface of the reference: per-layer kernel "
                                                    "+ sync + host copy loop"}
    vc.close()
    vf.close()
    return out


def _diff_tools(torch, case):
    """Forward, adjoint and FD-check closures of the differentiable integrate
    for one case (a dict of synthetic.diff_case_*)."""
    from cuphoto import diff as DF
    from cuphoto import synthetic as S
    cfg = DF.DiffConfig(case["grid"], tuple(float(v) for v in case["vs"]), tuple(float(v) for v in case["off"]),
                        *case["K"], truncation=case["trunc"], max_weight=case["max_weight"],
                        max_depth=case["max_depth"], min_z=case["min_z"])
    shape = case["grid"][::-1]
    F = len(case["R"])

    def inputs(R, t, dep, dt):
        return [torch.as_tensor(np.ascontiguousarray(x), device="cuda", dtype=dt) for x in (dep, R.reshape(-1, 9), t)]

    def forward(R, t, dep, dt, ckpt=False, sig=False):
        D = torch.full(shape, case["trunc"], dtype=dt, device="cuda")
        W = torch.zeros(shape, dtype=dt, device="cuda")
        ck = torch.empty(DF.checkpoint_shape(F, shape), dtype=dt, device="cuda") if ckpt else None
        sg = torch.empty(shape, dtype=torch.int32, device="cuda") if sig else None
        a = inputs(R, t, dep, dt)
        DF.forward_raw(cfg, D, W, *a, ck, sg)
        return D, W, ck, sg, a

    def adjoint(D, W, ck, a, mask, dt):
        gt = torch.as_tensor(case["gt"], device="cuda", dtype=dt)
        gD = (2 * W * (D - gt) * mask).contiguous()
        gW = ((D - gt) ** 2 * mask).contiguous()
        D0 = torch.full(shape, case["trunc"], dtype=dt, device="cuda")
        W0 = torch.zeros(shape, dtype=dt, device="cuda")
        gdep = torch.zeros_like(a[0])
        gpose = torch.zeros((F, 12), dtype=torch.float64, device="cuda")
        return (gD, gW, D0, W0, gdep, gpose), lambda: DF.backward_raw(cfg, gD, gW, D0, W0, ck, *a, gdep, gpose)

    def fd_check(which, h):
        """FP64 and FP32 adjoints against FP64 central differences (steps h
        and h/2, Richardson-extrapolated) of L = sum W (D - sdf_gt)^2 along a
        unit direction over all poses or over every valid depth pixel, on the
        voxels whose discrete decisions are the same at every perturbed input."""
        rng = np.random.default_rng(3)
        dphi = rng.normal(size=(F, 3))
        dtr = rng.normal(size=(F, 3))
        ddep = rng.normal(size=case["depth"].shape) * (case["depth"] > 0)
        if which == "pose":
            ddep = ddep * 0
        else:
            dphi, dtr = dphi * 0, dtr * 0
        nrm = np.sqrt((dphi ** 2).sum() + (dtr ** 2).sum() + (ddep ** 2).sum())
        dphi, dtr, ddep = dphi / nrm, dtr / nrm, ddep / nrm

        def perturbed(h):
            R = np.stack([S.axis_angle_matrix(h * dphi[k]) @ case["R"][k] for k in range(F)])
            return R, case["t"] + h * dtr, case["depth"] + h * ddep

        runs = {k: perturbed(k * h) for k in (1, 0.5, -0.5, -1)}
        D, W, ck, s0, a = forward(case["R"], case["t"], case["depth"], torch.float64, ckpt=True, sig=True)
        mask = torch.ones(shape, dtype=torch.bool, device="cuda")
        for k in runs:
            mask &= forward(*runs[k], torch.float64, sig=True)[3] == s0
        gt = torch.as_tensor(case["gt"], device="cuda", dtype=torch.float64)

        def loss(k):
            D2, W2 = forward(*runs[k], torch.float64)[:2]
            return float((W2 * (D2 - gt) ** 2)[mask].sum().item())

        L = {k: loss(k) for k in runs}
        d1 = (L[1] - L[-1]) / (2 * h)
        fd = (4 * (L[0.5] - L[-0.5]) / h - d1) / 3

        def directional(dt):
            Dx, Wx, ckx, _, ax = forward(case["R"], case["t"], case["depth"], dt, ckpt=True)
            b, run = adjoint(Dx, Wx, ckx, ax, mask, dt)
            run()
            gdep, gpose = b[4].double().cpu().numpy(), b[5].cpu().numpy()
            s = float(np.sum(gdep * ddep))
            for k in range(F):
                dR = np.cross(np.eye(3), dphi[k]) @ case["R"][k]   # hat(dphi) R
                s += float(np.sum(gpose[k, :9].reshape(3, 3) * dR) + gpose[k, 9:] @ dtr[k])
            return s

        an64 = directional(torch.float64)
        an32 = directional(torch.float32)
        return {"step": h, "fd": fd, "fd_plain": d1, "adjoint_fp64": an64, "adjoint_fp32": an32,
                "rel_err_fp64": abs(an64 - fd) / abs(fd), "rel_err_fp32": abs(an32 - fd) / abs(fd),
                "rel_err_fp64_vs_plain_fd": abs(an64 - d1) / abs(d1),
                "voxels_compared": float(mask.float().mean().item())}

    return cfg, forward, adjoint, fd_check


def differentiable_c3(torch, reps=20):
    """Forward + adjoint of the differentiable integrate on the 128^3,
    16-frame 320x240 configuration (seeded plane + 6 spheres, circle cameras,
    uint16 depth with noise and dropped pixels; FP32): CUDA-event times of
    the plain forward, the forward that writes the adjoint's checkpoints and
    the adjoint, their ratio; the directional-derivative errors of the FP64
    and FP32 adjoints against FP64 central differences on the GPU along all
    poses (steps 1e-4 and 1e-5) and all valid depth pixels (1e-4); the same
    pose check at steps 1e-4 and 1e-5 on the ground plane alone with exact
    depth (no depth edges in view); FP32 against FP64 gradients."""
    from cuphoto import diff as DF
    from cuphoto import synthetic as S
    case = S.diff_case_c3(128, 16)
    cfg, forward, adjoint, fd_check = _diff_tools(torch, case)
    shape = case["grid"][::-1]
    F = len(case["R"])

    # timing, FP32
    D, W, ck, _, a = forward(case["R"], case["t"], case["depth"], torch.float32, ckpt=True)
    bufs, run_adj = adjoint(D, W, ck, a, torch.ones(shape, dtype=torch.bool, device="cuda"), torch.float32)
    Dp = torch.empty_like(D)
    Wp = torch.empty_like(W)

    def fwd_plain():
        Dp.fill_(case["trunc"])
        Wp.zero_()
        DF.forward_raw(cfg, Dp, Wp, *a)

    def fwd_ckpt():
        Dp.fill_(case["trunc"])
        Wp.zero_()
        DF.forward_raw(cfg, Dp, Wp, *a, ck)

    def fill_only():
        Dp.fill_(case["trunc"])
        Wp.zero_()

    def adj():
        bufs[4].zero_()
        bufs[5].zero_()
        run_adj()

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    t_fill = timed(fill_only)
    t_plain = timed(fwd_plain) - t_fill
    t_ckpt = timed(fwd_ckpt) - t_fill
    t_adj = timed(adj) - timed(lambda: (bufs[4].zero_(), bufs[5].zero_()))
    nvf = int(np.prod(shape)) * F

    def fp32_vs_fp64():
        D64, W64, ck64, s64, a64 = forward(case["R"], case["t"], case["depth"], torch.float64, ckpt=True, sig=True)
        D32, W32, ck32, s32, a32 = forward(case["R"], case["t"], case["depth"], torch.float32, ckpt=True, sig=True)
        m = s32 == s64
        b64, run64 = adjoint(D64, W64, ck64, a64, m, torch.float64)
        b32, run32 = adjoint(D32, W32, ck32, a32, m, torch.float32)
        run64()
        run32()
        rel = lambda x, y: float((x.double() - y).norm().item() / y.norm().item())
        return {"voxels_same_decisions": float(m.float().mean().item()), "grad_depth_rel_l2": rel(b32[4], b64[4]),
                "grad_pose_rel_l2": rel(b32[5], b64[5])}

    smooth = S.diff_case_c3(128, 16, smooth=True)
    _, _, _, fd_smooth = _diff_tools(torch, smooth)
    return {"config": "128^3 voxels of 2 cm, 16 frames 320x240 (fx=fy=262.5, cx=159.5, cy=119.5) on the 1.5 m "
                      "circle, seeded plane + 6 spheres, uint16 mm depth with 1 mm noise and 2% dropped pixels, "
                      "truncation 4 voxels, L = sum W (D - sdf_gt)^2",
            "forward_ms": t_plain, "forward_with_checkpoints_ms": t_ckpt, "adjoint_ms": t_adj,
            "fwd_plus_adjoint_over_fwd": (t_ckpt + t_adj) / t_plain,
            "forward_voxel_updates_per_s": nvf / (t_plain * 1e-3),
            "fd_pose": [fd_check("pose", 1e-4), fd_check("pose", 1e-5)], "fd_depth": fd_check("depth", 1e-4),
            "fd_pose_plane_scene": {"scene": "ground plane alone, exact depth (no depth edges in view)",
                                    "checks": [fd_smooth("pose", 1e-4), fd_smooth("pose", 1e-5)]},
            "fp32_vs_fp64": fp32_vs_fp64()}


def refine_workload(args, torch):
    """Large pose refinement.  A seeded scene of a ground plane and 20 spheres,
    `frames` 1280x720 uint16 depth frames (fx = fy = 920) from a circle of
    cameras; `refine_frames` of them, evenly spaced, get a 1 deg / 5 mm pose
    error.  (1) Plain forward: the engine's fixed-mode integrate of all
    frames (jittered ones at their erroneous poses) into a grid^3 volume
    over the 2.56 m cube, then marching cubes; CUDA-event timed.  (2) The
    model: the same integrate of the other frames only.  (3) Refinement: for
    `refine_steps` steps on the jittered frames' se(3) left updates
    (Gauss-Newton-preconditioned adjoint gradients, or Adam with
    --refine-method adam), integrate them (differentiable, FP32, 8-frame
    recompute chunks) into a fresh volume and minimise the frame-to-model
    loss L = sum c W (D - D_model)^2 / sum c W, c = [W_model > 0], through
    the autograd Function (forward + adjoint timed per step).  Reports the
    rotation, camera-centre and surface-registration errors before and
    after, and the adjoint's cost against the forward."""
    import ctypes as C
    from cuphoto import TSDFVolume, TSDFVolumeConfig
    from cuphoto import _lib as L
    from cuphoto import diff as DF
    from cuphoto import synthetic as S
    n, nf, nj = args.grid, args.frames, args.refine_frames
    cam = S.Camera.hd()
    scene = S.make_scene(7, n_spheres=20)
    poses = S.circle_poses(nf)
    frames = S.render_sequence_torch(scene, poses, cam, seed=7)          # (nf, H, W) u16 bits in int16
    R_true = np.stack([S.matrix_from_quat(p[:4]) for p in poses])
    t_true = np.stack([p[4:] for p in poses])
    moved = [int(k) for k in np.linspace(3, nf - 1, nj).round().astype(int)]
    fixed = [k for k in range(nf) if k not in set(moved)]
    Rj, tj = S.jitter_poses(R_true, t_true, moved, 1.0, 0.005, seed=17)
    est = np.stack([S.pose7(Rj[k], tj[k]) for k in range(nf)])
    depths = [frames[k] for k in range(nf)]
    tr = args.refine_trunc
    tc = TSDFVolumeConfig(**S.grid_for(n, 2.56), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy,
                          camera_width=cam.width, camera_height=cam.height, max_weight=128.0, mode="fixed",
                          truncation=tr, max_depth=8.0, min_z=0.05)
    lib = L.lib()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # (1) plain forward + extract, timed (a warm-up pass first)
    vol = TSDFVolume(tc)
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    for it in range(2):
        e = [ev() for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record()
        vol.reset()
        vol.integrate_sequence(depths, est, frames_per_pass=32)
        e[1].record()
        n_tris = C.c_int64()
        L.check(lib.gbt_extract_mesh(vol.handle, None, None, 0, 0, C.byref(n_tris),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        cap = n_tris.value
        verts = torch.empty((max(cap, 1), 3, 3), dtype=torch.float32, device="cuda")
        tris = torch.empty((max(cap, 1), 3), dtype=torch.int32, device="cuda")
        e[1].synchronize()
        e1b = ev()
        e1b.record()
        L.check(lib.gbt_extract_mesh_async(vol.handle, C.c_void_p(verts.data_ptr()), C.c_void_p(tris.data_ptr()),
                                           cap, 0, C.c_void_p(count.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        e[2].record()
        torch.cuda.synchronize()
    plain_int_ms = e[0].elapsed_time(e[1])
    mesh_ms = e1b.elapsed_time(e[2])
    del verts, tris
    vol.close()
    # (2) the model
    model = TSDFVolume(tc)
    model.integrate_sequence([depths[k] for k in fixed], est[fixed], frames_per_pass=32)
    Dm = model.voxel_distances_data()
    cmask = (model.voxel_weights_data() > 0).to(torch.float32)
    # the engine's plain integrate of just the jittered frames, for scale
    v64 = TSDFVolume(tc)
    torch.cuda.synchronize()
    e = [ev(), ev()]
    e[0].record()
    v64.integrate_sequence([depths[k] for k in moved], est[moved], frames_per_pass=32)
    e[1].record()
    torch.cuda.synchronize()
    plain64_ms = e[0].elapsed_time(e[1])
    v64.close()
    # (3) refinement
    dj = (frames[moved].to(torch.int32) & 0xFFFF).to(torch.float32) * np.float32(0.001)
    vs = tuple(float(v) for v in model.scale_voxel_size())
    cfg = DF.DiffConfig((n, n, n), vs, tuple(model.global_offset()), cam.fx, cam.fy, cam.cx, cam.cy,
                        truncation=tr, max_weight=128.0, max_depth=8.0, min_z=0.05)
    shape = (n, n, n)
    D0 = torch.full(shape, tr, dtype=torch.float32, device="cuda")
    W0 = torch.zeros(shape, dtype=torch.float32, device="cuda")
    R = torch.as_tensor(Rj[moved], dtype=torch.float32, device="cuda")
    t = torch.as_tensor(tj[moved], dtype=torch.float32, device="cuda")
    Rt = torch.as_tensor(R_true[moved], dtype=torch.float32, device="cuda")
    tt = torch.as_tensor(t_true[moved], dtype=torch.float32, device="cuda")

    def errors(R, t):
        rot = torch.arccos(torch.clamp((torch.einsum("kij,kij->k", R.double(), Rt.double()) - 1) / 2, -1, 1))
        cen = ((R.double().transpose(1, 2) @ t.double()[..., None]) -
               (Rt.double().transpose(1, 2) @ tt.double()[..., None])).squeeze(-1).norm(dim=1)
        surf = DF.surface_alignment_error(dj, R, t, Rt, tt, cam.fx, cam.fy, cam.cx, cam.cy)
        return {"rotation_deg": float(torch.rad2deg(rot).mean().item()), "centre_mm": 1e3 * float(cen.mean().item()),
                "surface_rms_mm": 1e3 * float(surf.mean().item())}

    before = errors(R, t)
    if args.refine_method == "gn":
        res = _refine_gn(args, torch, DF, dj, R, t, D0, W0, cfg, Dm, cmask, model.voxel_weights_data(), cam, tr,
                         errors)
        after, f_ms, b_ms, losses, extra = res
        return {"workload": "pose refinement: %d^3 voxels of %.2f cm (FP32 D + W = %.1f GB), %d frames 1280x720 "
                            "uint16, %d jittered frames (1 deg / 5 mm), %d Gauss-Newton steps"
                            % (n, 256.0 / n, 8 * n ** 3 / 1e9, nf, nj, args.refine_steps),
                "truncation_m": tr, "plain_forward": {"integrate_ms": plain_int_ms, "mesh_ms": mesh_ms,
                                                      "triangles": int(count.item()),
                                                      "voxel_updates_per_s": n ** 3 * nf / (plain_int_ms * 1e-3)},
                "plain_integrate_of_jittered_frames_ms": plain64_ms,
                "refine_step_ms": {"forward": f_ms, "forward_plus_loss_and_adjoint": b_ms,
                                   "fwd_plus_adjoint_over_fwd": (f_ms + b_ms) / f_ms},
                "loss": {"first": losses[0], "last": losses[-1]}, "optimizer": extra,
                "pose_error_before": before, "pose_error_after": after,
                "reduction": {k: 1 - after[k] / before[k] for k in before}}
    m = v = None
    fwd_ms, bwd_ms, losses = [], [], []
    for it in range(1, args.refine_steps + 1):
        Rv = R.clone().requires_grad_(True)
        tv = t.clone().requires_grad_(True)
        e = [ev() for _ in range(3)]
        e[0].record()
        D, W = DF.integrate(dj, Rv, tv, D0, W0, cfg)
        e[1].record()
        cw = cmask * W
        den = cw.sum()
        loss = (cw * (D - Dm) ** 2).sum() / den
        loss.backward()
        e[2].record()
        torch.cuda.synchronize()
        fwd_ms.append(e[0].elapsed_time(e[1]))
        bwd_ms.append(e[1].elapsed_time(e[2]))
        losses.append(float(loss.item()))
        g = DF.se3_gradient(Rv.grad.double(), tv.grad.double(), R.double(), t.double())
        del D, W, cw, den, loss, Rv, tv
        if m is None:
            m = torch.zeros_like(g)
            v = torch.zeros_like(g)
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        xi = -args.refine_lr * (m / (1 - 0.9 ** it)) / ((v / (1 - 0.999 ** it)).sqrt() + 1e-12)
        R, t = DF.se3_left_update(R, t, xi)
    after = errors(R, t)
    f_ms = float(np.median(fwd_ms))
    b_ms = float(np.median(bwd_ms))
    return {"workload": "pose refinement: %d^3 voxels of %.2f cm (FP32 D + W = %.1f GB), %d frames 1280x720 uint16, "
                        "%d jittered frames (1 deg / 5 mm), %d Adam steps" % (n, 256.0 / n, 8 * n ** 3 / 1e9, nf, nj,
                                                                          args.refine_steps),
            "truncation_m": tr, "plain_forward": {"integrate_ms": plain_int_ms, "mesh_ms": mesh_ms,
                                                  "triangles": int(count.item()),
                                                  "voxel_updates_per_s": n ** 3 * nf / (plain_int_ms * 1e-3)},
            "plain_integrate_of_jittered_frames_ms": plain64_ms,
            "refine_step_ms": {"forward": f_ms, "forward_plus_loss_and_adjoint": b_ms,
                               "fwd_plus_adjoint_over_fwd": (f_ms + b_ms) / f_ms},
            "loss": {"first": losses[0], "last": losses[-1]},
            "pose_error_before": before, "pose_error_after": after,
            "reduction": {k: 1 - after[k] / before[k] for k in before}}


def _refine_gn(args, torch, DF, dj, R, t, D0, W0, cfg, Dm, cmask, Wm, cam, tr, errors):
    """The refinement of cuphoto.diff.refine_poses: adjoint gradients, per-frame
    6x6 Gauss-Newton preconditioning, backtracking line search with the step
    capped at 1 cm of motion and a sufficient-decrease test."""
    r = DF.refine_poses(dj, R, t, Dm, Wm, cfg, steps=args.refine_steps, D0=D0, W0=W0)
    after = errors(r["R"], r["t"])
    losses = r["losses"]
    extra = {"method": "adjoint gradient, per-frame 6x6 Gauss-Newton preconditioner (frame-to-model SDF), "
                       "backtracking line search (steps capped at 1 cm of motion, sufficient decrease 1e-4)",
             "forward_evaluations": r["forward_evaluations"],
             "steps": args.refine_steps, "loss_trace": losses[:: max(1, len(losses) // 10)]}
    return after, float(np.median(r["forward_ms"])), float(np.median(r["adjoint_ms"])), losses, extra


def points_workload(args, torch, nframes=30, reps=5):
    """Point clouds: 30 ray-cast 640x480 frames around a plane + 6 spheres
    back-projected into one 9.2 M-point cloud (gbt_points_extract, CUDA
    events per frame), then the cloud projected to colour + depth at another
    pose (gbt_points_project: 64-bit atomic-min z-buffer + resolve).  Beside
    them: the reference's own point_cloud_extract kernel launched as
    extract_points launches it (one launch + sync per frame), and its
    project_to_color_depth host loop restated single-threaded (the oracle)
    on the same cloud, whose images the engine must match bit for bit."""
    import ctypes as C
    import oracle
    from cuphoto import _lib as L
    from cuphoto import synthetic as S
    cam = S.Camera()
    W, H = cam.width, cam.height
    K = [cam.fx, 0, cam.cx, 0, cam.fy, cam.cy, cam.cx, cam.cy, 1.0]   # both readings agree
    scene = S.make_scene(0)
    poses = S.circle_poses(nframes)
    raw = S.render_sequence_torch(scene, poses, cam, seed=0)
    depth = (raw.to(torch.int32) & 0xFFFF).to(torch.float32) * np.float32(0.001)
    inv = []
    for p in poses:
        R = S.matrix_from_quat(p[:4])
        inv.append(S.pose7(R.T, -R.T @ p[4:]))
    n = nframes * W * H
    cloud = torch.zeros((n, 33), dtype=torch.uint8, device="cuda")
    lib = L.lib()
    Kc = (C.c_double * 9)(*K)
    # the launches go on the stream the timing events are recorded on
    sh = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def extract(k):
        L.check(lib.gbt_points_extract(C.byref(Kc), C.c_void_p(depth[k].data_ptr()), W * 4, L.DEPTH_F32_M, 1.0, None,
                                       0, W, H, C.byref((C.c_double * 7)(*inv[k])), k * W * H,
                                       C.c_void_p(cloud.data_ptr()), n, sh))

    for k in range(nframes):
        extract(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        for k in range(nframes):
            extract(k)
    e1.record()
    torch.cuda.synchronize()
    ext_ms = e0.elapsed_time(e1) / reps
    view = S.circle_poses(nframes * 2)[1]
    dimg = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    cimg = torch.zeros((H, W, 3), dtype=torch.uint8, device="cuda")
    scratch = torch.empty(W * H, dtype=torch.int64, device="cuda")
    Vp = (C.c_double * 7)(*view)

    def project():
        L.check(lib.gbt_points_project(C.c_void_p(cloud.data_ptr()), n, C.byref(Kc), C.byref(Vp),
                                       C.c_void_p(dimg.data_ptr()), W * 4, C.c_void_p(cimg.data_ptr()), W * 3, W, H,
                                       C.c_void_p(scratch.data_ptr()), sh))

    project()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        project()
    e1.record()
    torch.cuda.synchronize()
    proj_ms = e0.elapsed_time(e1) / reps
    out = {"workload": "points: %d frames %dx%d -> %d points, projected to a %dx%d view" % (nframes, W, H, n, W, H),
           "extract": {"ms_per_frame": ext_ms / nframes, "points_per_s": n / (ext_ms * 1e-3)},
           "project": {"ms": proj_ms, "points_per_s": n / (proj_ms * 1e-3), "pixels_hit": int((dimg > 0).sum())}}
    host = cloud.cpu().numpy()
    t0 = time.perf_counter()
    ed, ec = oracle.points_project(host, K, view, W, H)
    cpu_s = time.perf_counter() - t0
    out["reference_host_loop"] = {"kind": "port", "cores": 1, "s": cpu_s, "points_per_s": n / cpu_s,
                                  "what": "project_to_color_depth's host z-buffer loop, restated (the oracle)"}
    out["parity_with_host_loop"] = bool(np.array_equal(dimg.cpu().numpy().view(np.uint32), ed.view(np.uint32))
                                        and np.array_equal(cimg.cpu().numpy(), ec))
    if oracle.RefHarness.available():
        ref = torch.full_like(cloud[: W * H], 0)
        oracle.RefHarness.lib()
        t0 = time.perf_counter()
        for k in range(nframes):
            oracle.RefHarness.points_extract(K, depth[k].data_ptr(), W * 4, W, H, 0, 0, inv[k], 0, ref.data_ptr())
        wall = time.perf_counter() - t0
        out["reference_extract"] = {"ms_per_frame": 1e3 * wall / nframes, "points_per_s": n / wall,
                                    "what": "point_cloud_extract of the reference, one launch + sync per frame"}
    return out


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    S, cam, scene, poses = workload(args, 0)
    import oracle
    from cuphoto import synthetic as SS
    oracle.ensure_built()
    tc = volume_cfg(args, cam, "compat")
    c = oracle.cfg_from(tc)
    D, W = oracle.init_volume(c)
    cores = os.cpu_count() or 1
    frames = [SS.u16_to_metres(SS.render_depth_u16(scene, p, cam, frame_seed=k)) for k, p in enumerate(poses[:4])]
    nvox = args.grid ** 3
    # each step integrates a bounded sample of the frames (sized to ~4 s of host time)
    t = time.perf_counter()
    oracle.integrate_compat(c, D, W, frames[0], poses[0], threads=cores)
    per_frame = time.perf_counter() - t
    fps = max(1, min(4, int(4.0 / max(per_frame, 1e-3))))
    for _ in range(args.warmup):
        for k in range(fps):
            oracle.integrate_compat(c, D, W, frames[k % 4], poses[k % 4], threads=cores)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        for k in range(fps):
            oracle.integrate_compat(c, D, W, frames[k % 4], poses[k % 4], threads=cores)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = nvox * fps * args.steps / total
    sample = "%d frames per step into the full %d^3 grid (compat arithmetic, OpenMP over rows)" % (fps, args.grid)
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "batched integrate, %d^3 voxels of 0.5 cm, 640x480 uint16 depth (CPU sample)" % args.grid,
                      "grid": args.grid, "frames_per_step": fps},
           "comparison": "a rate: voxel-updates/s over a sample of %d frames per step, where the GPU arm integrates "
                         "all 300 frames per step; a voxel-update costs the CPU loop the same whatever the number "
                         "of frames, so a ratio of the two lines compares rates, not one identical step" % fps,
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def multiscene(args, torch, rank, world, local):
    """16 independent seeded scenes, grids drawn from 64^3..384^3 (multiples of
    8), 10..120 frames of 640x480 each, all integrated by the batched launches
    in one captured graph, then a mesh per scene.  With N ranks every rank
    runs its own 16 scenes (seeds offset by rank; weak scaling), or, with
    --split-scenes, the ranks split one set of 16 scenes balanced by
    voxel-updates (strong scaling)."""
    import ctypes as C
    from cuphoto import TSDFVolume, TSDFVolumeConfig, extract_mesh_device
    from cuphoto import _lib as L
    from cuphoto import synthetic as S
    from cuphoto.batch import BatchIntegrator
    from cuphoto import shard
    split = args.split_scenes and world > 1
    rng = np.random.default_rng(77 if split else 77 + rank)
    specs = [(int(rng.integers(8, 49)) * 8, int(rng.integers(10, 121))) for _ in range(16)]
    if split:
        mine = shard.partition_by_cost([n ** 3 * f for n, f in specs], world)[rank]
    else:
        mine = list(range(16))
    cam = S.Camera()
    vols, depths, poses, sizes, nfs, frames3d = [], [], [], [], [], []
    for i in mine:
        n, nf = specs[i]
        sid = i if split else shard.scene_seed(0, rank, i)
        scene = S.make_scene(scene_id=sid)
        ps = S.circle_poses(nf, phase=0.1 * i)
        fr = S.render_sequence_torch(scene, ps, cam, seed=sid)
        tc = TSDFVolumeConfig(**S.grid_for(n, 2.56), focal_x=cam.fx, focal_y=cam.fy, cx=cam.cx, cy=cam.cy,
                              max_weight=128.0, mode=args.mode)
        vols.append(TSDFVolume(tc))
        frames3d.append(fr)
        depths.append([fr[k] for k in range(nf)])
        poses.append(ps)
        sizes.append(n)
        nfs.append(nf)
    updates = sum(n ** 3 * f for n, f in zip(sizes, nfs))
    batch = BatchIntegrator(max_scenes=len(vols), max_frames=sum(nfs))
    # autotune: brick x frames per launch x CTAs/SM on the whole batch
    if args.config:
        brick, fpl, ctas = (int(x) for x in args.config.split(","))
        table = []
    else:
        table = []
        for fpl in (32, 64, 128):
            for brick in (0, 1, 2, 3):
                for ctas in (0, 8, 16):   # 0: as many as the kernel keeps resident
                    for v in vols:
                        v.reset()
                    batch.integrate(vols, depths, poses, brick=brick, ctas_per_sm=ctas, frames_per_launch=fpl)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    batch.integrate(vols, depths, poses, brick=brick, ctas_per_sm=ctas, frames_per_launch=fpl)
                    e1.record()
                    e1.synchronize()
                    table.append((e0.elapsed_time(e1), brick, fpl, ctas))
        _, brick, fpl, ctas = min(table)
    caps = []
    for v in vols:
        v.reset()
    batch.integrate(vols, depths, poses, brick=brick, ctas_per_sm=ctas, frames_per_launch=fpl)
    for v in vols:
        V, _ = extract_mesh_device(v)
        caps.append(max(1024, int(len(V) * 1.25) + 1024))
    outs = [(torch.empty((c, 3, 3), dtype=torch.float32, device="cuda"), torch.empty((c, 3), dtype=torch.int32,
             device="cuda"), torch.zeros(1, dtype=torch.int64, device="cuda")) for c in caps]
    lib = L.lib()
    stream = torch.cuda.Stream()

    def step_integrate():
        for v in vols:
            v.reset()
        batch.integrate(vols, depths, poses, brick=brick, ctas_per_sm=ctas, frames_per_launch=fpl)

    def step_mesh():
        sh = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for v, (vb, tb, cb), cap in zip(vols, outs, caps):
            L.check(lib.gbt_extract_mesh_async(v.handle, C.c_void_p(vb.data_ptr()), C.c_void_p(tb.data_ptr()), cap,
                                               0, C.c_void_p(cb.data_ptr()), sh))

    graphs = []
    with torch.cuda.stream(stream):
        step_integrate()
        step_mesh()
        torch.cuda.synchronize()
        for fn in (step_integrate, step_mesh):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                fn()
            graphs.append(g)
    g_int, g_mesh = graphs
    torch.cuda.set_stream(stream)
    for _ in range(args.warmup):
        g_int.replay()
        g_mesh.replay()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    shard.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            ev[i][0].record(stream)
            g_int.replay()
            ev[i][1].record(stream)
            g_mesh.replay()
            ev[i][2].record(stream)
        torch.cuda.synchronize()
    total_ms = shard.max_over_ranks(ev[0][0].elapsed_time(ev[-1][2]))
    job_updates = shard.sum_over_ranks(updates)
    int_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in ev]))
    mesh_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in ev]))
    ntri = sum(int(o[2].item()) for o in outs)
    # per scene: the same batched path with one scene
    per_scene = []
    for v, ds, ps, n, f in zip(vols, depths, poses, sizes, nfs):
        v.reset()
        batch.integrate([v], [ds], [ps], brick=brick, ctas_per_sm=ctas, frames_per_launch=fpl)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.integrate([v], [ds], [ps], brick=brick, ctas_per_sm=ctas, frames_per_launch=fpl)
        e1.record(stream)
        e1.synchronize()
        per_scene.append({"grid": n, "frames": f, "voxel_updates_per_s": n ** 3 * f / (e0.elapsed_time(e1) * 1e-3)})
    # end to end through the public API: depth frames from pinned host memory
    # (copied window by window while the previous window integrates), the
    # meshes of all scenes, their counts and triangles back to the host
    host = [torch.empty(f.shape, dtype=f.dtype, pin_memory=True).copy_(f) for f in frames3d]
    counts = torch.zeros(len(vols), dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    e2e = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for v in vols:
            v.reset()
        batch.integrate_streamed(vols, host, frames3d, poses, brick=brick, ctas_per_sm=ctas, frames_per_launch=fpl)
        sh = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for k, (v, (vb, tb, _), cap) in enumerate(zip(vols, outs, caps)):
            L.check(lib.gbt_extract_mesh_async(v.handle, C.c_void_p(vb.data_ptr()), C.c_void_p(tb.data_ptr()), cap,
                                               0, C.c_void_p(counts[k:k + 1].data_ptr()), sh))
        ns = counts.cpu().tolist()
        d2h = 8 * len(ns)
        for n, (vb, tb, _) in zip(ns, outs):
            d2h += vb[:n].cpu().numel() * 4 + tb[:n].cpu().numel() * 4
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    h2d = sum(h.numel() * h.element_size() for h in host)
    value = job_updates * args.steps / (total_ms * 1e-3)
    e2e_value = shard.whole_job_rate(updates, float(np.mean(e2e)))
    if rank != 0:
        return None
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "strong" if split else "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: 16 seeded plane + 6 sphere scenes, ray-cast uint16 depth, circle poses",
        "config": {"workload": "multi-scene batched integrate + marching cubes: %d volumes %s^3, %s frames 640x480"
                               "%s" % (len(vols), sizes, nfs, " (rank 0's share of 16 split over %d ranks)" % world
                                       if split else ""),
                   "mode": args.mode, "frames_per_launch": fpl, "brick": brick, "ctas_per_sm": ctas,
                   "voxel_updates_per_step": updates, "graph": "resets + batched launches, meshes: CUDA graphs",
                   "triangles": ntri},
        "breakdown_ms": {"integrate": int_ms, "mesh": mesh_ms},
        "integrate_only": {"value": updates / (int_ms * 1e-3), "unit": UNIT},
        "per_scene": per_scene,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * float(np.mean(e2e))},
        # per step: a reset per volume, the batched launches, four mesh launches per volume
        "gpu_launches": args.steps * (5 * len(vols) + ((max(nfs) + fpl - 1) // fpl)),
        "clocks": clocks.summary(),
        "autotune": {"candidates": len(table)},
    }


def onepass_workload(args, torch):
    """One frame per pass over the full volume, as TSDFVolume::integrate is
    called: for each brick shape, with the depth gathered from the image
    (bricks 0-3) and staged in shared memory per warp (4-7), and for the
    bricks streamed into shared memory by the Tensor Memory Accelerator
    (brick 8), the mean CUDA-event time of a pass over the frames of the helix
    (after one warm-up sweep), voxel-updates/s and the algorithmic 16 B per
    voxel-update against the measured copy bandwidth."""
    from cuphoto import TSDFVolume
    S, cam, scene, poses = workload(args, 0)
    nf = len(poses)
    nvox = args.grid ** 3
    frames = S.render_sequence_torch(scene, poses, cam, seed=0)
    depths = [frames[k] for k in range(nf)]
    vol = TSDFVolume(volume_cfg(args, cam, args.mode))
    peak, peak_kind = peaks()
    rows = []
    for brick in range(9):
        def sweep():
            vol.reset()
            for k in range(nf):
                vol.integrate_frames(depths[k:k + 1], poses[k:k + 1], brick=brick)
        sweep()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        sweep()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / nf
        gbs = 16.0 * nvox / (ms * 1e-3) / 1e9
        kind = "streamed" if brick == 8 else ("staged" if brick >= 4 else "gathered")
        rows.append({"brick": brick, "depth": kind, "ms_per_frame": ms,
                     "voxel_updates_per_s": nvox / (ms * 1e-3), "algorithmic_gbs": gbs, "frac_of_peak": gbs / peak})
    vol.close()
    best = {d: min((r for r in rows if r["depth"] == d), key=lambda r: r["ms_per_frame"])
            for d in ("gathered", "staged", "streamed")}
    return {"workload": "one frame per pass, %d^3 voxels, %d frames 640x480 uint16, %s mode" % (args.grid, nf, args.mode),
            "peak_gbs": peak, "peak_kind": peak_kind, "rows": rows, "best": best,
            "staged_over_gathered": best["staged"]["ms_per_frame"] / best["gathered"]["ms_per_frame"],
            "streamed_over_gathered": best["streamed"]["ms_per_frame"] / best["gathered"]["ms_per_frame"]}


def onepass_summary(args, torch):
    """One frame per pass over the default workload's 512^3 volume (the
    reference's calling pattern, one TSDFVolume::integrate per frame) inside
    the default line: `--workload onepass` for every brick shape, the depth
    gathered, staged in shared memory and the bricks streamed by tensor
    copies.  A failure here is reported in the object and leaves the rest of
    the line intact."""
    import copy
    a2 = copy.copy(args)
    a2.mode = "compat"
    try:
        r = onepass_workload(a2, torch)
    except Exception as e:
        return {"error": "%s: %s" % (type(e).__name__, e)}
    finally:
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return r


def points_summary(args, torch):
    """`--workload points` inside the default line: extraction of 30 frames
    into a 9.2 M-point cloud and its z-buffer projection, beside the
    reference's extraction kernel and its host projection loop.  A failure
    here is reported in the object and leaves the rest of the line intact."""
    try:
        return points_workload(args, torch)
    except Exception as e:
        return {"error": "%s: %s" % (type(e).__name__, e)}
    finally:
        torch.cuda.synchronize()
        torch.cuda.empty_cache()


def refine_summary(args, torch):
    """The large pose-refinement configuration (1024^3 voxels of 0.25 cm,
    1000 frames 1280x720, 50 Gauss-Newton-preconditioned steps on 64
    jittered frames; `--workload refine` with its defaults) run inside the
    default line and reduced to its figures.  A failure here is reported in
    the object and leaves the rest of the line intact."""
    import copy
    a2 = copy.copy(args)
    a2.grid, a2.frames, a2.refine_frames, a2.refine_steps, a2.refine_method = 1024, 1000, 64, 50, "gn"
    try:
        r = refine_workload(a2, torch)
    except Exception as e:
        return {"error": "%s: %s" % (type(e).__name__, e)}
    finally:
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    keep = ("workload", "plain_forward", "refine_step_ms", "loss", "pose_error_before", "pose_error_after",
            "reduction")
    return {k: r[k] for k in keep if k in r}


def multiscene_summary(args, torch, local):
    """The multi-scene configuration (16 seeded scenes, 64^3..384^3, 10..120
    frames, one batched launch per window, autotuned, graph-captured) run
    inside the default line: its aggregate, integrate-only and end-to-end
    rates and the per-scene rates (3 timed steps after 1 warm-up)."""
    import copy
    a2 = copy.copy(args)
    a2.steps, a2.warmup, a2.config, a2.mode, a2.split_scenes = 3, 1, "", "compat", False
    r = multiscene(a2, torch, 0, 1, local)
    return {"value": r["value"], "unit": r["unit"], "ms_per_step": r["ms_per_step"], "steps": 3, "warmup": 1,
            "config": r["config"], "breakdown_ms": r["breakdown_ms"], "integrate_only": r["integrate_only"],
            "e2e": r["e2e"], "per_scene": r["per_scene"], "clocks": r["clocks"]}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.workload == "refine":
        import torch
        import importlib.util
        spec = importlib.util.spec_from_file_location("gbt_engine_build", os.path.join(PKG, "build.py"))
        eb = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(eb)
        eb.build()
        print(json.dumps(refine_workload(args, torch)), flush=True)
        return
    if args.workload == "points":
        import torch
        import importlib.util
        spec = importlib.util.spec_from_file_location("gbt_engine_build", os.path.join(PKG, "build.py"))
        eb = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(eb)
        eb.build()
        print(json.dumps(points_workload(args, torch)), flush=True)
        return
    if args.workload == "onepass":
        import torch
        import importlib.util
        spec = importlib.util.spec_from_file_location("gbt_engine_build", os.path.join(PKG, "build.py"))
        eb = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(eb)
        eb.build()
        print(json.dumps(onepass_workload(args, torch)), flush=True)
        return
    if args.workload == "diff":
        import torch
        import importlib.util
        spec = importlib.util.spec_from_file_location("gbt_engine_build", os.path.join(PKG, "build.py"))
        eb = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(eb)
        eb.build()
        print(json.dumps({"workload": "differentiable integrate, 128^3 x 16 frames 320x240",
                          "differentiable": differentiable_c3(torch)}), flush=True)
        return
    if args.workload == "multiscene":
        import torch
        rank, world, local = dist_env()
        torch.cuda.set_device(local)
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        import importlib.util
        spec = importlib.util.spec_from_file_location("gbt_engine_build", os.path.join(PKG, "build.py"))
        eb = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(eb)
        if rank == 0:
            eb.build()
        if world > 1:
            torch.distributed.barrier()
        out = multiscene(args, torch, rank, world, local)
        if out is not None:
            print(json.dumps(out), flush=True)
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import importlib.util
    spec = importlib.util.spec_from_file_location("gbt_engine_build", os.path.join(PKG, "build.py"))
    eb = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(eb)
    if rank == 0:
        eb.build()
    if world > 1:
        torch.distributed.barrier()
    import ctypes as C
    from cuphoto import TSDFVolume, extract_mesh_device, make_frame
    from cuphoto import _lib as L
    from cuphoto.autotune import tune_batched, tune_integrate
    from cuphoto.batch import BatchIntegrator

    S, cam, scene, poses = workload(args, rank)
    nf = len(poses)
    nvox = args.grid ** 3
    frames_dev = S.render_sequence_torch(scene, poses, cam, seed=rank)          # (n, H, W) int16 = u16 bits
    frames_host = torch.empty(frames_dev.shape, dtype=torch.int16, pin_memory=True)
    frames_host.copy_(frames_dev)
    torch.cuda.synchronize()
    tc = volume_cfg(args, cam, args.mode)
    vol = TSDFVolume(tc)
    depths = [frames_dev[k] for k in range(nf)]

    # two paths of the engine integrate one volume: passes of up to 32 frames
    # (gbt_integrate) and the batched launch with windows of up to 128 frames
    # (gbt_integrate_batch with this one volume); each is autotuned and the
    # faster on the whole sequence is timed
    batch = BatchIntegrator(max_scenes=1, max_frames=nf)
    if args.config:
        parts = args.config.split(",")
        b_, k_, c_ = (int(x) for x in parts[:3])
        path = parts[3] if len(parts) > 3 else "single"
        tune = {"brick": b_, "frames": k_, "ctas": c_, "ns_per_update": None, "table": []}
        candidates = 0
    else:
        t_single = tune_integrate(vol, depths, poses)
        t_batched = tune_batched(vol, depths, poses, batch)
        candidates = len(t_single["table"]) + len(t_batched["table"])

        def full_ms(fn):
            fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(2):
                fn()
            e1.record()
            e1.synchronize()
            return e0.elapsed_time(e1) / 2

        ms_single = full_ms(lambda: (vol.reset(), vol.integrate_sequence(
            depths, poses, frames_per_pass=t_single["frames"], brick=t_single["brick"],
            ctas_per_sm=t_single["ctas"])))
        ms_batched = full_ms(lambda: (vol.reset(), batch.integrate(
            [vol], [depths], [poses], brick=t_batched["brick"], ctas_per_sm=t_batched["ctas"],
            frames_per_launch=t_batched["frames"])))
        path, tune = ("batched", t_batched) if ms_batched < ms_single else ("single", t_single)
    K, brick, ctas = tune["frames"], tune["brick"], tune["ctas"]
    n_passes = (nf + K - 1) // K
    # the fastest tuned candidate inside the configuration's 8-32 frames per launch
    in_cfg = None
    if not args.config:
        cands = [(ns, "batched", b_, k_, c_) for (b_, k_, c_, ns) in t_batched["table"] if k_ <= 32]
        cands += [(ns, "single", b_, k_, c_) for (b_, k_, c_, ns) in t_single["table"] if k_ <= 32]
        if cands:
            in_cfg = min(cands)[1:]

    def integrate_all():
        if path == "batched":
            batch.integrate([vol], [depths], [poses], brick=brick, ctas_per_sm=ctas, frames_per_launch=K)
        else:
            vol.integrate_sequence(depths, poses, frames_per_pass=K, brick=brick, ctas_per_sm=ctas)

    # mesh capacity from an untimed run
    vol.reset()
    integrate_all()
    V0, T0 = extract_mesh_device(vol)
    cap = max(1024, int(len(V0) * 1.25) + 1024)
    verts = torch.empty((cap, 3, 3), dtype=torch.float32, device="cuda")
    tris = torch.empty((cap, 3), dtype=torch.int32, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    lib = L.lib()

    def step_reset():
        vol.reset()

    def step_integrate():
        integrate_all()

    def step_mesh():
        L.check(lib.gbt_extract_mesh_async(vol.handle, C.c_void_p(verts.data_ptr()), C.c_void_p(tris.data_ptr()),
                                           cap, 0, C.c_void_p(count.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream)))

    stream = torch.cuda.Stream()
    graphs = []
    with torch.cuda.stream(stream):
        for fn in (step_reset, step_integrate, step_mesh):   # warm the path once outside capture
            fn()
        torch.cuda.synchronize()
        for fn in (step_reset, step_integrate, step_mesh):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                fn()
            graphs.append(g)
    g_reset, g_int, g_mesh = graphs

    # graphs replay on the current stream: make it the stream the events go on
    torch.cuda.set_stream(stream)
    for _ in range(args.warmup):
        for g in graphs:
            g.replay()
    torch.cuda.synchronize()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t_wall = time.perf_counter()
        for i in range(args.steps):
            ev[i][0].record(stream)
            g_reset.replay()
            ev[i][1].record(stream)
            g_int.replay()
            ev[i][2].record(stream)
            g_mesh.replay()
            ev[i][3].record(stream)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    if world > 1:
        torch.distributed.barrier()
    step_ms = [ev[i][0].elapsed_time(ev[i][3]) for i in range(args.steps)]
    int_ms = [ev[i][1].elapsed_time(ev[i][2]) for i in range(args.steps)]
    mesh_ms = [ev[i][2].elapsed_time(ev[i][3]) for i in range(args.steps)]
    from cuphoto import shard
    total_ms = shard.max_over_ranks(ev[0][0].elapsed_time(ev[-1][3]))
    ntri = int(count.item())
    value = world * nvox * nf * args.steps / (total_ms * 1e-3)

    # roofline of the dominant kernel (the integrate pass), from the timed region
    launch_ms = float(np.mean(int_ms)) / n_passes
    frame_px = cam.width * cam.height
    alg_bytes = 16.0 * nvox + (nf / n_passes) * frame_px * 2 + (nf / n_passes) * 64
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    # DRAM bytes and warp instructions: one ncu capture of the five
    # integrate_batch_kernel launches of a step of this workload (512^3, 300
    # frames in windows of 64 and 44, brick 2, resident CTAs): 4.372 GB read +
    # 3.176 GB written and 28.17 G warp instructions for the step (bricks no
    # frame sees are neither loaded nor stored).  Only for that launch shape;
    # other grids, shapes and the fixed mode were not captured.
    captured = (path == "batched" and args.mode == "compat" and args.grid == 512 and nf == 300 and K == 64)
    traffic = (4.37171e9 + 3.17576e9) / n_passes if captured else None
    peak, peak_kind = peaks()
    # The kernel is bound by instruction issue, not by HBM (a window of K
    # frames shares each voxel's 16 bytes).  Its issue roofline: the captured
    # warp instructions per voxel-update, times the measured update rate,
    # against one instruction per clock on each of the 4 schedulers of every
    # SM at the median SM clock sampled while timing.
    issue = None
    if captured:
        warp_inst_per_update = 28.16625e9 / (512 ** 3 * 300)
        sm_count = torch.cuda.get_device_properties(local).multi_processor_count
        sm_mhz = (clocks.summary().get("sm_mhz") or 0.0)
        upd_per_s = nvox * (nf / n_passes) / (launch_ms * 1e-3)
        if sm_mhz > 0:
            achieved_i = warp_inst_per_update * upd_per_s
            peak_i = 4.0 * sm_count * sm_mhz * 1e6
            issue = {"unit": "warp instructions/s", "achieved": achieved_i, "peak": peak_i, "frac": achieved_i / peak_i,
                     "warp_instructions_per_update": warp_inst_per_update, "sm_mhz": sm_mhz, "sms": sm_count,
                     "source": "ncu capture of the step's integrate_batch_kernel launches at 512^3, 300 frames"}

    # end to end through the public API with host buffers: H2D of the step's
    # depth frames from pinned memory (on the batched path window by window,
    # overlapped with the previous window's launch), integrate, mesh, D2H of
    # the mesh
    e2e_ms = []
    h2d = frames_host.numel() * 2
    d2h = 0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vol.reset()
        if path == "batched":
            # window w + 1 copies while window w integrates
            batch.integrate_streamed([vol], [frames_host], [frames_dev], [poses], brick=brick, ctas_per_sm=ctas,
                                     frames_per_launch=K)
        else:
            frames_dev.copy_(frames_host, non_blocking=True)
            integrate_all()
        V, T = extract_mesh_device(vol, capacity=cap)
        Vh = V.cpu()
        Th = T.cpu()
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
            d2h = Vh.numel() * 4 + Th.numel() * 4 + 8
    e2e_value = shard.whole_job_rate(nvox * nf, float(np.mean(e2e_ms)) * 1e-3)

    # the configuration's own launch shape (8-32 frames per launch): reset +
    # integrate captured as one graph and timed the same way as the step
    integrate_in_config = None
    if in_cfg is not None and world == 1:
        p_, b_, k_, c_ = in_cfg

        def integ_cfg():
            vol.reset()
            if p_ == "batched":
                batch.integrate([vol], [depths], [poses], brick=b_, ctas_per_sm=c_, frames_per_launch=k_)
            else:
                vol.integrate_sequence(depths, poses, frames_per_pass=k_, brick=b_, ctas_per_sm=c_)
        with torch.cuda.stream(stream):
            integ_cfg()
            torch.cuda.synchronize()
            g_cfg = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g_cfg, stream=stream):
                integ_cfg()
            for _ in range(args.warmup):
                g_cfg.replay()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                g_cfg.replay()
            e1.record(stream)
            torch.cuda.synchronize()
        ms_cfg = e0.elapsed_time(e1) / args.steps
        integrate_in_config = {"value": nvox * nf / (ms_cfg * 1e-3), "unit": UNIT, "ms_per_step": ms_cfg,
                               "path": p_, "frames_per_launch": k_, "brick": b_, "ctas_per_sm": c_,
                               "what": "reset + integrate of the 300 frames, fastest tuned candidate with at "
                                       "most 32 frames per launch, graph replay x %d" % args.steps}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    extras = {}
    # the legs below time their own work on torch's current stream: give them
    # back the default stream the graphs' replays were moved off
    torch.cuda.synchronize()
    torch.cuda.set_stream(torch.cuda.default_stream())
    if not args.no_extras and world == 1:
        extras["reference_cuda"] = reference_cuda(args, cam, scene, poses, torch)
        extras["fixed_mode_mesh"] = fixed_mode_mesh(args, torch, cam, depths, poses, K, brick, ctas)
        extras["differentiable"] = differentiable_c3(torch)
        extras["multiscene"] = multiscene_summary(args, torch, local)
        torch.cuda.synchronize()
        torch.cuda.set_stream(torch.cuda.default_stream())
        extras["one_frame_per_call"] = onepass_summary(args, torch)
        extras["points"] = points_summary(args, torch)
        extras["refine"] = refine_summary(args, torch)
        cpu = cpu_baseline(args, cam, scene, poses)
    else:
        cpu = None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: seeded plane + 6 spheres, ray-cast uint16 depth, helix trajectory",
        "config": {"workload": "batched integrate + marching cubes, %d^3 voxels of %.2g cm, %d frames 640x480 uint16"
                               % (args.grid, 256.0 / args.grid, nf),
                   "mode": args.mode, "path": path, "frames_per_pass": K, "brick": brick, "ctas_per_sm": ctas,
                   "passes_per_step": n_passes, "graph": "reset, integrate passes, mesh captured as CUDA graphs",
                   "l2": "inputs larger than L2: 1 GiB volume + %d MB depth per step" % (frames_dev.numel() * 2 // 2**20),
                   "triangles": ntri},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "kernel": "integrate_batch_kernel" if path == "batched" else "integrate_kernel",
                     "launch_ms": launch_ms,
                     "algorithmic_bytes_per_launch": alg_bytes, "peak_kind": peak_kind,
                     "issue": issue},
        "breakdown_ms": {"reset": float(np.mean([ev[i][0].elapsed_time(ev[i][1]) for i in range(args.steps)])),
                         "integrate": float(np.mean(int_ms)), "mesh": float(np.mean(mesh_ms))},
        "integrate_only": {"value": nvox * nf / (float(np.mean(int_ms)) * 1e-3), "unit": UNIT},
        "mesh": {"triangles_per_s": ntri / (float(np.mean(mesh_ms)) * 1e-3) if ntri else 0.0, "triangles": ntri},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": float(np.mean(e2e_ms))},
        # per step: reset, the integrate launches, four mesh launches (count, reduce, scan, emit)
        "gpu_launches": args.steps * (1 + n_passes + 4),
        "clocks": clocks.summary(),
        "wall_s_timed": t_wall,
        "autotune": {"ns_per_update": tune["ns_per_update"], "candidates": candidates},
    }
    if integrate_in_config is not None:
        out["integrate_in_config"] = integrate_in_config
    if "fixed_mode_mesh" in extras:
        # marching cubes of a field with a surface (the fixed-mode field of the same frames)
        out["mesh_with_surface"] = extras["fixed_mode_mesh"]["mesh_fixed"]
    if cpu is not None:
        out["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    out.update(extras)
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
