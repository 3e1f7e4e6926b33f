"""CPU checks of the oracle: case tables, known-answer integrates, single-cube
meshes, a pure-Python restatement on tiny grids, and the golden vectors
produced by the reference's own GPU build."""
import glob
import os

import numpy as np
import pytest

from cuphoto import TSDFVolumeConfig
from cuphoto import synthetic as S

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = os.path.join(HERE, "..", "cu-reconstruction_gb300", "csrc", "mc_tables.inc")
def _reference_root():
    # the reference checkout the oracle recipe builds from (REFERENCE_ROOT)
    import oracle.build
    return oracle.build.REF_ROOT


REF_ROOT = _reference_root()
REF_TABLES = os.path.join(REF_ROOT, "modules", "include", "cuda", "marching_cubes_tables.cuh")

# reference corner numbering (marching_cubes.cu:118-127)
DX = [0, 1, 1, 0, 0, 1, 1, 0]
DY = [0, 0, 0, 0, 1, 1, 1, 1]
DZ = [0, 0, 1, 1, 0, 0, 1, 1]


def load_tables():
    import re
    txt = open(TABLES).read()

    def arr(name):
        body = re.search(name + r"\[\d+\] = \{(.*?)\}", txt, re.S).group(1)
        return [int(t.rstrip("ul"), 0) for t in re.findall(r"0x[0-9a-f]+ull|0x[0-9a-f]+|\d+", body)]
    ends = arr("GBT_MC_EDGE_ENDS")
    count = arr("GBT_MC_TRI_COUNT")
    mask = arr("GBT_MC_EDGE_MASK")
    packed = arr("GBT_MC_TRI_PACKED")
    return [(e & 15, e >> 4) for e in ends], count, mask, packed


def tri_edges(packed, case, k):
    return (packed[case] >> (4 * k)) & 15


def test_tables_consistent():
    ends, count, mask, packed = load_tables()
    assert len(ends) == 12 and len(count) == 256 and len(mask) == 256 and len(packed) == 256
    for c in range(256):
        sign = [(c >> k) & 1 for k in range(8)]
        geo = sum(1 << e for e in range(12) if sign[ends[e][0]] != sign[ends[e][1]])
        used = 0
        for k in range(3 * count[c]):
            used |= 1 << tri_edges(packed, c, k)
        assert used == mask[c] == geo, c
    # edges join corners that differ in exactly one coordinate
    for a, b in ends:
        assert abs(DX[a] - DX[b]) + abs(DY[a] - DY[b]) + abs(DZ[a] - DZ[b]) == 1
    assert count[0] == count[255] == 0


@pytest.mark.skipif(not os.path.exists(REF_TABLES), reason="reference checkout not present")
def test_tables_match_reference_file():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "gen", os.path.join(HERE, "..", "cu-reconstruction_gb300", "csrc", "gen_mc_tables.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    ends, edge_table, tri = gen.load_reference_tables(REF_ROOT)
    e2, count, mask, packed = load_tables()
    assert ends == e2
    assert mask == edge_table
    for c in range(256):
        row = [tri_edges(packed, c, k) for k in range(3 * count[c])]
        assert row + [-1] * (16 - len(row)) == tri[c]


def fastdiv_host(d):
    if d <= 1:
        return d, 0, 0
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    return d, m & 0xFFFFFFFF, l


def fastdiv_dev(n, f):
    d, m, s = f
    if d == 1:
        return n
    t = (m * n) >> 32
    return (t + ((n - t) >> 1)) >> (s - 1)


def test_fastdiv_matches_integer_division():
    rng = np.random.default_rng(0)
    divisors = [1, 2, 3, 5, 7, 63, 64, 65, 127, 255, 256, 511, 1023, 1024, 4095, 65535, 65536, 99991]
    divisors += [int(x) for x in rng.integers(2, 1 << 24, size=40)]
    for d in divisors:
        f = fastdiv_host(d)
        ns = [0, 1, d - 1, d, d + 1, 2 * d - 1, (1 << 32) - 1, (1 << 31)] + [int(x) for x in rng.integers(0, 1 << 32, 200)]
        for n in ns:
            assert fastdiv_dev(n, f) == n // d, (n, d)


def test_fused_uint16_conversion_is_the_rounded_product():
    """The integrate kernels form a uint16 sample as fma(2^23 + raw, scale,
    -2^23 * scale), 2^23 + raw being the float with the bits of 2^23 OR raw,
    for scales whose biased exponent lies in 1..231.  Restated here with the
    exact sum in float64 (a 24-bit by 24-bit product and a 40-bit result fit
    its 53 bits) rounded once to float32, as the fused multiply-add rounds:
    equal to float32(raw) * scale for every raw value, none of the products
    subnormal, and 2^23 * scale exact."""
    raw = np.arange(65536, dtype=np.uint32)
    a = (raw | np.uint32(0x4B000000)).view(np.float32)
    assert np.array_equal(a.astype(np.float64), raw + 8388608.0)
    rng = np.random.default_rng(3)
    scales = [np.float32(2.0 ** -126), np.nextafter(np.float32(2.0 ** 105), np.float32(0)), np.float32(0.001),
              np.float32(1e-3 / 3), np.float32(0.0002), np.float32(1.0), np.float32(-0.001)]
    scales += [np.float32(x) for x in 2.0 ** rng.uniform(-126, 105, 40)]
    for sc in scales:
        e = (int(np.float32(sc).view(np.uint32)) >> 23) & 0xFF
        assert 1 <= e <= 231
        bias = np.float32(-8388608.0) * sc
        assert float(bias) == -8388608.0 * float(sc)              # exact
        fused = (a.astype(np.float64) * float(sc) + float(bias)).astype(np.float32)
        plain = raw.astype(np.float32) * sc
        assert np.array_equal(fused.view(np.uint32)[1:], plain.view(np.uint32)[1:]), sc
        assert fused[0] == 0 and plain[0] == 0                    # (signs of zero aside)
        assert np.all(np.abs(plain[1:]) >= np.finfo(np.float32).tiny)


def small_cfg(**kw):
    base = dict(voxel_grid_size=(16, 12, 8), physical_size=(0.8, 0.6, 0.4), global_offset=(-0.4, -0.3, 0.6),
                focal_x=100.0, focal_y=100.0, cx=31.5, cy=23.5, camera_width=64, camera_height=48, max_weight=64)
    base.update(kw)
    return TSDFVolumeConfig(**base)


def test_derived_voxel_size_and_truncation(oracle):
    c = oracle.cfg_from(small_cfg())
    vs, tr = oracle.derive(c)
    np.testing.assert_array_equal(vs, np.float32([0.8, 0.6, 0.4]) / np.float32([16, 12, 8]))
    v = vs.astype(np.float32)
    dot = np.float32(v[0] * v[0] + v[1] * v[1]) + np.float32(v[2] * v[2])
    assert tr == np.float32(1.1) * np.sqrt(np.float32(dot))
    c2 = oracle.cfg_from(small_cfg(truncation=0.07))
    assert oracle.derive(c2)[1] == np.float32(0.07)


def voxel_centres(cfg, vs):
    ax = []
    for i in range(3):
        v = np.arange(cfg.voxel_grid_size[i], dtype=np.float64)
        ax.append(((v + 0.5) * np.float64(vs[i]) + np.float64(np.float32(cfg.global_offset[i]))))
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return X, Y, Z


def test_compat_identity_pose_known_answer(oracle):
    """Identity pose, constant depth: one frame gives D = min(d - z, trunc)
    where sdf >= -trunc, W = 1; two frames average exactly."""
    tc = small_cfg()
    c = oracle.cfg_from(tc)
    vs, tr = oracle.derive(c)
    D, W = oracle.init_volume(c)
    assert np.all(D == np.float32(tr)) and np.all(W == 0)
    depth = np.full((48, 64), 0.8, np.float32)
    pose = np.array([1.0, 0, 0, 0, 0, 0, 0])
    oracle.integrate_compat(c, D, W, depth, pose)
    X, Y, Z = voxel_centres(tc, vs)
    qu = X * tc.focal_x / Z + tc.cx
    qv = Y * tc.focal_y / Z + tc.cy
    inside = (qu > -1 + 1e-3) & (qu < 64 - 1e-3) & (qv > -1 + 1e-3) & (qv < 48 - 1e-3)
    far = (np.abs(qu - np.rint(qu)) > 1e-3) & (np.abs(qv - np.rint(qv)) > 1e-3)
    sdf = np.float32(0.8) - Z.astype(np.float32)
    upd = inside & (sdf >= -np.float32(tr))
    m = far
    assert np.array_equal(W[m], upd[m].astype(np.float32))
    exp = np.where(sdf > 0, np.minimum(sdf, np.float32(tr)), sdf)
    assert np.array_equal(D[m & upd], exp[m & upd])
    assert np.all(D[m & ~upd] == np.float32(tr))
    assert upd.sum() > 100
    D1 = D.copy()
    depth2 = np.full((48, 64), 0.7, np.float32)
    oracle.integrate_compat(c, D, W, depth2, pose)
    sdf2 = np.float32(0.7) - Z.astype(np.float32)
    upd2 = inside & (sdf2 >= -np.float32(tr))
    t2 = np.where(sdf2 > 0, np.minimum(sdf2, np.float32(tr)), sdf2).astype(np.float32)
    both = m & upd & upd2
    assert both.sum() > 50
    exp2 = ((D1[both] * np.float32(1) + t2[both]).astype(np.float32) / np.float32(2)).astype(np.float32)
    assert np.array_equal(D[both], exp2)
    assert np.all(W[both] == 2)


def test_fixed_plane_known_answer(oracle):
    """Fixed mode, identity pose, fronto-parallel plane at z0: D = clamp(z0 - z)."""
    tc = small_cfg(mode="fixed", max_weight=3)
    c = oracle.cfg_from(tc)
    vs, tr = oracle.derive(c)
    D, W = oracle.init_volume(c)
    raw = np.full((48, 64), 800, np.uint16)
    pose = np.array([1.0, 0, 0, 0, 0, 0, 0])
    for _ in range(5):
        oracle.integrate_fixed(c, D, W, raw, pose, 0.001)
    X, Y, Z = voxel_centres(tc, vs)
    u = X * tc.focal_x / Z + tc.cx
    v = Y * tc.focal_y / Z + tc.cy
    inside = (u > -0.5 + 1e-3) & (u < 63.5 - 1e-3) & (v > -0.5 + 1e-3) & (v < 47.5 - 1e-3)
    z0 = np.float32(800) * np.float32(0.001)
    sdf = (z0 - Z.astype(np.float32)).astype(np.float32)
    upd = inside & (sdf >= -np.float32(tr))
    assert upd.sum() > 100
    assert np.all(W[upd] == 3)            # clamped at max_weight
    # five identical observations: the running mean stays at the observation
    np.testing.assert_allclose(D[upd], np.minimum(sdf[upd], np.float32(tr)), rtol=0, atol=2e-7)
    bad = ~inside
    assert np.all(W[bad] == 0)


def cube_grid(case, value=1.0):
    D = np.empty((2, 2, 2), np.float32)
    for k in range(8):
        D[DZ[k], DY[k], DX[k]] = -value if (case >> k) & 1 else value
    return D


@pytest.mark.parametrize("mode", ["compat", "fixed"])
def test_all_256_single_cube_cases(oracle, mode):
    """Every cube case on a 2x2x2 grid: triangle count from the table and
    each vertex at the midpoint of its edge (corner values +-1)."""
    ends, count, mask, packed = load_tables()
    tc = TSDFVolumeConfig(voxel_grid_size=(2, 2, 2), physical_size=(2.0, 2.0, 2.0), global_offset=(0, 0, 0),
                          mode=mode, max_weight=8)
    c = oracle.cfg_from(tc)
    for case in range(256):
        D = cube_grid(case)
        W = np.ones_like(D)
        if mode == "compat":
            V, T = oracle.mc_compat(c, D.ravel(), index_base=5)
        else:
            V, T = oracle.mc_fixed(c, D.ravel(), W.ravel(), index_base=5)
        assert len(V) == count[case], case
        assert np.array_equal(T.ravel(), 5 + np.arange(3 * len(T)))
        for t in range(len(V)):
            for j in range(3):
                e = tri_edges(packed, case, 3 * t + j)
                a, b = ends[e]
                mid = np.array([(DX[a] + DX[b]) / 2 + 0.5, (DY[a] + DY[b]) / 2 + 0.5, (DZ[a] + DZ[b]) / 2 + 0.5])
                np.testing.assert_array_equal(V[t, j], mid.astype(np.float32))


def test_fixed_mc_skips_unobserved_cubes(oracle):
    tc = TSDFVolumeConfig(voxel_grid_size=(2, 2, 2), physical_size=(2.0, 2.0, 2.0), mode="fixed", max_weight=8)
    c = oracle.cfg_from(tc)
    D = cube_grid(1)
    W = np.ones_like(D)
    W[1, 1, 1] = 0
    V, T = oracle.mc_fixed(c, D.ravel(), W.ravel())
    assert len(V) == 0


def py_mc_compat(grid, vs, off, D):
    """Pure-Python restatement of marching_cubes.cu:102-189 (tiny grids only)."""
    ends, count, mask, packed = load_tables()
    gx, gy, gz = grid
    layer = gx + gy
    f32 = np.float32
    out = []
    for vz in range(gz - 1):
        for vy in range(gy - 1):
            for vx in range(gx - 1):
                b0 = vz * layer + vy * gx + vx
                b1 = b0 + layer
                lin = [b0, b0 + 1, b1 + 1, b1, b0 + gx, b0 + gx + 1, b1 + gx + 1, b1 + gx]
                val = [f32(D[i]) for i in lin]
                case = sum(1 << k for k in range(8) if val[k] < 0)
                for t in range(count[case]):
                    tri = []
                    for j in range(3):
                        e = tri_edges(packed, case, 3 * t + j)
                        a, b = ends[e]
                        s, en = val[a], val[b]
                        if s > 0 and en < 0:
                            a, b, s, en = b, a, en, s
                        r = f32(-s) / f32(en - s)
                        pa = [f32((f32(i) + f32(0.5)) * f32(vs[k])) + f32(off[k]) for k, i in
                              enumerate((lin[a] % gx, (lin[a] // gx) % gy, lin[a] // (gx * gy)))]
                        pb = [f32((f32(i) + f32(0.5)) * f32(vs[k])) + f32(off[k]) for k, i in
                              enumerate((lin[b] % gx, (lin[b] // gx) % gy, lin[b] // (gx * gy)))]
                        tri.append([f32(pa[k] + f32(r * f32(pb[k] - pa[k]))) for k in range(3)])
                    out.append(tri)
    return np.array(out, np.float32).reshape(-1, 3, 3)


@pytest.mark.parametrize("grid", [(4, 3, 3), (5, 4, 3), (3, 3, 5)])
def test_compat_mc_layer_stride_quirk_matches_python(oracle, grid):
    """The oracle's compat mesh reads layers gx+gy apart (marching_cubes.cu:211)
    exactly like a direct Python restatement; vertices agree to 4 ulp (the
    Python version rounds the multiply-adds separately)."""
    rng = np.random.default_rng(sum(grid))
    tc = TSDFVolumeConfig(voxel_grid_size=grid, physical_size=tuple(0.1 * g for g in grid), global_offset=(-0.2, 0.1, 0.5))
    c = oracle.cfg_from(tc)
    vs, _ = oracle.derive(c)
    D = rng.uniform(-1, 1, size=grid[0] * grid[1] * grid[2]).astype(np.float32)
    V, T = oracle.mc_compat(c, D)
    P = py_mc_compat(grid, vs, tc.global_offset, D)
    assert V.shape == P.shape and len(V) > 0
    np.testing.assert_allclose(V, P, rtol=0, atol=4 * np.finfo(np.float32).eps * 2)


def test_synthetic_sequence_is_deterministic():
    a = S.make_sequence(2, scene_id=3, camera=S.Camera.half())
    b = S.make_sequence(2, scene_id=3, camera=S.Camera.half())
    assert np.array_equal(a.depth_u16, b.depth_u16) and np.array_equal(a.poses, b.poses)
    valid = (a.depth_u16 > 0).mean()
    assert 0.5 < valid < 0.99
    R = S.matrix_from_quat(a.poses[0][:4])
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)


GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "ref_*.npz")))


@pytest.mark.skipif(not GOLDEN, reason="no golden vectors from the reference build")
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_against_reference_golden(oracle, path):
    """The reference's own kernels (run on a GB300 by tests/golden/make_golden.py)
    against the oracle: distances and weights identical except at voxels
    whose pixel index sits within a few ulp of a truncation boundary (the
    reference divides approximately), and the same mesh from the same field."""
    g = np.load(path)
    tc = TSDFVolumeConfig(voxel_grid_size=tuple(int(x) for x in g["grid"]), physical_size=tuple(g["phys"]),
                          global_offset=tuple(g["offset"]), focal_x=float(g["K"][0]), focal_y=float(g["K"][1]),
                          cx=float(g["K"][2]), cy=float(g["K"][3]), max_weight=float(g["max_weight"]))
    c = oracle.cfg_from(tc)
    D, W = oracle.init_volume(c)
    flags = np.zeros(D.shape, np.uint8)
    depth = g["depth_u16"].astype(np.float32) * np.float32(g["depth_scale"])
    h, w = depth.shape[1:]
    for k in range(len(depth)):
        oracle.integrate_compat(c, D, W, depth[k], g["poses"][k])
        oracle.compat_ambiguous(c, g["poses"][k], w, h, 8.0, flags)
    Dr, Wr = g["D"], g["W"]
    ok = flags == 0
    trunc = float(oracle.derive(c)[1])
    tol = 1e-6 * trunc * len(depth)
    # weights differ only where a pixel index is ambiguous
    assert np.all(W[ok] == Wr[ok])
    # away from ambiguous pixels the distances agree to the reference's division error
    np.testing.assert_allclose(D[ok], Dr[ok], rtol=0, atol=tol)
    # and the ambiguous voxels that did flip to another pixel are few
    flipped = (~ok) & ((W != Wr) | (np.abs(D - Dr) > tol))
    assert flipped.sum() <= max(10, 1e-3 * D.size)
    # mesh of the reference's own field
    V, T = oracle.mc_compat(c, Dr.ravel())
    assert len(V) == int(g["ntri"])
    tol = max(1e-5 * float(np.max(oracle.derive(c)[0])), 2 * float(np.spacing(np.float32(np.abs(V).max(initial=1)))))
    np.testing.assert_allclose(V, g["verts"], rtol=0, atol=tol)
    assert np.array_equal(T, g["tris"])


# ---------------------------------------------------------------------------
# Differentiable integrate: the oracle's FP64 gradient against FP64 central
# differences, on voxels whose discrete decisions do not change in the step.
import diffcase  # noqa: E402


def _oracle_run(oracle, case, R, t, depth, D0=None, W0=None):
    cfg = oracle.diff_cfg(case["grid"], case["vs"], case["off"], case["K"], case["trunc"], case["max_weight"],
                          case["max_depth"], case["min_z"], case["width"], case["height"], 1)
    shape = case["grid"][::-1]
    D = np.full(shape, case["trunc"], np.float64) if D0 is None else D0.copy()
    W = np.zeros(shape, np.float64) if W0 is None else W0.copy()
    sig = oracle.diff_forward(cfg, D, W, np.asarray(depth, np.float64), R.reshape(-1, 9), t)
    return D, W, sig, cfg


def _fd_check(oracle, case, dphi, dt, ddep, h, D0=None, W0=None):
    """(finite difference, analytic) directional derivative of
    L = sum W (D - gt)^2 over voxels whose decisions do not change.

    The difference is Richardson-extrapolated from central differences at h
    and h/2, (4 D(h/2) - D(h)) / 3, whose error is O(h^4): bilinear depth
    gives the loss large third derivatives near depth edges, so a plain
    central difference at a step the FP64 round-off allows is only good to
    a few 1e-5."""
    runs = {}
    for k in (1, 0.5, -0.5, -1):
        R, t, dep = diffcase.perturbed(case, k * h, dphi, dt, ddep)
        runs[k] = _oracle_run(oracle, case, R, t, dep, D0, W0)
    D, W, s0, cfg = _oracle_run(oracle, case, case["R"], case["t"], case["depth"], D0, W0)
    mask = np.logical_and.reduce([r[2] == s0 for r in runs.values()])
    loss = lambda r: float(np.sum((r[1] * (r[0] - case["gt"]) ** 2)[mask]))
    d1 = (loss(runs[1]) - loss(runs[-1])) / (2 * h)
    d2 = (loss(runs[0.5]) - loss(runs[-0.5])) / h
    fd = (4 * d2 - d1) / 3
    shape = case["grid"][::-1]
    gD = 2 * W * (D - case["gt"]) * mask
    gW = (D - case["gt"]) ** 2 * mask
    D0 = np.full(shape, case["trunc"]) if D0 is None else D0
    W0 = np.zeros(shape) if W0 is None else W0
    gdep, gpose, _, _ = oracle.diff_backward(cfg, gD, gW, D0, W0, case["depth"], case["R"].reshape(-1, 9), case["t"])
    an = diffcase.directional(gpose[:, :9].reshape(-1, 3, 3), gpose[:, 9:], gdep, case, dphi, dt, ddep)
    return fd, an, mask


@pytest.mark.parametrize("seed", [0, 1])
def test_oracle_gradient_matches_fp64_central_differences(oracle, seed):
    case = diffcase.make_case(seed=seed)
    dphi, dt, ddep = diffcase.perturbation(case, seed=seed + 10)
    fd, an, mask = _fd_check(oracle, case, dphi, dt, ddep, 1e-6)
    assert mask.mean() > 0.5
    assert abs(fd) > 1e-6
    assert abs(an - fd) <= 1e-7 * abs(fd), (an, fd)


def test_oracle_gradient_with_saturated_weights(oracle):
    """Weights at max_weight before the frames: the running mean is an
    exponential average; the gradient still matches central differences."""
    case = diffcase.make_case(seed=3, frames=4)
    case["max_weight"] = 2.0
    dphi, dt, ddep = diffcase.perturbation(case, seed=7)
    shape = case["grid"][::-1]
    fd, an, _ = _fd_check(oracle, case, dphi, dt, ddep, 1e-6, np.full(shape, 0.01), np.full(shape, 2.0))
    assert abs(an - fd) <= 1e-7 * abs(fd), (an, fd)


def test_oracle_loss_is_smooth_along_the_gradient(oracle):
    """With continuous sample weights the loss has no jumps: along -grad its
    deviation from the linear model shrinks in proportion to the step (a
    sample appearing or leaving would add a step-independent jump, which
    dominates at the smallest steps), and it keeps falling up to 1e-3."""
    case = diffcase.make_case(seed=5, frames=6)
    D, W, _, cfg = _oracle_run(oracle, case, case["R"], case["t"], case["depth"])
    shape = case["grid"][::-1]
    gdep, gpose, _, _ = oracle.diff_backward(cfg, 2 * W * (D - case["gt"]), (D - case["gt"]) ** 2,
                                             np.full(shape, case["trunc"]), np.zeros(shape), case["depth"],
                                             case["R"].reshape(-1, 9), case["t"])
    gR = gpose[:, :9].reshape(-1, 3, 3)
    gt = gpose[:, 9:]
    A = gR @ case["R"].transpose(0, 2, 1)
    phi = np.stack([A[:, 2, 1] - A[:, 1, 2], A[:, 0, 2] - A[:, 2, 0], A[:, 1, 0] - A[:, 0, 1]], -1)
    phi = phi + np.cross(case["t"], gt)
    L0 = float(np.sum(W * (D - case["gt"]) ** 2))
    norm = np.sqrt((phi ** 2).sum() + (gt ** 2).sum())
    for s in (1e-9, 1e-8, 1e-7, 1e-6, 1e-5, 1e-4, 1e-3):
        R = np.stack([diffcase.rot_exp(-s * phi[k] / norm) @ case["R"][k] for k in range(len(phi))])
        t = np.stack([diffcase.rot_exp(-s * phi[k] / norm) @ case["t"][k] - s * gt[k] / norm for k in range(len(phi))])
        D2, W2, _, _ = _oracle_run(oracle, case, R, t, case["depth"])
        dL = float(np.sum(W2 * (D2 - case["gt"]) ** 2)) - L0
        rel = abs(dL + s * norm) / (s * norm)
        assert dL < 0, (s, dL)
        if s <= 1e-6:
            assert rel <= 1e3 * s, (s, dL, -s * norm)
