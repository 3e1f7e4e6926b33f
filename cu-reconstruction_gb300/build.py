"""Build the engine's shared library ``_build/libgbt_tsdf.so`` for sm_103a.

The translation units compile in parallel; ``k_ref.cu`` alone gets
``-use_fast_math`` (the compat mode's reference arithmetic).  Host code is
compiled with ``-ffp-contract=off`` so that host-side pose arithmetic gives the
same bits on x86-64 and AArch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgbt_tsdf.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]

UNITS = {
    "k_ref.cu": ["-use_fast_math"],
    "k_ieee.cu": [],
    "k_util.cu": [],
    "capi.cu": [],
    "k_noalloc.cu": [],
    "k_diff.cu": [],
    "k_points.cu": [],
}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cuh", ".h", ".inc")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT_DIR, unit.replace(".cu", ".o"))
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr))
    return obj, r.stderr


CPP = os.path.join(HERE, "cpp")
SHIM = os.path.join(OUT_DIR, "libcuphoto_gb300.so")
EXAMPLE = os.path.join(OUT_DIR, "tsdf_surface_headless")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_cpp(force=False):
    """The C++ layer over the C ABI (cuphoto::TSDFVolume, TSDFSurface, Mesh,
    Config) and the headless example driver."""
    srcs = sorted(os.path.join(CPP, "src", f) for f in os.listdir(os.path.join(CPP, "src")) if f.endswith(".cpp"))
    hdrs = sorted(os.path.join(CPP, "include", "cuphoto", f) for f in os.listdir(os.path.join(CPP, "include", "cuphoto")))
    ex = os.path.join(CPP, "examples", "tsdf_surface_headless.cpp")
    inc = ["-I" + os.path.join(CPP, "include"), "-I" + os.path.join(HERE, "..", "include"),
           "-I" + os.path.join(CUDA_HOME, "include")]
    libs = ["-L" + OUT_DIR, "-lgbt_tsdf", "-L" + os.path.join(CUDA_HOME, "lib64"), "-lcudart",
            "-Wl,-rpath," + OUT_DIR, "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")]
    flags = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off"]
    if force or _stale(SHIM, srcs + hdrs + [LIB]):
        r = subprocess.run(flags + ["-shared"] + inc + srcs + ["-o", SHIM + ".tmp"] + libs, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("C++ layer build failed:\n%s" % r.stderr[-4000:])
        os.replace(SHIM + ".tmp", SHIM)
    if force or _stale(EXAMPLE, [ex, SHIM] + hdrs):
        r = subprocess.run(flags + inc + [ex, "-o", EXAMPLE + ".tmp", "-L" + OUT_DIR, "-lcuphoto_gb300"] + libs,
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("example build failed:\n%s" % r.stderr[-4000:])
        os.replace(EXAMPLE + ".tmp", EXAMPLE)
    return SHIM, EXAMPLE


def build(force=False, verbose=False):
    """Compile every translation unit and link the shared library; returns its path."""
    lib = build_engine(force, verbose)
    build_cpp(force)
    return lib


def build_engine(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = _sources() + [os.path.join(HERE, "..", "include", "gbt_tsdf.h"), os.path.abspath(__file__)]
    if not force and not _stale(LIB, deps):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, u, e, verbose) for u, e in UNITS.items()]
        results = [f.result() for f in futs]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
