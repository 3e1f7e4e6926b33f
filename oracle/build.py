"""Build the CPU oracle and, where the reference sources are present, the
reference's own CUDA kernels.

TEST INFRASTRUCTURE ONLY -- nothing here is part of the engine.

Outputs
  oracle/_build/liboracle.so       the CPU restatement (tsdf_oracle.cpp)
  oracle/_build/libref_harness.so  host driver for the reference's kernels
  oracle/_ref/ref_tsdf.cubin       the reference's kernels, compiled from
                                   modules/src/cuda/{tsdf_volume,marching_cubes,
                                   camera_util,cuda_point_cloud,util}.cu with the reference's own
                                   device flags (-use_fast_math -rdc=true,
                                   modules/CMakeLists.txt:17-22,73,79), linked
  oracle/_ref/ref_kernels.txt      mangled names of its kernels, read from the
                                   cubin's ELF symbol table

The reference cubin is only built where the reference checkout exists
(REFERENCE_ROOT, default /root/reference); elsewhere a cubin built earlier is
used if present.  OpenCV is not installed, so ref_shim/ supplies the
image-view types the reference's headers name and declarations of the host
image type its point-cloud source uses (only its kernels are compiled).
"""
import os
import shutil
import struct
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("REFERENCE_ROOT", "/root/reference")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
REF_UNITS = ["tsdf_volume", "marching_cubes", "camera_util", "cuda_point_cloud", "util"]
# key -> a substring of the kernel's mangled name
REF_KERNELS = {"cu_tsdf_integrate": "cu_tsdf_integrate", "set_array_to_value": "set_array_to_value",
               "init_voxel_transofrmation": "init_voxel_transofrmation",
               "marching_cubes_kernel": "marching_cubes_kernel",
               "point_cloud_extract": "point_cloud_extractILb0E", "point_cloud_extract_rgb": "point_cloud_extractILb1E",
               "transform_points": "transform_points", "filter_image_if": "filter_image_if"}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "tsdf_oracle.cpp")
    tables = os.path.join(HERE, "..", "cu-reconstruction_gb300", "csrc", "mc_tables.inc")
    out = os.path.join(BUILD, "liboracle.so")
    if force or _stale(out, [src, tables, __file__]):
        _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def _elf_symbols(path):
    """Names in the .symtab of an ELF64 file (exported symbol names only)."""
    data = open(path, "rb").read()
    assert data[:4] == b"\x7fELF" and data[4] == 2
    shoff = struct.unpack_from("<Q", data, 0x28)[0]
    shentsize, shnum = struct.unpack_from("<HH", data, 0x3A)
    secs = [struct.unpack_from("<IIQQQQIIQQ", data, shoff + i * shentsize) for i in range(shnum)]
    names = []
    for s in secs:
        if s[1] != 2:  # SHT_SYMTAB
            continue
        strtab = secs[s[6]]
        for off in range(s[4], s[4] + s[5], 24):
            name_off = struct.unpack_from("<I", data, off)[0]
            start = strtab[4] + name_off
            end = data.index(b"\x00", start)
            names.append(data[start:end].decode())
    return names


def build_reference_cubin(force=False):
    """Compile the reference's TSDF kernels; returns the cubin path or None."""
    cubin = os.path.join(REF_OUT, "ref_tsdf.cubin")
    names_file = os.path.join(REF_OUT, "ref_kernels.txt")
    if not os.path.isdir(os.path.join(REF_ROOT, "modules")):
        return cubin if os.path.exists(cubin) and os.path.exists(names_file) else None
    srcs = [os.path.join(REF_ROOT, "modules/src/cuda/%s.cu" % u) for u in REF_UNITS]
    shims = [os.path.join(HERE, "ref_shim/opencv2/core/core.hpp"), os.path.join(HERE, "ref_shim/opencv2/core/cuda/common.hpp")]
    if not force and not _stale(cubin, srcs + shims + [__file__]) and os.path.exists(names_file):
        return cubin
    os.makedirs(REF_OUT, exist_ok=True)
    nvcc = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    inc = ["-I" + os.path.join(HERE, "ref_shim"), "-I" + os.path.join(REF_ROOT, "modules/include"),
           "-I" + os.path.join(REF_ROOT, "modules/include/cuda"), "-I" + os.path.join(REF_ROOT, "3dparty")]
    parts = []
    for u, src in zip(REF_UNITS, srcs):
        obj = os.path.join(REF_OUT, u + ".rdc.cubin")
        _run([nvcc, "-arch=sm_103a", "-use_fast_math", "-rdc=true", "-std=c++14", "-cubin", "-w"] + inc +
             [src, "-o", obj])
        parts.append(obj)
    nvlink = shutil.which("nvlink") or os.path.join(CUDA_HOME, "bin", "nvlink")
    _run([nvlink, "-arch=sm_103a"] + parts + ["-o", cubin + ".tmp"])
    os.replace(cubin + ".tmp", cubin)
    syms = _elf_symbols(cubin)
    with open(names_file, "w") as f:
        for k, pat in REF_KERNELS.items():
            hits = [s for s in syms if ("cuphoto" in s and pat in s and s.startswith("_Z"))]
            if not hits:
                raise RuntimeError("kernel %s not found in the reference cubin" % k)
            f.write("%s %s\n" % (k, sorted(hits, key=len)[0]))
    return cubin


def build_ref_harness(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref_harness.cpp")
    out = os.path.join(BUILD, "libref_harness.so")
    if force or _stale(out, [src, __file__, os.path.join(HERE, "ref_shim/opencv2/core/cuda/common.hpp"),
                             os.path.join(HERE, "ref_shim/opencv2/core/core.hpp")]):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", src,
              "-I" + os.path.join(HERE, "ref_shim"), "-I" + os.path.join(CUDA_HOME, "include"),
              "-L" + os.path.join(CUDA_HOME, "lib64"), "-lcudart_static", "-ldl", "-lpthread", "-lrt",
              "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def build_ref_project(force=False):
    """The reference's host z-buffer loop (cudaPointCloud::project_to_color_depth,
    cuda_point_cloud.cu:292-353) in an x86 host program (ref_project_main.cu),
    compiled from the reference's sources as its Release build compiles them
    (host code -O3, no -march: no fused multiply-adds on x86-64; device code
    -use_fast_math -rdc=true).  Returns the program's path, or None where the
    reference checkout is absent.  Only used to make golden vectors."""
    exe = os.path.join(REF_OUT, "ref_project")
    if not os.path.isdir(os.path.join(REF_ROOT, "modules")):
        return exe if os.path.exists(exe) else None
    main = os.path.join(HERE, "ref_project_main.cu")
    srcs = [os.path.join(REF_ROOT, "modules/src/cuda/cuda_point_cloud.cu"), os.path.join(REF_ROOT, "modules/src/cuda/util.cu")]
    log_src = os.path.join(REF_ROOT, "3dparty/CudaUtils/logging.cpp")
    shims = [os.path.join(HERE, "ref_shim/opencv2/core/core.hpp"), os.path.join(HERE, "ref_shim/opencv2/core/cuda/common.hpp")]
    if not force and not _stale(exe, srcs + [main, log_src] + shims + [__file__]):
        return exe
    os.makedirs(REF_OUT, exist_ok=True)
    nvcc = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    inc = ["-I" + os.path.join(HERE, "ref_shim"), "-I" + os.path.join(REF_ROOT, "modules/include"),
           "-I" + os.path.join(REF_ROOT, "modules/include/cuda"), "-I" + os.path.join(REF_ROOT, "3dparty")]
    flags = ["-arch=sm_103a", "-use_fast_math", "-rdc=true", "-std=c++14", "-O3", "-Xcompiler", "-O3", "-w"]
    objs = []
    for src in srcs + [main]:
        obj = os.path.join(REF_OUT, "host_" + os.path.basename(src) + ".o")
        _run([nvcc] + flags + inc + ["-c", src, "-o", obj])
        objs.append(obj)
    log_obj = os.path.join(REF_OUT, "host_logging.o")
    _run(["g++", "-O3", "-std=c++14", "-w", "-c", log_src, "-o", log_obj])
    _run([nvcc, "-arch=sm_103a", "-rdc=true"] + objs + [log_obj, "-o", exe + ".tmp"])
    os.replace(exe + ".tmp", exe)
    return exe


def build_all(force=False):
    out = {"oracle": build_oracle(force)}
    try:
        out["ref_cubin"] = build_reference_cubin(force)
    except Exception as e:  # the reference build is optional evidence, never required
        sys.stderr.write("reference cubin not built: %s\n" % e)
        out["ref_cubin"] = None
    out["ref_harness"] = build_ref_harness(force)
    try:
        out["ref_project"] = build_ref_project(force)
    except Exception as e:  # optional evidence, like the cubin
        sys.stderr.write("reference host-loop harness not built: %s\n" % e)
        out["ref_project"] = None
    return out


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
