"""Build libqlpix.so in-tree (qlens_gb300/_lib/) with nvcc for sm_103a.

Every translation unit is compiled separately so that the ray-shooting and
mapping kernels that reproduce QLens's bits can be built with --fmad=false
(QLens's operation order, no contracted multiply-adds) while the dense algebra
and the surrogate ray shooting keep FMA.  Compiles run in
parallel and only when a source is newer than its object.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libqlpix.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + CSRC,
          "-I" + os.path.join(ROOT, "include")] + ARCH

# (source, extra flags)
UNITS = [
    ("raytrace.cu", ["--fmad=false"]),
    ("mapping.cu", ["--fmad=false"]),
    ("psf.cu", ["--fmad=false"]),
    ("linalg.cu", []),
    ("sparseops.cu", []),
    ("noalloc.cu", []),
    ("mixed.cu", []),
    ("surrogate.cu", []),
    ("sur_exact.cu", ["--fmad=false"]),
    ("outside.cu", ["--fmad=false"]),
    ("ctx.cpp", []),
    ("autotune.cpp", []),
    ("fits.cpp", []),
    ("sampler.cpp", []),
    ("fitparam.cpp", []),
    ("qlpix_api.cpp", []),
]
HEADERS = ["qlpix_internal.h", "qlpix_ctx.h", "lens_device.cuh", "nfw_device.cuh", "patterson_rule.h", "chol.cuh", "chol128.cuh", "tc_common.cuh", "tc_syrk.cuh", "brent.h"]


def _newer(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def _compile(src, flags):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    deps = [os.path.join(CSRC, h) for h in HEADERS if os.path.exists(os.path.join(CSRC, h))]
    deps.append(os.path.join(ROOT, "include", "qlpix.h"))
    if not _newer(src, obj, deps):
        return obj
    cmd = [NVCC] + COMMON + flags + ["-x", "cu" if src.endswith(".cu") else "c++"]
    if src.endswith(".cpp"):
        cmd = [NVCC] + COMMON + flags
    cmd += ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    units = [(os.path.join(CSRC, s), f) for s, f in UNITS]
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), units))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
