"""Builds libpars_gpu.so (the sm_103a kernels + C ABI) in the package directory.

Each translation unit is compiled by nvcc in parallel for the single target
architecture sm_103a, then linked into one shared library.  Build products stay
in-tree (pars_gb300/_build/ and pars_gb300/libpars_gpu.so).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBRARY = os.path.join(HERE, "libpars_gpu.so")

SOURCES = ["pars_gpu.cu", "trace_kernels.cu", "curve_kernels.cu", "ftle_kernels.cu", "field_kernels.cu", "batch_kernels.cu",
           "service.cu", "render_kernels.cu", "field_io.cu", "vtk_export.cu", "calibrate.cu",
           "transport.cu"]
# Per-source flags: the ray tracer rounds every operation separately (no FMA
# contraction), as its CPU restatement does.
SOURCE_FLAGS = {"render_kernels.cu": ["--fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp"))]
    headers.append(os.path.join(ROOT, "include", "pars_gpu.h"))
    objects, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objects.append(o)
        if _stale(o, [s] + headers):
            jobs.append([nvcc(), *ARCH, *FLAGS, *SOURCE_FLAGS.get(src, []), *extra_flags, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("nvcc failed for " + cmd[-3])

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        list(pool.map(run, jobs))
    if jobs or _stale(LIBRARY, objects):
        run([nvcc(), *ARCH, "-shared", "-o", LIBRARY, *objects])
    return LIBRARY


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
