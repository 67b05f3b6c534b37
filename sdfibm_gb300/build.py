"""Build recipe of the in-tree shared library ``sdfibm_gb300/libsdfibm_cuda.so`` (sm_103a only).

``python -m sdfibm_gb300.build`` or ``sdfibm_gb300.build.build()``.  Translation units are compiled in parallel
with nvcc; ``-fmad=false`` keeps every FP64 operation unfused so the exact path reproduces host FP64 arithmetic
(FP32 hot loops use explicit fused multiply-add intrinsics), except in the translation units of CONTRACT_SOURCES,
which hold FP32 arithmetic only.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libsdfibm_cuda.so")
BUILD_DIR = os.path.join(HERE, "_build")
CU_SOURCES = ["classify.cu", "coupling.cu", "evolve.cu", "capi.cu", "noalloc.cu", "mlp.cu", "poly.cu", "stencil.cu"]
# pure FP32 kernels with no exact path: compiled with multiply-add contraction
CONTRACT_SOURCES = {"stencil.cu"}
CXX_SOURCES = ["host.cpp", "host_dict.cpp", "host_io.cpp", "host_poly.cpp"]
# the host half alone (no CUDA): what CPU-only builds of the host code (sanitizer runs, test doubles) compile
HOST_SOURCES = [os.path.join("sdfibm_gb300", "csrc", f) for f in CXX_SOURCES]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in CU_SOURCES + CXX_SOURCES + ["device_math.cuh", "kernels.cuh", "common.cuh",
                                                                   "host_text.hpp", "mlp.cuh", "poly.hpp",
                                                                   "poly_dev.cuh"]] + [
        os.path.join(HERE, "..", "include", h) for h in ("sdfibm_cuda.h", "sdfibm_host.h")]


def up_to_date():
    if not os.path.exists(OUT):
        return False
    t = os.path.getmtime(OUT)
    return all(os.path.getmtime(s) <= t for s in _sources() if os.path.exists(s))


def build(force=False, verbose=False):
    if not force and up_to_date():
        return OUT
    os.makedirs(BUILD_DIR, exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(HERE, "..", "include")]
    jobs = []
    for f in CU_SOURCES:
        obj = os.path.join(BUILD_DIR, f + ".o")
        fmad = [] if f in CONTRACT_SOURCES else ["-fmad=false"]
        cmd = [nv] + ARCH + common + ["-lineinfo"] + fmad + ["-Xptxas", "-warn-spills", "-c", os.path.join(CSRC, f),
                                                             "-o", obj]
        jobs.append((cmd, obj))
    for f in CXX_SOURCES:
        obj = os.path.join(BUILD_DIR, f + ".o")
        cmd = [nv] + common + ["-Xcompiler", "-ffp-contract=off", "-c", os.path.join(CSRC, f), "-o", obj]
        jobs.append((cmd, obj))

    def run(job):
        cmd, obj = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = OUT + ".tmp"
    link = [nv] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(link), r.stdout, r.stderr))
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
