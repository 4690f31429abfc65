"""Build recipe for libqmc_gb300.so (sm_103a).

Each CUDA translation unit is compiled by its own nvcc process, in parallel,
then linked with the host runtime into one shared library next to this file.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libqmc_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--use_fast_math", "-Xcompiler", "-fPIC",
              "-I" + os.path.join(ROOT, "include")]
CU_SOURCES = ["qmc_kernels.cu", "qmc_shape_h2.cu", "qmc_shape_li.cu", "qmc_shape_ch4_measure.cu",
              "qmc_shape_ch4_sweep.cu", "qmc_shape_ch4_allstep.cu", "qmc_shape_ch4min_measure.cu",
              "qmc_shape_ch4min_sweep.cu", "qmc_shape_c6h6.cu", "qmc_shape_heg.cu",
              "qmc_shape_ch4_batch.cu", "qmc_shape_ch4min_batch.cu", "qmc_shape_c6h6_batch.cu",
              "qmc_shape_heg_batch.cu", "qmc_noalloc.cu"]
CPP_SOURCES = ["qmc_api.cpp", "qmc_roofline.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "qmc.h"))
    jobs, objs = [], []
    for src in CU_SOURCES + CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            if src.endswith(".cu"):
                cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o]
            else:
                cmd = [nvcc, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
                       "-c", s, "-o", o]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            for err in ex.map(_run, jobs):
                if verbose and err:
                    sys.stderr.write(err)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
