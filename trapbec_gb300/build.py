"""Build libtrapbec.so in-tree with nvcc for sm_103a (no cmake, no torch).

Translation units are compiled in parallel; the result is
trapbec_gb300/lib/libtrapbec.so.  Device code is built for sm_103a only.
Host code is compiled with -ffp-contract=off so host-side coordinate and
coefficient arithmetic rounds the same way on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["trapbec.cu", "tiled_dispatch.cu", "tiled_f32_s0.cu", "tiled_f32_s1.cu", "tiled_f32_s2.cu",
                "tiled_f32_s3.cu", "tiled_f32_s4.cu", "tiled_f64_s0.cu", "tiled_f64_s1.cu", "batch.cu", "noalloc.cu", "peaks.cu",
                "sg_conv.cu", "sg_conv_tc.cu", "sg_conv_tcs.cu", "sg_wgrad_tc.cu", "sg_ops.cu"]
CXX_SOURCES = ["params_io.cpp"]
HEADERS_GLOB = (".cuh", ".h")


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newest_dep() -> float:
    t = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    t = max(t, os.path.getmtime(__file__))
    return t


def _compile(src: str, verbose_ptxas: bool) -> tuple[str, str]:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ_DIR, src + ".o")
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "--expt-relaxed-constexpr", "-c", path, "-o", obj]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I/usr/local/cuda/include",
               "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build_library(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    out = os.path.join(LIB_DIR, "libtrapbec.so")
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = [s for s in CUDA_SOURCES + CXX_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    drv = os.path.join(LIB_DIR, "trapbec_run")
    if not force and os.path.exists(out) and os.path.exists(drv) and os.path.getmtime(out) >= _newest_dep():
        return out
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, s, verbose_ptxas) for s in srcs]
        objs = []
        for f in futs:
            o, log = f.result()
            objs.append(o)
            logs.append(log)
    tmp = out + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lpthread", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    # the run.f90-style driver program, linked against the library
    drv = os.path.join(LIB_DIR, "trapbec_run")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(CSRC, "trapbec_run.cpp"), "-o", drv,
           "-L", LIB_DIR, "-ltrapbec", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write("\n".join(logs))
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_library(force=force, verbose_ptxas="-v" in sys.argv))
