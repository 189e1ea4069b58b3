"""Build libjuesgpu.so for sm_103a from csrc/ (in-tree; no cmake, no setuptools).

Each translation unit is compiled by nvcc in parallel, then linked into
``jues.jl_gb300/lib/libjuesgpu.so``.  Usage: ``python jues.jl_gb300/build.py [-j N]``.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def sources():
    return sorted(f for f in os.listdir(SRC) if f.endswith(".cu"))


def compile_one(src, extra):
    out = os.path.join(OBJ, src[:-3] + ".o")
    inp = os.path.join(SRC, src)
    deps = [inp] + [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith(".cuh")]
    deps.append(os.path.join(HERE, "..", "include", "jues_gpu.h"))
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out, ""
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", inp, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return out, r.stderr


def build(jobs=None, verbose=False, extra=None):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    extra = list(extra or [])
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: compile_one(s, extra), srcs))
    if verbose:
        for _, err in results:
            if err:
                print(err, file=sys.stderr)
    so = os.path.join(LIB, "libjuesgpu.so")
    cmd = [nvcc()] + ARCH + ["-shared", "-o", so] + [o for o, _ in results] + ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    return so


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("-j", type=int, default=None)
    ap.add_argument("-v", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print register/smem usage")
    a = ap.parse_args()
    extra = ["-Xptxas", "-v"] if a.ptxas_info else []
    if a.ptxas_info:
        shutil.rmtree(OBJ, ignore_errors=True)
    print(build(a.j, a.v or a.ptxas_info, extra))
