"""In-tree build of libpdgpu.so (the CUDA path and its C ABI) for sm_103a.

Each translation unit under csrc/ is compiled by nvcc in parallel and linked
into pd_gb300/_build/libpdgpu.so.  No CMake, no torch extension machinery: the
library is a plain C-ABI shared object that any host (C++, Python via ctypes,
PD's SWIG module) can load.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpdgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# FP32 denormals flush to zero: the special-function instructions (rsqrt, rcp,
# ex2) then run without their denormal fix-up sequences (the three GB passes of
# the 64-peptide batch: 1.96 -> 1.81 ms); no FP32 quantity of the path comes
# near 1e-38, and FP64 arithmetic is unaffected.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-ftz=true"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
           "-c", src, "-o", obj, *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(ROOT, "include", "pdgpu.h"))
    deps.append(os.path.abspath(__file__))
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False, extra=()):
    """Compile every CUDA source for sm_103a and link libpdgpu.so; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), sources()))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=("-Xptxas", "-v") if "--ptxas" in sys.argv else ()))
