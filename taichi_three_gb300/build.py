"""Builds libtina3.so, the sm_103a CUDA library behind the Tina drop-in API.

Each csrc/*.cu translation unit is compiled by nvcc in parallel
(-gencode arch=compute_103a,code=sm_103a, -O3, -lineinfo, C++17, no fast-math),
then linked into taichi_three_gb300/_lib/libtina3.so with the CUDA runtime
linked statically, so the library only needs the driver at load time.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtina3.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    p = shutil.which("nvcc")
    if p:
        return p
    p = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(p):
        return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtina3.so")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + [
        os.path.join(ROOT, "include", "tina3.h"), os.path.abspath(__file__)]


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def _compile(src, extra, verbose):
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    cmd = [nvcc_path(), "-c", src, "-o", obj] + _flags() + list(extra)
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout.strip() or r.stderr.strip()):
        print(r.stdout + r.stderr, flush=True)
    return obj


def build(force=False, verbose=False, extra=()):
    """Compile libtina3.so if missing or older than its sources; returns its path."""
    if not force and not stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc_path(), "-shared", *ARCH, "-o", tmp, *objs, "-lcuda"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    extra = [a for a in sys.argv[1:] if a.startswith("-X")]
    print(build(force="--force" in sys.argv, verbose=True, extra=extra))
