"""Build libraftgb.so in-tree for GB300 (sm_103a).

Each translation unit under csrc/ is compiled by nvcc in parallel and the
objects are linked into pyraft_gb300/lib/libraftgb.so (git-ignored).  Takes a
few seconds; needs no GPU (nvcc cross-compiles).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libraftgb.so")
UNITS = ("api", "slantstack", "aux", "filter", "bresenham", "em", "batch", "noalloc", "f64", "mesh",
         "radon_tma", "gather_rot")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: libraftgb.so needs the CUDA toolkit to build")
    return exe


def _sources():
    return [os.path.join(CSRC, u + ".cu") for u in UNITS
            if os.path.exists(os.path.join(CSRC, u + ".cu"))]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = _sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "raftgb.h"))
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the path of libraftgb.so."""
    if not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    cc = nvcc()
    with tempfile.TemporaryDirectory() as tmp:
        def one(src):
            obj = os.path.join(tmp, os.path.basename(src)[:-3] + ".o")
            # RG_NVCC_EXTRA: extra compile flags (development experiments)
            extra = os.environ.get("RG_NVCC_EXTRA", "").split()
            cmd = [cc, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
            if verbose and r.stderr:
                print(r.stderr)
            return obj
        with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
            objs = list(ex.map(one, _sources()))
        tmp_lib = LIB + ".tmp"
        cmd = [cc, "-shared", *ARCH, "-o", tmp_lib, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp_lib, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
