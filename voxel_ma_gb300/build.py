"""Build libvoxelcore_gb300.so (the C-ABI library) in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled in parallel into _build/ and
linked into voxel_ma_gb300/libvoxelcore_gb300.so.  A rebuild happens only
when a source or header is newer than the library (or the library was built
for another host architecture).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvoxelcore_gb300.so")
STAMP = os.path.join(BUILD, "host_arch.txt")
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-DNDEBUG"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))


def _up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(STAMP):
        return False
    if open(STAMP).read().strip() != platform.machine():
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    if not force and _up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []

    def compile_one(args):
        src, obj = args
        cmd = [nvcc(), *ARCH_FLAGS, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r.returncode, r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, zip(srcs, objs)))
    failed = [(s, out) for s, rc, out in results if rc != 0]
    for s, rc, out in results:
        if verbose or rc != 0 or ptxas_verbose:
            if out.strip():
                print(f"--- {os.path.basename(s)}\n{out}", file=sys.stderr)
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(os.path.basename(s) for s, _ in failed))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH_FLAGS, "-shared", "-cudart", "shared", "-o", tmp, *objs,
           "-Xlinker", "-rpath=/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(platform.machine())
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
