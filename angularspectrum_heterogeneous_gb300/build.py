"""Build the CUDA library ``libasgb300.so`` in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel and the
objects are linked into one shared library next to this file.  The build is
incremental (a unit is rebuilt when it or any header is newer than its
object).  Run ``python -m angularspectrum_heterogeneous_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libasgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(extra_ptxas_v: bool = False):
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", CSRC, "-I", INCLUDE] + ARCH
    if extra_ptxas_v:
        f += ["-Xptxas", "-v"]
    return f


def _needs(obj: str, src: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(x) > t for x in [src, *headers])


def build(verbose: bool = False, ptxas_v: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    cc = nvcc()
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if ptxas_v or _needs(o, s, headers):
            todo.append((s, o))

    def run(so):
        s, o = so
        cmd = [cc, *_flags(ptxas_v), "-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return s, cmd, r

    failed = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo) or 1, os.cpu_count() or 4)) as ex:
        for s, cmd, r in ex.map(run, todo):
            if verbose or ptxas_v or r.returncode != 0:
                sys.stderr.write(f"[nvcc] {os.path.basename(s)} rc={r.returncode}\n")
                sys.stderr.write(r.stdout[-20000:] + r.stderr[-20000:])
            if r.returncode != 0:
                failed.append(s)
    if failed:
        raise RuntimeError(f"nvcc failed for {', '.join(map(os.path.basename, failed))}")
    if todo or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [cc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_v="--ptxas" in sys.argv))
