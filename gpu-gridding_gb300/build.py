"""Builds libgpugrid.so in-tree with nvcc for sm_103a (GB300).

Each CUDA translation unit is compiled in parallel into ``_build/`` and
linked into ``_build/libgpugrid.so`` with the CUDA runtime linked
statically, so the library needs only the driver at run time.  Symbols are
hidden by default; only the ``GG_API`` entry points of include/gpugrid.h are
exported.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgpugrid.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["gg_api.cu", "gg_sort.cu", "gg_stack.cu", "gg_place.cu",
           "gg_grid.cu", "gg_degrid.cu", "gg_calib.cu", "gg_noalloc.cu",
           "gg_batch.cu", "gg_weights.cu", "gg_kgen.cu", "gg_loaders.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(verbose_ptxas: bool) -> list[str]:
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17",
                "-Xcompiler", "-fPIC,-fvisibility=hidden,-O3",
                "-I" + os.path.join(HERE, "..", "include")]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _up_to_date(obj: str, deps: list[str]) -> bool:
    if not os.path.isfile(obj):
        return False
    t = os.path.getmtime(obj)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False,
          jobs: int | None = None) -> str:
    """Compile and link; returns the path of libgpugrid.so."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC)
               if h.endswith((".cuh", ".h"))]
    headers += [os.path.join(HERE, "..", "include", h)
                for h in ("gpugrid.h", "gpugrid_io.h")]
    objs = []
    cmds = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _up_to_date(o, [s] + headers):
            cmds.append([cc, "-c", s, "-o", o] + _flags(verbose_ptxas))
    logs = []

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with concurrent.futures.ThreadPoolExecutor(
            max_workers=jobs or min(len(SOURCES), os.cpu_count() or 4)) as ex:
        for cmd, r in ex.map(run, cmds):
            logs.append(r.stdout + r.stderr)
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if cmds or not os.path.isfile(LIB):
        link = [cc, "-shared", "-o", LIB] + objs + ARCH + [
            "-Xcompiler", "-fPIC", "-cudart", "static"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    if verbose_ptxas:
        with open(os.path.join(BUILD, "ptxas.log"), "w") as f:
            f.write("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv,
                verbose_ptxas="-v" in sys.argv))
