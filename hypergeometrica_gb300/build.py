"""Build the CUDA library libhg_gb300.so in-tree (sm_103a only).

Each translation unit compiles in parallel with nvcc; the objects link into
hypergeometrica_gb300/libhg_gb300.so with the CUDA runtime linked statically,
so the library loads next to PyTorch without a separate libcudart search.
Usage:  python -m hypergeometrica_gb300.build [--checked]   (or import and call
build()).  --checked compiles the checked build, libhg_gb300_checked.so, with
-DHG_CHECKED=1.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhg_gb300.so")
CHECKED_LIB = os.path.join(HERE, "libhg_gb300_checked.so")

SOURCES = ["hg_ntt_strided.cu", "hg_ntt_contig.cu", "hg_crt.cu", "hg_api.cu", "hg_service.cu", "hg_sum.cu", "hg_series.cu", "hg_peak.cu", "hg_persist.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
         "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> str:
    """Compile the library; with checked=True the checked build
    (-DHG_CHECKED=1: range, bounds and product checks in every kernel) into
    libhg_gb300_checked.so, from objects of its own."""
    bdir = os.path.join(BUILD, "checked") if checked else BUILD
    lib = CHECKED_LIB if checked else LIB
    os.makedirs(bdir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    headers.append(os.path.join(ROOT, "include", "hypergeometrica_gb300.h"))
    cc = nvcc()
    flags = FLAGS + (["-DHG_CHECKED=1"] if checked else [])
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc, *ARCH, *flags, "-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(lib, objs):
        tmp = lib + ".tmp"
        run([cc, *ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv, checked="--checked" in sys.argv))
