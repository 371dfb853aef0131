"""Build recipe for libmcrt.so (CUDA for sm_103a) — no cmake, plain nvcc.

The translation units are compiled in parallel into objects and linked into
``mcrt_gb300/_lib/libmcrt.so`` inside the package, where the Python host code loads
it. Run ``python build.py`` from anywhere; ``__graft_entry__.build()`` calls
:func:`build` as well.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import platform
import shutil
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "mcrt_gb300", "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmcrt.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
    "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr",
]
# Each unit instantiates a subset of the kernels so that they compile in parallel.
UNITS = ["mcrt_api.cu", "mcrt_k_fp32.cu", "mcrt_k_fp64.cu", "mcrt_k_plain.cu", "mcrt_mie.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libmcrt")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _fingerprint(nvcc: str, unit: str, extra: list[str]) -> str:
    """Hash of everything an object depends on: the unit, every header beside it and in
    include/, the host architecture, the compiler's path and the flags. An object whose
    recorded fingerprint matches is reused."""
    h = hashlib.sha256()
    h.update(" ".join([platform.machine(), nvcc, *NVCC_FLAGS, *extra]).encode())
    for path in [os.path.join(CSRC, unit)] + sorted(glob.glob(os.path.join(CSRC, "*.cuh")) +
                                                    glob.glob(os.path.join(CSRC, "*.h")) +
                                                    glob.glob(os.path.join(INCLUDE, "*.h"))):
        h.update(path.encode())
        with open(path, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compiles every unit for sm_103a (reusing objects whose sources, headers and flags
    are unchanged) and links libmcrt.so; returns its path."""
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    t0 = time.time()

    def compile_one(u: str) -> str:
        obj = os.path.join(OBJ_DIR, u.replace(".cu", ".o"))
        stamp = obj + ".sha256"
        fp = _fingerprint(nvcc, u, extra)
        if not ptxas_info and os.path.exists(obj) and os.path.exists(stamp):
            with open(stamp) as f:
                if f.read().strip() == fp:
                    return obj
        cmd = [nvcc, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, u), "-o", obj]
        if ptxas_info:
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(r.stdout + r.stderr)
            sys.stderr.write(r.stderr)
        else:
            _run(cmd)
        with open(stamp, "w") as f:
            f.write(fp)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread", "-ldl"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB} in {time.time() - t0:.1f}s")
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
