"""Build recipe of the native library multifebe_gb300/_lib/libmfbem.so.

Device code (one translation unit) is compiled by nvcc for sm_103a only; the
host-side tables and mesh preparation by the host C++ compiler with FP
contraction off, so their results match the CPU oracle bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libmfbem.so")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(nv))
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(SRC, f) for f in os.listdir(SRC)]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _sources() + [os.path.join(HERE, "..", "include", "mfbem.h"), __file__])


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT, exist_ok=True)
    inc = ["-I", SRC, "-I", os.path.join(HERE, "..", "include")]
    cxx = os.environ.get("CXX", "g++")
    jobs = {
        "host_tables.o": [cxx, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", *inc, "-I", os.path.join(cuda, "include"),
                          "-c", os.path.join(SRC, "host_tables.cpp"), "-o", os.path.join(OUT, "host_tables.o")],
        "host_prep.o": [cxx, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", *inc, "-I", os.path.join(cuda, "include"),
                        "-c", os.path.join(SRC, "host_prep.cpp"), "-o", os.path.join(OUT, "host_prep.o")],
        "host_msh.o": [cxx, "-std=c++17", "-O2", "-fPIC", *inc,
                       "-c", os.path.join(SRC, "host_msh.cpp"), "-o", os.path.join(OUT, "host_msh.o")],
        "host_nso.o": [cxx, "-std=c++17", "-O2", "-fPIC", *inc,
                       "-c", os.path.join(SRC, "host_nso.cpp"), "-o", os.path.join(OUT, "host_nso.o")],
        "mfbem_abi.o": [nvcc, ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *inc,
                        "-Xptxas", "-v" if verbose else "-O3",
                        "-c", os.path.join(SRC, "mfbem_abi.cu"), "-o", os.path.join(OUT, "mfbem_abi.o")],
        "mfbem_noalloc.o": [nvcc, ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *inc,
                            "-c", os.path.join(SRC, "mfbem_noalloc.cu"), "-o", os.path.join(OUT, "mfbem_noalloc.o")],
    }

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for cmd, r in ex.map(run, jobs.values()):
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("build failed: " + " ".join(cmd[:4]))
            if verbose and (r.stdout or r.stderr):
                sys.stderr.write(r.stderr)
    link = [nvcc, ARCH, "-shared", "-o", LIB + ".tmp"] + [os.path.join(OUT, o) for o in jobs] + ["-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link failed")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
