"""Compile the engine (csrc/*.cu) into simplehydrology_gb300/libshy.so.

Every translation unit is compiled by nvcc for sm_103a only, in parallel, and
linked into one shared library with the CUDA runtime linked statically.  The
library is built in place (never installed) so that the tests and the bench
load exactly this file.

Numerics flags that the parity guarantees depend on:
  --fmad=false            no multiply-add contraction on the device
  -Xcompiler -ffp-contract=off   nor on the host
  (IEEE-rounded division and square root are nvcc's defaults; fast-math is
   never enabled)
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libshy.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I" + INCLUDE, "-I" + CSRC,
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, "shy.h"), os.path.join(INCLUDE, "shy_surrogate.h")]
    return sorted(hs)


def _digest(paths, extra=""):
    h = hashlib.sha256(extra.encode())
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def build(verbose: bool = False, force: bool = False) -> str:
    """Build libshy.so if any source changed; return its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    stamp = os.path.join(BUILD, "stamp")
    key = _digest(srcs + headers(), " ".join(NVCC_FLAGS) + os.uname().machine)
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == key:
                return LIB
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [exe, *NVCC_FLAGS, "-Xptxas", "-v" if verbose else "-O3", "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([exe, ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(key)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
