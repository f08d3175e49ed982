"""In-tree build of the CUDA library and the CPU oracle.

``build_library()`` compiles ``csrc/`` into ``finitevolume_gb300/_lib/
libfvgb300.so`` for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``);
``build_oracle()`` compiles ``oracle/fv_oracle.cpp`` (the CPU restatement used
by the tests and the CPU baseline) and, when the reference checkout is
present, the reference itself into ``oracle/_ref``.  Translation units are
compiled in parallel; a stamp of the source hashes skips unchanged builds.
Host code is built with ``-ffp-contract=off`` so results do not depend on
whether the host compiler would fuse multiply-adds (x86-64 vs aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIB_DIR, "libfvgb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "libfvoracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + os.path.join(ROOT, "include")]
# Per-file extra flags: the strict kernels are built without FMA contraction.
EXTRA = {"kernels_strict.cu": ["--fmad=false"], "diffusion.cu": ["--fmad=false"], "gradients.cu": ["--fmad=false"],
         "ns.cu": ["--fmad=false"], "rans.cu": ["--fmad=false"],
         "geometry.cu": ["--fmad=false"]}
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _hash(paths, extra="") -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        h.update(p.encode())
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    hdr = sorted(f for f in os.listdir(CSRC) if f.endswith((".h", ".cuh")))
    return cu, cpp, hdr


def reference_dir() -> str:
    """The reference checkout: $FV_REFERENCE, else the directory named
    ``reference`` beside this repository (used only to build the oracle's
    reference binaries and the fixtures; absent on machines without it)."""
    return os.environ.get("FV_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")


def build_library(force: bool = False, verbose: bool = False, jobs: int = 0) -> str:
    cu, cpp, hdr = _sources()
    allsrc = [os.path.join(CSRC, f) for f in cu + cpp + hdr] + [os.path.join(ROOT, "include", "fv_gb300.h")]
    stamp = _hash(allsrc, " ".join(NVCC_FLAGS + ARCH + CXX_FLAGS) + repr(EXTRA))
    stamp_file = os.path.join(LIB_DIR, "stamp.txt")
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file) and open(stamp_file).read() == stamp:
        return LIB
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = _nvcc()
    cmds = []
    objs = []
    for f in cu:
        o = os.path.join(obj_dir, f + ".o")
        objs.append(o)
        cmds.append([nvcc, *ARCH, *NVCC_FLAGS, *EXTRA.get(f, []), "-c", os.path.join(CSRC, f), "-o", o])
    for f in cpp:
        o = os.path.join(obj_dir, f + ".o")
        objs.append(o)
        cmds.append([os.environ.get("CXX", "g++"), *CXX_FLAGS, "-I" + os.path.dirname(nvcc) + "/../include",
                     "-c", os.path.join(CSRC, f), "-o", o])
    n = jobs or min(len(cmds), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=n) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for o in outs:
            if o.strip():
                print(o, file=sys.stderr)
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB


def build_oracle(force: bool = False, reference: str = None) -> str:
    """Compile the CPU restatement; also the reference when its sources exist."""
    src = os.path.join(ORACLE_DIR, "fv_oracle.cpp")
    hdrs = [os.path.join(ORACLE_DIR, f) for f in os.listdir(ORACLE_DIR) if f.endswith(".h")]
    stamp = _hash([src] + hdrs)
    stamp_file = os.path.join(ORACLE_BUILD, "stamp.txt")
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    if force or not (os.path.exists(ORACLE_LIB) and os.path.exists(stamp_file) and open(stamp_file).read() == stamp):
        tmp = ORACLE_LIB + ".tmp"
        _run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC",
              "-shared", "-o", tmp, src])
        os.replace(tmp, ORACLE_LIB)
        with open(stamp_file, "w") as f:
            f.write(stamp)
    ref = reference or reference_dir()
    if os.path.isdir(os.path.join(ref, "src")) and shutil.which("make"):
        _run(["make", "-s", "-C", ORACLE_DIR, "ref", "REF=" + ref])
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
