"""Build and load the native libraries of the package.

* ``libqltg.so``       - the CUDA library behind include/qltg.h (sm_103a only);
* ``libqltg_synth.so`` - the deterministic workload generator (host code).

Both are built in-tree with nvcc / g++ (no cmake) so the same commands run in the
x86 development container and on the aarch64 GPU host. Loading ``libqltg.so`` fails
loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from typing import List

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB_QLTG = os.path.join(PKG, "libqltg.so")
LIB_SYNTH = os.path.join(PKG, "libqltg_synth.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden"]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources() -> List[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers() -> List[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.h"))) + [os.path.join(ROOT, "include", "qltg.h")]


def _stale(target: str, deps: List[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_qltg(force: bool = False, jobs: int = 8, verbose: bool = False) -> str:
    """Compile every csrc/*.cu for sm_103a in parallel and link libqltg.so."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    srcs = _sources()
    hdrs = _headers()
    objs = []
    cmds = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmds.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", os.path.join(ROOT, "include"), "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max(1, jobs)) as ex:
        list(ex.map(run, cmds))
    if force or cmds or _stale(LIB_QLTG, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB_QLTG, *objs, "-cudart", "shared", "-lcuda"])
    return LIB_QLTG


def build_synth(force: bool = False) -> str:
    src = os.path.join(CSRC, "synth_capi.cc")
    deps = [src, os.path.join(CSRC, "synth.h")]
    if force or _stale(LIB_SYNTH, deps):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-o", LIB_SYNTH])
    return LIB_SYNTH


_qltg = None
_synth = None


def load_qltg():
    """Load libqltg.so (build it first with build_qltg / __graft_entry__.build)."""
    global _qltg
    if _qltg is None:
        if not os.path.exists(LIB_QLTG):
            raise RuntimeError(f"{LIB_QLTG} is missing: run __graft_entry__.build() (no CPU fallback exists)")
        _qltg = C.CDLL(LIB_QLTG)
    return _qltg


def load_synth():
    global _synth
    if _synth is None:
        build_synth()
        _synth = C.CDLL(LIB_SYNTH)
    return _synth
