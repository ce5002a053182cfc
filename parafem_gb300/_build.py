"""Build recipe for libpfgpu.so and the p121 executable (sm_103a only).

Compiles the CUDA and C++ translation units of ``parafem_gb300/csrc`` in
parallel with nvcc and links them in-tree under ``parafem_gb300/_build``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libpfgpu.so")
EXE = os.path.join(OUT, "p121")
EXE123 = os.path.join(OUT, "p123")
EXE122 = os.path.join(OUT, "p122")
PROGRAMS = [("p121_main.cpp", EXE), ("p123_main.cpp", EXE123), ("p122_main.cpp", EXE122)]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["pf_kernels.cu", "pf_elem_sym.cu", "pf_elem_h16.cu", "pf_shared.cu", "pf_scalar8.cu",
                "pf_solid8.cu", "pf_plastic.cu", "pf_batch.cu", "pf_multi.cu", "pf_abi.cu", "pf_noalloc.cu"]
CXX_SOURCES = ["pf_host.cpp"]
HEADERS = ["pf_internal.h", "pf_device.cuh", "pf_tc.cuh"]

_lock = threading.Lock()


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpfgpu.so")


def _sources():
    return ([os.path.join(SRC, s) for s in CUDA_SOURCES + CXX_SOURCES + HEADERS + [m for m, _ in PROGRAMS]]
            + [os.path.join(INCLUDE, "pfgpu.h"), os.path.abspath(__file__)])


def _stale(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile everything if any source is newer than the library; return its path."""
    with _lock:
        if not force and not _stale(LIB) and not any(_stale(x) for _, x in PROGRAMS):
            return LIB
        os.makedirs(OUT, exist_ok=True)
        cc = nvcc()
        common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", SRC]
        jobs = []
        objs = []
        for s in CUDA_SOURCES + CXX_SOURCES:
            obj = os.path.join(OUT, os.path.splitext(s)[0] + ".o")
            objs.append(obj)
            cmd = [cc] + ARCH + common + ["-c", os.path.join(SRC, s), "-o", obj]
            if s.endswith(".cpp"):
                cmd = [cc] + common + ["-x", "c++", "-c", os.path.join(SRC, s), "-o", obj]
            jobs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        failed = []
        for cmd, pr in jobs:
            out, _ = pr.communicate()
            if pr.returncode != 0:
                failed.append((cmd, out.decode(errors="replace")))
            elif verbose and out:
                print(out.decode(errors="replace"))
        if failed:
            msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
            raise RuntimeError("libpfgpu build failed:\n" + msg)
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call([cc] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
        cxx = shutil.which("g++") or shutil.which("c++") or "g++"
        for main, exe in PROGRAMS:
            tmpx = exe + f".tmp{os.getpid()}"
            subprocess.check_call([cxx, "-O2", "-std=c++17", "-I", INCLUDE, os.path.join(SRC, main),
                                   "-L", OUT, "-lpfgpu", "-Wl,-rpath,$ORIGIN", "-o", tmpx])
            os.replace(tmpx, exe)
        return LIB
