"""Build the GB300 engine library (libimpec2d.so) and the Impec2D command-line driver.

Every CUDA translation unit is compiled for sm_103a only; units are compiled in parallel.
Outputs stay in-tree (git-ignored): ``impec2d_gb300/libimpec2d.so`` and
``impec2d_gb300/Impec2D``.
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
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libimpec2d.so")
CLI = os.path.join(HERE, "Impec2D")

CU_SOURCES = ["ctx.cu", "pressure.cu", "transport.cu", "dispersion.cu", "step.cu", "graph.cu", "project.cu", "learned.cu", "learned_net.cu"]
CPP_SOURCES = ["host/SimParams.cpp", "host/Impec2DSolver.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd, log):
    r = subprocess.run(cmd, capture_output=True, text=True)
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return log


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _arch_stamp_ok() -> bool:
    """Objects built on another host architecture (x86_64 vs aarch64) are discarded."""
    import platform
    stamp = os.path.join(OBJ, "ARCH")
    mach = platform.machine()
    ok = os.path.exists(stamp) and open(stamp).read().strip() == mach
    if not ok:
        shutil.rmtree(OBJ, ignore_errors=True)
        os.makedirs(OBJ, exist_ok=True)
        for f in (LIB, CLI):
            if os.path.exists(f):
                os.remove(f)
        with open(stamp, "w") as fh:
            fh.write(mach)
    return ok


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    _arch_stamp_ok()
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", "impec2d.h")]
    hostdir = os.path.join(CSRC, "host")
    if os.path.isdir(hostdir):
        headers += [os.path.join(hostdir, h) for h in os.listdir(hostdir) if h.endswith(".h")]
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(([nvcc] + NVFLAGS + ["-c", s, "-o", o], o + ".log"))
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(OBJ, os.path.basename(src).replace(".cpp", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append((["g++"] + CXXFLAGS + [f"-I{os.path.join(ROOT, 'include')}", f"-I{_cuda_home()}/include",
                                               "-c", s, "-o", o], o + ".log"))
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for log in ex.map(lambda a: _run(*a), jobs):
            if verbose:
                print(open(log).read())
    if _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"], os.path.join(OBJ, "link.log"))
    main = os.path.join(CSRC, "host", "main.cpp")
    if os.path.exists(main) and _stale(CLI, [main, LIB]):
        _run(["g++", "-O2", "-std=c++17", main, "-o", CLI, f"-I{os.path.join(ROOT, 'include')}",
              f"-I{os.path.join(CSRC, 'host')}", f"-L{HERE}", "-limpec2d", f"-Wl,-rpath,{HERE}",
              f"-L{_cuda_home()}/lib64", "-lcudart"], os.path.join(OBJ, "cli.log"))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
