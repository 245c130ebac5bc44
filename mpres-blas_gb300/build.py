"""Builds libmpres_gb300.so in-tree (mpres-blas_gb300/_build/) for sm_103a.

Every translation unit compiles in parallel; the kernels with
    nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3 -fmad=false
and the host helpers with g++ -ffp-contract=off (the host conversion must not
fuse multiply-adds).  Objects are rebuilt only when a source or header is newer.
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libmpres_gb300.so"
INCLUDE = HERE.parent / "include"

CU_SOURCES = ["dot.cu", "gemv.cu", "gemm.cu", "spmv.cu", "capi.cu", "probe.cu", "elementwise.cu", "convert.cu",
              "batch.cu", "solver.cu", "probe_fx.cu"]
CPP_SOURCES = ["host_tables.cpp", "host_convert.cpp", "host_mpfr.cpp", "server.cpp", "mtx.cpp"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and pathlib.Path(c, "bin", "nvcc").exists():
            return pathlib.Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return pathlib.Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found")


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _stale(obj, src):
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src] + _headers())


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(map(str, cmd)), r.stdout))
    return r.stdout


def build(verbose=False, ptxas_info=False):
    """Compiles the library if needed and returns the path of the .so."""
    home = cuda_home()
    nvcc = str(home / "bin" / "nvcc")
    OUT.mkdir(exist_ok=True)
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src, obj = CSRC / s, OUT / (s + ".o")
        objs.append(obj)
        if _stale(obj, src) or ptxas_info:
            cmd = [nvcc, ARCH, "-lineinfo", "-O3", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for s in CPP_SOURCES:
        src, obj = CSRC / s, OUT / (s + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math",
                         "-I", str(CSRC), "-I", str(home / "include"), "-c", str(src), "-o", str(obj)])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            logs = list(ex.map(_run, jobs))
    if jobs or not LIB.exists():
        _run([nvcc, ARCH, "-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lpthread"])
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    return LIB


if __name__ == "__main__":
    info = "--ptxas" in sys.argv
    p = build(verbose=True, ptxas_info=info)
    print(p)
