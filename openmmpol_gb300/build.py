"""Build libommp_gb300.so in-tree for GB300 (sm_103a).

CUDA sources go through nvcc with ``-gencode arch=compute_103a,code=sm_103a``,
C++ host sources through g++; the translation units compile in parallel and
link with a static CUDA runtime.  No cmake, no PyTorch extension machinery.

    python -m openmmpol_gb300.build          # or openmmpol_gb300.build.build()
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libommp_gb300.so")

CU_SOURCES = ["kernels.cu", "engine.cu", "solvers.cu", "noalloc.cu", "tmu32.cu", "ds_kernels.cu", "external.cu", "grad.cu",
              "grad_ds.cu", "qm_helper.cu", "fmm.cu",
              "fixedelec.cu", "block_cg.cu", "multisolve.cu"]
# per-file nvcc flags: the FP32 operators flush subnormals (plain MUFU rsqrt);
# the double-single kernel fuses nothing implicitly (its FMAs are explicit)
CU_EXTRA = {"tmu32.cu": ["-ftz=true"], "ds_kernels.cu": ["-ftz=true", "--fmad=false"],
            "grad_ds.cu": ["-ftz=true", "--fmad=false"]}
CXX_SOURCES = ["setup.cpp", "capi.cpp", "log.cpp", "server.cpp", "precond.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libommp_gb300.so")


def _cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))), "include")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "openmmpol_gb300.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-c", s, "-o", o]
            cmd[1:1] = CU_EXTRA.get(src, [])
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off",
                         "-I", _cuda_include(), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
