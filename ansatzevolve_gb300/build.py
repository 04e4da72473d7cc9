"""Builds the in-tree extension libansatzevolve_gb300.so (CUDA engine + C++ host +
the reference-compatible C ABI) for sm_103a.  Plain nvcc / g++, translation units
compiled in parallel; no CMake.  Usage: python -m ansatzevolve_gb300.build"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libansatzevolve_gb300.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["engine.cu", "mlp.cu", "dense.cu"]
CPP = ["setup.cpp", "otf_tables.cpp", "manager.cpp", "newton.cpp", "interface.cpp", "optimise.cpp", "runfiles.cpp", "properties.cpp", "diis.cpp"]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def sources():
    return [os.path.join(CSRC, f) for f in CU + CPP] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".h")] + \
        [os.path.join(HERE, "..", "include", h) for h in ("aegpu.h", "AnsatzSynthInterface.h", "aegpu_runfiles.h")]


def up_to_date():
    if not os.path.exists(OUT):
        return False
    t = os.path.getmtime(OUT)
    return all(os.path.getmtime(s) <= t for s in sources())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    jobs = []
    for f in CU:
        o = os.path.join(BUILD, f + ".o")
        jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
                     os.path.join(CSRC, f), "-o", o])
    for f in CPP:
        o = os.path.join(BUILD, f + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-parameter", "-I" + cuda_inc, "-c",
                     os.path.join(CSRC, f), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    objs = [os.path.join(BUILD, f + ".o") for f in CU + CPP]
    tmp = OUT + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
