"""Builds libnlfem_gpu.so in-tree with nvcc for sm_103a (five translation units in parallel)."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libnlfem_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cpp", ".cuh", ".inl"))] + [
        os.path.join(ROOT, "include", "nlfem_gpu.h"), os.path.join(ROOT, "include", "Cassemble_compat.h")]


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force=False, verbose=False):
    if not force and not needs_build():
        return LIB
    objdir = os.path.join(HERE, "_build")
    os.makedirs(objdir, exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-lineinfo", "-I" + os.path.join(ROOT, "include")]
    jobs = [
        [NVCC] + ARCH + common + ["-Xptxas", "-warn-spills", "-c", os.path.join(CSRC, "assemble.cu"),
                                  "-o", os.path.join(objdir, "assemble.o")],
        [NVCC] + common + ["-x", "cu", "-c", os.path.join(CSRC, "compat.cpp"),
                           "-o", os.path.join(objdir, "compat.o")] + ARCH,
        [NVCC] + ARCH + common + ["-c", os.path.join(CSRC, "noalloc.cu"),
                                  "-o", os.path.join(objdir, "noalloc.o")],
        [NVCC] + ARCH + common + ["-c", os.path.join(CSRC, "peaks.cu"),
                                  "-o", os.path.join(objdir, "peaks.o")],
        [NVCC] + ARCH + common + ["-c", os.path.join(CSRC, "mass.cu"),
                                  "-o", os.path.join(objdir, "mass.o")],
    ]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + p.stdout + p.stderr)
        return p.stdout + p.stderr

    with ThreadPoolExecutor(len(jobs)) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    tmp = LIB + ".tmp"
    run([NVCC] + ARCH + ["-shared", "-o", tmp, os.path.join(objdir, "assemble.o"),
                         os.path.join(objdir, "compat.o"), os.path.join(objdir, "noalloc.o"), os.path.join(objdir, "peaks.o"),
                         os.path.join(objdir, "mass.o"), "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
