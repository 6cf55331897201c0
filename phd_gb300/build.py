"""Build the in-tree shared libraries.

* phd_gb300/_lib/libizem_gpu.so  -- the CUDA library (nvcc, sm_103a only)
* oracle/_build/libizem_oracle.so -- the CPU oracle (g++), test infrastructure

Both are rebuilt only when a source is newer than the library.
"""
import glob
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "phd_gb300", "csrc")
LIBDIR = os.path.join(ROOT, "phd_gb300", "_lib")
GPU_LIB = os.path.join(LIBDIR, "libizem_gpu.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libizem_oracle.so")

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-shared"]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.exists(cand) or cand == "nvcc"):
            return cand
    return "nvcc"


def build_gpu(force=False, verbose=False):
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(CSRC, "*.h")) + [os.path.join(ROOT, "include", "izem_gpu.h")])
    if not force and not _stale(GPU_LIB, srcs):
        return GPU_LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tus = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs = []
    procs = []
    for tu in tus:
        obj = os.path.join(LIBDIR, os.path.basename(tu) + ".o")
        cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
               "-Xcompiler", "-fPIC", "-rdc=false", "-c", tu, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
        objs.append(obj)
    for p, tu in zip(procs, tus):
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode())
            raise RuntimeError("nvcc failed on %s" % tu)
    cmd = [_nvcc(), "-shared", "-o", GPU_LIB] + objs + ["-lcudart"]
    subprocess.check_call(cmd)
    for o in objs:
        os.remove(o)
    return GPU_LIB


def build_oracle(force=False):
    srcs = sorted(glob.glob(os.path.join(ORACLE_DIR, "*.cpp")) + glob.glob(os.path.join(ORACLE_DIR, "*.inc")) +
                  [os.path.join(ROOT, "include", "izem_gpu.h")])
    if not force and not _stale(ORACLE_LIB, srcs):
        return ORACLE_LIB
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", ORACLE_LIB] + sorted(glob.glob(os.path.join(ORACLE_DIR, "*.cpp")))
    subprocess.check_call(cmd)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_gpu(force="-f" in sys.argv, verbose=True))
