"""Build the engine's shared library (kronspice_gb300/_lib/libkronspice_gpu.so).

Every translation unit is compiled by nvcc for sm_103a only, in parallel, then
linked with the host planner into one shared library.  No cmake, no torch build
machinery: the library has a plain C ABI (include/kronspice_gpu.h).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libkronspice_gpu.so")
OBJ_DIR = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-diag-suppress", "550"]

UNITS = ["ks_host.cpp", "ks_api.cu", "ks_kernels.cu", "ks_tran.cu", "ks_mlp.cu"]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "kronspice_gpu.h"))
    return files


def _compile(unit):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OBJ_DIR, unit + ".o")
    cmd = [NVCC] + CU_FLAGS + ["-c", src, "-o", obj]
    if unit.endswith(".cpp"):
        cmd = [NVCC, "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    newest = max(os.path.getmtime(f) for f in _deps())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
