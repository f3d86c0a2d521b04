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

UNITS = ["ks_host.cpp", "ks_api.cu", "ks_kernels.cu", "ks_tran.cu", "ks_mlp.cu", "ks_jit.cpp", "ks_noalloc.cu", "ks_ac.cu", "ks_torn.cu", "ks_sparse.cpp",
         "ks_multi.cu", "ks_peak.cu"]
# device headers embedded in the library for the per-topology kernels (NVRTC),
# under the names their #include lines use
JIT_HEADERS = [("ks_tran.cuh", "ks_tran.cuh"), ("ks_newton.cuh", "ks_newton.cuh"), ("ks_start32.cuh", "ks_start32.cuh"),
               ("ks_solve.cuh", "ks_solve.cuh"),
               ("ks_devices.cuh", "ks_devices.cuh"), ("ks_mos.cuh", "ks_mos.cuh"), ("ks_engine.h", "ks_engine.h"),
               ("../../include/kronspice_gpu.h", os.path.join("..", "..", "include", "kronspice_gpu.h"))]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "kronspice_gpu.h"))
    return files


def _write_jit_headers():
    """C++ source holding the device headers as string literals."""
    out = os.path.join(OBJ_DIR, "ks_jit_headers.cpp")
    parts = ["// generated by kronspice_gb300/build.py from csrc/*.cuh: headers of the per-topology kernels\n"]
    names, srcs = [], []
    for name, rel in JIT_HEADERS:
        with open(os.path.join(CSRC, rel)) as f:
            text = f.read()
        assert ')KSJIT"' not in text
        # split into pieces below the compilers' string-literal limits
        chunks = [text[i:i + 8000] for i in range(0, len(text), 8000)] or [""]
        srcs.append("\n".join('R"KSJIT(%s)KSJIT"' % c for c in chunks))
        names.append('"%s"' % name)
    parts.append("extern const int ks_jit_n_headers = %d;\n" % len(names))
    parts.append("extern const char* const ks_jit_header_names[] = {%s};\n" % ", ".join(names))
    parts.append("extern const char* const ks_jit_header_srcs[] = {\n%s};\n" % ",\n".join(srcs))
    text = "".join(parts)
    if not os.path.exists(out) or open(out).read() != text:
        with open(out, "w") as f:
            f.write(text)
    return out


def _compile(unit):
    src = os.path.join(CSRC, unit)
    if os.path.isabs(unit):
        src = unit
        unit = os.path.basename(unit)
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
    units = UNITS + [_write_jit_headers()]
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(_compile, units))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + [
        "-lcudart", "-lnvrtc"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
