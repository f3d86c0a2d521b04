"""The per-topology kernels compile: NVRTC, with the engine's own options and its
embedded headers, on the generated source of a small transient.  NVRTC compiles for sm_103a without a
GPU, so a header change that breaks the run-time compilation fails here, on the
CPU, before any GPU run."""
import os

import pytest

from kronspice_gb300 import analysis, build, workloads

nvrtc = pytest.importorskip("cuda.bindings.nvrtc")

CSRC = os.path.join(os.path.dirname(build.__file__), "csrc")


def compile_nvrtc(src):
    names, texts = [], []
    for name, rel in build.JIT_HEADERS:
        with open(os.path.join(CSRC, rel), "rb") as f:
            texts.append(f.read())
        names.append(name.encode())
    err, prog = nvrtc.nvrtcCreateProgram(src.encode(), b"ks_spec.cu", len(names), texts, names)
    assert err == nvrtc.nvrtcResult.NVRTC_SUCCESS
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", b"--generate-line-info", b"-DKS_JIT=1"]
    (rc,) = nvrtc.nvrtcCompileProgram(prog, len(opts), opts)
    err, n = nvrtc.nvrtcGetProgramLogSize(prog)
    log = b" " * n
    nvrtc.nvrtcGetProgramLog(prog, log)
    nvrtc.nvrtcDestroyProgram(prog)
    return rc, log.decode(errors="replace")


def test_generated_transient_kernel_compiles():
    """The transient kernel of the RC ladder (the smallest compile that takes in
    every header: transient, Newton, devices, solve, FP32 start stage)."""
    el, nn, vals = workloads.rc_ladder_batch(4, sections=4)
    src = analysis.Plan(el, nn, vals.shape[1]).kernel_source("tran")
    rc, log = compile_nvrtc(src)
    assert rc == nvrtc.nvrtcResult.NVRTC_SUCCESS, log[-2000:]
