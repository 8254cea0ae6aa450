"""Loader of the measurement probes (tests/native/probes.cu) -- test and bench infrastructure.

The probes are not part of the product library: ``pqt_fp32_fma_probe`` gives the
FP32 peak that the bench's roofline divides by, ``pqt_guard_band_probe`` the bound
the packed sweep's exact decision relies on, ``pqt_settle_threshold`` the per-step
threshold of its quiet-site rule.  ``build()`` compiles them for sm_103a
(called by ``__graft_entry__.build()``); ``lib()`` loads them.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(HERE, "probes.cu")
OUT = os.path.join(HERE, "_build", "libpiqmc_probes.so")
CSRC = os.path.join(ROOT, "pathintegral-qmc_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")


def build(force=False):
    deps = [SRC, os.path.join(CSRC, "common.cuh"), os.path.join(CSRC, "sweep_core.cuh"),
            os.path.join(INCLUDE, "piqmc_gb300.h")]
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp%d" % os.getpid()
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo",
                           "--fmad=false", "-Xcompiler", "-fPIC", "-shared", "-I", INCLUDE, "-I", CSRC, SRC, "-o", tmp])
    os.replace(tmp, OUT)
    return OUT


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(OUT):
            build()
        L = ctypes.CDLL(OUT)
        V, I32, I64, U32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint32
        L.pqt_fp32_fma_probe.argtypes = [V, I32, I32, I32, V]
        L.pqt_fp32_fma_probe.restype = I32
        L.pqt_guard_band_probe.argtypes = [U32, I64, V, V]
        L.pqt_guard_band_probe.restype = I32
        L.pqt_settle_threshold.argtypes = [V, I32, V, V]
        L.pqt_settle_threshold.restype = I32
        _lib = L
    return _lib
