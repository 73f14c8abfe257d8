"""ctypes binding and build recipe of the FP32 CPU restatement (cpu_fp32.cpp).

TEST INFRASTRUCTURE AND CPU BASELINE ONLY: imported by the tests and by the
benchmark's CPU arm, never by the product. ``build()`` compiles
``oracle/_build/libcpuf32.so`` with g++ and OpenMP (portable flags: no
``-march=native``, so the same source builds on x86-64 and aarch64).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_fp32.cpp")
LIB = os.path.join(HERE, "_build", "libcpuf32.so")
CXXFLAGS = ["-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=fast"]

_lib = None


def build(force=False):
    """Compiles the library if it is missing or older than its source; returns its path."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        r = subprocess.run(["g++"] + CXXFLAGS + ["-o", LIB, SRC], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("g++ failed for cpu_fp32.cpp:\n" + r.stdout + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        P = C.c_void_p
        lib.cpuf32_create.restype = P
        lib.cpuf32_create.argtypes = [C.c_int, P, P, C.c_int, C.c_int, P, C.c_int, C.c_int]
        lib.cpuf32_destroy.restype = None
        lib.cpuf32_destroy.argtypes = [P]
        lib.cpuf32_nparams.restype = C.c_size_t
        lib.cpuf32_nparams.argtypes = [P]
        lib.cpuf32_grad.restype = C.c_int
        lib.cpuf32_grad.argtypes = [P, P, C.c_double, C.c_double, P, C.c_int, C.c_double, C.c_double,
                                    C.c_longlong, P, C.c_int, C.POINTER(C.c_double), P, P, P, P]
        _lib = lib
    return _lib


class CpuNeuralODE:
    """One network (flat Lux parameters p) and batch size B on the host cores.

    ``grad(u0, tspan, saveat, abstol, reltol, target, loss_kind)`` runs one
    gradient evaluation -- forward solve with saves, the save-point loss (0:
    sum of squares, 1: mean), InterpolatingAdjoint -- and returns
    ``(loss, usave (S,B,nsave), dL/du0 (S,B), dL/dp, counts)``."""

    COUNTS = ("nf", "naccept", "nreject", "nf_adj", "naccept_adj", "nreject_adj", "retcode", "retcode_adj")

    def __init__(self, dims, acts, p, B, cube=False, time_input=False, nthreads=0):
        self.lib = load()
        self.dims = np.ascontiguousarray(dims, np.int32)
        self.acts = np.ascontiguousarray(acts, np.int32)
        self.p = np.ascontiguousarray(p, np.float32)
        self.S = int(dims[-1])
        self.B = int(B)
        self.h = self.lib.cpuf32_create(len(acts), self.dims.ctypes.data, self.acts.ctypes.data, int(cube),
                                        int(time_input), self.p.ctypes.data, self.B, int(nthreads))
        if not self.h:
            raise ValueError("cpuf32_create rejected the network")
        self.nparams = int(self.lib.cpuf32_nparams(self.h))
        if self.nparams != self.p.size:
            raise ValueError(f"parameter count {self.p.size} != {self.nparams}")

    def close(self):
        if self.h:
            self.lib.cpuf32_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grad(self, u0, tspan, saveat, abstol, reltol, target, loss_kind=1, maxiters=100000):
        S, B = self.S, self.B
        u0cm = np.ascontiguousarray(np.asarray(u0, np.float32).T)            # B x S = col-major S x B
        sv = np.ascontiguousarray(saveat, np.float64)
        ns = sv.size
        tg = np.ascontiguousarray(np.transpose(np.asarray(target, np.float32), (2, 1, 0)))
        us = np.empty((ns, B, S), np.float32)
        du0 = np.empty((B, S), np.float32)
        dp = np.empty(self.nparams, np.float32)
        cnt = np.zeros(8, np.int64)
        loss = C.c_double(0.0)
        rc = self.lib.cpuf32_grad(self.h, u0cm.ctypes.data, float(tspan[0]), float(tspan[1]), sv.ctypes.data, ns,
                                  float(abstol), float(reltol), int(maxiters), tg.ctypes.data, int(loss_kind),
                                  C.byref(loss), us.ctypes.data, du0.ctypes.data, dp.ctypes.data,
                                  cnt.ctypes.data)
        counts = dict(zip(self.COUNTS, cnt.tolist()))
        if rc != 0:
            raise RuntimeError(f"forward solve failed: {counts}")
        return loss.value, np.transpose(us, (2, 1, 0)), du0.T, dp, counts
