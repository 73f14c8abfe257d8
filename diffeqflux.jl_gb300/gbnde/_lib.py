"""ctypes binding of the C ABI in ``include/gbnde.h`` (libgbnde.so).

This is the Python counterpart of the ``ccall`` stubs a Julia host would
write. Loading fails loudly when the library is missing: there is no CPU
fallback for the solver.
"""
import ctypes as C
import os

from . import _build

MAX_LAYERS = 8

ACT = {"identity": 0, "tanh": 1, "softplus": 2}
PREC = {"fp32": 0, "bf16": 1}
SENSE = {"interpolating": 0, "backsolve": 1, "gauss": 2}
FLAG_FP32_TIME = 1  # gbnde_solve_desc.flags

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_UNSUPPORTED = -4
ERR_STATE = -5
ERR_TIMEOUT = -6

RET_SUCCESS = 0
RET_MAXITERS = 1
RET_DTLESSTHANMIN = 2
RET_UNSTABLE = 3
RET_BARRIER_TIMEOUT = 4
RETCODE_NAMES = {0: "Success", 1: "MaxIters", 2: "DtLessThanMin", 3: "Unstable", 4: "BarrierTimeout"}

# gbnde_stats.fwd_path / adj_path (gbnde_path)
PATH_NONE, PATH_FP32, PATH_FP32_RECOMPUTE, PATH_TC, PATH_TC_RECOMPUTE = 0, 1, 2, 3, 4
PATH_NAMES = {0: "none", 1: "fp32", 2: "fp32_recompute", 3: "tc", 4: "tc_recompute"}


class MlpDesc(C.Structure):
    _fields_ = [
        ("nlayers", C.c_int),
        ("dims", C.c_int * (MAX_LAYERS + 1)),
        ("act", C.c_int * MAX_LAYERS),
        ("cube_input", C.c_int),
        ("time_input", C.c_int),
    ]


class SolveDesc(C.Structure):
    _fields_ = [
        ("t0", C.c_double), ("t1", C.c_double),
        ("abstol", C.c_double), ("reltol", C.c_double),
        ("dt0", C.c_double), ("dtmin", C.c_double),
        ("maxiters", C.c_longlong),
        ("saveat", C.POINTER(C.c_double)),
        ("nsave", C.c_int),
        ("sensealg", C.c_int),
        ("flags", C.c_int),
    ]


class Segment(C.Structure):
    _fields_ = [("t0", C.c_double), ("t1", C.c_double), ("save_off", C.c_int), ("nsave", C.c_int)]


class Adam(C.Structure):
    _fields_ = [("lr", C.c_double), ("beta1", C.c_double), ("beta2", C.c_double), ("eps", C.c_double)]


class Stats(C.Structure):
    _fields_ = [
        ("nf", C.c_longlong), ("naccept", C.c_longlong), ("nreject", C.c_longlong),
        ("nf_recompute", C.c_longlong),
        ("nf_adj", C.c_longlong), ("naccept_adj", C.c_longlong), ("nreject_adj", C.c_longlong),
        ("retcode", C.c_int), ("retcode_adj", C.c_int),
        ("t_final", C.c_double),
        ("nf_adj_vjp", C.c_longlong),
        ("fwd_path", C.c_int), ("adj_path", C.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every symbol the header declares, with its signature.
_P = C.c_void_p
_FP = C.POINTER(C.c_float)
_SIGS = {
    "gbnde_create": (C.c_int, [C.POINTER(_P), C.POINTER(MlpDesc), C.c_int, C.c_int]),
    "gbnde_destroy": (None, [_P]),
    "gbnde_nparams": (C.c_size_t, [_P]),
    "gbnde_set_params": (C.c_int, [_P, _P, C.c_size_t]),
    "gbnde_set_params_device": (C.c_int, [_P, _P, C.c_size_t]),
    "gbnde_set_stage_memory": (C.c_int, [_P, C.c_size_t]),
    "gbnde_set_grid_cap": (C.c_int, [_P, C.c_int]),
    "gbnde_forward": (C.c_int, [_P, C.POINTER(SolveDesc), C.c_int, C.c_int, _P, _P, C.POINTER(Stats)]),
    "gbnde_forward_device": (C.c_int, [_P, C.POINTER(SolveDesc), C.c_int, C.c_int, _P, _P, C.POINTER(Stats)]),
    "gbnde_backward": (C.c_int, [_P, _P, _P, _P, C.POINTER(Stats)]),
    "gbnde_backward_device": (C.c_int, [_P, _P, _P, _P, C.POINTER(Stats)]),
    "gbnde_loss_device": (C.c_int, [_P, _P, _P, C.c_int, _P, C.POINTER(C.c_double)]),
    "gbnde_ffjord_forward": (C.c_int, [_P, C.POINTER(SolveDesc), C.c_int, C.c_int, _P, _P, _P, _P,
                                      C.POINTER(Stats)]),
    "gbnde_ffjord_backward": (C.c_int, [_P, _P, _P, _P, _P, C.POINTER(Stats)]),
    "gbnde_ffjord_forward_reg": (C.c_int, [_P, C.POINTER(SolveDesc), C.c_int, C.c_int, _P, _P, C.c_int, _P, _P,
                                          _P, _P, C.POINTER(Stats)]),
    "gbnde_ffjord_backward_reg": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, C.POINTER(Stats)]),
    "gbnde_multishoot_forward": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(Segment), C.POINTER(C.c_double),
                                          C.c_int, _P, C.c_double, C.c_double, C.c_longlong, _P,
                                          C.POINTER(C.c_int), C.POINTER(Stats)]),
    "gbnde_multishoot_saves": (C.c_int, [_P, _P]),
    "gbnde_multishoot_backward": (C.c_int, [_P, _P, _P, _P, C.POINTER(Stats)]),
    "gbnde_multishoot_loss": (C.c_int, [_P, _P, _P, C.c_int, C.c_double, C.POINTER(C.c_double)]),
    "gbnde_loss_noalloc": (C.c_int, [_P, _P, C.c_size_t, C.c_int, _P, C.POINTER(C.c_double), _P]),
    "gbnde_train_step": (C.c_int, [_P, C.POINTER(SolveDesc), C.c_int, C.c_int, _P, _P, C.c_int,
                                   C.POINTER(Adam), C.c_longlong, _P, _P, _P, C.POINTER(C.c_double),
                                   C.POINTER(Stats)]),
    "gbnde_graph_train_step": (C.c_int, [_P, C.POINTER(SolveDesc), C.c_int, C.c_int, _P, _P, C.c_int,
                                         C.POINTER(Adam), C.c_longlong, _P, _P, _P, C.POINTER(C.c_double),
                                         C.POINTER(Stats), C.POINTER(C.c_int)]),
    "gbnde_forward_steps": (C.c_longlong, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_longlong]),
    "gbnde_forward_trace": (C.c_longlong, [_P, C.POINTER(C.c_double), C.c_longlong]),
    "gbnde_stream": (C.c_void_p, [_P]),
    "gbnde_set_stream": (C.c_int, [_P, _P]),
    "gbnde_last_kernel_ms": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gbnde_autotune": (C.c_int, [_P, C.POINTER(SolveDesc), C.c_int, C.c_int, _P, C.POINTER(C.c_int)]),
    "gbnde_tc_selftest": (C.c_int, [_FP, _FP, C.c_int, C.c_int, C.c_int, _FP]),
    "gbnde_act_selftest": (C.c_int, [_FP, C.c_int, C.c_int, _FP, _FP]),
    "gbnde_barrier_selftest": (C.c_int, [C.c_int, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "gbnde_strerror": (C.c_char_p, [C.c_int]),
    "gbnde_last_error": (C.c_char_p, []),
}

_lib = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=False):
    """Load libgbnde.so (optionally building it first) and bind the prototypes."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libgbnde.so not found at {path}; run __graft_entry__.build() first")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GbndeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbnde error {code} ({msg})")
        self.code = code


def check(code):
    if code != OK:
        lib = load()
        msg = lib.gbnde_last_error().decode() or lib.gbnde_strerror(code).decode()
        raise GbndeError(code, msg)
    return code
