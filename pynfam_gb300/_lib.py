"""ctypes binding of the C ABI declared in include/pnfam_gpu.h.

The library is loaded from the package directory (in-tree build).  There is
no fallback: if the library is missing or no GPU is usable, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libpnfam_gb300.so")

EXPORTS = ("pnfam_gpu_init", "pnfam_gpu_set_operator", "pnfam_gpu_solve", "pnfam_gpu_calc_hamiltonian",
           "pnfam_gpu_nxy", "pnfam_gpu_last_profile", "pnfam_gpu_free", "pnfam_gpu_last_error",
           "pnfam_gpu_engine_create", "pnfam_gpu_engine_admit", "pnfam_gpu_engine_launch",
           "pnfam_gpu_engine_finish", "pnfam_gpu_engine_active", "pnfam_gpu_engine_ready", "pnfam_gpu_engine_free",
           "pnfam_gpu_calc_hamiltonian_mixed", "pnfam_gpu_set_occupations", "pnfam_gpu_task_tables",
           "pnfam_gpu_solve_state", "pnfam_gpu_state_size", "pnfam_gpu_2bc_field", "pnfam_gpu_hfb_basis",
           "pnfam_gpu_hfb_matrices", "pnfam_gpu_sym_eigen", "pnfam_gpu_hfb_densities")

TASK_TERMS = 4
TASK_RECORD = 7 + 10 * TASK_TERMS

ERRORS = {1: "EINVAL", 2: "ENOMEM", 3: "ECUDA", 4: "ENONFINITE", 5: "ESTATE"}


class PnfamGPUError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Basis(C.Structure):
    _fields_ = [("nb", C.c_int), ("db", C.POINTER(C.c_int)), ("num_spin_up", C.POINTER(C.c_int)),
                ("ns", C.POINTER(C.c_int)), ("nghl", C.c_int)]


class Coupl(C.Structure):
    _fields_ = [("crho", C.POINTER(C.c_double)), ("cs", C.POINTER(C.c_double)),
                ("cpair", C.POINTER(C.c_double)), ("cspair", C.POINTER(C.c_double)),
                ("scalars", C.c_double * 12)]


class TwoBodyInput(C.Structure):
    """pnfam_2bc_input_t"""
    _fields_ = [("ntx", C.c_int), ("nbx", C.c_int), ("block_size", C.POINTER(C.c_int)),
                ("nz", C.POINTER(C.c_int)), ("nr", C.POINTER(C.c_int)), ("nl", C.POINTER(C.c_int)),
                ("ns", C.POINTER(C.c_int)), ("bz", C.c_double), ("bp", C.c_double),
                ("rk_n", C.POINTER(C.c_double)), ("rk_p", C.POINTER(C.c_double)),
                ("K", C.c_int), ("beta_minus", C.c_int), ("use_p", C.c_int),
                ("op_cols", C.POINTER(C.c_int)), ("op_offsets", C.POINTER(C.c_longlong)), ("nxy", C.c_longlong)]


class SolverOpts(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("broyden_history_size", C.c_int),
                ("convergence_epsilon", C.c_double), ("alpha_mix", C.c_double),
                ("quench_residual_int", C.c_double), ("precision", C.c_int),
                ("reserved", C.c_int * 7)]


_lib = None


def load(path: str = LIBPATH):
    """Load the library (raises OSError if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it with `python -m pynfam_gb300.build`")
    lib = C.CDLL(path)
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    lib.pnfam_gpu_init.argtypes = [C.POINTER(Basis), dp, dp, dp, dp, dp, dp, dp, dp, C.POINTER(Coupl), C.POINTER(C.c_void_p)]
    lib.pnfam_gpu_init.restype = C.c_int
    lib.pnfam_gpu_set_operator.argtypes = [C.c_void_p, C.c_int, ip, dp, C.c_int, C.POINTER(dp)]
    lib.pnfam_gpu_set_operator.restype = C.c_int
    lib.pnfam_gpu_solve.argtypes = [C.c_void_p, C.c_int, dp, dp, C.POINTER(SolverOpts), dp, dp, ip, dp, dp]
    lib.pnfam_gpu_solve.restype = C.c_int
    lib.pnfam_gpu_solve_state.argtypes = [C.c_void_p, C.c_int, dp, dp, C.POINTER(SolverOpts), dp, dp, dp, ip, dp, dp,
                                          dp]
    lib.pnfam_gpu_solve_state.restype = C.c_int
    lib.pnfam_gpu_state_size.argtypes = [C.c_void_p]
    lib.pnfam_gpu_state_size.restype = C.c_longlong
    lib.pnfam_gpu_calc_hamiltonian.argtypes = [C.c_void_p] + [dp] * 16
    lib.pnfam_gpu_calc_hamiltonian.restype = C.c_int
    lib.pnfam_gpu_calc_hamiltonian_mixed.argtypes = [C.c_void_p] + [dp] * 16
    lib.pnfam_gpu_calc_hamiltonian_mixed.restype = C.c_int
    lib.pnfam_gpu_nxy.argtypes = [C.c_void_p]
    lib.pnfam_gpu_nxy.restype = C.c_longlong
    lib.pnfam_gpu_last_profile.argtypes = [C.c_void_p, dp, C.c_int, C.POINTER(C.c_longlong)]
    lib.pnfam_gpu_last_profile.restype = C.c_int
    lib.pnfam_gpu_free.argtypes = [C.c_void_p]
    lib.pnfam_gpu_free.restype = None
    lib.pnfam_gpu_last_error.argtypes = []
    lib.pnfam_gpu_last_error.restype = C.c_char_p
    lp = C.POINTER(C.c_longlong)
    lib.pnfam_gpu_engine_create.argtypes = [C.c_void_p, C.c_int, C.POINTER(SolverOpts), C.POINTER(C.c_void_p)]
    lib.pnfam_gpu_engine_create.restype = C.c_int
    lib.pnfam_gpu_engine_admit.argtypes = [C.c_void_p, C.c_int, dp, dp, lp]
    lib.pnfam_gpu_engine_admit.restype = C.c_int
    lib.pnfam_gpu_engine_launch.argtypes = [C.c_void_p]
    lib.pnfam_gpu_engine_launch.restype = C.c_int
    lib.pnfam_gpu_engine_finish.argtypes = [C.c_void_p, C.c_int, lp, dp, dp, ip, dp, ip]
    lib.pnfam_gpu_engine_finish.restype = C.c_int
    lib.pnfam_gpu_engine_active.argtypes = [C.c_void_p]
    lib.pnfam_gpu_engine_active.restype = C.c_int
    lib.pnfam_gpu_engine_ready.argtypes = [C.c_void_p]
    lib.pnfam_gpu_engine_ready.restype = C.c_int
    lib.pnfam_gpu_engine_free.argtypes = [C.c_void_p]
    lib.pnfam_gpu_engine_free.restype = None
    lib.pnfam_gpu_set_occupations.argtypes = [C.c_void_p, dp, dp]
    lib.pnfam_gpu_set_occupations.restype = C.c_int
    lib.pnfam_gpu_task_tables.argtypes = [C.c_int, ip, ip, C.c_int, ip, C.c_int, C.c_int, dp, C.c_int, ip, lp, lp]
    lib.pnfam_gpu_task_tables.restype = C.c_int
    lib.pnfam_gpu_2bc_field.argtypes = [C.POINTER(TwoBodyInput), dp, dp]
    lib.pnfam_gpu_2bc_field.restype = C.c_int
    lib.pnfam_gpu_hfb_basis.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, C.c_double, C.c_double, C.c_int, ip, ip, ip,
                                        dp]
    lib.pnfam_gpu_hfb_basis.restype = C.c_int
    lib.pnfam_gpu_hfb_matrices.argtypes = [C.c_int, ip, C.c_int, ip, dp, dp, dp, dp, dp, dp]
    lib.pnfam_gpu_hfb_matrices.restype = C.c_int
    lib.pnfam_gpu_sym_eigen.argtypes = [C.c_int, ip, dp, dp, dp, dp, ip]
    lib.pnfam_gpu_sym_eigen.restype = C.c_int
    lib.pnfam_gpu_hfb_densities.argtypes = [C.c_int, ip, C.c_int, ip, dp, dp, dp, dp, dp, dp, dp, dp]
    lib.pnfam_gpu_hfb_densities.restype = C.c_int
    _lib = lib
    return lib


def check(rc: int):
    if rc != 0:
        msg = _lib.pnfam_gpu_last_error().decode(errors="replace") if _lib else ""
        raise PnfamGPUError(rc, msg)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int))


def task_tables(db, num_spin_up, fcols, beta_minus: bool, statistical: bool, stage: int):
    """The block-GEMM tasks of one stage (host only, no device): (records [n, TASK_RECORD],
    nxy, scratch elements per plane); see pnfam_gpu_task_tables."""
    lib = load()
    db = np.ascontiguousarray(db, dtype=np.int32)
    nup = np.ascontiguousarray(num_spin_up, dtype=np.int32)
    fc = np.ascontiguousarray(fcols, dtype=np.int32)
    n = C.c_int(); nxy = C.c_longlong(); scr = C.c_longlong()
    check(lib.pnfam_gpu_task_tables(len(db), iptr(db), iptr(nup), int(bool(beta_minus)), iptr(fc),
                                    int(bool(statistical)), int(stage), None, 0, C.byref(n), C.byref(nxy),
                                    C.byref(scr)))
    out = np.zeros((max(n.value, 1), TASK_RECORD))
    check(lib.pnfam_gpu_task_tables(len(db), iptr(db), iptr(nup), int(bool(beta_minus)), iptr(fc),
                                    int(bool(statistical)), int(stage), dptr(out), n.value, C.byref(n),
                                    C.byref(nxy), C.byref(scr)))
    return out[:n.value], int(nxy.value), int(scr.value)
