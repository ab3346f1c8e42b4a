"""ctypes binding of libspde_gb300 (the C ABI declared in include/spde_gb300.h).

The library is built in-tree (``spdepy_gb300/build.py``); importing this module
never falls back to anything else: a missing library or a missing CUDA device
raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libspde_gb300.so")

SPDE_OK = 0
_ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "matrix is not positive definite", 4: "out of memory",
           5: "invalid state", 6: "not converged"}


class NotPositiveDefiniteError(RuntimeError):
    """Raised where the reference's CHOLMOD raises CholmodNotPositiveDefiniteError."""


class SpdeError(RuntimeError):
    pass


class PlanInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("nfronts", ctypes.c_int64), ("max_depth", ctypes.c_int32),
                ("max_front", ctypes.c_int32), ("nslots", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("factor_flops", ctypes.c_double), ("selinv_flops", ctypes.c_double), ("nnz_l", ctypes.c_double),
                ("bytes_factor", ctypes.c_double), ("bytes_work", ctypes.c_double), ("launches", ctypes.c_int64)]


class ModelDesc(ctypes.Structure):
    _fields_ = [("Mx", ctypes.c_int32), ("Ny", ctypes.c_int32), ("T", ctypes.c_int32), ("bc", ctypes.c_int32),
                ("hx", ctypes.c_double), ("hy", ctypes.c_double), ("dt", ctypes.c_double),
                ("diff_form", ctypes.c_int32), ("var_h", ctypes.c_int32), ("adv", ctypes.c_int32),
                ("nbasis", ctypes.c_int32), ("bs", ctypes.c_void_p), ("bsH", ctypes.c_void_p),
                ("bsA", ctypes.c_void_p), ("ww", ctypes.c_void_p), ("mod0_diff_form", ctypes.c_int32),
                ("mod0_bc", ctypes.c_int32), ("temporal", ctypes.c_int32)]


_lib = None

# name -> (restype, argtypes) for every entry point the header declares
_P, _I, _D, _I64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64
SIGNATURES = {
    "spde_diffusion_triplets": (_I, [_I, _I, _P, _I, _D, _D, _I, _P, _P, _P, _P]),
    "spde_advection_triplets": (_I, [_I, _I, _P, _P, _I, _D, _D, _I, _I, _P, _P, _P, _P]),
    "spde_plan_create": (_I, [_I, _I, _I, _I, _I, ctypes.POINTER(_P)]),
    "spde_plan_create_separable": (_I, [_I, _I, _I, _I, _I, ctypes.POINTER(_P)]),
    "spde_plan_destroy": (_I, [_P]),
    "spde_plan_set_stream": (_I, [_P, _P]),
    "spde_plan_info": (_I, [_P, ctypes.POINTER(PlanInfo)]),
    "spde_last_error": (ctypes.c_char_p, [_P]),
    "spde_plan_set_profiling": (_I, [_P, _I]),
    "spde_plan_read_profile": (_I, [_P, _P, _P, _P, _I]),
    "spde_plan_read_sites": (_I, [_P, _P, _P, _P, _I]),
    "spde_plan_set_pipelines": (_I, [_P, _I]),
    "spde_plan_set_wait_limit": (_I, [_P, _I64]),
    "spde_symbolic_info": (_I, [_I, _I, _I, _I, ctypes.POINTER(PlanInfo)]),
    "spde_symbolic_export": (_I, [_I, _I, _I, _I, _P, _P, _P, _P, _I64]),
    "spde_set_model": (_I, [_P, ctypes.POINTER(ModelDesc)]),
    "spde_assemble": (_I, [_P, _P, _I]),
    "spde_export_q": (_I, [_P, _I, _D, _P]),
    "spde_spmv": (_I, [_P, _I, _D, _P, _P, _I]),
    "spde_set_obs": (_I, [_P, _P, _I]),
    "spde_set_obs_weighted": (_I, [_P, _P, _P, _I]),
    "spde_factor": (_I, [_P, _I, _D, ctypes.POINTER(_D)]),
    "spde_solve": (_I, [_P, _P, _P, _I, _I, _D, ctypes.POINTER(_D)]),
    "spde_sample": (_I, [_P, _P, _P, _I]),
    "spde_selinv": (_I, [_P, _P]),
    "spde_adjoint": (_I, [_P, _P, _P]),
    "spde_adjoint_noalloc": (_I, [_P, _P, _P]),
    "spde_loglike": (_I, [_P, _P, _I, _P, _I, _I, _P, _I, ctypes.POINTER(_D), _P]),
    "spde_conditional_mean": (_I, [_P, _D, _P, _P, _P]),
    "spde_precond_nparams": (_I, []),
    "spde_precond_weights": (_I, [_P, _I, _D, _P, _P, _P]),
    "spde_precond_compact_size": (_I, [_P, ctypes.POINTER(_I64)]),
    "spde_precond_weights_compact": (_I, [_P, _I, _D, _P, _P]),
    "spde_precond_grad": (_I, [_P, _I, _D, _P, _P, _P, _P, _I, ctypes.POINTER(_D), _P]),
    "spde_adam_step": (_I, [_P, _P, _P, _P, _P, _I, _D, _D, _D, _D, _I]),
    "spde_qsqrt": (_I, [_P, _I, _P, _P, _I]),
    "spde_jacobi_smooth": (_I, [_P, _I, _D, _D, _I, _P, _I]),
    "spde_loglike_grad_pcg": (_I, [_P, _D, _P, _I, _P, _I, _I, _P, _P, _D, _I, _P, ctypes.POINTER(_I)]),
    "spde_pcg": (_I, [_P, _I, _D, _I, _P, _P, _P, _I, _D, _I, ctypes.POINTER(_I), ctypes.POINTER(_D)]),
}


def lib():
    """Load the native library (built by ``spdepy_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libspde_gb300.so is not built ({LIB_PATH}); run spdepy_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc, plan=None, what=""):
    if rc == SPDE_OK:
        return
    msg = _ERRORS.get(rc, f"status {rc}")
    if plan is not None:
        detail = lib().spde_last_error(plan)
        if detail:
            msg += ": " + detail.decode()
    if rc == 3:
        raise NotPositiveDefiniteError(msg)
    raise SpdeError(f"{what}: {msg}" if what else msg)


def ptr(a):
    """Raw pointer of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def symbolic_info(Mx, Ny, T, leaf_max=128):
    info = PlanInfo()
    check(lib().spde_symbolic_info(Mx, Ny, T, leaf_max, ctypes.byref(info)), what="symbolic analysis")
    return info


def symbolic_export(Mx, Ny, T, leaf_max=128):
    info = symbolic_info(Mx, Ny, T, leaf_max)
    nf = int(info.nfronts)
    perm = np.zeros(int(info.n), np.int32)
    ns, nb, par = (np.zeros(nf, np.int32) for _ in range(3))
    check(lib().spde_symbolic_export(Mx, Ny, T, leaf_max, ptr(perm), ptr(ns), ptr(nb), ptr(par), nf))
    return perm, ns, nb, par
