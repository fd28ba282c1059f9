"""ctypes binding of the C ABI in ``include/adscf.h``.

The shared library is the product; this module only loads it and declares
the signatures.  Loading fails loudly when the library is missing: there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libadscf_gb300.so"

ADSCF_OK = 0
ADSCF_E_ARG = 1
ADSCF_E_CUDA = 2
ADSCF_E_PIVOT = 3
ADSCF_E_NONFINITE = 4
ADSCF_E_TIMEOUT = 5
ADSCF_E_OOM = 6
ADSCF_E_STATE = 7
ADSCF_E_TOO_LARGE = 8

BULK, FILM_1D, FILM_3D, BRUSH = 0, 1, 2, 3
FP64, SPLIT = 0, 1
MIX_SIMPLE, MIX_LAMBDA, MIX_ANDERSON = 1, 2, 3

_dp = C.POINTER(C.c_double)


class Params(C.Structure):
    _fields_ = [
        ("geometry", C.c_int),
        ("gx", C.c_int), ("gy", C.c_int), ("gz", C.c_int),
        ("sizex", C.c_double), ("sizey", C.c_double), ("sizez", C.c_double),
        ("ds", C.c_double),
        ("dss", _dp),
        ("ns", C.c_int),
        ("n_a", C.c_int),
        ("block_length", C.c_double * 2),
        ("ensemble", C.c_int),
        ("rho", C.c_double), ("mu", C.c_double),
        ("kappa", C.c_double), ("chi", C.c_double),
        ("monomer_volume", C.c_double * 2),
        ("precision", C.c_int),
        ("mixing_type", C.c_int),
        ("mixing_dim", C.c_int),
        ("lam", C.c_double),
        ("lam_warm", C.c_double),
        ("warm_iters", C.c_int),
        ("dz", _dp),
        ("int_scheme", C.c_int),
        ("int_span", C.c_int),
        ("ext_potential", _dp),
        ("ww", C.c_double),
        ("graft", _dp),
        ("nblocks", C.c_int),
        ("blocks", _dp),
        ("block_types", C.POINTER(C.c_int)),
    ]


class ChainResult(C.Structure):
    _fields_ = [("Qsum", C.c_double), ("logQ", C.c_double), ("mu", C.c_double),
                ("rho", C.c_double), ("energy", C.c_double)]


class IterResult(C.Structure):
    _fields_ = [("accuracy", C.c_double), ("free_energy", C.c_double),
                ("Qsum", C.c_double), ("logQ", C.c_double), ("mu", C.c_double),
                ("rho", C.c_double), ("lam", C.c_double), ("iter", C.c_int),
                ("status", C.c_int)]


# name -> (restype, argtypes); every symbol include/adscf.h declares
SIGNATURES = {
    "adscf_abi_version": (C.c_int, []),
    "adscf_status_string": (C.c_char_p, [C.c_int]),
    "adscf_last_error": (C.c_char_p, [C.c_void_p]),
    "adscf_ctx_create": (C.c_int, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "adscf_ctx_destroy": (C.c_int, [C.c_void_p]),
    "adscf_field_points": (C.c_longlong, [C.c_void_p]),
    "adscf_contour_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "adscf_propagate_diblock": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(ChainResult)]),
    "adscf_propagate_diblock_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(ChainResult)]),
    "adscf_propagate_homopolymer": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(ChainResult)]),
    "adscf_propagate_step": (C.c_int, [C.c_void_p, _dp, _dp, C.c_double]),
    "adscf_real2fourier": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_fourier2real": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_integrator": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_mean_fields": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_update_solvent": (C.c_int, [C.c_void_p, _dp, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp]),
    "adscf_interaction_energy": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_mix": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int]),
    "adscf_mix_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "adscf_mix_reset": (C.c_int, [C.c_void_p]),
    "adscf_set_field": (C.c_int, [C.c_void_p, _dp]),
    "adscf_set_density": (C.c_int, [C.c_void_p, _dp]),
    "adscf_get_field": (C.c_int, [C.c_void_p, _dp]),
    "adscf_get_density": (C.c_int, [C.c_void_p, _dp]),
    "adscf_scf_run": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(IterResult)]),
    "adscf_scf_iteration": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(IterResult)]),
    "adscf_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "adscf_enqueue": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "adscf_stage_launches": (C.c_int, [C.c_void_p, C.c_int]),
    "adscf_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int]),
    "adscf_probe_l2_copy": (C.c_int, [C.c_longlong, C.c_int, C.POINTER(C.c_double)]),
    "adscf_tuning": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "adscf_set_pass_plan": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "adscf_set_adi_plan": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "adscf_forward": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_backward": (C.c_int, [C.c_void_p, _dp]),
    "adscf_forward_dev": (C.c_int, [C.c_void_p, C.c_void_p, _dp]),
    "adscf_backward_surface": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_set_adjoint_checkpoint": (C.c_int, [C.c_void_p, C.c_int]),
    "adscf_ddft_set_mobility": (C.c_int, [C.c_void_p, C.c_int, C.c_double, _dp, C.c_double]),
    "adscf_ddft_rhs": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_conjugate_fields": (C.c_int, [C.c_void_p, _dp, C.c_double, C.c_int, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]),
    "adscf_ddft_step": (C.c_int, [C.c_void_p, _dp, C.c_double, C.c_int, C.c_double, C.c_int,
                                  C.POINTER(C.c_int)]),
    "adscf_free_energy_fp64": (C.c_int, [C.c_void_p, C.POINTER(IterResult)]),
    "adscf_set_box": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double]),
    "adscf_batch_create": (C.c_int, [C.POINTER(Params), C.c_int, C.POINTER(C.c_void_p)]),
    "adscf_batch_destroy": (C.c_int, [C.c_void_p]),
    "adscf_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "adscf_batch_offset": (C.c_longlong, [C.c_void_p, C.c_int]),
    "adscf_batch_set_fields": (C.c_int, [C.c_void_p, _dp]),
    "adscf_batch_get_fields": (C.c_int, [C.c_void_p, _dp]),
    "adscf_batch_get_densities": (C.c_int, [C.c_void_p, _dp]),
    "adscf_batch_scf_run": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(IterResult)]),
    "adscf_batch_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "adscf_batch_enqueue": (C.c_int, [C.c_void_p, C.c_int]),
    "adscf_batch_results": (C.c_int, [C.c_void_p, C.POINTER(IterResult)]),
    "adscf_batch_launches": (C.c_int, [C.c_void_p]),
    "adscf_batch_forward": (C.c_int, [C.c_void_p, _dp, _dp]),
    "adscf_batch_backward": (C.c_int, [C.c_void_p, _dp]),
    "adscf_propagate_step_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                               C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                                               C.c_void_p]),
}

STAGE_ITERATION, STAGE_PROPAGATE, STAGE_CONTOUR, STAGE_UPDATE = 0, 1, 2, 3

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the library (once) and declare every signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -m adscf_gb300.build` "
            "(there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class AdscfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"adscf status {code}: {msg}")
        self.code = code


def check(lib, ctx, rc: int):
    if rc != ADSCF_OK:
        detail = lib.adscf_last_error(ctx).decode() if ctx else ""
        raise AdscfError(rc, f"{lib.adscf_status_string(rc).decode()} ({detail})")


def c_double_out(fn, *args):
    """Call fn(*args, &out) for an entry point with a trailing double*
    result; None when it returns a non-zero status."""
    out = C.c_double()
    return out.value if fn(*args, C.byref(out)) == ADSCF_OK else None


def dptr(a):
    """Pointer to a C-contiguous float64 numpy array."""
    return a.ctypes.data_as(_dp)
