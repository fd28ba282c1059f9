"""adscf_gb300 -- the ADSCF SCF inner loop on one GB300 (sm_103a).

The compute lives in ``libadscf_gb300.so`` (hand-written CUDA behind the C
ABI of ``include/adscf.h``); :mod:`adscf_gb300.scf` mirrors the reference
module procedures over that ABI.
"""
from . import _lib
from ._lib import (BULK, FILM_1D, FILM_3D, BRUSH, FP64, SPLIT, MIX_SIMPLE,
                   MIX_LAMBDA, MIX_ANDERSON, AdscfError)
from .scf import Batch, Context, make_params

__all__ = ["Batch", "Context", "make_params", "AdscfError", "BULK", "FILM_1D", "FILM_3D", "BRUSH",
           "FP64", "SPLIT", "MIX_SIMPLE", "MIX_LAMBDA", "MIX_ANDERSON"]
