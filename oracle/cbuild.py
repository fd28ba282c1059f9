"""Build recipe of the oracle's C++ restatement (test infrastructure).

``build()`` compiles ``oracle/scf_cpu.cpp`` (FP64, OpenMP) into
``oracle/_build/libscf_cpu.so`` with g++; ``load()`` returns it through
ctypes.  Only the tests, ``__graft_entry__`` and ``bench.py``'s CPU legs use
it -- the GPU library never does.
"""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "scf_cpu.cpp"
OUT = HERE / "_build" / "libscf_cpu.so"
FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared"]

_lib = None


def build(verbose: bool = False) -> Path:
    """Compile the restatement (skipped when the library is newer than its source)."""
    if OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the oracle's restatement")
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    r = subprocess.run([cxx, *FLAGS, str(SRC), "-o", str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {SRC.name}:\n{r.stderr}")
    tmp.replace(OUT)
    if verbose:
        print(f"built {OUT}")
    return OUT


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        dp = C.POINTER(C.c_double)
        lib.scfcpu_threads.restype = C.c_int
        lib.scfcpu_set_threads.argtypes = [C.c_int]
        lib.scfcpu_create.restype = C.c_void_p
        lib.scfcpu_create.argtypes = [C.POINTER(C.c_int), dp, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.c_int, C.c_double, C.c_double, C.c_int]
        lib.scfcpu_destroy.argtypes = [C.c_void_p]
        lib.scfcpu_contour_steps.argtypes = [C.c_void_p]
        lib.scfcpu_contour_steps.restype = C.c_int
        for fn in ("scfcpu_set_field", "scfcpu_get_field", "scfcpu_get_density"):
            getattr(lib, fn).argtypes = [C.c_void_p, dp]
        lib.scfcpu_iterate.argtypes = [C.c_void_p, C.c_int, dp]
        lib.scfcpu_propagate.argtypes = [C.c_void_p, dp, dp, dp]
        lib.scfcpu_fft3d.argtypes = [C.c_int, C.c_int, C.c_int, dp, C.c_int]
        lib.scfcpu_fft3d.restype = C.c_int
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class ScfCpu:
    """Canonical bulk diblock melt with Anderson mixing, on the host cores."""

    def __init__(self, grid, size, ds, f_a, kappa, chi, m=10, lam=0.1, lam_warm=0.1,
                 warm_iters=10):
        import numpy as np
        self.lib = load()
        self.grid = tuple(grid)
        g = (C.c_int * 3)(*grid)
        b = (C.c_double * 3)(*size)
        self.h = self.lib.scfcpu_create(g, b, ds, f_a, kappa, chi, m, lam, lam_warm, warm_iters)
        if not self.h:
            raise RuntimeError("scfcpu_create failed")
        self.n2 = 2 * grid[0] * grid[1] * grid[2]
        self.np = np

    def close(self):
        if getattr(self, "h", None):
            self.lib.scfcpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def ns(self):
        return self.lib.scfcpu_contour_steps(self.h)

    def set_field(self, w):
        a = self.np.ascontiguousarray(w, dtype=self.np.float64).reshape(-1)
        self.lib.scfcpu_set_field(self.h, _dp(a))

    def get_field(self):
        out = self.np.empty(self.n2)
        self.lib.scfcpu_get_field(self.h, _dp(out))
        return out

    def get_density(self):
        out = self.np.empty(self.n2)
        self.lib.scfcpu_get_density(self.h, _dp(out))
        return out

    def iterate(self, n=1):
        """n SCF iterations; returns (accuracy, F per chain, log Q, iteration)."""
        out = self.np.empty(4)
        self.lib.scfcpu_iterate(self.h, int(n), _dp(out))
        return out[0], out[1], out[2], int(out[3])

    def propagate(self, w):
        """Propagate_Diblock at w: (density [2][N], Qsum, logQ, mu, energy)."""
        a = self.np.ascontiguousarray(w, dtype=self.np.float64).reshape(-1)
        dens = self.np.empty(self.n2)
        out = self.np.empty(4)
        self.lib.scfcpu_propagate(self.h, _dp(a), _dp(dens), _dp(out))
        return dens, out[0], out[1], out[2], out[3]


def fft3d(a, sign=-1):
    """Unnormalised 3D complex FFT of a [gz][gy][gx] complex array."""
    import numpy as np
    lib = load()
    buf = np.ascontiguousarray(np.stack([a.real, a.imag], axis=-1), dtype=np.float64)
    gz, gy, gx = a.shape
    if lib.scfcpu_fft3d(gx, gy, gz, _dp(buf), int(sign)) != 0:
        raise ValueError("grid length with a prime factor above 5")
    return buf[..., 0] + 1j * buf[..., 1]
