"""Pins the FP64 oracle (CPU) with analytic known answers -- the reference
ships no golden vectors, so these are the pins (oracle/bulk.py, iterate.py)."""
import numpy as np
import pytest

from oracle import bulk as ob
from oracle import interactions as oi
from oracle import iterate as oit


def test_fft_normalisation_matches_reference_convention(rng):
    q = rng.standard_normal((6, 5, 8))
    f = ob.real2fourier(q)
    assert np.isclose(f[0, 0, 0].real, q.mean())             # mod_fourier.f90:102
    assert np.allclose(ob.fourier2real(f, q.shape), q)        # round trip


def test_wavenumber_wrap():
    k = ob.wavenumbers(8, 2 * np.pi)
    assert list(k) == [0, 1, 2, 3, 4, -3, -2, -1]             # mod_fourier.f90:181-186


def test_constant_field_partition_function():
    grid, size, ds = (6, 4, 5), (3.0, 2.0, 2.5), 0.01
    w = np.full((2, 5, 4, 6), 0.4)
    r = ob.propagate_diblock(w, grid, size, ds, (0.25, 0.75), keep_chains=True)
    V = 15.0
    assert np.isclose(r["Qsum"], V * np.exp(-0.4), rtol=1e-13)
    for s in range(r["segments"] + 1):
        assert np.allclose(r["qq"][s], np.exp(-0.4 * s * ds), rtol=1e-12)
    assert np.allclose(r["density"][0], 0.25) and np.allclose(r["density"][1], 0.75)


def test_partition_function_is_contour_invariant(rng):
    """sum q_s qdag_{N-s} is the same for every s (each step operator is
    symmetric), a property the GPU contour pass relies on."""
    grid, size, ds = (8, 6, 4), (3.0, 3.0, 2.0), 0.05
    w = rng.standard_normal((2, 4, 6, 8))
    r = ob.propagate_diblock(w, grid, size, ds, (0.4, 0.6), keep_chains=True)
    N = r["segments"]
    vals = [np.sum(r["qq"][s] * r["qqdag"][N - s]) * r["dvol"] for s in range(N + 1)]
    assert np.allclose(vals, r["Qsum"], rtol=1e-12)


def test_block_segments_nint():
    assert ob.block_segments((0.3, 0.7), 0.01) == [30, 70]
    assert ob.block_segments((0.4, 0.6), 0.005) == [80, 120]


def test_grand_canonical_closure(rng):
    grid, size, ds = (4, 4, 4), (2.0, 2.0, 2.0), 0.05
    w = 0.3 * rng.standard_normal((2, 4, 4, 4))
    r = ob.propagate_diblock(w, grid, size, ds, (0.5, 0.5), ensemble=2, mu=1.2)
    assert np.allclose(r["density"], np.exp(1.2) * r["distribution"])
    assert np.isclose(r["energy"], -r["rho"] * r["volume"])


def test_lu_matches_dense_solve(rng):
    a = rng.standard_normal((6, 6)) + 6 * np.eye(6)
    b = rng.standard_normal(6)
    assert np.allclose(oit.solve_linear_system_lu(a, b), np.linalg.solve(a, b), rtol=1e-12)


def test_anderson_reduces_to_least_squares(rng):
    """Mixing_Anderson's coefficients solve min |r0 - sum c_i (r0 - r_i)|."""
    n, m = 50, 3
    field = rng.standard_normal((m + 1, n))
    dfield = rng.standard_normal((m + 1, n))
    d0 = dfield.copy()
    c = oit.mixing_anderson(field, dfield, 0.5, it=m + 1)
    D = (d0[0][None, :] - d0[1:]).T
    c_ls, *_ = np.linalg.lstsq(D, d0[0], rcond=None)
    assert np.allclose(c, c_ls, rtol=1e-9)


def test_lambda_mixing_step():
    f = np.zeros((3, 4)); d = np.zeros((3, 4))
    f[0] = 1.0; d[0] = 2.0
    lam = oit.mixing_lambda(f, d, 0.5, it=1)
    assert lam == 1e-5 and np.allclose(f[0], 1.0 + 2e-5) and np.allclose(f[1], 1.0)


def test_mean_field_helfand_model():
    dens = np.array([[0.6], [0.5]])
    w = oi.mean_fields(dens, kappa=10.0, chi=20.0)
    assert np.allclose(w[:, 0], [10 * 0.1 + 20 * 0.5, 10 * 0.1 + 20 * 0.6])
