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


def test_multiblock_two_blocks_is_the_diblock(rng):
    grid, size, ds = (6, 4, 5), (3.0, 2.0, 2.5), 0.02
    w = 0.5 * rng.standard_normal((2, 5, 4, 6))
    d = ob.propagate_diblock(w, grid, size, ds, (0.3, 0.7))
    m = ob.propagate_multiblock(w, grid, size, ds, (0.3, 0.7), (0, 1))
    assert m["Qsum"] == d["Qsum"]
    assert np.array_equal(m["density"], d["density"])
    assert np.array_equal(m["density_type"], ob.density_by_type(d["density"]))


def test_multiblock_constant_fields():
    """Constant w_A, w_B: q_N = exp(-sum over blocks of w_type * length) and
    each block's density is rho * (its length) (mod_multiblock.f90:170)."""
    grid, size, ds = (4, 4, 4), (2.0, 2.0, 2.0), 0.01
    w = np.stack([np.full((4, 4, 4), 0.3), np.full((4, 4, 4), -0.2)])
    blocks, types = (0.5, 0.1, 0.1, 0.1, 0.1, 0.1), (0, 1, 0, 1, 0, 1)
    r = ob.propagate_multiblock(w, grid, size, ds, blocks, types, rho=0.8)
    assert np.isclose(r["Qsum"], 8.0 * np.exp(-(0.3 * 0.7 - 0.2 * 0.3)), rtol=1e-12)
    for k, b in enumerate(blocks):
        assert np.allclose(r["density"][k], 0.8 * b, rtol=1e-12)
    assert np.allclose(r["density_type"][0], 0.8 * 0.7) and np.allclose(r["density_type"][1], 0.8 * 0.3)


def test_multiblock_reversed_sequence_is_the_same_chain(rng):
    """A linear chain read from its other end: same Q, block densities reversed."""
    grid, size, ds = (6, 4, 4), (3.0, 2.0, 2.0), 0.02
    w = 0.5 * rng.standard_normal((2, 4, 4, 6))
    blocks, types = (0.2, 0.3, 0.1, 0.4), (0, 1, 1, 0)
    a = ob.propagate_multiblock(w, grid, size, ds, blocks, types)
    b = ob.propagate_multiblock(w, grid, size, ds, blocks[::-1], types[::-1])
    assert np.isclose(a["Qsum"], b["Qsum"], rtol=1e-12)
    assert np.allclose(a["density"], b["density"][::-1], rtol=1e-10, atol=1e-14)


def test_update_solvent_known_answers(rng):
    """Update_Solvent (mod_solvent.f90:85-110): a uniform field w gives
    Qsum = V exp(-w); canonical density rho everywhere and mu = log(rho) + w;
    grand canonical density exp(mu - w) and rho equal to it; both ensembles
    agree when mu is the canonical one."""
    grid, size = (4, 5, 6), (2.0, 2.5, 3.0)
    V = 2.0 * 2.5 * 3.0
    w = np.full((6, 5, 4), 0.7)
    c = ob.update_solvent(w, grid, size, 1, rho=0.8)
    assert np.isclose(c["Qsum"], V * np.exp(-0.7))
    assert np.allclose(c["density"], 0.8)
    assert np.isclose(c["mu"], np.log(0.8) + 0.7)
    assert np.isclose(c["energy"], 0.8 * V * (c["mu"] - 1.0))
    g = ob.update_solvent(w, grid, size, 2, mu=0.3)
    assert np.allclose(g["density"], np.exp(0.3 - 0.7))
    assert np.isclose(g["rho"], np.exp(0.3 - 0.7))
    assert np.isclose(g["energy"], -g["rho"] * V)
    w = rng.standard_normal((6, 5, 4))
    c = ob.update_solvent(w, grid, size, 1, rho=1.3)
    g = ob.update_solvent(w, grid, size, 2, mu=c["mu"])
    assert np.allclose(g["density"], c["density"]) and np.isclose(g["rho"], 1.3)
    with pytest.raises(ValueError):
        ob.update_solvent(w, grid, size, 3)
