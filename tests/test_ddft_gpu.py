"""The DDFT step of the multiblock driver on the device (adscf_ddft_*,
adscf_conjugate_fields) against the oracle's restatement (oracle/ddft.py)."""
import numpy as np
import pytest

from adscf_gb300 import BULK, FP64, SPLIT, MIX_ANDERSON, Context
from oracle import ddft as od
from oracle import interactions as oi

pytestmark = pytest.mark.gpu

TABLE = np.array([[0.56, 0.14, 0.16], [0.50, 0.12, 0.15], [0.42, 0.10, 0.13], [0.33, 0.07, 0.11],
                  [0.25, 0.05, 0.09], [0.18, 0.03, 0.07], [0.12, 0.02, 0.05], [0.08, 0.01, 0.04]])
DQ, WCUT = 0.5, 10.0
KAPPA, CHI = 20.0, 12.0
SEQ = ((0.5, 0.1, 0.1, 0.1, 0.1, 0.1), (0, 1, 0, 1, 0, 1))


def ctx(grid, size, ds, prec=FP64, **kw):
    return Context(BULK, grid=grid, size=size, ds=ds, precision=prec, blocks=SEQ[0], block_types=SEQ[1],
                   kappa=KAPPA, chi=CHI, mixing_type=MIX_ANDERSON, mixing_dim=4, lam=0.5, lam_warm=1e-3,
                   warm_iters=4, **kw)


@pytest.mark.parametrize("grid,prec,tol", [((12, 10, 8), FP64, 1e-12), ((15, 9, 10), FP64, 1e-12),
                                           ((32, 32, 32), FP64, 1e-12), ((32, 32, 32), SPLIT, 2e-6)])
def test_ddft_rhs_matches_oracle(grid, prec, tol, rng):
    gx, gy, gz = grid
    size = (6.0, 5.0, 4.0)
    mu = rng.standard_normal((2, gz, gy, gx))
    mob = od.mobility_qq(grid, size, len(TABLE), DQ, TABLE, WCUT)
    ref = od.ddft_rhs(mu, mob)
    with ctx(grid, size, 0.05, prec) as c:
        c.ddft_set_mobility(TABLE, DQ, WCUT)
        out = c.ddft_rhs(mu)
    assert np.max(np.abs(out - ref)) <= tol * np.max(np.abs(ref))
    assert abs(out[0].sum()) <= 1e-9 * np.abs(out[0]).sum()


def test_conjugate_fields_reach_the_density(rng):
    grid, size, ds = (12, 8, 8), (4.0, 3.0, 3.0), 0.05
    w0 = 0.4 * rng.standard_normal((2, 8, 8, 12))
    fn = lambda w: od.calculate_densities(w, grid, size, ds, SEQ[0], SEQ[1])
    target = fn(w0)
    with ctx(grid, size, ds) as c:
        c.set_field(np.zeros_like(w0))
        st, it = c.conjugate_fields(target, accuracy=1e-6, itermax=3000)
        w = c.get_field().reshape(w0.shape)
    assert st == 0 and 1 < it < 3000
    assert np.max(np.abs(fn(w) - target)) <= 0.5e-6 * (1 + 1e-9)


def test_ddft_step_matches_oracle_euler_step(rng):
    """The step's Euler update from the conjugate field of the density: the
    new density equals rho + dt * ddft_rhs(w_mean(rho) - w_conj), and the
    mass of each type is conserved."""
    grid, size, ds = (12, 8, 8), (4.0, 3.0, 3.0), 0.05
    w0 = 0.4 * rng.standard_normal((2, 8, 8, 12))
    fn = lambda w: od.calculate_densities(w, grid, size, ds, SEQ[0], SEQ[1])
    rho = fn(w0)
    dt = 0.01
    mob = od.mobility_qq(grid, size, len(TABLE), DQ, TABLE, WCUT)
    with ctx(grid, size, ds) as c:
        c.ddft_set_mobility(TABLE, DQ, WCUT)
        c.set_field(np.zeros_like(w0))
        st, _it = c.conjugate_fields(rho, accuracy=1e-8, itermax=4000)
        assert st == 0
        wc = c.get_field().reshape(w0.shape)
        rho1, st1 = c.ddft_step(rho, dt, accuracy=1e-8, itermax=4000)
        w1 = c.get_field().reshape(w0.shape)
    expect = rho + dt * od.ddft_rhs(oi.mean_fields(rho, KAPPA, CHI) - wc, mob)
    assert st1 == 0
    assert np.max(np.abs(rho1 - expect)) <= 1e-12 * np.max(np.abs(rho))
    assert np.allclose(rho1.sum(axis=(1, 2, 3)), rho.sum(axis=(1, 2, 3)), rtol=1e-13)
    # the field afterwards is the conjugate field of the new density
    assert np.max(np.abs(fn(w1) - rho1)) <= 0.5e-8 * (1 + 1e-6)
