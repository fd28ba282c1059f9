"""Reverse-mode adjoint of the bulk diblock free energy (adscf_forward /
adscf_backward) against central finite differences of the oracle's free
energy at fixed fields, and against the difference of converged free
energies of neighbouring box sizes."""
import numpy as np
import pytest

from adscf_gb300 import BULK, FP64, SPLIT, MIX_ANDERSON, AdscfError, Context
from oracle import bulk as ob, interactions as oi

pytestmark = pytest.mark.gpu

KAPPA, CHI, F_A = 10.0, 15.0, 0.4


def oracle_free_energy(w, grid, size, ds, chi=CHI):
    """Calculate_Energy (main_diblock.f90:295-307) at the densities of w."""
    r = ob.propagate_diblock(w, grid, size, ds, (F_A, 1.0 - F_A))
    phi = ob.density_by_type(r["density"])
    eint = oi.interaction_energy(phi, KAPPA, chi, r["dvol"])
    phiw = r["dvol"] * np.sum(phi * w)
    return (r["energy"] - phiw + eint) / (r["rho"] * r["volume"])


def ctx(grid, size, ds, prec=FP64, chi=CHI, **kw):
    return Context(BULK, grid=grid, size=size, ds=ds, block_length=(F_A, 1.0 - F_A),
                   kappa=KAPPA, chi=chi, precision=prec, **kw)


def fields(grid, size, rng, amp=1.0, noise=0.3):
    gx, gy, gz = grid
    x = np.arange(gx) * size[0] / gx
    y = np.arange(gy) * size[1] / gy
    s = np.cos(2 * np.pi * x / size[0])[None, None, :] * np.cos(2 * np.pi * y / size[1])[None, :, None]
    s = np.broadcast_to(s, (gz, gy, gx))
    w = np.stack([amp * s, -amp * s]) + noise * rng.standard_normal((2, gz, gy, gx))
    return w


def test_forward_free_energy_matches_oracle(rng):
    grid, size, ds = (16, 12, 10), (3.3, 3.1, 2.9), 0.05
    w = fields(grid, size, rng)
    with ctx(grid, size, ds) as c:
        F = c.forward(w)
    assert abs(F - oracle_free_energy(w, grid, size, ds)) < 1e-12 * max(1.0, abs(F))


def test_gradient_matches_oracle_central_differences(rng):
    grid, size, ds = (16, 12, 10), (3.3, 3.1, 2.9), 0.05
    w = fields(grid, size, rng)
    with ctx(grid, size, ds) as c:
        c.forward(w)
        g = c.backward()
    d = 1e-5
    for i in range(3):
        sp = list(size); sm = list(size)
        sp[i] += d; sm[i] -= d
        fd = (oracle_free_energy(w, grid, tuple(sp), ds) - oracle_free_energy(w, grid, tuple(sm), ds)) / (2 * d)
        assert abs(g[i] - fd) < 1e-6 * max(1e-2, abs(fd)), (i, g[i], fd)
    dc = 1e-4
    fd = (oracle_free_energy(w, grid, size, ds, CHI + dc) - oracle_free_energy(w, grid, size, ds, CHI - dc)) / (2 * dc)
    assert abs(g[3] - fd) < 1e-8 * max(1.0, abs(fd))


def test_gradient_matches_gpu_central_differences_register_path(rng):
    # 32^3 runs the FP64 forward on the register-FFT passes
    grid, size, ds = (32, 32, 32), (3.9, 4.1, 3.7), 0.04
    w = fields(grid, size, rng, amp=2.0, noise=0.2)
    with ctx(grid, size, ds) as c:
        F0 = c.forward(w)
        g = c.backward()
    assert abs(F0 - oracle_free_energy(w, grid, size, ds)) < 1e-11 * max(1.0, abs(F0))
    d = 1e-5
    for i in range(3):
        sp = list(size); sm = list(size)
        sp[i] += d; sm[i] -= d
        with ctx(grid, tuple(sp), ds) as c:
            fp = c.forward(w)
        with ctx(grid, tuple(sm), ds) as c:
            fm = c.forward(w)
        fd = (fp - fm) / (2 * d)
        assert abs(g[i] - fd) < 1e-6 * max(1e-2, abs(fd)), (i, g[i], fd)


def test_backward_is_repeatable_and_deterministic(rng):
    grid, size, ds = (16, 16, 16), (3.5, 3.5, 3.5), 0.05
    w = fields(grid, size, rng)
    with ctx(grid, size, ds) as c:
        c.forward(w)
        g1 = c.backward()
        g2 = c.backward()
        c.forward(w)
        g3 = c.backward()
    assert np.array_equal(g1, g2) and np.array_equal(g1, g3)


def test_backward_state_errors(rng):
    grid, size, ds = (16, 16, 16), (3.5, 3.5, 3.5), 0.05
    w = fields(grid, size, rng)
    with ctx(grid, size, ds) as c:
        with pytest.raises(AdscfError):
            c.backward()                       # no forward yet
        c.forward(w)
        c.propagate_diblock(w)                 # overwrites the slices
        with pytest.raises(AdscfError):
            c.backward()
    with ctx(grid, size, ds, prec=SPLIT) as c:
        with pytest.raises(AdscfError):
            c.forward(w)


def test_stress_at_saddle_matches_neighbouring_box_free_energies(rng):
    """At a converged saddle point dF/dL_x equals the slope of the
    equilibrium free energy between neighbouring box sizes."""
    grid, ds = (32, 8, 8), 0.05
    size = (4.2, 2.0, 2.0)
    x = np.arange(grid[0]) * size[0] / grid[0]
    s = np.broadcast_to(np.cos(2 * np.pi * x / size[0])[None, None, :], grid[::-1])
    w0 = np.stack([2.0 * s, -2.0 * s]) + 0.01 * rng.standard_normal((2,) + grid[::-1])

    def converge(sz, start):
        with ctx(grid, sz, ds, mixing_type=MIX_ANDERSON, mixing_dim=10, lam=0.1,
                 lam_warm=0.1, warm_iters=10) as c:
            c.set_field(start)
            res = c.scf_run(3000, tol=1e-26)
            wf = c.get_field().reshape(start.shape)
            F = c.forward(wf)
            g = c.backward()
        return wf, F, g, res

    wc, Fc, gc, res = converge(size, w0)
    assert res.accuracy < 1e-18
    d = 2e-3
    _, Fp, _, _ = converge((size[0] + d,) + size[1:], wc)
    _, Fm, _, _ = converge((size[0] - d,) + size[1:], wc)
    slope = (Fp - Fm) / (2 * d)
    assert abs(gc[0] - slope) < 1e-5 * max(1e-2, abs(slope)) + 1e-8, (gc[0], slope)
