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


def ctx(grid, size, ds, prec=FP64, chi=CHI, kappa=KAPPA, **kw):
    return Context(BULK, grid=grid, size=size, ds=ds, block_length=(F_A, 1.0 - F_A),
                   kappa=kappa, chi=chi, precision=prec, **kw)


# an ordered lamellar phase along x: chiN = 25, kappa = 25 at f_A = 0.4
# (the free energy of converged lamellae has its minimum near L_x = 4.1)
LAM = dict(chi=25.0, kappa=25.0, mixing_type=MIX_ANDERSON, mixing_dim=10, lam=0.1, lam_warm=0.1,
           warm_iters=10)


def lamellar_start(grid, size, rng, amp=5.0):
    x = np.arange(grid[0]) * size[0] / grid[0]
    s = np.broadcast_to(np.cos(2 * np.pi * x / size[0])[None, None, :], grid[::-1])
    return np.stack([amp * s, -amp * s]) + 0.01 * rng.standard_normal((2,) + grid[::-1])


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


@pytest.mark.parametrize("grid,size,ds,every", [
    ((16, 12, 10), (3.3, 3.1, 2.9), 0.05, -1),   # Ns 20, segments of 5 (generic passes)
    ((16, 12, 10), (3.3, 3.1, 2.9), 0.05, 3),    # ragged last segment
    ((16, 12, 10), (3.3, 3.1, 2.9), 0.05, 1),
    ((16, 12, 10), (3.3, 3.1, 2.9), 0.05, 20),   # one segment
    ((32, 32, 32), (3.9, 4.1, 3.7), 0.04, -1),   # Ns 25; the stored pass runs the register FFTs
    ((24, 20, 18), (3.6, 3.3, 3.1), 0.03, -1),   # Ns 34 (odd segment count), odd block boundary
])
def test_checkpointed_adjoint_matches_stored_slices(rng, grid, size, ds, every):
    w = fields(grid, size, rng, amp=1.5, noise=0.3)
    with ctx(grid, size, ds) as c:
        F0 = c.forward(w)
        g0 = c.backward()
        c.set_adjoint_checkpoint(every)
        F1 = c.forward(w)
        g1 = c.backward()
        g1b = c.backward()
    assert abs(F1 - F0) < 1e-12 * max(1.0, abs(F0))
    assert np.allclose(g1, g0, rtol=1e-10, atol=1e-12), (g0, g1)
    assert np.array_equal(g1, g1b)


def test_checkpointing_releases_and_restores_the_slices(rng):
    grid, size, ds = (16, 16, 16), (3.5, 3.5, 3.5), 0.05
    w = fields(grid, size, rng)
    with ctx(grid, size, ds) as c:
        c.forward(w)
        g0 = c.backward()
        c.set_adjoint_checkpoint(-1)
        with pytest.raises(AdscfError):
            c.propagate_diblock(w)             # the slices are released
        with pytest.raises(AdscfError):
            c.backward()                       # the forward predates the mode change
        c.forward(w)
        assert np.allclose(c.backward(), g0, rtol=1e-10, atol=1e-12)
        c.set_adjoint_checkpoint(0)
        c.forward(w)
        assert np.array_equal(c.backward(), g0)   # the stored-slice pass again
        c.set_field(w)
        r = c.scf_run(3, tol=0.0)
        assert np.isfinite(r.free_energy)
    with ctx(grid, size, ds, prec=SPLIT) as c:
        with pytest.raises(AdscfError):
            c.set_adjoint_checkpoint(-1)


def test_stress_at_saddle_matches_neighbouring_box_free_energies(rng):
    """At a converged (ordered) saddle point dF/dL_x equals the slope of the
    equilibrium free energy between neighbouring box sizes."""
    grid, ds = (32, 8, 8), 0.02
    size = (3.8, 2.0, 2.0)
    w0 = lamellar_start(grid, size, rng)

    def converge(sz, start):
        with ctx(grid, sz, ds, **LAM) as c:
            c.set_field(start)
            res = c.scf_run(3000, tol=1e-26)
            wf = c.get_field().reshape(start.shape)
            F = c.forward(wf)
            g = c.backward()
            dens = c.get_density()
        return wf, F, g, res, dens

    wc, Fc, gc, res, dens = converge(size, w0)
    assert res.accuracy < 1e-18
    assert np.ptp(dens[: dens.size // 2]) > 0.5          # lamellae, not the disordered melt
    d = 2e-3
    _, Fp, _, _, _ = converge((size[0] + d,) + size[1:], wc)
    _, Fm, _, _, _ = converge((size[0] - d,) + size[1:], wc)
    slope = (Fp - Fm) / (2 * d)
    assert abs(slope) > 1e-2                              # a real stress at L = 3.8
    assert abs(gc[0] - slope) < 1e-5 * abs(slope), (gc[0], slope)


def test_unit_cell_relaxation_reaches_zero_stress(rng):
    """Lamellae along x: relax L_x from 3.6 with the adjoint stress to
    |dF/dL_x| < 1e-6; the converged free energy there is below its
    neighbours', and the lamellae persist."""
    from adscf_gb300.relax import relax_box
    grid, ds = (32, 8, 8), 0.02
    size = (3.6, 2.0, 2.0)
    w0 = lamellar_start(grid, size, rng)
    with ctx(grid, size, ds, **LAM) as c:
        L, F, g, hist = relax_box(c, w0, axes=(0,), tol=1e-6)
        dens = c.get_density()
    print("relaxation:", [(round(h[0][0], 6), h[1], h[2][0]) for h in hist])
    assert abs(g[0]) < 1e-6, hist
    assert len(hist) < 25
    assert 3.9 < L[0] < 4.4
    assert np.ptp(dens[: dens.size // 2]) > 0.5

    def converged_F(lx):
        with ctx(grid, (lx,) + size[1:], ds, **LAM) as c2:
            c2.set_field(lamellar_start(grid, (lx,) + size[1:], rng))
            c2.scf_run(3000, tol=1e-16)
            return c2.forward(c2.get_field())

    d = 0.01
    assert converged_F(L[0] - d) > F and converged_F(L[0] + d) > F


def test_batched_adjoint_matches_single_contexts(rng):
    """adscf_batch_forward / adscf_batch_backward over uneven instances equal
    each instance's single-context forward / backward."""
    from adscf_gb300 import Batch
    insts = [
        dict(grid=(32, 32, 32), size=(3.9, 4.1, 3.7), ds=0.04, block_length=(0.4, 0.6), chi=18.0),
        dict(grid=(24, 24, 24), size=(3.3, 3.3, 3.3), ds=0.05, block_length=(0.3, 0.7), chi=22.0),
        dict(grid=(16, 12, 10), size=(3.3, 3.1, 2.9), ds=0.02, block_length=(0.45, 0.55), chi=15.0),
        dict(grid=(40, 32, 24), size=(4.6, 3.9, 3.0), ds=0.025, block_length=(0.35, 0.65), chi=25.0),
    ]
    for kw in insts:
        kw.update(geometry=BULK, kappa=KAPPA, precision=FP64)
    fields = []
    for kw in insts:
        gx, gy, gz = kw["grid"]
        fields.append(0.5 * rng.standard_normal((2, gz, gy, gx)))
    with Batch(insts) as b:
        Fb = b.forward(fields)
        gb = b.backward()
    for kw, w, F, g in zip(insts, fields, Fb, gb):
        kw = dict(kw)
        kw.pop("geometry")
        with Context(BULK, **kw) as c:
            F1 = c.forward(w)
            g1 = c.backward()
        assert abs(F - F1) < 1e-12 * max(1.0, abs(F1))
        assert np.allclose(g, g1, rtol=1e-9, atol=1e-12), (g, g1)
