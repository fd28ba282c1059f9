"""Bulk pseudo-spectral path on the GPU, through the C ABI, against the
FP64 oracle (oracle/bulk.py restating Bulk_3D_FFT/...).

Tolerances: FP64 path relative 1e-11 (FFT rounding); split path (FP32
propagators) relative 2e-5 on single steps and densities, |d log Q| 2e-6."""
import numpy as np
import pytest

from oracle import bulk as ob
from oracle import interactions as oi
from oracle import iterate as oit
from oracle import scf as oscf

pytestmark = pytest.mark.gpu

from adscf_gb300 import BULK, FP64, SPLIT, MIX_SIMPLE, MIX_LAMBDA, MIX_ANDERSON
from adscf_gb300 import Context


def mkctx(grid, size=(4.0, 3.5, 4.5), ds=0.01, prec=FP64, f=(0.3, 0.7), **kw):
    return Context(BULK, grid=grid, size=size, ds=ds, block_length=f, precision=prec, **kw)


# generic mixed-radix lines (8, 12, 10, 20, 24, 40, 48, 6) and the register
# kernels (32, 64, 128, 256-point lines, power-of-two gx)
GRIDS = [(8, 8, 8), (12, 10, 20), (24, 1, 40), (16, 32, 8), (40, 48, 6),
         (32, 32, 32), (64, 32, 128), (128, 16, 64), (32, 256, 16), (24, 64, 32)]


@pytest.mark.parametrize("grid", GRIDS)
@pytest.mark.parametrize("prec", [FP64, SPLIT])
def test_propagate_step(grid, prec, rng):
    gx, gy, gz = grid
    size = (4.0, 3.5, 4.5)
    ds = 0.01
    q = 1.0 + 0.3 * rng.standard_normal((gz, gy, gx))
    w = rng.standard_normal((gz, gy, gx))
    e = ob.calculate_expfield(w, ds)
    ref = ob.propagate_step(q, e, ob.calculate_laplace(grid, size, ds))
    with mkctx(grid, size, ds, prec) as c:
        out = c.propagate_step(q, e)
    tol = 1e-12 if prec == FP64 else 2e-6
    assert np.max(np.abs(out - ref)) <= tol * np.max(np.abs(ref))


@pytest.mark.parametrize("grid", [(8, 8, 8), (12, 10, 20), (16, 1, 6), (64, 32, 128)])
def test_real2fourier_fourier2real(grid, rng):
    gx, gy, gz = grid
    q = rng.standard_normal((gz, gy, gx))
    with mkctx(grid) as c:
        spec = c.real2fourier(q)
        ref = ob.real2fourier(q)
        assert np.max(np.abs(spec - ref)) <= 1e-14 * np.max(np.abs(ref)) * 10
        back = c.fourier2real(ref)
    assert np.max(np.abs(back - q)) <= 1e-12


def test_single_mode_decay():
    """w = 0: a single Fourier mode decays by exp(-k^2 ds) per step."""
    grid, size, ds = (16, 16, 16), (4.0, 4.0, 4.0), 0.02
    z = np.arange(16) * size[2] / 16
    q = np.cos(2 * np.pi * 2 * z / size[2])[:, None, None] * np.ones((16, 16, 16))
    with mkctx(grid, size, ds) as c:
        out = c.propagate_step(q, np.ones_like(q))
    k2 = (2 * np.pi * 2 / size[2]) ** 2
    assert np.allclose(out, q * np.exp(-k2 * ds), atol=1e-13)


@pytest.mark.parametrize("prec", [FP64, SPLIT])
@pytest.mark.parametrize("grid", [(16, 8, 12), (256, 256, 256)])
def test_constant_field_known_answer(prec, grid):
    """w = const: q(s) = exp(-w s), Q = V exp(-w), phi_A = rho f_A; also at
    the largest register line length (256^3, 20 contour steps)."""
    size, ds = (3.0, 2.0, 2.5), (0.02 if grid[0] == 16 else 0.05)
    w0 = 0.7
    gx, gy, gz = grid
    field = np.full((2, gz, gy, gx), w0)
    with mkctx(grid, size, ds, prec, f=(0.3, 0.7)) as c:
        dens, res = c.propagate_diblock(field)
    V = 15.0
    # FP32 storage of a constant field rounds every point the same way, so the
    # split tolerance is a few ulp per step accumulated over the contour
    assert abs(res.Qsum / (V * np.exp(-w0)) - 1) < (1e-13 if prec == FP64 else 2e-6)
    assert np.allclose(dens[0], 0.3, rtol=1e-6)
    assert np.allclose(dens[1], 0.7, rtol=1e-6)


@pytest.mark.parametrize("grid,f", [((8, 8, 8), (0.3, 0.7)), ((12, 10, 20), (0.45, 0.55)),
                                     ((24, 1, 40), (0.5, 0.5)), ((32, 32, 32), (0.4, 0.6))])
@pytest.mark.parametrize("ensemble", [1, 2])
def test_propagate_diblock_fp64(grid, f, ensemble, rng):
    gx, gy, gz = grid
    size, ds = (4.0, 3.5, 4.5), 0.02
    field = 0.5 * rng.standard_normal((2, gz, gy, gx))
    ref = ob.propagate_diblock(field, grid, size, ds, f, ensemble=ensemble, rho=1.0, mu=0.3)
    with mkctx(grid, size, ds, FP64, f=f, ensemble=ensemble, rho=1.0, mu=0.3) as c:
        dens, res = c.propagate_diblock(field)
    rd = ob.density_by_type(ref["density"])
    assert abs(res.Qsum / ref["Qsum"] - 1) < 1e-12
    assert np.max(np.abs(dens - rd)) < 1e-11 * np.max(np.abs(rd))
    assert abs(res.mu - ref["mu"]) < 1e-11
    assert abs(res.energy - ref["energy"]) < 1e-10 * abs(ref["energy"])


@pytest.mark.parametrize("grid", [(16, 16, 16), (12, 10, 20), (32, 32, 32), (64, 64, 32)])
def test_propagate_diblock_split(grid, rng):
    gx, gy, gz = grid
    size, ds = (3.8, 3.8, 3.8), 0.01
    field = 2.0 * rng.standard_normal((2, gz, gy, gx))
    ref = ob.propagate_diblock(field, grid, size, ds, (0.4, 0.6))
    with mkctx(grid, size, ds, SPLIT, f=(0.4, 0.6)) as c:
        dens, res = c.propagate_diblock(field)
    rd = ob.density_by_type(ref["density"])
    assert abs(np.log(res.Qsum) - np.log(ref["Qsum"])) < 2e-6
    assert np.max(np.abs(dens - rd)) < 1e-5


def test_mean_fields_and_energy(rng):
    grid = (8, 6, 10)
    dens = rng.random((2, 10, 6, 8))
    with mkctx(grid, kappa=25.0, chi=17.0, monomer_volume=(1.0, 1.3)) as c:
        w = c.mean_fields(dens)
        e = c.interaction_energy(dens)
        dvol = (4.0 * 3.5 * 4.5) / (8 * 6 * 10)
    assert np.allclose(w, oi.mean_fields(dens, 25.0, 17.0, (1.0, 1.3)), rtol=1e-14, atol=1e-13)
    assert abs(e - oi.interaction_energy(dens, 25.0, 17.0, dvol, (1.0, 1.3))) < 1e-11 * abs(e)


@pytest.mark.parametrize("mtype,m,warm", [(MIX_SIMPLE, 2, None), (MIX_LAMBDA, 2, None),
                                          (MIX_ANDERSON, 2, None), (MIX_ANDERSON, 10, 20),
                                          (MIX_ANDERSON, 4, 6)])
def test_mixing_matches_oracle(mtype, m, warm, rng):
    grid = (8, 4, 6)
    nv = 2 * 8 * 4 * 6
    lam = 0.1
    with mkctx(grid, mixing_type=mtype, mixing_dim=m, lam=lam, lam_warm=1e-3,
               warm_iters=warm or 0) as c:
        ref = oit.Mixer(nv, mtype, lam, m=m, lam00=1e-3, warm=warm)
        x = rng.standard_normal(nv)
        for it in range(1, 30):
            # a contracting residual so Anderson sees a sensible system
            r = -0.3 * x + 0.05 * rng.standard_normal(nv) / it
            xg = c.mix(x, r, it)
            xr = ref(x, r, it)
            assert np.max(np.abs(xg - xr)) <= 1e-9 * (1 + np.max(np.abs(xr))), it
            x = xr


@pytest.mark.parametrize("mtype,m,warm", [(MIX_LAMBDA, 2, None), (MIX_ANDERSON, 3, 5)])
def test_scf_run_matches_oracle(mtype, m, warm, rng):
    """Whole device SCF loop vs the oracle loop.  The warm-up step is 0.05:
    with the reference's 1e-3 the residuals entering the first Anderson step
    are nearly equal, U is nearly singular and even the oracle's two algebraic
    forms of the same system (direct and Gram) disagree at 1e-3 in F."""
    grid, size, ds = (12, 12, 12), (3.8, 3.8, 3.8), 0.02
    f = (0.4, 0.6)
    kappa, chi = 25.0, 15.0
    z = np.arange(12) * size[2] / 12
    lam_shape = np.cos(2 * np.pi * z / size[2])[:, None, None] * np.ones((12, 12, 12))
    field = np.stack([3.0 * lam_shape, -3.0 * lam_shape]) + 0.1 * rng.standard_normal((2, 12, 12, 12))
    n = 10
    # the device forms the Anderson system from the residual Gram matrix; the
    # oracle's Gram form is the tight reference, the reference's direct form
    # (ill-conditioned U amplifies rounding) the loose one
    xr, hist = oscf.bulk_scf(field, n, grid, size, ds, f, kappa, chi, mixing_type=mtype,
                             lam=0.1, m=m, lam00=0.05, warm=warm, gram=True)
    xd, hd = oscf.bulk_scf(field, n, grid, size, ds, f, kappa, chi, mixing_type=mtype,
                           lam=0.1, m=m, lam00=0.05, warm=warm, gram=False)
    with mkctx(grid, size, ds, FP64, f=f, kappa=kappa, chi=chi, mixing_type=mtype,
               mixing_dim=m, lam=0.1, lam_warm=0.05, warm_iters=warm or 0) as c:
        c.set_field(field)
        res = c.scf_run(n)
        xg = c.get_field()
        dg = c.get_density()
    assert res.iter == n
    assert abs(res.free_energy - hist[-1]["F"]) < 1e-9 * abs(hist[-1]["F"]) + 1e-12
    assert abs(res.accuracy - hist[-1]["accuracy"]) <= 1e-8 * hist[-1]["accuracy"] + 1e-20
    assert np.max(np.abs(dg - hist[-1]["density"].reshape(-1))) < 1e-9
    assert np.max(np.abs(xg - xr.reshape(-1))) < 1e-8 * (1 + np.max(np.abs(xr)))
    assert abs(res.free_energy - hd[-1]["F"]) < 1e-9 * abs(hd[-1]["F"])


def test_scf_iteration_host_buffers(rng):
    """adscf_scf_iteration (one loop body with host buffers) = scf_run(1)."""
    grid = (8, 8, 8)
    field = rng.standard_normal((2, 8, 8, 8))
    with mkctx(grid, mixing_type=MIX_ANDERSON, mixing_dim=2) as c:
        c.set_field(field)
        c.scf_run(1)
        x1 = c.get_field()
        d1 = c.get_density()
    with mkctx(grid, mixing_type=MIX_ANDERSON, mixing_dim=2) as c:
        c.set_field(field)
        x2, d2, res = c.scf_iteration(field.reshape(-1))
    assert res.iter == 1
    assert np.array_equal(x1, x2) and np.array_equal(d1, d2)
    # page-locked buffers advanced in place (DMA without staging)
    import torch
    xp = torch.empty(field.size, dtype=torch.float64, pin_memory=True).numpy()
    dp = torch.empty(field.size, dtype=torch.float64, pin_memory=True).numpy()
    xp[:] = field.reshape(-1)
    with mkctx(grid, mixing_type=MIX_ANDERSON, mixing_dim=2) as c:
        c.set_field(field)
        x3, d3, _r = c.scf_iteration(xp, dp, inplace=True)
        x4, d4, _r = c.scf_iteration(x2.copy())       # the pageable path continues the same loop
    assert x3 is xp and np.array_equal(xp, x2) and np.array_equal(dp, d2)
    with mkctx(grid, mixing_type=MIX_ANDERSON, mixing_dim=2) as c:
        c.set_field(field)
        c.scf_run(2)
        assert np.array_equal(c.get_field(), x4) and np.array_equal(c.get_density(), d4)


@pytest.mark.parametrize("ensemble", [1, 2])
def test_update_solvent_vs_oracle(ensemble, rng):
    """Update_Solvent (mod_solvent.f90:85-110) on the GPU against the FP64
    oracle, both ensembles (relative 1e-13: exp and the sums in FP64)."""
    grid, size = (24, 20, 16), (4.0, 3.5, 4.5)
    w = 0.5 * rng.standard_normal((grid[2], grid[1], grid[0]))
    ref = ob.update_solvent(w, grid, size, ensemble, rho=0.9, mu=0.4)
    with mkctx(grid, size) as c:
        out = c.update_solvent(w, ensemble, rho=0.9, mu=0.4)
        again = c.update_solvent(w, ensemble, rho=0.9, mu=0.4)
    for k in ("Qsum", "mu", "rho", "energy"):
        assert abs(out[k] - ref[k]) <= 1e-13 * max(1.0, abs(ref[k])), k
        assert out[k] == again[k], k
    for k in ("distribution", "density"):
        assert np.max(np.abs(out[k] - ref[k])) <= 1e-13 * np.max(np.abs(ref[k])), k


def test_bad_arguments_return_status():
    from adscf_gb300 import AdscfError
    with pytest.raises(AdscfError):
        Context(BULK, grid=(7, 8, 8))     # 7 is not a product of 2, 3, 5
    with pytest.raises(AdscfError):
        Context(BULK, grid=(8, 8, 8), mixing_type=3, mixing_dim=40)


@pytest.mark.parametrize("n", [64, 128])
def test_tma_passes_match_register_passes(n, rng, monkeypatch):
    """The TMA-fed Y/Z passes move data differently but compute the same
    arithmetic as the register passes: results must be bitwise identical."""
    grid, size, ds = (n, n, n), (3.8, 3.8, 3.8), 0.05
    field = 0.5 * rng.standard_normal((2, n, n, n))
    monkeypatch.delenv("ADSCF_NO_TMA", raising=False)
    with mkctx(grid, size, ds, SPLIT, f=(0.4, 0.6)) as c:
        d1, r1 = c.propagate_diblock(field)
    monkeypatch.setenv("ADSCF_NO_TMA", "1")
    with mkctx(grid, size, ds, SPLIT, f=(0.4, 0.6)) as c:
        d2, r2 = c.propagate_diblock(field)
    assert r1.Qsum == r2.Qsum
    assert np.array_equal(d1, d2)


def test_split_64cube_against_oracle(rng):
    grid, size, ds = (64, 64, 64), (3.8, 3.8, 3.8), 0.05
    field = 2.0 * rng.standard_normal((2, 64, 64, 64))
    ref = ob.propagate_diblock(field, grid, size, ds, (0.4, 0.6))
    with mkctx(grid, size, ds, SPLIT, f=(0.4, 0.6)) as c:
        dens, res = c.propagate_diblock(field)
    assert abs(np.log(res.Qsum) - np.log(ref["Qsum"])) < 1e-6
    assert np.max(np.abs(dens - ob.density_by_type(ref["density"]))) < 1e-5


@pytest.mark.parametrize("n,prec", [(64, SPLIT), (128, SPLIT), (64, FP64), (32, FP64)])
def test_every_pass_plan_gives_identical_results(n, prec, rng):
    """The autotuner may pick any available kernel per pass (plain,
    persistent, TMA); all compute the same arithmetic, bit for bit."""
    from adscf_gb300 import AdscfError
    grid, size, ds = (n, n, n), (3.8, 3.8, 3.8), 0.05
    field = 0.5 * rng.standard_normal((2, n, n, n))
    ref = None
    tried = 0
    with mkctx(grid, size, ds, prec, f=(0.4, 0.6)) as c:
        assert "plan" in c.tuning()
        for y in (0, 1, 2):
            for z in (0, 1, 2):
                for x in (0, 1, 3):
                    try:
                        c.set_pass_plan(y, z, x)
                    except AdscfError:
                        continue
                    d, r = c.propagate_diblock(field)
                    tried += 1
                    if ref is None:
                        ref = (d, r.Qsum)
                    else:
                        assert r.Qsum == ref[1], (y, z, x)
                        assert np.array_equal(d, ref[0]), (y, z, x)
    assert tried >= 4
