"""Linear block sequences in the bulk (Propagate_Multiblock, mod_multiblock.f90;
Propagate_Triblock and the homopolymer as its 3- and 1-block cases) against
the oracle's restatement, on the generic, register, TMA and fused passes."""
import numpy as np
import pytest

from adscf_gb300 import BULK, FP64, SPLIT, AdscfError, Batch, Context
from oracle import bulk as ob
from oracle import interactions as oi

pytestmark = pytest.mark.gpu

SIX = ((0.5, 0.1, 0.1, 0.1, 0.1, 0.1), (0, 1, 0, 1, 0, 1))   # Main_Multiblock's chain
ABA = ((0.25, 0.5, 0.25), (0, 1, 0))
BAAB = ((0.2, 0.3, 0.1, 0.4), (1, 0, 0, 1))                   # adjacent blocks of one type
HOMO = ((1.0,), (0,))
ZERO = ((0.5, 0.0, 0.5), (0, 1, 0))                             # a zero-length block
SIXTEEN = (tuple([0.0625] * 16), tuple(k % 2 for k in range(16)))   # the maximum count
SEQS = [SIX, ABA, BAAB, HOMO, ZERO, SIXTEEN]


def mbctx(grid, size, ds, prec, seq, **kw):
    return Context(BULK, grid=grid, size=size, ds=ds, precision=prec, blocks=seq[0],
                   block_types=seq[1], **kw)


@pytest.mark.parametrize("seq", SEQS)
@pytest.mark.parametrize("grid", [(12, 10, 8), (32, 32, 32)])
@pytest.mark.parametrize("ensemble", [1, 2])
def test_block_sequence_fp64_matches_oracle(seq, grid, ensemble, rng):
    gx, gy, gz = grid
    size, ds = (4.0, 3.5, 4.5), 0.02
    field = 0.5 * rng.standard_normal((2, gz, gy, gx))
    ref = ob.propagate_multiblock(field, grid, size, ds, seq[0], seq[1], ensemble=ensemble,
                                  rho=0.9, mu=0.3)
    with mbctx(grid, size, ds, FP64, seq, ensemble=ensemble, rho=0.9, mu=0.3) as c:
        assert c.ns == ref["segments"]
        dens, res = c.propagate_diblock(field)
    rd = ref["density_type"]
    assert abs(res.Qsum / ref["Qsum"] - 1) < 1e-12
    assert np.max(np.abs(dens - rd)) < 1e-11 * np.max(np.abs(rd))
    assert abs(res.mu - ref["mu"]) < 1e-11
    assert abs(res.energy - ref["energy"]) < 1e-10 * abs(ref["energy"])


@pytest.mark.parametrize("prec", [FP64, SPLIT])
@pytest.mark.parametrize("grid", [(12, 10, 8), (32, 32, 32), (64, 64, 64)])
def test_two_block_sequence_is_the_diblock_bit_for_bit(prec, grid, rng):
    gx, gy, gz = grid
    size, ds = (3.8, 3.8, 3.8), 0.02
    field = 0.5 * rng.standard_normal((2, gz, gy, gx))
    with Context(BULK, grid=grid, size=size, ds=ds, precision=prec, block_length=(0.3, 0.7)) as c:
        d1, r1 = c.propagate_diblock(field)
    with mbctx(grid, size, ds, prec, ((0.3, 0.7), (0, 1))) as c:
        d2, r2 = c.propagate_diblock(field)
    assert r1.Qsum == r2.Qsum
    assert np.array_equal(d1, d2)


@pytest.mark.parametrize("seq", [SIX, ABA])
@pytest.mark.parametrize("grid", [(32, 32, 32), (64, 64, 64)])
def test_block_sequence_split_matches_oracle(seq, grid, rng):
    gx, gy, gz = grid
    size, ds = (3.8, 3.8, 3.8), 0.01
    field = 2.0 * rng.standard_normal((2, gz, gy, gx))
    ref = ob.propagate_multiblock(field, grid, size, ds, seq[0], seq[1])
    with mbctx(grid, size, ds, SPLIT, seq) as c:
        dens, res = c.propagate_diblock(field)
    assert abs(np.log(res.Qsum) - np.log(ref["Qsum"])) < 2e-6
    assert np.max(np.abs(dens - ref["density_type"])) < 1e-5


def test_block_sequence_every_pass_plan_identical(rng):
    """The TMA and fused passes choose each chain's Boltzmann factor per step
    from the block table, like the plain passes."""
    n = 64
    grid, size, ds = (n, n, n), (3.8, 3.8, 3.8), 0.02
    field = 0.5 * rng.standard_normal((2, n, n, n))
    ref, tried = None, 0
    with mbctx(grid, size, ds, SPLIT, SIX) as c:
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
                        assert r.Qsum == ref[1] and np.array_equal(d, ref[0]), (y, z, x)
    assert tried >= 4


def oracle_free_energy(w, grid, size, ds, seq, kappa, chi):
    """Calculate_Energy of Main_Multiblock (main_multiblock.f90:547-556)."""
    r = ob.propagate_multiblock(w, grid, size, ds, seq[0], seq[1])
    phi = r["density_type"]
    eint = oi.interaction_energy(phi, kappa, chi, r["dvol"])
    return (r["energy"] - r["dvol"] * np.sum(phi * w) + eint) / (r["rho"] * r["volume"])


def test_block_sequence_free_energy_and_adjoint(rng):
    """forward = the driver's energy per chain; backward's dF/dL and dF/dchi
    against central differences of the oracle."""
    grid, size, ds = (12, 10, 8), (3.3, 3.1, 2.9), 0.05
    kappa, chi = 10.0, 15.0
    w = 0.5 * rng.standard_normal((2, 8, 10, 12))
    with mbctx(grid, size, ds, FP64, ABA, kappa=kappa, chi=chi) as c:
        F = c.forward(w)
        g = c.backward()
    assert abs(F - oracle_free_energy(w, grid, size, ds, ABA, kappa, chi)) < 1e-12 * max(1.0, abs(F))
    d = 1e-5
    for i in range(3):
        sp, sm = list(size), list(size)
        sp[i] += d
        sm[i] -= d
        fd = (oracle_free_energy(w, grid, tuple(sp), ds, ABA, kappa, chi) -
              oracle_free_energy(w, grid, tuple(sm), ds, ABA, kappa, chi)) / (2 * d)
        assert abs(g[i] - fd) < 1e-6 * max(1e-2, abs(fd)), (i, g[i], fd)
    dc = 1e-4
    fd = (oracle_free_energy(w, grid, size, ds, ABA, kappa, chi + dc) -
          oracle_free_energy(w, grid, size, ds, ABA, kappa, chi - dc)) / (2 * dc)
    assert abs(g[3] - fd) < 1e-8 * max(1.0, abs(fd))


def test_block_sequence_scf_iterations_follow_the_oracle_density(rng):
    """Three SCF iterations of the six-block chain run on the device; the
    density of the final field equals the oracle's."""
    grid, size, ds = (16, 8, 8), (4.0, 2.0, 2.0), 0.02
    w = 0.5 * rng.standard_normal((2, 8, 8, 16))
    with mbctx(grid, size, ds, FP64, SIX, kappa=25.0, chi=20.0) as c:
        c.set_field(w)
        res = c.scf_run(3, tol=0.0)
        wf = c.get_field().reshape(w.shape)
        dens, _r = c.propagate_diblock(wf)
    assert res.iter == 3 and np.isfinite(res.free_energy)
    ref = ob.propagate_multiblock(wf, grid, size, ds, SIX[0], SIX[1])
    assert np.max(np.abs(dens - ref["density_type"])) < 1e-11 * np.max(ref["density_type"])


def test_block_sequence_argument_errors():
    with pytest.raises(AdscfError):
        Context(BULK, grid=(8, 8, 8), blocks=(0.5, 0.5), block_types=(0, 2))
    with pytest.raises(AdscfError):
        Context(BULK, grid=(8, 8, 8), blocks=(0.1,) * 17, block_types=(0,) * 17)
    with pytest.raises(AdscfError):
        Batch([dict(grid=(8, 8, 8), blocks=(0.5, 0.5), block_types=(0, 1))])
