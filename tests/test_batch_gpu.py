"""Batches of independent bulk instances (adscf_batch_*): every instance must
follow its own single-context SCF trajectory, match the oracle, and the
split-precision batch must track the FP64 batch."""
import numpy as np
import pytest

from adscf_gb300 import BULK, FP64, SPLIT, MIX_ANDERSON, MIX_LAMBDA, Batch, Context
from oracle import bulk as ob, interactions as oi

pytestmark = pytest.mark.gpu

# uneven grids, contour steps, compositions, chi and boxes
INSTANCES = [
    dict(grid=(24, 24, 24), size=(3.2, 3.2, 3.2), ds=0.01, block_length=(0.30, 0.70), chi=25.0),
    dict(grid=(32, 32, 32), size=(4.1, 4.1, 4.1), ds=1 / 150, block_length=(0.40, 0.60), chi=18.0),
    dict(grid=(40, 32, 24), size=(4.6, 3.9, 3.0), ds=0.005, block_length=(0.45, 0.55), chi=16.0),
    dict(grid=(48, 48, 48), size=(4.8, 4.8, 4.8), ds=1 / 120, block_length=(0.35, 0.65), chi=22.0),
    dict(grid=(16, 12, 10), size=(3.0, 2.8, 2.5), ds=0.02, block_length=(0.25, 0.75), chi=30.0),
]


def with_common(inst, prec, mixing=MIX_LAMBDA):
    kw = dict(inst, geometry=BULK, kappa=20.0, precision=prec, mixing_type=mixing,
              mixing_dim=4, lam=0.1, lam_warm=0.1, warm_iters=4)
    return kw


def start_fields(rng):
    out = []
    for inst in INSTANCES:
        gx, gy, gz = inst["grid"]
        lx = inst["size"][0]
        x = np.arange(gx) * lx / gx
        s = np.broadcast_to(np.cos(2 * np.pi * x / lx)[None, None, :], (gz, gy, gx))
        w = np.stack([1.5 * s, -1.5 * s]) + 0.1 * rng.standard_normal((2, gz, gy, gx))
        out.append(w)
    return out


@pytest.mark.parametrize("mixing", [MIX_LAMBDA, MIX_ANDERSON])
def test_batch_follows_single_contexts(rng, mixing):
    w = start_fields(rng)
    singles = [Context(**with_common(inst, FP64, mixing)) for inst in INSTANCES]
    for c, wi in zip(singles, w):
        c.set_field(wi)
    with Batch([with_common(inst, FP64, mixing) for inst in INSTANCES]) as b:
        b.set_fields(w)
        for it in range(8):
            rb = b.scf_run(1)
            for i, c in enumerate(singles):
                rs = c.scf_run(1)
                assert rb[i].iter == rs.iter == it + 1
                # the batch sums Q over a different block partition (rounding
                # order); Anderson's small least-squares solve amplifies that
                # 1e-16 difference, so its trajectory is compared more loosely
                rtol = 1e-10 if mixing == MIX_LAMBDA else 1e-5
                assert abs(rb[i].free_energy - rs.free_energy) < rtol * max(1.0, abs(rs.free_energy)), (it, i)
                assert abs(rb[i].accuracy - rs.accuracy) <= rtol * 100 * rs.accuracy + 1e-20, (it, i)
        fb = b.get_fields()
        db = b.get_densities()
    tol = 1e-9 if mixing == MIX_LAMBDA else 1e-5
    for i, c in enumerate(singles):
        assert np.max(np.abs(fb[i].ravel() - c.get_field())) < tol
        assert np.max(np.abs(db[i].ravel() - c.get_density())) < tol
        c.close()


def test_batch_instance_matches_oracle(rng):
    w = start_fields(rng)
    with Batch([with_common(inst, FP64) for inst in INSTANCES]) as b:
        b.set_fields(w)
        res = b.scf_run(1)
        dens = b.get_densities()
    for i in (0, 2, 4):
        inst = INSTANCES[i]
        r = ob.propagate_diblock(w[i], inst["grid"], inst["size"], inst["ds"], inst["block_length"])
        phi = ob.density_by_type(r["density"])
        eint = oi.interaction_energy(phi, 20.0, inst["chi"], r["dvol"])
        F = (r["energy"] - r["dvol"] * np.sum(phi * w[i]) + eint) / (r["rho"] * r["volume"])
        assert abs(res[i].free_energy - F) < 1e-11 * max(1.0, abs(F))
        assert np.max(np.abs(dens[i] - phi)) < 1e-11


def test_split_batch_tracks_fp64_batch(rng):
    """Away from a saddle point F is first-order in the density error (FP32
    propagators and FFTs); log Q and the densities are the precision gauge.
    The per-instance numbers equal those of single split contexts."""
    w = start_fields(rng)
    out = {}
    for prec in (FP64, SPLIT):
        with Batch([with_common(inst, prec) for inst in INSTANCES]) as b:
            b.set_fields(w)
            out[prec] = (b.scf_run(1), b.get_densities())
    for i in range(len(INSTANCES)):
        rs, rd = out[SPLIT][0][i], out[FP64][0][i]
        assert abs(rs.logQ - rd.logQ) < 5e-7
        assert abs(rs.free_energy - rd.free_energy) < 5e-6
        assert np.max(np.abs(out[SPLIT][1][i] - out[FP64][1][i])) < 1e-5


def test_batch_converges_every_instance(rng):
    w = start_fields(rng)
    with Batch([dict(with_common(inst, FP64, MIX_ANDERSON), mixing_dim=10, warm_iters=10)
                for inst in INSTANCES]) as b:
        b.set_fields(w)
        res = b.scf_run(3000, tol=1e-8)
    assert all(r.accuracy <= 1e-8 for r in res)
    assert all(r.status == 0 for r in res)
    assert res[0].iter < 3000              # stopped once every instance was converged


@pytest.mark.parametrize("prec", [SPLIT, FP64])
def test_persistent_sweep_matches_launch_per_pass(rng, prec, monkeypatch):
    """The persistent sweep (every pass of every instance in one launch) runs
    the same tile functions as the launch-per-pass schedule, so three SCF
    iterations give the same bits; it takes at most a handful of launches."""
    w = start_fields(rng)
    insts = [with_common(inst, prec, MIX_ANDERSON) for inst in INSTANCES]
    out = {}
    for sweep in ("1", "0"):
        monkeypatch.setenv("ADSCF_BATCH_SWEEP", sweep)
        with Batch(insts) as b:
            b.set_fields(w)
            res = b.scf_run(3)
            out[sweep] = (b.get_fields(), [r.free_energy for r in res], b.lib.adscf_batch_launches(b.h))
    f1, F1, l1 = out["1"]
    f0, F0, l0 = out["0"]
    assert l1 <= 10 < l0
    assert F1 == F0
    for a, c in zip(f1, f0):
        assert np.array_equal(a, c)
