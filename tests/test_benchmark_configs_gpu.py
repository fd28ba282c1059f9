"""Parity at the benchmark's own configurations, through the C ABI, against
the FP64 oracle (oracle/bulk.py, oracle/film.py):

- C3: bulk diblock 128^3, Ns = 200 (ds = 0.005), f_A = 0.40, chi N = 20,
  L = 3.8, {211} fields plus noise (bench.c3_fields).  FP64 path: |dlogQ| <=
  1e-11 and max|dphi| <= 1e-10; split path: |dlogQ| <= 1e-6, max|dphi| <=
  1e-5 (FP32 propagators).  At a field 800 split iterations toward the
  saddle, the FP64 evaluation of F (adscf_free_energy_fp64) within 1e-10 of
  the oracle's F and the split path's own F within 2e-7 per chain.
- C4: Film_3D ADI film, 64 x 64 lateral, 64-interval tanh mesh, Ns = 150
  end-refined (bench.c4_film3d): FP64 relative 1e-10, split 1e-5.
- C2: the 4096-film batch (bench.c2_films), one iteration; the films with
  the most planes and the most contour steps and two others against the
  oracle at their start fields: split relative 1e-5.

The oracle at C3 holds every slice of both chains (about 6.7 GB of host
memory) and takes about a minute per propagation.
"""
import numpy as np
import pytest

import bench
from oracle import bulk as ob
from oracle import film as of
from oracle import interactions as oi

pytestmark = pytest.mark.gpu

from adscf_gb300 import (BULK, FILM_1D, FILM_3D, FP64, SPLIT, Batch, Context,
                         MIX_ANDERSON)

GRID = (bench.GRID,) * 3
SIZE = (bench.L,) * 3


def c3_context(prec):
    return Context(BULK, grid=GRID, size=SIZE, ds=bench.DS,
                   block_length=(bench.F_A, 1.0 - bench.F_A), ensemble=1, rho=1.0,
                   kappa=bench.KAPPA, chi=bench.CHI, precision=prec, mixing_type=MIX_ANDERSON,
                   mixing_dim=bench.M_HIST, lam=bench.LAM, lam_warm=bench.LAM,
                   warm_iters=bench.M_HIST)


def oracle_c3(field):
    """Densities by type, log Q and the free energy per chain of the oracle at
    `field` (Calculate_Energy at the iterate, oracle/scf.py)."""
    r = ob.propagate_diblock(field, GRID, SIZE, bench.DS, (bench.F_A, 1.0 - bench.F_A))
    dens = ob.density_by_type(r["density"])
    eint = oi.interaction_energy(dens, bench.KAPPA, bench.CHI, r["dvol"])
    F = (r["energy"] - r["dvol"] * np.sum(dens * field) + eint) / (r["rho"] * r["volume"])
    out = {"density": dens, "logQ": float(np.log(r["Qsum"])), "F": float(F)}
    del r
    return out


@pytest.fixture(scope="module")
def c3_start():
    w = bench.c3_fields()
    return w, oracle_c3(w)


@pytest.mark.parametrize("prec,tq,tphi", [(FP64, 1e-11, 1e-10), (SPLIT, 1e-6, 1e-5)])
def test_c3_propagate_diblock_vs_oracle(c3_start, prec, tq, tphi):
    w, ref = c3_start
    with c3_context(prec) as c:
        dens, res = c.propagate_diblock(w)
    dq = abs(res.logQ - ref["logQ"])
    dphi = float(np.max(np.abs(dens - ref["density"])))
    print(f"C3 precision={prec}: |dlogQ| {dq:.2e}, max|dphi| {dphi:.2e}")
    assert dq <= tq
    assert dphi <= tphi


def test_c3_split_saddle_free_energy_vs_oracle():
    """800 split iterations from the C3 start field, then F at the field
    reached: FP64 evaluation on the GPU against the oracle (FP64 parity at
    128^3), and the split path's own F (FP32 log Q error) against it."""
    w = bench.c3_fields()
    with c3_context(SPLIT) as c:
        c.set_field(w)
        run = c.scf_run(800, tol=1e-12)
        ws = c.get_field().reshape(w.shape)
        pol = c.free_energy_fp64()
        _x, _d, own = c.scf_iteration(ws.reshape(-1).copy())
    ref = oracle_c3(ws)
    d64 = abs(pol.free_energy - ref["F"])
    dsplit = abs(own.free_energy - ref["F"])
    print(f"C3 after {run.iter} split iterations (accuracy {run.accuracy:.2e}): "
          f"|dF| FP64 evaluation {d64:.2e}, split {dsplit:.2e} per chain")
    assert np.isfinite(run.accuracy)
    assert d64 <= 1e-10 * max(1.0, abs(ref["F"]))
    assert dsplit <= 2e-7


@pytest.mark.parametrize("prec,tol", [(FP64, 1e-10), (SPLIT, 1e-5)])
def test_c4_film3d_propagate_diblock_vs_oracle(prec, tol):
    import adscf_gb300 as A
    kw, w = bench.c4_film3d(A)
    kw = dict(kw, precision=prec)
    gx, gy, gz = kw["grid"]
    size = kw["size"]
    dz = kw["dz"]
    step = lambda p, f, h: of.adi_step_3d(p, f, dz, size[0] / gx, size[1] / gy, h)
    ref = of.film_propagate_diblock(w, dz, kw["dss"], kw["n_a"], step, rho=1.0,
                                    dx=size[0] / gx, dy=size[1] / gy, int_scheme=kw["int_scheme"],
                                    span="full", sizes=size, ensemble=kw["ensemble"], mu=kw["mu"])
    with Context(FILM_3D, **kw) as c:
        dens, res = c.propagate_diblock(w)
    dq = abs(np.log(res.Qsum) - np.log(ref["Qsum"]))
    rel = float(np.max(np.abs(dens - ref["density"])) / np.max(np.abs(ref["density"])))
    print(f"C4 precision={prec}: |dlogQ| {dq:.2e}, max|dphi|/max phi {rel:.2e}")
    assert dq <= tol
    assert rel <= tol


def test_c2_film_batch_vs_oracle():
    import adscf_gb300 as A
    inst, fields = bench.c2_films(A)
    with Batch(inst) as b:
        b.set_fields(fields)
        res = b.scf_run(1)
        dens = b.get_densities()
    nz = [k["grid"][2] for k in inst]
    ns = [len(k["dss"]) - 1 for k in inst]
    pick = sorted({int(np.argmax(nz)), int(np.argmax(ns)), 1, 2049})
    for i in pick:
        k = inst[i]
        dz = k["dz"]
        step = lambda p, f, h, dz=dz: of.cn_step_1d(p, f, dz, h)
        w = fields[i].reshape(2, -1)
        ref = of.film_propagate_diblock(w, dz, k["dss"], k["n_a"], step, rho=1.0,
                                        int_scheme=k["int_scheme"], span="interior",
                                        sizes=k["size"], ensemble=k["ensemble"], mu=k["mu"])
        got = np.asarray(dens[i]).reshape(2, -1)
        dq = abs(res[i].logQ - np.log(ref["Qsum"]))
        rel = float(np.max(np.abs(got - ref["density"])) / np.max(np.abs(ref["density"])))
        print(f"C2 film {i} (nz {nz[i]}, Ns {ns[i]}): |dlogQ| {dq:.2e}, rel dphi {rel:.2e}")
        assert dq <= 1e-5, i
        assert rel <= 1e-5, i
