"""Failure detection without a GPU fault.

The reference stops on a non-finite accuracy (its convergence test is NaN
safe, Bulk_3D_FFT/Main_Diblock_Melt/main_diblock.f90:421,433) and on a zero
tridiagonal pivot (Film_CK_AD/Film_3D/Geometry_Modules/mod_realspace.f90:
194-207, tested in test_film_gpu.py).  Here the failures are made on the
host and the library must report them as status codes, with the context
still usable:

- a field with a NaN (bulk FP64 / split, films, batches) gives
  ADSCF_E_NONFINITE, and the next call with a finite field is correct;
- the pipeline wait of the TMA passes set to give up at once (0 polls: the
  wait runs out without depending on timing) gives ADSCF_E_TIMEOUT -- each
  kernel sets its flag, drains its copies in flight and returns -- and the
  same context with the default bound, and a fresh one, match the oracle.
"""
import numpy as np
import pytest

from oracle import bulk as ob
from oracle import film as of

pytestmark = pytest.mark.gpu

from adscf_gb300 import (BULK, FILM_1D, FILM_3D, FP64, SPLIT, AdscfError, Batch,
                         Context)
from adscf_gb300 import _lib as L


def bulk_ctx(grid, prec, **kw):
    return Context(BULK, grid=grid, size=(3.8, 3.8, 3.8), ds=0.02, block_length=(0.4, 0.6),
                   precision=prec, **kw)


def check_bulk(c, field, grid, tol):
    ref = ob.propagate_diblock(field, grid, (3.8, 3.8, 3.8), 0.02, (0.4, 0.6))
    dens, res = c.propagate_diblock(field)
    assert abs(res.logQ - np.log(ref["Qsum"])) < tol
    assert np.max(np.abs(dens - ob.density_by_type(ref["density"]))) < 50 * tol


@pytest.mark.parametrize("prec,tol", [(FP64, 1e-11), (SPLIT, 2e-6)])
def test_nan_field_bulk_reports_nonfinite(prec, tol, rng):
    grid = (16, 16, 16)
    w = rng.standard_normal((2, 16, 16, 16))
    bad = w.copy()
    bad[1, 3, 5, 7] = np.nan
    with bulk_ctx(grid, prec) as c:
        with pytest.raises(AdscfError) as e:
            c.propagate_diblock(bad)
        assert e.value.code == L.ADSCF_E_NONFINITE
        check_bulk(c, w, grid, tol)             # the context is still usable
        c.set_field(bad)
        with pytest.raises(AdscfError) as e:
            c.scf_run(1)
        assert e.value.code == L.ADSCF_E_NONFINITE


@pytest.mark.parametrize("geom", [FILM_1D, FILM_3D])
def test_nan_field_film_reports_nonfinite(geom, rng):
    gz = 24
    grid = (1, 1, gz) if geom == FILM_1D else (6, 4, gz)
    dz, zr = of.tanh_mesh(gz, 3.0)
    shape = (2, gz + 1, grid[1], grid[0])
    w = 0.3 * rng.standard_normal(shape)
    bad = w.copy()
    bad[0, gz // 2, 0, 0] = np.nan
    with Context(geom, grid=grid, size=(3.0, 2.0, 3.0), ds=0.02, block_length=(0.5, 0.5),
                 dz=dz, precision=SPLIT) as c:
        with pytest.raises(AdscfError) as e:
            c.propagate_diblock(bad)
        assert e.value.code == L.ADSCF_E_NONFINITE
        dens, res = c.propagate_diblock(w)
        assert np.isfinite(res.Qsum) and np.all(np.isfinite(dens))


def test_nan_field_batch_names_the_instance(rng):
    inst = [dict(geometry=BULK, grid=(g, g, g), size=(4.0, 4.0, 4.0), ds=0.02,
                 block_length=(0.4, 0.6), chi=15.0, kappa=25.0, precision=SPLIT)
            for g in (16, 24, 16)]
    fields = [0.2 * rng.standard_normal((2, g, g, g)) for g in (16, 24, 16)]
    fields[1][0, 1, 2, 3] = np.nan
    with Batch(inst) as b:
        b.set_fields(fields)
        with pytest.raises(AdscfError) as e:
            b.scf_run(1)
        assert e.value.code == L.ADSCF_E_NONFINITE
        assert "instance 1" in str(e.value)


def test_tma_wait_limit_expiry_reports_timeout(rng):
    """64^3 split context on the TMA Z pass and the fused XY pass (every
    pipeline wait of both is bounded by the context's limit)."""
    grid = (64, 64, 64)
    w = 0.5 * rng.standard_normal((2, 64, 64, 64))
    with bulk_ctx(grid, SPLIT) as c:
        c.set_pass_plan(2, 2, 3)
        c.set_wait_limit(0)
        with pytest.raises(AdscfError) as e:
            c.propagate_diblock(w)
        assert e.value.code == L.ADSCF_E_TIMEOUT
        c.set_wait_limit(-1)
        check_bulk(c, w, grid, 2e-6)
    with bulk_ctx(grid, SPLIT) as c:
        c.set_pass_plan(2, 2, 3)
        check_bulk(c, w, grid, 2e-6)
