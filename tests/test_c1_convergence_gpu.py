"""C1, the reference's CPU-runnable case (32^3 FP64 bulk diblock melt run to
convergence), on the GPU against the oracle's converged state stored in
tests/golden/c1_bulk_converged.json (tests/golden/make_c1.py)."""
import json
from pathlib import Path

import numpy as np
import pytest

from adscf_gb300 import BULK, FP64, SPLIT, MIX_ANDERSON, Context

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).parent / "golden" / "c1_bulk_converged.json").read_text())


def c1_context(prec):
    import sys
    sys.path.insert(0, str(Path(__file__).parent / "golden"))
    from make_c1 import CHI, DS, F_A, KAPPA, L, N
    return Context(BULK, grid=(N, N, N), size=(L, L, L), ds=DS, block_length=(F_A, 1 - F_A),
                   kappa=KAPPA, chi=CHI, precision=prec, mixing_type=MIX_ANDERSON,
                   mixing_dim=10, lam=0.1, lam_warm=0.1, warm_iters=20)


def start_field():
    import sys
    sys.path.insert(0, str(Path(__file__).parent / "golden"))
    from make_c1 import c1_field
    return c1_field()


def test_c1_fp64_converges_to_the_oracle_saddle():
    with c1_context(FP64) as c:
        c.set_field(start_field())
        res = c.scf_run(2000, tol=1e-16)
        field = c.get_field().reshape(2, 32, 32, 32)
    assert res.accuracy <= 1e-16
    assert abs(res.iter - GOLD["iterations"]) <= 10
    assert abs(res.free_energy - GOLD["free_energy"]) < 1e-10 * abs(GOLD["free_energy"])
    # densities converge to accuracy 1e-16; the fields only to ~1e-5 relative
    # along directions the densities barely see
    sub = np.asarray(GOLD["field_sub"]).reshape(2, 8, 8, 8)
    assert np.max(np.abs(field[:, ::4, ::4, ::4] - sub)) < 1e-5 * np.max(np.abs(sub))


def test_c1_split_free_energy_at_the_saddle():
    """Split path (FP32 propagators, FP64 accumulation/mixing) converged on
    its own, then F evaluated once in FP64 at that field: |Delta F| per chain
    against the FP64 oracle's saddle.  The split path's own F carries the
    FP32 log Q error (~1.7e-7 here); the FP64 evaluation at the converged
    field is second order in the field error."""
    with c1_context(SPLIT) as c:
        c.set_field(start_field())
        res = c.scf_run(2000, tol=1e-8)   # the split path's accuracy floor is ~6e-9 here
        pol = c.free_energy_fp64()
    raw = abs(res.free_energy - GOLD["free_energy"])
    dF = abs(pol.free_energy - GOLD["free_energy"])
    print(f"C1 split: iterations {res.iter}, accuracy {res.accuracy:.2e}, "
          f"|dF| split {raw:.2e}, FP64 at the split field {dF:.2e}")
    assert res.accuracy <= 1e-8
    assert raw < 5e-7
    assert dF < 1e-8
