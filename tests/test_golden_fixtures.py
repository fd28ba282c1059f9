"""The committed oracle fixtures match the configurations they stand for
(CPU only): the C3 start-field fixture that bench.py compares its first
iteration with, and its sample points lie inside the grid."""
import json
from pathlib import Path

import bench

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_c3_start_fixture_matches_the_benchmark_config():
    fx = json.loads((GOLDEN / "c3_start.json").read_text())
    assert (fx["grid"], fx["L"], fx["ds"], fx["f_A"], fx["chi"], fx["kappa"], fx["seed"]) == \
        (bench.GRID, bench.L, bench.DS, bench.F_A, bench.CHI, bench.KAPPA, bench.SEED)
    assert len(fx["sample_index"]) == len(fx["sample_density"]) == 256
    for c, z, y, x in fx["sample_index"]:
        assert 0 <= c < 2 and all(0 <= v < bench.GRID for v in (z, y, x))
    # canonical closure: the densities integrate to rho V split by block length
    n = bench.GRID ** 3
    tot = sum(fx["density_sum"]) / n
    assert abs(tot - 1.0) < 1e-10
    assert abs(fx["density_sum"][0] / n - bench.F_A) < 1e-10
