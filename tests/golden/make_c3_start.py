"""Generate tests/golden/c3_start.json: the FP64 oracle at the C3 benchmark's
start field (bench.c3_fields(): 128^3, L = 3.8, f_A = 0.40, chiN = 20,
kappa = 25, ds = 0.005, Ns = 200, {211} pattern plus noise, seed 7 of the
benchmark): log Q, the free energy per chain at the iterate (Calculate_Energy,
as oracle/scf.py forms it), density sums and the densities at 256 seeded
sample points.  bench.py compares the split and FP64 GPU paths' first
iteration with it (no oracle code runs in the benchmark).  The oracle holds
every slice of both chains (about 6.7 GB of host memory) for about a minute.
Run from the repo root: python tests/golden/make_c3_start.py"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402
from oracle import bulk as ob  # noqa: E402
from oracle import interactions as oi  # noqa: E402

NSAMPLE = 256


def sample_indices(shape, n=NSAMPLE, seed=2026):
    rng = np.random.default_rng(seed)
    return [tuple(int(rng.integers(0, s)) for s in shape) for _ in range(n)]


def main():
    grid = (bench.GRID,) * 3
    size = (bench.L,) * 3
    w = bench.c3_fields()
    r = ob.propagate_diblock(w, grid, size, bench.DS, (bench.F_A, 1.0 - bench.F_A))
    dens = ob.density_by_type(r["density"])
    eint = oi.interaction_energy(dens, bench.KAPPA, bench.CHI, r["dvol"])
    F = (r["energy"] - r["dvol"] * np.sum(dens * w) + eint) / (r["rho"] * r["volume"])
    idx = sample_indices(dens.shape)
    out = {
        "workload": "C3 start field (bench.c3_fields), FP64 oracle, one propagation",
        "grid": bench.GRID, "L": bench.L, "ds": bench.DS, "f_A": bench.F_A, "chi": bench.CHI,
        "kappa": bench.KAPPA, "seed": bench.SEED,
        "logQ": float(np.log(r["Qsum"])), "F": float(F),
        "density_sum": [float(dens[0].sum()), float(dens[1].sum())],
        "sample_index": idx, "sample_density": [float(dens[i]) for i in idx],
    }
    path = ROOT / "tests" / "golden" / "c3_start.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {path}: logQ {out['logQ']:.15g}, F {out['F']:.15g}")


if __name__ == "__main__":
    main()
