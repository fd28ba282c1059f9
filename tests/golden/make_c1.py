"""Generate tests/golden/c1_bulk_converged.json: the C1 bulk diblock melt
(32^3, L = 4.0, f_A = 0.30, chiN = 25, kappa = 25, ds = 0.01) converged by the
FP64 oracle (Anderson m = 10 after 20 lambda = 0.1 steps, Gram form) from
w_A/B = +-chiN (phi_A0 - f_A) + N(0, 0.1^2), phi_A0 = f_A + 0.1 cos(2 pi x/L),
seed 1.  Run from the repo root: python tests/golden/make_c1.py"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import scf as oscf  # noqa: E402

N, L, F_A, CHI, KAPPA, DS = 32, 4.0, 0.30, 25.0, 25.0, 0.01


def c1_field(seed=1):
    rng = np.random.default_rng(seed)
    x = np.arange(N) * L / N
    phi0 = F_A + 0.1 * np.broadcast_to(np.cos(2 * np.pi * x / L)[None, None, :], (N, N, N))
    w = np.empty((2, N, N, N))
    w[0] = CHI * (phi0 - F_A) + rng.normal(0.0, 0.1, (N, N, N))
    w[1] = -CHI * (phi0 - F_A) + rng.normal(0.0, 0.1, (N, N, N))
    return w


def main(max_iter=1500, tol=1e-16):
    w0 = c1_field()
    field, hist = oscf.bulk_scf(w0, max_iter, (N, N, N), (L, L, L), DS, (F_A, 1 - F_A), KAPPA, CHI,
                                mixing_type=3, lam=0.1, m=10, lam00=0.1, warm=20, gram=True,
                                stop_accuracy=tol)
    last = hist[-1]
    out = {
        "config": "C1: 32^3, L=4.0, f_A=0.30, chiN=25, kappa=25, ds=0.01, Anderson m=10 after 20 "
                  "lambda=0.1 steps; start w = +-chiN(phi_A0 - f_A) + N(0, 0.1^2), "
                  "phi_A0 = f_A + 0.1 cos(2 pi x / L), seed 1",
        "iterations": last["iter"], "accuracy": last["accuracy"], "free_energy": last["F"],
        "Qsum": last["Qsum"],
        "field_sub": field[:, ::4, ::4, ::4].ravel().tolist(),
    }
    (Path(__file__).parent / "c1_bulk_converged.json").write_text(json.dumps(out))
    print(out["iterations"], out["accuracy"], out["free_energy"])


if __name__ == "__main__":
    main()
