"""The C++17/OpenMP FP64 restatement (oracle/scf_cpu.cpp, the timed CPU
baseline) against numpy.fft and the numpy oracle, on the CPU.

- its FFT against numpy.fft.fftn (power-of-two and 2/3/5 lengths), 1e-13;
- Propagate_Diblock against oracle.bulk.propagate_diblock, 1e-12;
- whole SCF iterations (Anderson m = 3 after a 3-step warm-up) against
  oracle.scf.bulk_scf: accuracy, free energy and the mixed field, 1e-10.
"""
import numpy as np
import pytest

from oracle import bulk as ob
from oracle import cbuild
from oracle import scf as oscf


@pytest.fixture(scope="module")
def lib():
    try:
        return cbuild.load()
    except RuntimeError as e:
        pytest.skip(str(e))


@pytest.mark.parametrize("shape", [(8, 8, 8), (4, 6, 10), (12, 15, 16), (3, 5, 2), (32, 32, 32)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft_matches_numpy(lib, shape, sign, rng):
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    got = cbuild.fft3d(a, sign)
    want = np.fft.fftn(a) if sign < 0 else np.fft.ifftn(a) * a.size
    assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))


@pytest.mark.parametrize("grid,f", [((16, 16, 16), 0.4), ((12, 10, 8), 0.3)])
def test_propagate_diblock_matches_oracle(lib, grid, f, rng):
    gx, gy, gz = grid
    size, ds = (3.8, 3.3, 4.1), 0.05
    w = rng.standard_normal((2, gz, gy, gx))
    ref = ob.propagate_diblock(w, grid, size, ds, (f, 1 - f))
    with cbuild.ScfCpu(grid, size, ds, f, 25.0, 20.0) as c:
        dens, qsum, logq, mu, energy = c.propagate(w)
    assert abs(qsum / ref["Qsum"] - 1) < 1e-12
    want = ob.density_by_type(ref["density"]).reshape(-1)
    assert np.max(np.abs(dens - want)) < 1e-12 * np.max(np.abs(want))
    assert abs(mu - ref["mu"]) < 1e-12


def test_scf_iterations_match_oracle_loop(lib, rng):
    grid, size, ds, f = (16, 16, 16), (4.0, 4.0, 4.0), 0.05, 0.3
    kappa, chi = 25.0, 18.0
    w = 2.0 * rng.standard_normal((2, 16, 16, 16))
    field, hist = oscf.bulk_scf(w, 6, grid, size, ds, (f, 1 - f), kappa, chi, mixing_type=3,
                                lam=0.1, m=3, lam00=0.1, warm=3)
    with cbuild.ScfCpu(grid, size, ds, f, kappa, chi, m=3, lam=0.1, lam_warm=0.1,
                       warm_iters=3) as c:
        c.set_field(w)
        for h in hist:
            acc, F, logq, it = c.iterate(1)
            assert it == h["iter"]
            assert abs(acc - h["accuracy"]) <= 1e-10 * abs(h["accuracy"])
            assert abs(F - h["F"]) <= 1e-10 * abs(h["F"])
        got = c.get_field()
    assert np.max(np.abs(got - field.reshape(-1))) <= 1e-10 * np.max(np.abs(field))
