"""Pins of the DDFT restatement (oracle/ddft.py) and the mobility reader."""
import numpy as np
import pytest

from adscf_gb300 import io
from oracle import bulk as ob
from oracle import ddft as od

MOBILITIES = """4     ! number of entries nq
0.5    ! delta q

! Description of entries: q, LAA, LAB, LBB

0.5 0.40 0.10 0.20
1.0 0.30 0.08 0.15
1.5 0.20 0.05 0.10
2.0 0.10 0.02 0.05
"""


def test_read_mobilities(tmp_path):
    p = tmp_path / "input_mobilities"
    p.write_text(MOBILITIES)
    dq, t = io.read_mobilities(p)
    assert dq == 0.5 and t.shape == (4, 3)
    assert np.array_equal(t[2], [0.20, 0.05, 0.10])
    p.write_text(MOBILITIES.replace("1.5 0.20", "1.6 0.20"))
    with pytest.raises(ValueError):
        io.read_mobilities(p)


def test_mobility_interpolation_follows_the_reference_rule():
    """q below dq scales the first row by q/dq; beyond the table the last
    row; in between the reference's weights (row iq at q - iq dq, row iq+1 at
    (iq+1) dq - q); all times q^2 and capped at wcutoff."""
    table = np.array([[0.40, 0.10, 0.20], [0.30, 0.08, 0.15], [0.20, 0.05, 0.10], [0.10, 0.02, 0.05]])
    grid, size = (8, 6, 4), (2 * np.pi * 4, 2 * np.pi * 2, 2 * np.pi)
    m = od.mobility_qq(grid, size, 4, 0.5, table, wcutoff=10.0)
    def expect(q, c):
        iq = int(q / 0.5)
        if iq == 0:
            v = table[0, c] * q / 0.5
        elif iq >= 4:
            v = table[3, c]
        else:
            v = (table[iq - 1, c] * (q - iq * 0.5) + table[iq, c] * ((iq + 1) * 0.5 - q)) / 0.5
        return min(q * q * v, 10.0)
    # kx = x/4, ky = y/2, kz = z
    for (z, y, x) in [(0, 0, 0), (0, 0, 1), (0, 1, 2), (1, 0, 3), (2, 3, 4), (1, 5, 2)]:
        kx, ky = ob.wavenumbers(8, size[0])[x], ob.wavenumbers(6, size[1])[y]
        kz = ob.wavenumbers(4, size[2])[z]
        q = np.sqrt(kx * kx + ky * ky + kz * kz)
        assert np.isclose(m[z, y, x, 0, 0], expect(q, 0), rtol=1e-14, atol=0)
        assert np.isclose(m[z, y, x, 0, 1], expect(q, 1), rtol=1e-14, atol=0)
        assert np.isclose(m[z, y, x, 1, 0], expect(q, 1), rtol=1e-14, atol=0)
        assert np.isclose(m[z, y, x, 1, 1], expect(q, 2), rtol=1e-14, atol=0)
    assert m[0, 0, 0].max() == 0.0


def test_ddft_rhs_conserves_mass_and_is_linear(rng):
    table = np.array([[0.40, 0.10, 0.20], [0.30, 0.08, 0.15], [0.20, 0.05, 0.10], [0.10, 0.02, 0.05]])
    grid, size = (8, 6, 4), (3.0, 2.5, 2.0)
    mob = od.mobility_qq(grid, size, 4, 0.5, table, wcutoff=10.0)
    mu1 = rng.standard_normal((2, 4, 6, 8))
    mu2 = rng.standard_normal((2, 4, 6, 8))
    r1, r2 = od.ddft_rhs(mu1, mob), od.ddft_rhs(mu2, mob)
    assert abs(r1[0].sum()) < 1e-12 and abs(r1[1].sum()) < 1e-12
    assert np.allclose(od.ddft_rhs(mu1 + 2 * mu2, mob), r1 + 2 * r2, atol=1e-12)
    # a uniform potential moves nothing
    assert np.allclose(od.ddft_rhs(np.ones((2, 4, 6, 8)), mob), 0.0, atol=1e-14)


def test_conjugate_fields_recover_the_density(rng):
    grid, size, ds = (6, 4, 4), (3.0, 2.0, 2.0), 0.05
    blocks, types = (0.6, 0.4), (0, 1)
    w0 = 0.4 * rng.standard_normal((2, 4, 4, 6))
    fn = lambda w: od.calculate_densities(w, grid, size, ds, blocks, types)
    target = fn(w0)
    w, st, it, acc = od.get_conjugate_fields(target, np.zeros_like(w0), 1e-6, 3000, fn, mixing_dim=4)
    assert st == 0 and acc <= 5e-7
    assert np.max(np.abs(fn(w) - target)) <= 5e-7
