"""Reference deck readers and output writers (adscf_gb300.io), on decks in
the reference's record layout (values of our own)."""
import numpy as np
import pytest

from adscf_gb300 import io

BULK_GENERAL = """3.7d0\t\tsizex
1.d0\t\tsizey
4.25d0\t\tsizez

1.0d0\t\tC
2.4d0\t \tmu_scf \t! a comment

0.002d0\tds

2000\t\titermax_scf
1.0d-10\t\taccuracy_scf

0.15d0\t\tlambda
"""

FILM_GENERAL = """1.d0\t\tsizex
1.d0\t\tsizey
3.5d0\t\tsizez  ! input from inline argument
1.0d0\t\tC
2.5d0\t \tmu_scf
0.02d0    ds
300        itermax_scf
1.0d-14     accuracy_scf
0.25d0       lambda
1           int_scheme ! 0 rectangle, 1 trapezoid
2           mesh_type
"""

INTERACTIONS = """22.0d0        ! kappa

17.5d0         ! chi

1.0d0          ! volume 1
0.9d0          ! volume 2
"""


def test_read_bulk_general(tmp_path):
    p = tmp_path / "input_general"
    p.write_text(BULK_GENERAL)
    d = io.read_input_general(p, "bulk")
    assert d == {"sizex": 3.7, "sizey": 1.0, "sizez": 4.25, "C": 1.0, "mu": 2.4, "ds": 0.002,
                 "itermax_scf": 2000, "accuracy_scf": 1e-10, "lambda": 0.15}


def test_read_film_general_and_interactions(tmp_path):
    (tmp_path / "g").write_text(FILM_GENERAL)
    (tmp_path / "i").write_text(INTERACTIONS)
    g = io.read_input_general(tmp_path / "g", "film")
    assert g["int_scheme"] == 1 and g["mesh_type"] == 2 and g["accuracy_scf"] == 1e-14
    i = io.read_input_interactions(tmp_path / "i")
    assert i["kappa"] == 22.0 and i["chi"][0, 1] == i["chi"][1, 0] == 17.5
    assert i["monomer_volume"] == [1.0, 0.9]
    kw = io.context_kwargs(g, i, grid=(1, 1, 64))
    assert kw["size"] == (1.0, 1.0, 3.5) and kw["rho"] == 1.0 and kw["chi"] == 17.5
    assert kw["lam"] == 0.25 and kw["int_scheme"] == 1


def test_truncated_deck_raises(tmp_path):
    p = tmp_path / "g"
    p.write_text("\n".join(BULK_GENERAL.splitlines()[:6]))
    with pytest.raises(ValueError):
        io.read_input_general(p, "bulk")


def test_saddle_files_round_trip(tmp_path, rng):
    grid = (5, 3, 4)
    dens = rng.random((2, 4, 3, 5))
    field = rng.standard_normal((2, 4, 3, 5))
    io.write_saddle(tmp_path / "d", tmp_path / "f", dens, field)
    assert np.array_equal(io.read_saddle(tmp_path / "d", grid), dens)
    assert np.array_equal(io.read_saddle(tmp_path / "f", grid), field)
    lines = (tmp_path / "d").read_text().splitlines()
    assert lines[0].split()[:3] == ["1", "1", "1"] and lines[5] == ""   # blank record per x row


def test_energy_and_film_density_records(tmp_path, rng):
    io.write_energy(tmp_path / "e", (3.6, 1.0, 3.6), -1.25, 0.98, 12)
    toks = (tmp_path / "e").read_text().split()
    assert [float(t) for t in toks[:5]] == [3.6, 1.0, 3.6, -1.25, 0.98] and toks[5] == "12"
    zr = np.linspace(0, 3, 7)
    d = rng.random((2, 7, 1, 1))
    f = rng.standard_normal((2, 7, 1, 1))
    io.write_film_density(tmp_path / "fd", zr, d, f)
    rows = [list(map(float, l.split())) for l in (tmp_path / "fd").read_text().splitlines()]
    assert np.allclose(np.array(rows), np.column_stack([zr, d[0, :, 0, 0], d[1, :, 0, 0],
                                                        f[0, :, 0, 0], f[1, :, 0, 0]]), rtol=0, atol=0)


@pytest.mark.gpu
def test_run_bulk_deck_matches_the_oracle_loop(tmp_path):
    """The bulk driver on its decks (grand canonical, lambda mixing, blocks
    0.7/0.3, zero start field) against the oracle's loop for 30 iterations."""
    from oracle import scf as oscf
    (tmp_path / "input_general").write_text(BULK_GENERAL.replace("2000", "30"))
    (tmp_path / "input_interactions").write_text(INTERACTIONS.replace("0.9d0", "1.0d0"))
    grid = (16, 8, 8)
    res = io.run_bulk_deck(tmp_path, grid, tmp_path / "out")
    dens = io.read_saddle(tmp_path / "out" / "saddle_dens.dat", grid)
    field = io.read_saddle(tmp_path / "out" / "saddle_field.dat", grid)
    g = io.read_input_general(tmp_path / "input_general")
    i = io.read_input_interactions(tmp_path / "input_interactions")
    xr, hist = oscf.bulk_scf(np.zeros((2, 8, 8, 16)), 30, grid, (g["sizex"], g["sizey"], g["sizez"]),
                             g["ds"], (0.7, 0.3), i["kappa"], i["chi"][0, 1], mixing_type=2,
                             lam=g["lambda"], ensemble=2, rho=g["C"], mu=g["mu"])
    assert res.iter == 30
    assert np.max(np.abs(field - xr)) < 1e-9 * (1 + np.max(np.abs(xr)))
    assert np.max(np.abs(dens - hist[-1]["density"])) < 1e-9
    e = (tmp_path / "out" / "energy.dat").read_text().split()
    assert abs(float(e[3]) - hist[-1]["F"]) < 1e-9 * max(1.0, abs(hist[-1]["F"]))
