"""The reference's input decks and output files.

Readers follow the reference's Fortran list-directed reads record by record
(one ``read(20,*) x`` takes the first value of a record and discards the
rest of it; a bare ``read(20,*)`` skips a record; ``1.0d-12`` is a valid
real):

* ``read_input_general``  -- read_input_parameters, Bulk_3D_FFT/
  Main_Diblock_Melt/main_diblock.f90:226-255 (``layout="bulk"``, blank
  records between groups) and Film_CK_AD/Film_1D/Main_Diblock_Melt/
  main_diblock_melt.f90:270-296 (``layout="film"``, adds int_scheme and
  mesh_type; the Film_3D deck has the same records).
* ``read_mobilities`` -- Read_Mobilities of the multiblock DDFT driver
  (Main_Multiblock/main_multiblock.f90:462-485).
* ``read_input_interactions`` -- Initialize_Interactions, Bulk_3D_FFT/
  Interaction_Modules/mod_FloryHuggins.f90:40-62 (kappa, the upper triangle
  of chi, monomer volumes).

Writers produce the reference's output layouts (main_diblock.f90:157-182;
main_diblock_melt.f90:200-238): ``saddle_dens.dat`` / ``saddle_field.dat``
("x y z value value" per point, 1-based, x fastest, a blank record after
each x row in the density file), the energy record ("sizex sizey sizez
Energy rho ...") and the film ``density.dat`` ("zr density... field..."
per point).  Reals are written with 17 significant digits.

``run_bulk_deck`` mirrors the bulk driver (main_diblock.f90): decks in,
SCF loop (grand canonical, lambda mixing, blocks 0.7/0.3 as the driver
sets them) on the GPU, output files out.
"""
from __future__ import annotations

import os
from pathlib import Path

import numpy as np


def _fortran_real(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "E"))


class _Records:
    """List-directed reading over the records (lines) of a deck."""

    def __init__(self, path):
        self.lines = Path(path).read_text().splitlines()
        self.k = 0

    def skip(self):
        self._need()
        self.k += 1

    def values(self, n=1, cast=_fortran_real):
        out = []
        while len(out) < n:
            self._need()
            toks = self.lines[self.k].replace(",", " ").split()
            self.k += 1
            for t in toks:
                if len(out) == n:
                    break
                if t.startswith("!"):
                    break
                out.append(cast(t))
        return out

    def value(self, cast=_fortran_real):
        return self.values(1, cast)[0]

    def _need(self):
        if self.k >= len(self.lines):
            raise ValueError("deck ends before all records were read")


def _int(tok: str) -> int:
    return int(float(tok.replace("d", "e").replace("D", "E")))


def read_input_general(path, layout="bulk") -> dict:
    r = _Records(path)
    d = {}
    d["sizex"], d["sizey"], d["sizez"] = r.value(), r.value(), r.value()
    if layout == "bulk":
        r.skip()
    d["C"], d["mu"] = r.value(), r.value()
    if layout == "bulk":
        r.skip()
    d["ds"] = r.value()
    if layout == "bulk":
        r.skip()
    d["itermax_scf"] = r.value(_int)
    d["accuracy_scf"] = r.value()
    if layout == "bulk":
        r.skip()
    d["lambda"] = r.value()
    if layout == "film":
        d["int_scheme"] = r.value(_int)
        d["mesh_type"] = r.value(_int)
    elif layout != "bulk":
        raise ValueError("layout must be 'bulk' or 'film'")
    return d


def read_input_interactions(path, components=2) -> dict:
    r = _Records(path)
    kappa = r.value()
    r.skip()
    chi = np.zeros((components, components))
    for a in range(components):
        for b in range(a + 1, components):
            chi[a, b] = chi[b, a] = r.value()
    r.skip()
    vol = [r.value() for _ in range(components)]
    return {"kappa": kappa, "chi": chi, "monomer_volume": vol}


def read_mobilities(path, small=1.0e-6):
    """Read_Mobilities, Bulk_3D_FFT/Main_Multiblock/main_multiblock.f90:
    462-485: nq, dq, three skipped records, then nq rows "q LAA LAB LBB" with
    q = i dq (1-based i, checked to `small`).  Returns (dq, table [nq][3])
    for Context.ddft_set_mobility."""
    r = _Records(path)
    nq = r.value(_int)
    dq = r.value()
    for _ in range(3):
        r.skip()
    table = np.zeros((nq, 3))
    for i in range(nq):
        q, aa, ab, bb = r.values(4)
        if abs(q - (i + 1) * dq) >= small:
            raise ValueError(f"q values in mobility are not consistent: {q} vs {(i + 1) * dq}")
        table[i] = (aa, ab, bb)
    return dq, table


def context_kwargs(general: dict, interactions: dict, **overrides) -> dict:
    """adscf_gb300.Context keywords from the two decks (C -> rho)."""
    kw = dict(size=(general["sizex"], general["sizey"], general["sizez"]), ds=general["ds"],
              rho=general["C"], mu=general["mu"], lam=general["lambda"],
              kappa=interactions["kappa"], chi=float(interactions["chi"][0, 1]),
              monomer_volume=tuple(interactions["monomer_volume"][:2]))
    if "int_scheme" in general:
        kw["int_scheme"] = general["int_scheme"]
    kw.update(overrides)
    return kw


def _g(x: float) -> str:
    return f"{x:25.17E}"


def write_saddle(dens_path, field_path, density, field):
    """density, field: [types][gz][gy][gx] (C order) -> the reference's
    saddle_dens.dat / saddle_field.dat."""
    density = np.asarray(density)
    field = np.asarray(field)
    nt, gz, gy, gx = density.shape
    with open(dens_path, "w") as fd, open(field_path, "w") as ff:
        for z in range(gz):
            for y in range(gy):
                for x in range(gx):
                    idx = f"{x + 1:12d}   {y + 1:12d}   {z + 1:12d}   "
                    fd.write(idx + "".join(_g(density[c, z, y, x]) for c in range(nt)) + "\n")
                    ff.write(idx + "".join(_g(field[c, z, y, x]) for c in range(nt)) + "\n")
                fd.write("\n")


def read_saddle(path, grid, types=2):
    """Inverse of write_saddle for one file: -> [types][gz][gy][gx]."""
    gx, gy, gz = grid
    out = np.zeros((types, gz, gy, gx))
    n = 0
    for line in Path(path).read_text().splitlines():
        toks = line.split()
        if not toks:
            continue
        x, y, z = (int(t) for t in toks[:3])
        out[:, z - 1, y - 1, x - 1] = [_fortran_real(t) for t in toks[3:3 + types]]
        n += 1
    if n != gx * gy * gz:
        raise ValueError(f"{path}: {n} points, expected {gx * gy * gz}")
    return out


def write_energy(path, sizes, energy, rho, *extra):
    """The energy record: sizex sizey sizez Energy rho [elapsed minutes, iter]."""
    vals = list(sizes) + [energy, rho] + list(extra)
    with open(path, "w") as f:
        f.write("    ".join(_g(float(v)) if not isinstance(v, (int, np.integer)) else f"{v:12d}"
                           for v in vals) + "\n")


def write_film_density(path, zr, density, field):
    """Film density.dat: zr, densities, fields per point (x fastest, then y, z)."""
    density = np.asarray(density)
    field = np.asarray(field)
    nt, nz, gy, gx = density.shape
    with open(path, "w") as f:
        for z in range(nz):
            for y in range(gy):
                for x in range(gx):
                    f.write(_g(zr[z]) + "  " + "".join(_g(density[c, z, y, x]) for c in range(nt)) +
                            "  " + "".join(_g(field[c, z, y, x]) for c in range(nt)) + "\n")


def run_bulk_deck(deck_dir, grid, out_dir, precision=None, block_length=(0.7, 0.3), ensemble=2,
                  mixing_type=2, max_iter=None, lib=None):
    """The bulk driver on its decks: reads input_general and
    input_interactions from `deck_dir`, runs the SCF loop from a zero field
    (the driver's uninitialised field) until accuracy_scf or itermax_scf, and
    writes saddle_dens.dat, saddle_field.dat and energy.dat to `out_dir`.
    Returns the last iteration's result."""
    from . import _lib as L
    from .scf import Context
    deck_dir, out_dir = Path(deck_dir), Path(out_dir)
    gen = read_input_general(deck_dir / "input_general", "bulk")
    inter = read_input_interactions(deck_dir / "input_interactions")
    kw = context_kwargs(gen, inter, grid=grid, block_length=block_length, ensemble=ensemble,
                        mixing_type=mixing_type, precision=L.FP64 if precision is None else precision)
    gx, gy, gz = grid
    iters = gen["itermax_scf"] if max_iter is None else min(max_iter, gen["itermax_scf"])
    with Context(L.BULK, lib=lib, **kw) as c:
        c.set_field(np.zeros((2, gz, gy, gx)))
        res = c.scf_run(iters, tol=gen["accuracy_scf"])
        field = c.get_field().reshape(2, gz, gy, gx)
        dens = c.get_density().reshape(2, gz, gy, gx)
    os.makedirs(out_dir, exist_ok=True)
    write_saddle(out_dir / "saddle_dens.dat", out_dir / "saddle_field.dat", dens, field)
    write_energy(out_dir / "energy.dat", (gen["sizex"], gen["sizey"], gen["sizez"]),
                 res.free_energy, res.rho)
    return res
