"""Film (Film_1D CN, Film_3D Douglas ADI) and brush propagators on the GPU,
through the C ABI, against the FP64 oracle (oracle/film.py).  Tolerances:
FP64 relative 1e-11; split (FP32 sweeps on a mildly graded mesh) 2e-5."""
import re

import numpy as np
import pytest

from oracle import film as of
from oracle import interactions as oi
from oracle import scf as oscf

pytestmark = pytest.mark.gpu

from adscf_gb300 import (FILM_1D, FILM_3D, BRUSH, FP64, SPLIT, MIX_LAMBDA,
                         MIX_ANDERSON, AdscfError, Context)


def film_ctx(geom, grid, dz, size, ds=0.01, f=(0.5, 0.5), prec=FP64, **kw):
    return Context(geom, grid=grid, size=size, ds=ds, block_length=f, dz=dz,
                   precision=prec, **kw)


@pytest.mark.parametrize("mesh", [0, 1])
def test_film1d_cn_step(mesh, rng):
    gz, D, ds = 40, 3.0, 0.01
    dz, zr = of.generate_mesh(mesh, gz, D, film3d=False)
    q = rng.random(gz + 1) + 0.5
    w = rng.standard_normal(gz + 1)
    ref = of.cn_step_1d(q, w, dz, ds, solver="inplace")
    with film_ctx(FILM_1D, (1, 1, gz), dz, (1.0, 1.0, D), ds) as c:
        out = c.propagate_step(q, w, ds)
    assert np.max(np.abs(out - ref)) < 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("ensemble", [1, 2])
def test_film1d_propagate_diblock(ensemble, rng):
    gz, D, ds = 64, 4.0, 0.02
    dz, zr = of.tanh_mesh(gz, D)
    field = 0.5 * rng.standard_normal((2, gz + 1))
    dss = np.r_[0.0, np.full(50, ds)]
    step = lambda p, w, h: of.cn_step_1d(p, w, dz, h)
    ref = of.film_propagate_diblock(field, dz, dss, 25, step, rho=1.0, int_scheme=1,
                                    span="interior", ensemble=ensemble, mu=0.4,
                                    sizes=(1.0, 1.0, D))
    with film_ctx(FILM_1D, (1, 1, gz), dz, (1.0, 1.0, D), ds, int_scheme=1, int_span=1,
                  ensemble=ensemble, mu=0.4) as c:
        dens, res = c.propagate_diblock(field)
    assert abs(res.Qsum / ref["Qsum"] - 1) < 1e-12
    assert np.max(np.abs(dens - ref["density"])) < 1e-11 * np.max(np.abs(ref["density"]))


def test_film1d_many_lines_adaptive_contour(rng):
    """gx*gy independent lines on one mesh, end-refined contour steps."""
    gx, gy, gz, D = 5, 3, 48, 3.0
    dz, zr = of.tanh_mesh(gz, D)
    dss = of.contour_steps(60, ds_scheme=1)
    field = rng.standard_normal((2, gz + 1, gy, gx))
    step = lambda p, w, h: of.cn_step_1d(p, w, dz, h)
    ref = of.film_propagate_diblock(field, dz, dss, 30, step, rho=1.0, dx=1.0, dy=1.0,
                                    int_scheme=1, span="full", sizes=(gx, gy, D))
    with film_ctx(FILM_1D, (gx, gy, gz), dz, (gx * 1.0, gy * 1.0, D), dss=dss, n_a=30,
                  int_scheme=1, int_span=0) as c:
        dens, res = c.propagate_diblock(field)
    assert abs(res.Qsum / ref["Qsum"] - 1) < 1e-12
    assert np.max(np.abs(dens - ref["density"])) < 1e-11 * np.max(np.abs(ref["density"]))


def test_film1d_split_precision(rng):
    gz, D, ds = 64, 3.0, 0.01
    dz, zr = of.generate_mesh(0, gz, D)
    field = rng.standard_normal((2, gz + 1))
    dss = np.r_[0.0, np.full(100, ds)]
    step = lambda p, w, h: of.cn_step_1d(p, w, dz, h)
    ref = of.film_propagate_diblock(field, dz, dss, 50, step, sizes=(1.0, 1.0, D))
    with film_ctx(FILM_1D, (1, 1, gz), dz, (1.0, 1.0, D), ds, prec=SPLIT) as c:
        dens, res = c.propagate_diblock(field)
    # FP32 sweeps in increment form: the rounding is relative to the O(ds)
    # increment of each step, not to the O(ds/dz^2) matrix entries
    assert abs(np.log(res.Qsum) - np.log(ref["Qsum"])) < 2e-6
    assert np.max(np.abs(dens - ref["density"])) < 2e-6 * np.max(np.abs(ref["density"]))


def test_film3d_adi_step(rng):
    gx, gy, gz, ds = 8, 6, 12, 0.02
    dz, zr = of.generate_mesh(1, gz, 2.5)
    size = (3.0, 2.4, 2.5)
    q = rng.random((gz + 1, gy, gx)) + 0.5
    w = rng.standard_normal((gz + 1, gy, gx))
    ref = of.adi_step_3d(q, w, dz, size[0] / gx, size[1] / gy, ds)
    with film_ctx(FILM_3D, (gx, gy, gz), dz, size, ds) as c:
        out = c.propagate_step(q, w, ds)
    assert np.max(np.abs(out - ref)) < 1e-12 * np.max(np.abs(ref))


def test_film3d_propagate_diblock(rng):
    gx, gy, gz, ds = 8, 6, 10, 0.05
    dz, zr = of.tanh_mesh(gz, 3.0)
    size = (3.0, 2.4, 3.0)
    field = 0.5 * rng.standard_normal((2, gz + 1, gy, gx))
    dss = np.r_[0.0, np.full(20, ds)]
    step = lambda p, w, h: of.adi_step_3d(p, w, dz, size[0] / gx, size[1] / gy, h)
    ref = of.film_propagate_diblock(field, dz, dss, 5, step, dx=size[0] / gx,
                                    dy=size[1] / gy, int_scheme=1, span="full", sizes=size)
    with film_ctx(FILM_3D, (gx, gy, gz), dz, size, ds, f=(0.25, 0.75)) as c:
        dens, res = c.propagate_diblock(field)
    assert abs(res.Qsum / ref["Qsum"] - 1) < 1e-11
    assert np.max(np.abs(dens - ref["density"])) < 1e-10 * np.max(np.abs(ref["density"]))


def test_film3d_split_precision(rng):
    """FP32 Douglas ADI sweeps (uniform mesh, so the split path sweeps in
    FP32) against the FP64 oracle over 100 contour steps."""
    gx, gy, gz, ds = 16, 12, 24, 0.01
    dz, zr = of.generate_mesh(0, gz, 3.0)
    size = (3.2, 2.4, 3.0)
    field = 0.5 * rng.standard_normal((2, gz + 1, gy, gx))
    dss = np.r_[0.0, np.full(100, ds)]
    step = lambda p, w, h: of.adi_step_3d(p, w, dz, size[0] / gx, size[1] / gy, h)
    ref = of.film_propagate_diblock(field, dz, dss, 25, step, dx=size[0] / gx,
                                    dy=size[1] / gy, int_scheme=1, span="full", sizes=size)
    with film_ctx(FILM_3D, (gx, gy, gz), dz, size, ds, f=(0.25, 0.75), prec=SPLIT) as c:
        dens, res = c.propagate_diblock(field)
    assert abs(np.log(res.Qsum) - np.log(ref["Qsum"])) < 2e-6
    assert np.max(np.abs(dens - ref["density"])) < 2e-6 * np.max(np.abs(ref["density"]))


def _adi_shapes(n, periodic, stageable, z):
    """(lanes, staged) of the warp-solver shapes for a line of n points, as
    the library enumerates them, plus (0, 0): one thread per line."""
    out = []
    for g in (2, 4, 8, 16, 32):
        if periodic:
            ok = any(n == g * k for k in (2, 4))
        else:
            k = max(2, -(-n // g))
            ok = k <= 4 or (k <= 8 and g >= 8)
        if ok:
            out.append((g, 0))
    if stageable and (3 if z else 2) * n * 33 * 4 <= 46 * 1024:
        out += [(g, 1) for g, _ in list(out) if g >= 4]
    return out + [(0, 0)]


def test_film3d_every_adi_shape_vs_oracle(rng):
    """Every ADI sweep shape the autotuner may pick (warp solver with each
    lane count, staged through shared memory or not, and one thread per
    line), one sweep at a time with the other two at the tuner's choice,
    against the FP64 oracle; the tuner's report names a shape per sweep."""
    gx, gy, gz, ds = 16, 32, 24, 0.01
    dz, zr = of.generate_mesh(0, gz, 3.0)
    size = (3.2, 4.0, 3.0)
    field = 0.5 * rng.standard_normal((2, gz + 1, gy, gx))
    dss = np.r_[0.0, np.full(60, ds)]   # blocks of 15 and 45 steps
    step = lambda p, w, h: of.adi_step_3d(p, w, dz, size[0] / gx, size[1] / gy, h)
    ref = of.film_propagate_diblock(field, dz, dss, 15, step, dx=size[0] / gx,
                                    dy=size[1] / gy, int_scheme=1, span="full", sizes=size)
    with film_ctx(FILM_3D, (gx, gy, gz), dz, size, ds, f=(0.15, 0.45), prec=SPLIT) as c:
        rep = c.tuning()
        chosen = re.findall(r"\b([xyz])=(\d+)x(\d+)(s?)", rep[rep.index("adi"):])
        assert sorted(a for a, _, _, _ in chosen) == ["x", "y", "z"]
        tuned = {a: (int(g), 1 if st else 0) for a, g, _, st in chosen}
        shapes = {"x": _adi_shapes(gx, True, False, False), "y": _adi_shapes(gy, True, True, False),
                  "z": _adi_shapes(gz + 1, False, True, True)}
        assert len(shapes["x"]) >= 3 and len(shapes["y"]) >= 5 and len(shapes["z"]) >= 6
        for axis in "xyz":
            for sh in shapes[axis]:
                plan = dict(tuned, **{axis: sh})
                mask = 2 * plan["y"][1] + 4 * plan["z"][1]
                c.set_adi_plan(plan["x"][0], plan["y"][0], plan["z"][0], mask)
                dens, res = c.propagate_diblock(field)
                assert abs(np.log(res.Qsum) - np.log(ref["Qsum"])) < 2e-6, (axis, sh)
                assert np.max(np.abs(dens - ref["density"])) < 2e-6 * np.max(np.abs(ref["density"])), (axis, sh)
        with pytest.raises(AdscfError):
            c.set_adi_plan(3, 0, 0)
        with pytest.raises(AdscfError):
            c.set_adi_plan(8, 16, 8, 1)   # the x sweep has no staged form


@pytest.mark.parametrize("n,lanes", [(32, 16), (32, 8), (64, 16)])
def test_film3d_fused_xy_sweep(n, lanes, rng):
    """The x and y ADI sweeps as one plane kernel (mask 8) against the two
    sweeps of the same shape (the same arithmetic) and against the FP64
    oracle; refused when the x and y shapes differ."""
    gx = gy = n
    gz, ds = 12, 0.01
    dz, zr = of.generate_mesh(0, gz, 3.0)
    size = (3.2, 3.2, 3.0)
    field = 0.5 * rng.standard_normal((2, gz + 1, gy, gx))
    dss = np.r_[0.0, np.full(40, ds)]   # blocks of 10 and 30 steps
    step = lambda p, w, h: of.adi_step_3d(p, w, dz, size[0] / gx, size[1] / gy, h)
    ref = of.film_propagate_diblock(field, dz, dss, 10, step, dx=size[0] / gx,
                                    dy=size[1] / gy, int_scheme=1, span="full", sizes=size)
    with film_ctx(FILM_3D, (gx, gy, gz), dz, size, ds, f=(0.1, 0.3), prec=SPLIT) as c:
        c.set_adi_plan(lanes, lanes, 8, 0)
        d0, r0 = c.propagate_diblock(field)
        c.set_adi_plan(lanes, lanes, 8, 8)
        d1, r1 = c.propagate_diblock(field)
        assert abs(np.log(r1.Qsum) - np.log(r0.Qsum)) < 1e-9
        assert np.max(np.abs(d1 - d0)) <= 1e-7 * np.max(np.abs(d0))
        assert abs(np.log(r1.Qsum) - np.log(ref["Qsum"])) < 2e-6
        assert np.max(np.abs(d1 - ref["density"])) < 2e-6 * np.max(np.abs(ref["density"]))
        other = 8 if lanes == 16 else 16
        with pytest.raises(AdscfError):
            c.set_adi_plan(lanes, other, 8, 8)


@pytest.mark.parametrize("geom,grid", [(FILM_3D, (8, 6, 16)), (FILM_1D, (1, 1, 24))])
def test_film_scf_iteration_host_buffers(geom, grid, rng):
    """adscf_scf_iteration on films (the densities copied to the host beside
    the solve and the mix) gives the field and densities of scf_run(1)."""
    gx, gy, gz = grid
    dz, zr = of.generate_mesh(0, gz, 3.0)
    size = (1.6, 1.2, 3.0) if geom == FILM_3D else (1.0, 1.0, 3.0)
    field = 0.3 * rng.standard_normal((2, gz + 1, gy, gx))
    kw = dict(ds=0.02, f=(0.3, 0.7), prec=SPLIT, kappa=10.0, chi=12.0, mixing_type=MIX_LAMBDA,
              lam=0.1, ensemble=2, mu=1.0)
    with film_ctx(geom, grid, dz, size, **kw) as c:
        c.set_field(field)
        c.scf_run(1)
        x1, d1 = c.get_field(), c.get_density()
    with film_ctx(geom, grid, dz, size, **kw) as c:
        c.set_field(field)
        x2, d2, res = c.scf_iteration(field.reshape(-1))
    assert res.iter == 1
    assert np.array_equal(x1.reshape(-1), x2) and np.array_equal(d1.reshape(-1), d2.reshape(-1))


def test_brush_propagate_homopolymer(rng):
    gz, D = 80, 5.0
    dz, zr = of.generate_mesh(0, gz, D)
    dss = of.contour_steps(120, ds_scheme=1)
    graft = np.zeros(gz + 1)
    graft[4] = 1.0
    wts = of.integrator_weights(dz, 1, "interior")
    graft /= np.dot(wts, graft)                      # mod_homopolymer.f90:145-150
    field = 0.3 * rng.standard_normal(gz + 1)
    ref = of.propagate_homopolymer(field, dz, dss, graft, 0.4, int_scheme=1,
                                   span="interior", sizes=(1.0, 1.0, D))
    with Context(BRUSH, grid=(1, 1, gz), size=(1.0, 1.0, D), dss=dss, dz=dz, graft=graft,
                 rho=0.4, int_scheme=1, int_span=1, ww=1.0) as c:
        dens, res = c.propagate_homopolymer(field)
    assert abs(res.Qsum / ref["Qsum"] - 1) < 1e-11
    assert np.max(np.abs(dens - ref["density"])) < 1e-10 * np.max(np.abs(ref["density"]))
    assert abs(res.mu - ref["mu"]) < 1e-10


@pytest.mark.parametrize("mtype", [MIX_LAMBDA, MIX_ANDERSON])
def test_film1d_scf_loop_with_walls(mtype, rng):
    gz, D, ds = 48, 3.0, 0.02
    dz, zr = of.tanh_mesh(gz, D)
    surf = np.stack([0.8 * oi.wall_potential_shape(zr, D, 0.4), -0.4 * oi.wall_potential_shape(zr, D, 0.4)])
    z = zr / D
    field = np.stack([2.0 * np.cos(2 * np.pi * z), -2.0 * np.cos(2 * np.pi * z)])
    field[:, 0] = field[:, -1] = 0.0
    dss = np.r_[0.0, np.full(50, ds)]
    step = lambda p, w, h: of.cn_step_1d(p, w, dz, h)
    xr, hist = oscf.film_scf(field, 8, dz, dss, 25, step, 25.0, 15.0, surf, (1.0, 1.0, D),
                             int_scheme=1, span="full", mixing_type=mtype, lam=0.1, m=2,
                             lam00=0.05, warm=3)
    with film_ctx(FILM_1D, (1, 1, gz), dz, (1.0, 1.0, D), ds, kappa=25.0, chi=15.0,
                  ext_potential=surf, int_scheme=1, int_span=0, mixing_type=mtype,
                  mixing_dim=2, lam=0.1, lam_warm=0.05, warm_iters=3) as c:
        c.set_field(field)
        res = c.scf_run(8)
        xg = c.get_field().reshape(2, gz + 1)
    assert res.iter == 8
    assert abs(res.accuracy - hist[-1]["accuracy"]) <= 1e-8 * hist[-1]["accuracy"] + 1e-18
    assert np.max(np.abs(xg - xr)) < 1e-9 * (1 + np.max(np.abs(xr)))


def test_zero_pivot_returns_status():
    """A zero Thomas pivot (the reference's 'TriDiag Error' stop) becomes
    ADSCF_E_PIVOT: uniform h = 0.5, ds = 0.25 gives b = 1 and a field of -16
    at plane 1 makes the first interior diagonal exactly zero."""
    gz = 8
    dz = np.r_[0.0, np.full(gz, 0.5)]
    w = np.zeros(gz + 1)
    w[1] = -16.0
    with film_ctx(FILM_1D, (1, 1, gz), dz, (1.0, 1.0, 4.0), 0.25) as c:
        with pytest.raises(AdscfError) as e:
            c.propagate_step(np.ones(gz + 1), w, 0.25)
    assert e.value.code == 3


def _film_kw(gz, D, dz, ext, ensemble=1, chi=15.0, **kw):
    return dict(grid=(1, 1, gz), size=(1.0, 1.0, D), ds=0.02, block_length=(0.5, 0.5), dz=dz,
                kappa=25.0, chi=chi, ext_potential=ext, int_scheme=1, int_span=1,
                ensemble=ensemble, mu=0.4, **kw)


@pytest.mark.parametrize("ensemble", [1, 2])
def test_film_free_energy_gradient_wrt_wall_potential(ensemble, rng):
    """adscf_forward / adscf_backward_surface on a Film_1D context: F equals
    the SCF loop's F of the same field, and dF/dU_c(z), dF/dchi match
    central differences of F at fixed fields."""
    gz, D = 40, 3.0
    dz, zr = of.tanh_mesh(gz, D)
    ext = np.stack([0.6 * oi.wall_potential_shape(zr, D, 0.4), -0.3 * oi.wall_potential_shape(zr, D, 0.4)])
    z = zr / D
    field = np.stack([1.5 * np.cos(2 * np.pi * z), -1.5 * np.cos(2 * np.pi * z)])
    field += 0.1 * rng.standard_normal(field.shape)
    field[:, 0] = field[:, -1] = 0.0
    with Context(FILM_1D, **_film_kw(gz, D, dz, ext, ensemble)) as c:
        F = c.forward(field)
        dchi, dU = c.backward_surface()
        c.set_field(field)
        _x, _d, r = c.scf_iteration(field.copy())
    assert abs(F - r.free_energy) < 1e-12 * max(1.0, abs(F))

    def F_of(ext2, chi=15.0):
        with Context(FILM_1D, **_film_kw(gz, D, dz, ext2, ensemble, chi)) as c2:
            return c2.forward(field)

    d = 1e-5
    for ctype, zi in ((0, 1), (0, 5), (1, 3), (1, gz - 2), (0, gz // 2)):
        ep, em = ext.copy(), ext.copy()
        ep[ctype, zi] += d
        em[ctype, zi] -= d
        fd = (F_of(ep) - F_of(em)) / (2 * d)
        assert abs(dU[ctype, zi] - fd) < 1e-7 * max(1e-3, abs(fd)), (ctype, zi, dU[ctype, zi], fd)
    fd = (F_of(ext, 15.0 + 1e-4) - F_of(ext, 15.0 - 1e-4)) / 2e-4
    assert abs(dchi - fd) < 1e-8 * max(1.0, abs(fd))


def test_brush_gradient_wrt_wall_potential(rng):
    gz, D = 50, 4.0
    dz, zr = of.tanh_mesh(gz, D)
    dss = of.contour_steps(60, ds_scheme=2)
    graft = np.zeros(gz + 1)
    graft[3] = 1.0
    graft /= np.dot(of.integrator_weights(dz, 1, "interior"), graft)
    ext = (0.4 * oi.wall_potential_shape(zr, D, 0.5))[None, :]
    field = 0.3 * rng.standard_normal((1, gz + 1))

    def make(ext2, ww=1.0):
        return Context(BRUSH, grid=(1, 1, gz), size=(1.0, 1.0, D), dss=dss, dz=dz, graft=graft,
                       rho=0.3, ww=ww, ext_potential=ext2, int_scheme=1, int_span=1)

    with make(ext) as c:
        F = c.forward(field)
        dww, dU = c.backward_surface()
    d = 1e-5
    for zi in (2, 10, 25):
        ep, em = ext.copy(), ext.copy()
        ep[0, zi] += d
        em[0, zi] -= d
        with make(ep) as a, make(em) as b:
            fd = (a.forward(field) - b.forward(field)) / (2 * d)
        assert abs(dU[0, zi] - fd) < 1e-7 * max(1e-3, abs(fd)), (zi, dU[0, zi], fd)
    with make(ext, 1.0 + 1e-4) as a, make(ext, 1.0 - 1e-4) as b:
        fd = (a.forward(field) - b.forward(field)) / 2e-4
    assert abs(dww - fd) < 1e-8 * max(1.0, abs(fd))


@pytest.mark.parametrize("geom,grid,scheme,span", [(FILM_3D, (6, 4, 20), 1, 0), (FILM_3D, (6, 4, 20), 0, 0),
                                                   (FILM_1D, (1, 1, 30), 1, 1), (FILM_1D, (1, 1, 30), 0, 1)])
def test_integrator_entry_point_vs_oracle(geom, grid, scheme, span, rng):
    """adscf_integrator (integrator, Film_3D/.../mod_realspace.f90:267-281;
    Film_1D/Brush interior form) on a host integrand against the oracle."""
    gx, gy, gz = grid
    dz, zr = of.tanh_mesh(gz, 3.0)
    size = (3.0, 2.0, 3.0) if geom == FILM_3D else (1.0, 1.0, 3.0)
    f = rng.random((gz + 1, gy, gx))
    with film_ctx(geom, grid, dz, size, int_scheme=scheme, int_span=span) as c:
        got = c.integrator(f)
    want = of.integrator(f, dz, size[0] / gx, size[1] / gy, int_scheme=scheme,
                         span="full" if span == 0 else "interior")
    assert abs(got - want) <= 1e-13 * abs(want)


def test_integrator_entry_point_bulk(rng):
    """Bulk: dvol * sum (the reference's dvol * sum(...) reductions)."""
    from adscf_gb300 import BULK
    f = rng.random((12, 10, 8))
    with Context(BULK, grid=(8, 10, 12), size=(2.0, 2.5, 3.0), ds=0.05, block_length=(0.5, 0.5)) as c:
        got = c.integrator(f)
    assert abs(got - f.sum() * (2.0 * 2.5 * 3.0) / f.size) <= 1e-13 * abs(got)
