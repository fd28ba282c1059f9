"""Host-side mirror of the ADSCF module procedures over the C ABI.

Each method keeps the reference routine's name and argument meaning, so a
test reads like a call into the Fortran modules:

* ``propagate_diblock``  -- Propagate_Diblock (Bulk_3D_FFT/Polymer_Modules/
  mod_diblock.f90:100-173) with Calculate_Expfield (mod_propagate.f90:22-32)
* ``propagate_step``     -- Propagate_Step (mod_propagate.f90:40-68; films
  Film_CK_AD/Film_1D/Geometry_Modules/mod_realspace.f90:24-79)
* ``real2fourier`` / ``fourier2real`` -- mod_fourier.f90:75-105
* ``mean_fields`` / ``interaction_energy`` -- mod_FloryHuggins.f90:74-129
* ``mix``                -- Mix_Fields (main_diblock.f90:315-372)
* ``scf_run``            -- the Calculate_Saddle_Point loop
  (main_diblock.f90:398-451), device resident.

Errors raise ``AdscfError`` carrying the C status code (the reference stops
the program instead).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def make_params(geometry=L.BULK, grid=(32, 32, 32), size=(4.0, 4.0, 4.0), ds=0.01,
                block_length=(0.5, 0.5), ensemble=1, rho=1.0, mu=0.0, kappa=25.0, chi=20.0,
                monomer_volume=(1.0, 1.0), precision=L.FP64, mixing_type=L.MIX_LAMBDA,
                mixing_dim=2, lam=0.1, lam_warm=1.0e-3, warm_iters=0, dss=None, n_a=0,
                dz=None, int_scheme=1, int_span=0, ext_potential=None, ww=1.0, graft=None,
                blocks=None, block_types=None):
    """adscf_params of one instance; returns (params, arrays it points into).
    ``blocks`` / ``block_types`` give a bulk linear block sequence (lengths and
    monomer types 0 = A, 1 = B) in place of the diblock of ``block_length``."""
    keep = []
    p = L.Params()
    p.geometry = geometry
    p.gx, p.gy, p.gz = grid
    p.sizex, p.sizey, p.sizez = size
    p.ds = ds
    if dss is not None:
        dss = _f64(dss)
        keep.append(dss)
        p.dss = L.dptr(dss)
        p.ns = dss.size - 1
        p.n_a = n_a
    p.block_length[0], p.block_length[1] = block_length
    p.ensemble = ensemble
    p.rho, p.mu = rho, mu
    p.kappa, p.chi = kappa, chi
    p.monomer_volume[0], p.monomer_volume[1] = monomer_volume
    p.precision = precision
    p.mixing_type = mixing_type
    p.mixing_dim = mixing_dim
    p.lam = lam
    p.lam_warm = lam_warm
    p.warm_iters = warm_iters
    for name, arr in (("dz", dz), ("ext_potential", ext_potential), ("graft", graft)):
        if arr is not None:
            arr = _f64(arr)
            keep.append(arr)
            setattr(p, name, L.dptr(arr))
    p.int_scheme = int_scheme
    p.int_span = int_span
    p.ww = ww
    if blocks is not None:
        bl = _f64(blocks)
        bt = np.ascontiguousarray(block_types, dtype=np.int32)
        if bt.size != bl.size:
            raise ValueError("blocks and block_types differ in length")
        keep += [bl, bt]
        p.nblocks = bl.size
        p.blocks = L.dptr(bl)
        p.block_types = bt.ctypes.data_as(C.POINTER(C.c_int))
    return p, keep


class Context:
    """One SCF context (geometry, grid, chain, interactions, mixing)."""

    def __init__(self, geometry=L.BULK, grid=(32, 32, 32), size=(4.0, 4.0, 4.0),
                 ds=0.01, block_length=(0.5, 0.5), ensemble=1, rho=1.0, mu=0.0,
                 kappa=25.0, chi=20.0, monomer_volume=(1.0, 1.0),
                 precision=L.FP64, mixing_type=L.MIX_LAMBDA, mixing_dim=2,
                 lam=0.1, lam_warm=1.0e-3, warm_iters=0, dss=None, n_a=0,
                 dz=None, int_scheme=1, int_span=0, ext_potential=None,
                 ww=1.0, graft=None, blocks=None, block_types=None, lib=None):
        self.lib = lib or L.load()
        p, self._keep = make_params(
            geometry=geometry, grid=grid, size=size, ds=ds, block_length=block_length,
            ensemble=ensemble, rho=rho, mu=mu, kappa=kappa, chi=chi,
            monomer_volume=monomer_volume, precision=precision, mixing_type=mixing_type,
            mixing_dim=mixing_dim, lam=lam, lam_warm=lam_warm, warm_iters=warm_iters,
            dss=dss, n_a=n_a, dz=dz, int_scheme=int_scheme, int_span=int_span,
            ext_potential=ext_potential, ww=ww, graft=graft, blocks=blocks,
            block_types=block_types)
        self.params = p
        h = C.c_void_p()
        rc = self.lib.adscf_ctx_create(C.byref(p), C.byref(h))
        if rc != L.ADSCF_OK:
            raise L.AdscfError(rc, self.lib.adscf_status_string(rc).decode())
        self.h = h
        self.npts = int(self.lib.adscf_field_points(h))
        ns, na = C.c_int(), C.c_int()
        self.lib.adscf_contour_info(h, C.byref(ns), C.byref(na))
        self.ns, self.n_a = ns.value, na.value
        self.ntypes = 1 if geometry == L.BRUSH else 2
        self.geometry = geometry

    # -- lifetime --------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.adscf_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        L.check(self.lib, self.h, rc)

    # -- propagators -----------------------------------------------------
    def propagate_diblock(self, field):
        """field [2][npts] -> (density [2][npts], ChainResult)."""
        w = _f64(field, 2 * self.npts)
        out = np.empty(2 * self.npts)
        res = L.ChainResult()
        self._ck(self.lib.adscf_propagate_diblock(self.h, L.dptr(w), L.dptr(out), C.byref(res)))
        return out.reshape(np.shape(field)), res

    def propagate_homopolymer(self, field):
        w = _f64(field, self.npts)
        out = np.empty(self.npts)
        res = L.ChainResult()
        self._ck(self.lib.adscf_propagate_homopolymer(self.h, L.dptr(w), L.dptr(out), C.byref(res)))
        return out.reshape(np.shape(field)), res

    def propagate_step(self, prop, aux, ds=0.0):
        """One step in place on a copy; aux = expfield (bulk) or field (films)."""
        q = _f64(prop, self.npts).copy()
        a = _f64(aux, self.npts)
        self._ck(self.lib.adscf_propagate_step(self.h, L.dptr(q), L.dptr(a), ds))
        return q.reshape(np.shape(prop))

    def real2fourier(self, prop):
        gx, gy, gz = self.params.gx, self.params.gy, self.params.gz
        q = _f64(prop, self.npts)
        out = np.empty((gz, gy, gx // 2 + 1, 2))
        self._ck(self.lib.adscf_real2fourier(self.h, L.dptr(q), L.dptr(out)))
        return out[..., 0] + 1j * out[..., 1]

    def fourier2real(self, spec):
        gx, gy, gz = self.params.gx, self.params.gy, self.params.gz
        s = np.ascontiguousarray(np.stack([spec.real, spec.imag], axis=-1), dtype=np.float64)
        out = np.empty((gz, gy, gx))
        self._ck(self.lib.adscf_fourier2real(self.h, L.dptr(s), L.dptr(out)))
        return out

    def integrator(self, integrand):
        f = _f64(integrand, self.npts)
        out = C.c_double()
        self._ck(self.lib.adscf_integrator(self.h, L.dptr(f), C.byref(out)))
        return out.value

    # -- interactions ----------------------------------------------------
    def mean_fields(self, density):
        d = _f64(density, self.ntypes * self.npts)
        out = np.empty_like(d)
        self._ck(self.lib.adscf_mean_fields(self.h, L.dptr(d), L.dptr(out)))
        return out.reshape(np.shape(density))

    def update_solvent(self, field, ensemble, rho=1.0, mu=0.0):
        """Update_Solvent (mod_solvent.f90:85-110) of a monomeric solvent in
        `field` ([npts]) on this bulk context's grid: dict of distribution,
        Qsum, density, mu, rho and energy (rho in and mu out when canonical,
        mu in and rho out when grand canonical)."""
        w = _f64(field, self.npts)
        dens = np.empty_like(w)
        dist = np.empty_like(w)
        r, m, q, e = C.c_double(rho), C.c_double(mu), C.c_double(), C.c_double()
        self._ck(self.lib.adscf_update_solvent(self.h, L.dptr(w), int(ensemble), C.byref(r), C.byref(m),
                                               C.byref(q), C.byref(e), L.dptr(dens), L.dptr(dist)))
        shape = np.shape(field)
        return {"distribution": dist.reshape(shape), "Qsum": q.value, "density": dens.reshape(shape),
                "mu": m.value, "rho": r.value, "energy": e.value}

    def interaction_energy(self, density):
        d = _f64(density, self.ntypes * self.npts)
        out = C.c_double()
        self._ck(self.lib.adscf_interaction_energy(self.h, L.dptr(d), C.byref(out)))
        return out.value

    # -- mixing -----------------------------------------------------------
    def mix(self, field, dfield, it):
        x = _f64(field).copy()
        r = _f64(dfield, x.size)
        self._ck(self.lib.adscf_mix(self.h, L.dptr(x), L.dptr(r), int(it)))
        return x.reshape(np.shape(field))

    def mix_reset(self):
        self._ck(self.lib.adscf_mix_reset(self.h))

    # -- device SCF loop ---------------------------------------------------
    def set_field(self, field):
        self._ck(self.lib.adscf_set_field(self.h, L.dptr(_f64(field, self.ntypes * self.npts))))

    def set_density(self, density):
        self._ck(self.lib.adscf_set_density(self.h, L.dptr(_f64(density, self.ntypes * self.npts))))

    def get_field(self):
        out = np.empty(self.ntypes * self.npts)
        self._ck(self.lib.adscf_get_field(self.h, L.dptr(out)))
        return out

    def get_density(self):
        out = np.empty(self.ntypes * self.npts)
        self._ck(self.lib.adscf_get_density(self.h, L.dptr(out)))
        return out

    def scf_run(self, n_iter, tol=-1.0):
        res = L.IterResult()
        self._ck(self.lib.adscf_scf_run(self.h, int(n_iter), float(tol), C.byref(res)))
        return res

    # -- pass-kernel autotuner (bulk) ---------------------------------------
    def tuning(self):
        """Chosen pass plan and the autotuner's per-candidate timings."""
        buf = C.create_string_buffer(2048)
        self._ck(self.lib.adscf_tuning(self.h, buf, len(buf)))
        return buf.value.decode()

    def set_wait_limit(self, polls):
        """Pipeline-wait bound of the TMA passes (polls; < 0 restores the default)."""
        self._ck(self.lib.adscf_set_wait_limit(self.h, int(polls)))

    def set_pass_plan(self, y, z, x):
        """Pin the kernel of the Y, Z and X passes (0 plain, 1 persistent, 2 TMA)."""
        self._ck(self.lib.adscf_set_pass_plan(self.h, int(y), int(z), int(x)))

    def set_adi_plan(self, x_lanes, y_lanes, z_lanes, staged=0):
        """Pin the lanes per line of the FP32 ADI sweeps of a Film_3D context
        (0: one thread per line), their staging through shared memory
        (mask: 2 for y, 4 for z) and the x and y sweeps as one plane kernel
        (mask 8: x and y with one shape on a square plane)."""
        self._ck(self.lib.adscf_set_adi_plan(self.h, int(x_lanes), int(y_lanes), int(z_lanes),
                                             int(staged)))

    # -- differentiation (FP64 bulk) ----------------------------------------
    def forward(self, field):
        """Free energy per chain at `field` [ntypes][npts], no mixing; keeps
        the propagator state for ``backward`` / ``backward_surface``."""
        w = _f64(field, self.ntypes * self.npts)
        out = C.c_double()
        self._ck(self.lib.adscf_forward(self.h, L.dptr(w), C.byref(out)))
        return out.value

    def set_box(self, size):
        """New box side lengths (bulk); fields and mixing history are kept."""
        self._ck(self.lib.adscf_set_box(self.h, *map(float, size)))
        self.params.sizex, self.params.sizey, self.params.sizez = size

    def free_energy_fp64(self):
        """FP64 free energy at the current SCF field (IterResult); on a split
        context this is the polished value at a converged field."""
        res = L.IterResult()
        self._ck(self.lib.adscf_free_energy_fp64(self.h, C.byref(res)))
        return res

    # -- DDFT (bulk) ------------------------------------------------------
    def ddft_set_mobility(self, table, dq, wcutoff):
        """Mobilities from input_mobilities rows: table [nq][3] (AA, AB, BB)."""
        t = _f64(table)
        self._ck(self.lib.adscf_ddft_set_mobility(self.h, int(t.size // 3), float(dq), L.dptr(t),
                                                  float(wcutoff)))

    def ddft_rhs(self, mu):
        """d rho / dt for mu [2][npts] (the k-space part of the DDFT step)."""
        m = _f64(mu, 2 * self.npts)
        out = np.empty(2 * self.npts)
        self._ck(self.lib.adscf_ddft_rhs(self.h, L.dptr(m), L.dptr(out)))
        return out.reshape(np.shape(mu))

    def conjugate_fields(self, density, accuracy=1.0e-3, itermax=2000):
        """Get_Conjugate_Fields from the current field: (status, iterations)."""
        d = _f64(density, 2 * self.npts)
        st, it = C.c_int(), C.c_int()
        self._ck(self.lib.adscf_conjugate_fields(self.h, L.dptr(d), float(accuracy), int(itermax),
                                                 C.byref(st), C.byref(it)))
        return st.value, it.value

    def ddft_step(self, density, timestep, floor_density=False, accuracy=1.0e-3, itermax=2000):
        """One DDFT_Timestep_Euler: returns (new density, status)."""
        d = _f64(density, 2 * self.npts).copy()
        st = C.c_int()
        self._ck(self.lib.adscf_ddft_step(self.h, L.dptr(d), float(timestep), int(bool(floor_density)),
                                          float(accuracy), int(itermax), C.byref(st)))
        return d.reshape(np.shape(density)), st.value

    def set_adjoint_checkpoint(self, every):
        """Checkpoint interval of forward/backward (0 off, < 0 ceil(sqrt(Ns)))."""
        self._ck(self.lib.adscf_set_adjoint_checkpoint(self.h, int(every)))

    def backward_surface(self):
        """Films / brushes: (dF/dchi or dF/dww, dF/dU [ntypes][gz+1]) at the
        fields of the last ``forward``."""
        nplanes = self.npts // (self.params.gx * self.params.gy)
        g = np.empty(self.ntypes * nplanes)
        dchi = C.c_double()
        self._ck(self.lib.adscf_backward_surface(self.h, C.byref(dchi), L.dptr(g)))
        return dchi.value, g.reshape(self.ntypes, nplanes)

    def backward(self):
        """(dF/dL_x, dF/dL_y, dF/dL_z, dF/dchi) at the fields of the last
        ``forward`` (reverse-mode adjoint of the discrete chain)."""
        g = np.empty(4)
        self._ck(self.lib.adscf_backward(self.h, L.dptr(g)))
        return g

    def scf_iteration(self, field, density_out=None, inplace=False):
        """One iteration with host buffers (adscf_scf_iteration).  With
        ``inplace`` the float64 C-contiguous ``field`` itself is advanced, so
        a page-locked array is copied by DMA without staging."""
        if inplace:
            if field.dtype != np.float64 or not field.flags.c_contiguous or field.size != self.ntypes * self.npts:
                raise ValueError("inplace needs a C-contiguous float64 field of ntypes * npts values")
            x = field
        else:
            x = _f64(field).copy()
        d = np.empty_like(x) if density_out is None else density_out
        res = L.IterResult()
        self._ck(self.lib.adscf_scf_iteration(self.h, L.dptr(x), L.dptr(d), C.byref(res)))
        return x, d, res


class Batch:
    """Independent instances advanced together (adscf_batch_*).

    ``instances`` is a list of keyword dicts for :func:`make_params`: all
    bulk, or all one-line films (FILM_1D) or brushes, one precision.  Fields
    and densities are lists of [ntypes][planes][gy][gx] arrays, one per
    instance."""

    def __init__(self, instances, lib=None):
        self.lib = lib or L.load()
        self.n = len(instances)
        arr = (L.Params * self.n)()
        self._keep = []
        self.shapes = []
        for i, kw in enumerate(instances):
            kw = dict(kw)
            kw.setdefault("geometry", L.BULK)
            p, keep = make_params(**kw)
            self._keep += keep
            arr[i] = p
            gx, gy, gz = kw.get("grid", (32, 32, 32))
            geom = kw["geometry"]
            if geom == L.BULK:
                self.shapes.append((2, gz, gy, gx))
            else:   # films and brushes carry both walls, planes 0..gz
                self.shapes.append((1 if geom == L.BRUSH else 2, gz + 1, gy, gx))
        h = C.c_void_p()
        rc = self.lib.adscf_batch_create(arr, self.n, C.byref(h))
        if rc != L.ADSCF_OK:
            raise L.AdscfError(rc, self.lib.adscf_status_string(rc).decode())
        self.h = h
        self.offsets = [int(self.lib.adscf_batch_offset(h, i)) for i in range(self.n + 1)]

    def close(self):
        if getattr(self, "h", None):
            self.lib.adscf_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != L.ADSCF_OK:
            detail = self.lib.adscf_batch_last_error(self.h).decode()
            raise L.AdscfError(rc, f"{self.lib.adscf_status_string(rc).decode()} ({detail})")

    def _pack(self, arrays):
        out = np.empty(self.offsets[-1])
        for i, a in enumerate(arrays):
            out[self.offsets[i]:self.offsets[i + 1]] = np.ravel(a)
        return out

    def _unpack(self, flat):
        return [flat[self.offsets[i]:self.offsets[i + 1]].reshape(sh) for i, sh in enumerate(self.shapes)]

    def set_fields(self, fields):
        self._ck(self.lib.adscf_batch_set_fields(self.h, L.dptr(self._pack(fields))))

    def get_fields(self):
        out = np.empty(self.offsets[-1])
        self._ck(self.lib.adscf_batch_get_fields(self.h, L.dptr(out)))
        return self._unpack(out)

    def get_densities(self):
        out = np.empty(self.offsets[-1])
        self._ck(self.lib.adscf_batch_get_densities(self.h, L.dptr(out)))
        return self._unpack(out)

    def scf_run(self, n_iter, tol=-1.0):
        res = (L.IterResult * self.n)()
        self._ck(self.lib.adscf_batch_scf_run(self.h, int(n_iter), float(tol), res))
        return list(res)

    def forward(self, fields):
        """FP64 bulk batch: free energy per chain of every instance at `fields`."""
        F = np.empty(self.n)
        self._ck(self.lib.adscf_batch_forward(self.h, L.dptr(self._pack(fields)), L.dptr(F)))
        return F

    def backward(self):
        """[n][4]: dF/dL_x, dF/dL_y, dF/dL_z, dF/dchi per instance."""
        g = np.empty((self.n, 4))
        self._ck(self.lib.adscf_batch_backward(self.h, L.dptr(g)))
        return g

    def results(self):
        res = (L.IterResult * self.n)()
        self._ck(self.lib.adscf_batch_results(self.h, res))
        return list(res)
