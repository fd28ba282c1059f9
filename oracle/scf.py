"""SCF loop restatement (FP64) -- test infrastructure.

Calculate_Saddle_Point loop body, Bulk_3D_FFT/Main_Diblock_Melt/
main_diblock.f90:410-429: densities of the current field, Check_Accuracy
(:380-390), Calculate_Mean_Fields, dfield = newfield - field, Mix_Fields,
density = newdensity.  The free energy per chain reported for iterate k is
[chain energy - dvol sum(phi_new * w_k) + Interaction_Energy(phi_new)]/(rho V)
(Calculate_Energy, main_diblock.f90:295-307, evaluated at the iterate).
"""
from __future__ import annotations

import numpy as np

from . import bulk, interactions, iterate


def bulk_scf(field, n_iter, grid, size, ds, block_length, kappa, chi,
             mixing_type=2, lam=0.1, m=2, lam00=1.0e-3, warm=None,
             ensemble=1, rho=1.0, mu=0.0, density0=None, vol=(1.0, 1.0),
             gram=False, stop_accuracy=None):
    field = np.array(field, dtype=np.float64, copy=True)
    density = np.zeros_like(field) if density0 is None else np.array(density0, dtype=np.float64)
    mixer = iterate.Mixer(field.size, mixing_type, lam, m=m, lam00=lam00, warm=warm,
                          gram=gram)
    hist = []
    for it in range(1, n_iter + 1):
        r = bulk.propagate_diblock(field, grid, size, ds, block_length,
                                   ensemble=ensemble, rho=rho, mu=mu)
        newdensity = bulk.density_by_type(r["density"])
        acc = interactions.check_accuracy(density, newdensity)
        newfield = interactions.mean_fields(newdensity, kappa, chi, vol)
        dvol = r["dvol"]
        eint = interactions.interaction_energy(newdensity, kappa, chi, dvol, vol)
        phiw = dvol * np.sum(newdensity * field)
        volume = r["volume"]
        rho_now = r["rho"]
        F = (r["energy"] - phiw + eint) / (rho_now * volume)
        hist.append(dict(iter=it, accuracy=acc, F=F, Qsum=r["Qsum"], mu=r["mu"],
                         density=newdensity, field=field.copy()))
        dfield = newfield - field
        field = mixer(field, dfield, it)
        density = newdensity
        if stop_accuracy is not None and not acc > stop_accuracy:
            break
    return field, hist


def film_scf(field, n_iter, dz, dss, n_a, step, kappa, chi, surface, sizes,
             int_scheme=1, span="full", mixing_type=2, lam=0.1, m=2,
             lam00=1.0e-3, warm=None, rho=1.0, density0=None, gram=True, ensemble=1, mu=0.0):
    """Film SCF loop, Film_CK_AD/Film_1D/Main_Diblock_Melt/main_diblock_melt.f90:
    155-169: densities (film Propagate_Diblock), Check_Accuracy over all
    planes, Calculate_Mean_Ext_Fields with the wall potential ``surface``
    ([2][0:gz]), and Mix_Fields over the interior planes 1..gz-1 only
    (:362-378).  ``step(prop, w, ds)`` is the geometry's propagator step."""
    from . import film
    field = np.array(field, dtype=np.float64, copy=True)
    density = np.zeros_like(field) if density0 is None else np.array(density0, dtype=np.float64)
    gz = dz.shape[0] - 1
    interior = (slice(None), slice(1, gz))
    nvar = field[interior].size
    mixer = iterate.Mixer(nvar, mixing_type, lam, m=m, lam00=lam00, warm=warm, gram=gram)
    dx = sizes[0] / (field.shape[-1] if field.ndim == 4 else 1)
    dy = sizes[1] / (field.shape[-2] if field.ndim == 4 else 1)
    ext = (slice(None), slice(None)) + (None,) * (field.ndim - 2)
    hist = []
    for it in range(1, n_iter + 1):
        r = film.film_propagate_diblock(field, dz, dss, n_a, step, rho=rho, dx=dx, dy=dy,
                                        int_scheme=int_scheme, span=span, sizes=sizes,
                                        ensemble=ensemble, mu=mu)
        newdensity = r["density"]
        acc = interactions.check_accuracy(density, newdensity)
        newfield = interactions.mean_fields(newdensity, kappa, chi, surface=surface[ext])
        hist.append(dict(iter=it, accuracy=acc, Qsum=r["Qsum"], density=newdensity,
                         field=field.copy()))
        dfield = newfield - field
        x = mixer(field[interior].copy(), dfield[interior].copy(), it)
        field[interior] = x
        density = newdensity
    return field, hist
