"""CPU restatement (numpy FP64) of the DDFT step of the multiblock driver,
Bulk_3D_FFT/Main_Multiblock/main_multiblock.f90.  Test infrastructure only:
the checker of the GPU build, never called by it.

* mobility_qq        -- Read_Mobilities, :441-506 (half spectrum, as there)
* ddft_rhs           -- the Fourier part of DDFT_Timestep_Euler, :828-861
* get_conjugate_fields -- Get_Conjugate_Fields, :566-640, with Mix_Fields /
                        Mixing_Anderson (mod_iterate.f90:92-150)
* ddft_step_euler    -- DDFT_Timestep_Euler, :794-880
"""
from __future__ import annotations

import numpy as np

from . import bulk as ob
from . import interactions as oi
from . import iterate as oit


def mobility_qq(grid, size, nq, dq, table, wcutoff):
    """mobility_qq[z][y][x(half)][t2][t1] = min(q^2 Lambda(q), wcutoff),
    Lambda from the table rows (row i at q = (i+1) dq) by the reference's
    interpolation (:490-500, including its weights), q = |k|."""
    gx, gy, gz = grid
    table = np.asarray(table, dtype=np.float64).reshape(nq, 3)
    tab = np.zeros((nq, 2, 2))
    tab[:, 0, 0], tab[:, 0, 1], tab[:, 1, 1] = table[:, 0], table[:, 1], table[:, 2]
    tab[:, 1, 0] = tab[:, 0, 1]                                   # :484
    kx = np.array([ob.wavenumbers(gx, size[0])[i] for i in range(gx // 2 + 1)])
    ky = ob.wavenumbers(gy, size[1])
    kz = ob.wavenumbers(gz, size[2])
    out = np.zeros((gz, gy, gx // 2 + 1, 2, 2))
    for z in range(gz):
        for y in range(gy):
            for x in range(gx // 2 + 1):
                qq = kx[x] ** 2 + ky[y] ** 2 + kz[z] ** 2
                q = np.sqrt(qq)
                iq = int(q / dq)
                if iq == 0:
                    m = tab[0] * q / dq
                elif iq >= nq:
                    m = tab[nq - 1]
                else:
                    m = (tab[iq - 1] * (q - iq * dq) + tab[iq] * ((iq + 1) * dq - q)) / dq
                out[z, y, x] = np.minimum(qq * m, wcutoff)
    return out


def ddft_rhs(mu, mob):
    """ddensity = Fourier2Real(-sum_t2 mobility_qq(t2, t1) Real2Fourier(mu_t2))."""
    shape = mu.shape[1:]
    mu_q = np.stack([ob.real2fourier(mu[t]) for t in range(2)])
    dq = np.zeros_like(mu_q)
    for t1 in range(2):
        for t2 in range(2):
            dq[t1] -= mob[..., t2, t1] * mu_q[t2]
    return np.stack([ob.fourier2real(dq[t], shape) for t in range(2)])


def calculate_densities(field, grid, size, ds, blocks, types, ensemble=1, rho=1.0, mu=0.0):
    r = ob.propagate_multiblock(field, grid, size, ds, blocks, types, ensemble=ensemble, rho=rho, mu=mu)
    return r["density_type"]


def get_conjugate_fields(density, field, accuracy, itermax, dens_fn, mixing_dim=10, lam=0.5,
                         lam00=1.0e-3):
    """Returns (field, status, iterations, accuracy).  The residual is
    newdensity - density, the accuracy its max abs (:597-603); iter_status =
    min(iter, mixing_dim + 1) restarts the Anderson warm-up on every call."""
    m = mixing_dim
    nvar = field.size
    var = np.zeros((m + 1, nvar))
    dvar = np.zeros((m + 1, nvar))
    field = field.copy()
    acc = np.nan
    it = 0
    for it in range(1, itermax + 1):
        newdensity = dens_fn(field)
        dfield = newdensity - density
        acc = np.max(np.abs(dfield))
        if not (acc > accuracy * 0.5):
            break
        it_status = min(it, m + 1)
        var[0] = field.reshape(-1)
        dvar[0] = dfield.reshape(-1)
        oit.mixing_anderson(var, dvar, lam, it_status, lam00=lam00)
        field = var[0].reshape(field.shape).copy()
    if not (acc < accuracy * 0.5):
        status = 1 if acc < accuracy else 2
    else:
        status = 0
    return field, status, it, acc


def ddft_step_euler(density, field, mob, timestep, qdmin, kappa, chi, dens_fn, accuracy=1.0e-3,
                    itermax=2000, mixing_dim=10):
    """DDFT_Timestep_Euler: returns (density, field, status)."""
    field, _st, _it, _acc = get_conjugate_fields(density, field, accuracy, itermax, dens_fn, mixing_dim)
    mulocal = oi.mean_fields(density, kappa, chi) - field
    ddensity = ddft_rhs(mulocal, mob)
    density = density + timestep * ddensity
    if qdmin and density.min() <= 1.0e-4:
        density = np.maximum(density, 1.0e-4)
    field, st, _it, _acc = get_conjugate_fields(density, field, accuracy, itermax, dens_fn, mixing_dim)
    if qdmin and st >= 1:
        density = dens_fn(field)
    return density, field, st
