"""Bulk pseudo-spectral SCF restatement (FP64, numpy) -- test infrastructure.

Follows Bulk_3D_FFT/Geometry_Modules/Bulk/mod_fourier.f90,
Bulk_3D_FFT/General_Routines/mod_propagate.f90 and
Bulk_3D_FFT/Polymer_Modules/mod_diblock.f90.  Arrays are C-ordered
``[z][y][x]`` (Fortran ``(x,y,z)``); the halved r2c axis is x, the last axis,
exactly as FFTW's Fortran interface halves the first Fortran axis.
"""
from __future__ import annotations

import numpy as np


def volume_parameters(grid, size):
    """Calculate_Volume_Parameters, mod_fourier.f90:152-157."""
    gx, gy, gz = grid
    volume = size[0] * size[1] * size[2]
    return volume, volume / float(gx * gy * gz)


def wavenumbers(n, length):
    """Signed wave numbers 2*pi*m/L with the wrap of mod_fourier.f90:178-186.

    0-based index m > n/2 maps to m - n (Fortran: y > gridy/2+1)."""
    m = np.arange(n, dtype=np.float64)
    m = np.where(m > n // 2, m - n, m)
    return 2.0 * np.pi * m / length


def calculate_laplace(grid, size, ds):
    """Calculate_Laplace, mod_fourier.f90:165-198: explaplace = exp(-ds q^2)
    on the r2c half spectrum, shape [gz][gy][gx//2+1]."""
    gx, gy, gz = grid
    qx = 2.0 * np.pi * np.arange(gx // 2 + 1, dtype=np.float64) / size[0]
    qy = wavenumbers(gy, size[1])
    qz = wavenumbers(gz, size[2])
    q2 = qz[:, None, None] ** 2 + qy[None, :, None] ** 2 + qx[None, None, :] ** 2
    return np.exp(-ds * q2)


def real2fourier(prop):
    """Real2Fourier, mod_fourier.f90:94-105 (r2c scaled by 1/N, :102)."""
    return np.fft.rfftn(prop) / prop.size


def fourier2real(propfourier, shape):
    """Fourier2Real, mod_fourier.f90:75-86 (unnormalised c2r)."""
    return np.fft.irfftn(propfourier, s=shape, axes=tuple(range(-len(shape), 0))) * float(np.prod(shape))


def calculate_expfield(field, ds):
    """Calculate_Expfield, mod_propagate.f90:22-32: exp(-0.5 ds w)."""
    return np.exp(-0.5 * ds * field)


def propagate_step(prop, expfield, explaplace):
    """Propagate_Step, mod_propagate.f90:40-68 (Strang split, :56-64)."""
    prop = expfield * prop
    pf = real2fourier(prop)
    pf = explaplace * pf
    prop = fourier2real(pf, prop.shape)
    return expfield * prop


def block_segments(block_length, ds):
    """Initialize_Diblock, mod_diblock.f90:74-75: nint(f/ds) (round half
    away from zero, as Fortran nint)."""
    out = []
    for f in block_length:
        x = f / ds
        out.append(int(np.floor(x + 0.5)) if x >= 0 else -int(np.floor(-x + 0.5)))
    return out


def propagate_diblock(field, grid, size, ds, block_length, ensemble=1, rho=1.0,
                      mu=0.0, monomer_type=(0, 1), keep_chains=False):
    """Propagate_Diblock, mod_diblock.f90:100-173.

    field: [2][gz][gy][gx] FP64 (monomer types 0=A, 1=B).
    ensemble 1 = canonical, 2 = grand canonical (mod_diblock.f90:156-167).
    Returns a dict with Qsum, distribution[block], density[block], mu, rho,
    energy and (optionally) the stored chains qq, qqdag [0..segments].
    """
    volume, dvol = volume_parameters(grid, size)
    shape = field.shape[1:]
    explaplace = calculate_laplace(grid, size, ds)
    expfield = calculate_expfield(field, ds)
    nseg = block_segments(block_length, ds)
    segments = sum(nseg)
    qq = np.empty((segments + 1,) + shape)
    qqdag = np.empty((segments + 1,) + shape)
    # forward chain, mod_diblock.f90:116-126
    prop = np.ones(shape)
    qq[0] = prop
    s0 = 0
    for block in range(2):
        e = expfield[monomer_type[block]]
        for s in range(s0 + 1, s0 + nseg[block] + 1):
            prop = propagate_step(prop, e, explaplace)
            qq[s] = prop
        s0 += nseg[block]
    # backward chain, mod_diblock.f90:128-138
    prop = np.ones(shape)
    qqdag[0] = prop
    s0 = 0
    for block in (1, 0):
        e = expfield[monomer_type[block]]
        for s in range(s0 + 1, s0 + nseg[block] + 1):
            prop = propagate_step(prop, e, explaplace)
            qqdag[s] = prop
        s0 += nseg[block]
    mono = segments
    qsum = dvol * qq[mono].sum()                       # :141
    dist = np.zeros((2,) + shape)
    s0 = 0
    for block in range(2):                              # :143-154
        d = 0.5 * ds * qq[s0] * qqdag[mono - s0]
        for s in range(s0 + 1, s0 + nseg[block]):
            d = d + ds * qq[s] * qqdag[mono - s]
        s0 += nseg[block]
        d = d + 0.5 * ds * qq[s0] * qqdag[mono - s0]
        dist[block] = d
    out = dict(Qsum=qsum, distribution=dist, segments=segments,
               block_segments=nseg, volume=volume, dvol=dvol)
    if ensemble == 1:                                   # :156-159
        out["density"] = rho * volume * dist / qsum
        out["mu"] = np.log(rho * volume / qsum)
        out["rho"] = rho
        out["energy"] = rho * volume * (out["mu"] - 1.0)
    elif ensemble == 2:                                 # :160-163
        out["density"] = np.exp(mu) * dist
        out["mu"] = mu
        out["rho"] = out["density"].sum() * dvol / volume / (ds * segments)
        out["energy"] = -out["rho"] * volume
    else:
        raise ValueError("Invalid ensemble")
    if keep_chains:
        out["qq"] = qq
        out["qqdag"] = qqdag
    return out


def propagate_multiblock(field, grid, size, ds, blocks, types, ensemble=1, rho=1.0, mu=0.0):
    """Propagate_Multiblock, Bulk_3D_FFT/Polymer_Modules/mod_multiblock.f90:112-180
    (Propagate_Triblock, mod_triblock.f90:103-170, is the same loop with three
    blocks), followed by the driver's sum of block densities by monomer type
    (Calculate_Densities, Main_Multiblock/main_multiblock.f90:531-536).

    blocks: block lengths; types: monomer type per block (0 = A, 1 = B);
    block segments nint(length / ds) (mod_multiblock.f90:80).  Returns a dict
    with Qsum, distribution[block], density[block], density_type[type], mu,
    rho and energy.
    """
    volume, dvol = volume_parameters(grid, size)
    shape = field.shape[1:]
    explaplace = calculate_laplace(grid, size, ds)
    expfield = calculate_expfield(field, ds)
    nseg = [int(np.floor(b / ds + 0.5)) for b in blocks]
    segments = sum(nseg)
    nb = len(blocks)
    qq = np.empty((segments + 1,) + shape)
    qqdag = np.empty((segments + 1,) + shape)
    prop = np.ones(shape)                               # :127-137
    qq[0] = prop
    s0 = 0
    for k in range(nb):
        for s in range(s0 + 1, s0 + nseg[k] + 1):
            prop = propagate_step(prop, expfield[types[k]], explaplace)
            qq[s] = prop
        s0 += nseg[k]
    prop = np.ones(shape)                               # :139-149
    qqdag[0] = prop
    s0 = 0
    for k in range(nb - 1, -1, -1):
        for s in range(s0 + 1, s0 + nseg[k] + 1):
            prop = propagate_step(prop, expfield[types[k]], explaplace)
            qqdag[s] = prop
        s0 += nseg[k]
    mono = segments
    qsum = dvol * qq[mono].sum()                        # :152
    dist = np.zeros((nb,) + shape)
    s0 = 0
    for k in range(nb):                                 # :154-165
        d = 0.5 * ds * qq[s0] * qqdag[mono - s0]
        for s in range(s0 + 1, s0 + nseg[k]):
            d = d + ds * qq[s] * qqdag[mono - s]
        s0 += nseg[k]
        dist[k] = d + 0.5 * ds * qq[s0] * qqdag[mono - s0]
    out = dict(Qsum=qsum, distribution=dist, segments=segments, block_segments=nseg,
               volume=volume, dvol=dvol)
    if ensemble == 1:                                   # :170-173
        out["density"] = rho * volume * dist / qsum
        out["mu"] = np.log(rho * volume / qsum)
        out["rho"] = rho
        out["energy"] = rho * volume * (out["mu"] - 1.0)
    elif ensemble == 2:                                 # :174-177
        out["density"] = np.exp(mu) * dist
        out["mu"] = mu
        out["rho"] = out["density"].sum() * dvol / volume / (ds * segments)
        out["energy"] = -out["rho"] * volume
    else:
        raise ValueError("Invalid ensemble")
    dt = np.zeros((2,) + shape)
    for k in range(nb):
        dt[types[k]] += out["density"][k]
    out["density_type"] = dt
    return out


def density_by_type(blk_density, monomer_type=(0, 1)):
    """Calculate_Densities, main_diblock.f90:277-283: block -> monomer type."""
    dens = np.zeros_like(blk_density)
    for i in range(2):
        dens[monomer_type[i]] += blk_density[i]
    return dens


def update_solvent(field, grid, size, ensemble, rho=1.0, mu=0.0):
    """Update_Solvent, Bulk_3D_FFT/Polymer_Modules/mod_solvent.f90:85-110.

    distribution = exp(-field), Qsum = dvol * sum; canonical (1):
    density = rho V dist / Qsum, mu = log(rho V / Qsum), energy = rho V (mu - 1);
    grand canonical (2): density = exp(mu) dist, rho = sum(density) dvol / V,
    energy = -rho V."""
    volume, dvol = volume_parameters(grid, size)
    dist = np.exp(-np.asarray(field, dtype=np.float64))
    qsum = dvol * dist.sum()
    if ensemble == 1:
        density = rho * volume * dist / qsum
        mu = np.log(rho * volume / qsum)
        energy = rho * volume * (mu - 1.0)
    elif ensemble == 2:
        density = np.exp(mu) * dist
        rho = density.sum() * dvol / volume
        energy = -rho * volume
    else:
        raise ValueError("Invalid ensemble; Cannot calculate Density")
    return {"distribution": dist, "Qsum": qsum, "density": density, "mu": mu, "rho": rho,
            "energy": energy}
