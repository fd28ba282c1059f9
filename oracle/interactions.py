"""Interaction restatement (FP64) -- test infrastructure.

Helfand-compressible Flory-Huggins model of
Bulk_3D_FFT/Interaction_Modules/mod_FloryHuggins.f90 and its film variant
with a wall potential, Film_CK_AD/Film_1D/Interaction_Modules/
mod_FloryHuggins.f90, plus the brush model of
Brush_CK_AD/Interaction_Modules/mod_virial_expansion.f90.
"""
from __future__ import annotations

import numpy as np


def chi_matrix(chi):
    """Initialize_Interactions, mod_FloryHuggins.f90:49-55 (two components)."""
    return np.array([[0.0, chi], [chi, 0.0]])


def mean_fields(density, kappa, chi, vol=(1.0, 1.0), surface=None):
    """Calculate_Mean_Fields, mod_FloryHuggins.f90:104-129; with ``surface``
    ([2][...] broadcastable) it is Calculate_Mean_Ext_Fields,
    Film_1D/Interaction_Modules/mod_FloryHuggins.f90:140-167."""
    chim = chi_matrix(chi)
    vf = np.stack([density[c] * vol[c] for c in range(2)])
    tot = vf.sum(axis=0)
    field = np.empty_like(density)
    for c in range(2):
        f = kappa * (tot - 1.0)
        for c2 in range(2):
            f = f + chim[c, c2] * vf[c2]
        if surface is not None:
            f = f + surface[c]
        field[c] = f * vol[c]
    return field


def interaction_energy(density, kappa, chi, dvol, vol=(1.0, 1.0)):
    """Interaction_Energy, mod_FloryHuggins.f90:74-96."""
    vf = np.stack([density[c] * vol[c] for c in range(2)])
    tot = vf.sum(axis=0)
    e = 0.5 * kappa * dvol * np.sum((tot - 1.0) ** 2)
    e += chi * dvol * np.sum(vf[0] * vf[1])
    return e


def check_accuracy(density, newdensity):
    """Check_Accuracy, main_diblock.f90:380-390."""
    return float(np.sum((density - newdensity) * (density - newdensity)))


def wall_potential_shape(zr, sizez, delta_z, walls=(True, True)):
    """Shape 1+cos(pi z/delta) within delta_z of a wall.

    Film: Calculate_Potential, Film_1D/.../mod_FloryHuggins.f90:203-226
    (interior points 1..gz-1, both walls).  Brush: mod_virial_expansion.f90:
    174-204 selects walls with ``wall_scheme``; pass ``walls`` accordingly."""
    gz = len(zr) - 1
    shape = np.zeros(gz + 1)
    z0 = sizez - delta_z
    for i in range(1, gz):
        if zr[i] <= delta_z and walls[0]:
            shape[i] = 1.0 + np.cos(np.pi * zr[i] / delta_z)
        elif zr[i] >= z0 and walls[1]:
            shape[i] = 1.0 + np.cos(np.pi * (sizez - zr[i]) / delta_z)
    return shape


def brush_mean_field(density, ww, surface):
    """Calculate_Mean_Ext_Fields, mod_virial_expansion.f90:111-137."""
    return ww * density + surface
