"""Host-side meshes, contour schedules and wall potentials for film and brush
contexts (the inputs a driver passes in ``adscf_params``: ``dz``, ``dss``,
``ext_potential``).

* ``generate_mesh`` -- generate_mesh, Film_CK_AD/Film_3D/Geometry_Modules/
  mod_realspace.f90:222-265 and its Film_1D variant (:155-198): uniform,
  cosine and wall-refined step meshes.
* ``tanh_mesh`` -- a wall-clustered z_i = D/2 (1 + tanh(a(2i/gz - 1))/tanh a)
  mesh, handed to the reference as an explicit dz array.
* ``contour_steps`` -- the dss schedules of Initialize_Homopolymer,
  Brush_CK_AD/Polymer_Modules/mod_homopolymer.f90:98-115 (uniform,
  half-cosine, quarter-cosine), normalised to a unit chain.
* ``wall_potential`` -- Calculate_Potential, Film_CK_AD/Film_1D/
  Interaction_Modules/mod_FloryHuggins.f90:203-226: amplitude times
  1 + cos(pi d / delta) within delta of a wall, on interior planes.

Every mesh is returned as (dz, zr) with dz[0] = 0 and dz[i] = zr[i] - zr[i-1].
"""
from __future__ import annotations

import numpy as np


def _dz(zr):
    zr = np.asarray(zr, dtype=np.float64)
    dz = np.empty_like(zr)
    dz[0] = 0.0
    dz[1:] = zr[1:] - zr[:-1]
    return dz


def generate_mesh(mesh_type, gz, sizez, delta_z=0.2, film3d=True):
    """mesh_type 0 uniform, 1 cosine, 2 wall-refined steps (the Film_3D rule
    when ``film3d``, else the Film_1D rule)."""
    i = np.arange(gz + 1, dtype=np.float64)
    if mesh_type == 0:
        h = sizez / gz
        return _dz(i * h), i * h
    if mesh_type == 1:
        zr = 0.5 * sizez * (1.0 - np.cos(np.pi * i / gz))
        zr[0] = 0.0
        return _dz(zr), zr
    if mesh_type != 2:
        raise ValueError("mesh_type must be 0, 1 or 2")
    steps = np.zeros(gz + 1)
    if film3d:
        ns_ = 20                                       # planes refined per wall
        h_s = delta_z / ns_
        h_b = (0.5 * sizez - delta_z) / (0.5 * gz - ns_)
        # the Film_3D rule tests the plane index against delta_z, so planes
        # ns_ < i <= delta_z (none for delta_z < ns_) take no step
        for k in range(1, gz + 1):
            if k <= ns_ or k > gz - ns_:
                steps[k] = h_s
            elif k > delta_z:
                steps[k] = h_b
    else:
        ns_ = int((0.8 - 0.2 * (gz - 100) / 2000.0) * gz / 2)
        h_s = delta_z / ns_
        h_b = (sizez - 2.0 * delta_z) / (gz - 2 * ns_)
        k = np.arange(gz + 1)
        steps = np.where((k <= ns_) | (k > gz - ns_), h_s, h_b)
        steps[0] = 0.0
    zr = np.cumsum(steps)
    return _dz(zr), zr


def tanh_mesh(gz, thickness, stretch=2.0):
    """Wall-clustered tanh mesh with both wall planes exact."""
    x = 2.0 * np.arange(gz + 1, dtype=np.float64) / gz - 1.0
    zr = 0.5 * thickness * (1.0 + np.tanh(stretch * x) / np.tanh(stretch))
    zr[0], zr[-1] = 0.0, thickness
    return _dz(zr), zr


def contour_steps(ns, ds_scheme=0):
    """dss[0..ns], dss[0] = 0, summing to 1: 0 uniform, 1 half-cosine
    (refined at both chain ends), 2 quarter-cosine (refined at s = 0)."""
    s = np.arange(ns + 1, dtype=np.float64)
    if ds_scheme == 0:
        c = s / ns
    elif ds_scheme == 1:
        c = 0.5 * (1.0 - np.cos(np.pi * s / ns))
    elif ds_scheme == 2:
        c = 1.0 - np.cos(0.5 * np.pi * s / ns)
    else:
        raise ValueError("ds_scheme must be 0, 1 or 2")
    dss = np.zeros(ns + 1)
    dss[1:] = np.diff(c)
    dss[1:] /= dss[1:].sum()
    return dss


def wall_potential(zr, sizez, delta_z, amplitudes, walls=(True, True)):
    """[len(amplitudes)][gz+1] wall potential: amplitude_c times the shape
    1 + cos(pi d / delta_z) at distance d < delta_z from an enabled wall,
    on the interior planes 1..gz-1 (zero on the wall planes)."""
    zr = np.asarray(zr, dtype=np.float64)
    shape = np.zeros_like(zr)
    inner = np.zeros_like(zr, dtype=bool)
    inner[1:-1] = True
    lo = inner & (zr <= delta_z) if walls[0] else np.zeros_like(inner)
    hi = inner & ~lo & (zr >= sizez - delta_z) if walls[1] else np.zeros_like(inner)
    shape[lo] = 1.0 + np.cos(np.pi * zr[lo] / delta_z)
    shape[hi] = 1.0 + np.cos(np.pi * (sizez - zr[hi]) / delta_z)
    return np.stack([a * shape for a in amplitudes])
