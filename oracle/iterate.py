"""Field mixing restatement (FP64) -- test infrastructure.

Follows Bulk_3D_FFT/General_Routines/mod_iterate.f90 (the four copies in
the reference tree are identical).  History arrays have the reference's
shape ``(fieldsize, 0:mixing_dim)`` stored here as ``[m+1][fieldsize]``.

The reference's ``Mix_Fields`` keeps the history in non-SAVEd locals
(main_diblock.f90:328); this restatement keeps it persistent, which is what
the algorithm needs to be defined.
"""
from __future__ import annotations

import numpy as np


def mixing_simple(field, dfield, lam, it):
    """Mixing_Simple, mod_iterate.f90:27-38."""
    field[0] = field[0] + lam * dfield[0]


def mixing_lambda(field, dfield, lammax, it, lammin=1.0e-5):
    """Mixing_Lambda, mod_iterate.f90:46-84."""
    if it == 1:
        lam = lammin
    else:
        num = np.sum((field[0] - field[1]) ** 2)
        nom = np.sum((dfield[0] - dfield[1]) ** 2)
        if nom > 1.0e-50:
            lam = np.sqrt(num / nom)
            if lam < lammin:
                lam = lammin
            elif lam > lammax:
                lam = lammax
        else:
            lam = lammin
    field[1] = field[0]
    dfield[1] = dfield[0]
    field[0] = field[0] + lam * dfield[0]
    return lam


def ludcmp(a):
    """ludcmp (Crout with implicit partial pivoting), mod_iterate.f90:232-298.
    Operates on a copy; returns (lu, indx, d) with 0-based indx."""
    a = np.array(a, dtype=np.float64, copy=True)
    n = a.shape[0]
    tiny = 1.0e-20
    indx = np.zeros(n, dtype=np.int64)
    vv = np.zeros(n)
    d = 1.0
    for i in range(n):
        aamax = np.max(np.abs(a[i, :]))
        vv[i] = 1.0 / aamax if aamax != 0.0 else np.inf
    for j in range(n):
        for i in range(j):
            dsum = a[i, j]
            for k in range(i):
                dsum -= a[i, k] * a[k, j]
            a[i, j] = dsum
        aamax = 0.0
        imax = j
        for i in range(j, n):
            dsum = a[i, j]
            for k in range(j):
                dsum -= a[i, k] * a[k, j]
            a[i, j] = dsum
            dum = vv[i] * abs(dsum)
            if dum >= aamax:
                imax = i
                aamax = dum
        if j != imax:
            a[[imax, j], :] = a[[j, imax], :]
            d = -d
            vv[imax] = vv[j]
        indx[j] = imax
        if a[j, j] == 0.0:
            a[j, j] = tiny
        if j != n - 1:
            a[j + 1:, j] *= 1.0 / a[j, j]
    return a, indx, d


def lubksb(a, indx, b):
    """lubksb, mod_iterate.f90:302-337."""
    b = np.array(b, dtype=np.float64, copy=True)
    n = a.shape[0]
    ii = -1
    for i in range(n):
        ll = indx[i]
        dsum = b[ll]
        b[ll] = b[i]
        if ii >= 0:
            for j in range(ii, i):
                dsum -= a[i, j] * b[j]
        elif dsum != 0.0:
            ii = i
        b[i] = dsum
    for i in range(n - 1, -1, -1):
        dsum = b[i]
        for j in range(i + 1, n):
            dsum -= a[i, j] * b[j]
        b[i] = dsum / a[i, i]
    return b


def solve_linear_system_lu(a, b):
    """Solve_LinearSystem_LU, mod_iterate.f90:203-224."""
    lu, indx, _ = ludcmp(a)
    return lubksb(lu, indx, b)


def mixing_anderson(field, dfield, lam_mix, it, lam00=1.0e-3, warm=None,
                    gram=False):
    """Mixing_Anderson, mod_iterate.f90:92-150, with the history depth m
    taken from the arrays (the reference fixes m = mixing_dim = 2, :13).

    ``warm`` generalises the reference's ``iter > mixing_dim`` switch (:110)
    to ``iter > warm`` (default warm = m) so a longer simple-mixing warm-up
    with step ``lam00`` can be requested; warm must be >= m.

    gram=True forms the same U and v from the Gram matrix of the residuals,
    U_ij = G00 - G0i - G0j + Gij, v_i = G00 - G0i (G_ab = <r_a, r_b>): equal
    in exact arithmetic, it is the form the GPU evaluates."""
    m = field.shape[0] - 1
    if warm is None:
        warm = m
    coeffs = None
    if it > warm:
        ddiff = dfield[0][None, :] - dfield[1:]                     # :112-114
        if gram:
            G = dfield @ dfield.T
            v = G[0, 0] - G[0, 1:]
            u = G[0, 0] - G[0, 1:][:, None] - G[0, 1:][None, :] + G[1:, 1:]
        else:
            v = ddiff @ dfield[0]                                   # :117
            u = ddiff @ ddiff.T                                     # :119
        coeffs = solve_linear_system_lu(u, v)                       # :123
        field_mix = field[0].copy()
        dfield_mix = dfield[0].copy()
        for i in range(m):                                          # :127-130
            field_mix = field_mix - coeffs[i] * (field[0] - field[i + 1])
            dfield_mix = dfield_mix - coeffs[i] * ddiff[i]
        lam = lam_mix
    else:
        field_mix = field[0].copy()
        dfield_mix = dfield[0].copy()
        lam = lam00
    for i in range(m, 0, -1):                                       # :143-146
        field[i] = field[i - 1]
        dfield[i] = dfield[i - 1]
    field[0] = field_mix + lam * dfield_mix                         # :148
    return coeffs


class Mixer:
    """Persistent-history driver for the three mixing routines, mirroring
    Mix_Fields (main_diblock.f90:315-372) with SAVEd var/dvar."""

    def __init__(self, nvar, mixing_type, lam, m=2, lam00=1.0e-3, warm=None,
                 gram=False):
        self.type = mixing_type
        self.lam = lam
        self.m = m if mixing_type == 3 else 1
        self.var = np.zeros((self.m + 1, nvar))
        self.dvar = np.zeros((self.m + 1, nvar))
        self.lam00 = lam00
        self.warm = warm
        self.gram = gram

    def __call__(self, field, dfield, it):
        self.var[0] = field.reshape(-1)
        self.dvar[0] = dfield.reshape(-1)
        if self.type == 1:
            mixing_simple(self.var, self.dvar, self.lam, it)
        elif self.type == 2:
            mixing_lambda(self.var, self.dvar, self.lam, it)
        elif self.type == 3:
            mixing_anderson(self.var, self.dvar, self.lam, it, self.lam00,
                            self.warm, self.gram)
        else:
            raise ValueError("Invalid mixing option")
        return self.var[0].reshape(field.shape).copy()
