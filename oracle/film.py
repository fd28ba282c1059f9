"""Real-space Crank-Nicolson / ADI restatement (FP64) -- test infrastructure.

Follows
  Film_CK_AD/Film_1D/Geometry_Modules/mod_realspace.f90   (1D CN, tridiag)
  Film_CK_AD/Film_3D/Geometry_Modules/mod_realspace.f90   (Douglas ADI,
                                                           cyclicTriDiag)
  Film_CK_AD/Film_{1D,3D}/Polymer_Modules/mod_diblock.f90 (film diblock)
  Brush_CK_AD/Geometry_Modules/mod_realspace.f90          (CN, per-call ds)
  Brush_CK_AD/Adaptive_Modules/mod_adaptive.f90           (meshes)
  Brush_CK_AD/Polymer_Modules/mod_homopolymer.f90         (adaptive contour)

Films are C-ordered ``[z][y][x]`` with z = 0..gz including both wall
planes, as the reference's ``(gridx, gridy, 0:gridz)``.  Line solves are
vectorised over all (x, y) lines; the recurrences run over z.
"""
from __future__ import annotations

import numpy as np


# ----------------------------------------------------------------------------
# tridiagonal solvers
# ----------------------------------------------------------------------------
def tridiag_nr(a, b, c, r):
    """Thomas solve, NR form, Film_3D/.../mod_realspace.f90:184-215.

    a: sub-diagonal (a[j] couples row j to j-1), b: diagonal, c: super-
    diagonal (c[j] couples row j to j+1); trailing axes are independent
    lines.  Raises ZeroDivisionError on a zero pivot (the reference stops,
    :194-207)."""
    n = b.shape[0]
    u = np.empty(np.broadcast(a, b, c, r).shape)
    gam = np.empty_like(u)
    bet = np.broadcast_to(b[0], u.shape[1:]).astype(np.float64)
    if np.any(bet == 0.0):
        raise ZeroDivisionError("TriDiag Error")
    u[0] = r[0] / bet
    for j in range(1, n):
        gam[j] = c[j - 1] / bet
        bet = b[j] - a[j] * gam[j]
        if np.any(bet == 0.0):
            raise ZeroDivisionError("TriDiag Error")
        u[j] = (r[j] - a[j] * u[j - 1]) / bet
    for j in range(n - 2, -1, -1):
        u[j] = u[j] - gam[j + 1] * u[j + 1]
    return u


def tridiag_inplace(a, b, c, r):
    """Thomas solve, in-place variant of Film_1D/.../mod_realspace.f90:
    120-148 (mutates copies of b and r, :137-141)."""
    b = np.array(np.broadcast_to(b, np.broadcast(a, b, c, r).shape), dtype=np.float64)
    r = np.array(np.broadcast_to(r, b.shape), dtype=np.float64)
    n = b.shape[0]
    if np.any(b[0] == 0.0):
        raise ZeroDivisionError("TriDiag Error")
    u = np.empty_like(b)
    for j in range(1, n):
        gam = a[j] / b[j - 1]
        b[j] = b[j] - c[j - 1] * gam
        r[j] = r[j] - r[j - 1] * gam
    u[n - 1] = r[n - 1] / b[n - 1]
    for j in range(n - 2, -1, -1):
        u[j] = (r[j] - u[j + 1] * c[j]) / b[j]
    return u


def cyclic_tridiag(a, b, c, r):
    """Sherman-Morrison periodic solve, Film_3D/.../mod_realspace.f90:
    149-176, with the N<3 fallback of :157-158.  Corner elements are
    m(1,N) = a(1) and m(N,1) = c(N)."""
    n = b.shape[0]
    shp = np.broadcast(a, b, c, r).shape
    if n < 3:
        x = np.broadcast_to(r[0] / (b[0] + a[0] + c[0]), shp[1:])
        return np.broadcast_to(x, shp).copy()
    gamma = -b[0]
    bb = np.array(np.broadcast_to(b, shp), dtype=np.float64)
    bb[0] = b[0] - gamma
    bb[n - 1] = b[n - 1] - a[0] * c[n - 1] / gamma
    y = tridiag_nr(a, bb, c, r)
    u = np.zeros(shp)
    u[0] = gamma
    u[n - 1] = c[n - 1]
    q = tridiag_nr(a, bb, c, u)
    fact = (y[0] + a[0] * y[n - 1] / gamma) / (1.0 + q[0] + a[0] * q[n - 1] / gamma)
    return y - fact * q


# ----------------------------------------------------------------------------
# meshes and integrators
# ----------------------------------------------------------------------------
def mesh_from_zr(zr):
    """dz(i) = zr(i) - zr(i-1), dz(0) = 0 (generate_mesh convention)."""
    zr = np.asarray(zr, dtype=np.float64)
    dz = np.zeros_like(zr)
    dz[1:] = np.diff(zr)
    return dz


def generate_mesh(mesh_type, gz, sizez, delta_z=0.2, film3d=True):
    """generate_mesh, Film_3D/.../mod_realspace.f90:222-265 (film3d=True)
    or Film_1D/.../mod_realspace.f90:155-198.  Returns (dz, zr)."""
    dz = np.zeros(gz + 1)
    zr = np.zeros(gz + 1)
    if mesh_type == 0:                                   # uniform
        dz[:] = sizez / gz
        dz[0] = 0.0
        zr = np.arange(gz + 1) * dz
        zr[0] = 0.0
    elif mesh_type == 1:                                 # cosine
        for i in range(1, gz + 1):
            zr[i] = sizez * 0.5 * (1.0 - np.cos(np.pi * i / gz))
            dz[i] = zr[i] - zr[i - 1]
    elif mesh_type == 2:                                 # step function
        if film3d:
            grid_surf = 20
            dz_surf = delta_z / grid_surf
            dz_bulk = (sizez / 2.0 - delta_z) / (gz / 2.0 - grid_surf)
            for i in range(1, gz + 1):
                if i <= grid_surf:
                    zr[i] = zr[i - 1] + dz_surf
                elif i > delta_z and i <= gz - grid_surf:
                    zr[i] = zr[i - 1] + dz_bulk
                elif i > gz - grid_surf:
                    zr[i] = zr[i - 1] + dz_surf
                dz[i] = zr[i] - zr[i - 1]
        else:
            grid_surf = int((0.8 - 0.2 * (gz - 100) / 2000.0) * gz / 2)
            dz_surf = delta_z / grid_surf
            dz_bulk = (sizez - 2.0 * delta_z) / (gz - 2 * grid_surf)
            for i in range(1, gz + 1):
                if i <= grid_surf or i > gz - grid_surf:
                    zr[i] = zr[i - 1] + dz_surf
                else:
                    zr[i] = zr[i - 1] + dz_bulk
                dz[i] = zr[i] - zr[i - 1]
    else:
        raise ValueError("mesh_type")
    return dz, zr


def tanh_mesh(gz, thickness, stretch=2.0):
    """Wall-clustered tanh mesh z_i = D/2 (1 + tanh(a(2i/gz-1))/tanh a);
    supplied to the reference as an explicit dz array."""
    i = np.arange(gz + 1, dtype=np.float64)
    zr = 0.5 * thickness * (1.0 + np.tanh(stretch * (2.0 * i / gz - 1.0)) / np.tanh(stretch))
    zr[0] = 0.0
    zr[-1] = thickness
    return mesh_from_zr(zr), zr


# integrator variants: (scheme, span)
#   span "full": Film_3D/.../mod_realspace.f90:267-281 (rect i=0..gz-1,
#                trap i=1..gz)
#   span "interior": Film_1D/.../mod_realspace.f90:201-218 and
#                Brush_CK_AD/Adaptive_Modules/mod_adaptive.f90:124-143
#                (both rules over i=1..gz-1)
def integrator(f, dz, dx=1.0, dy=1.0, int_scheme=1, span="full"):
    """integrator over [..., 0:gz, y, x] -> sum over the last three axes."""
    gz = dz.shape[0] - 1
    w = np.zeros(gz + 1)
    if int_scheme == 0:
        lo, hi = (0, gz - 1) if span == "full" else (1, gz - 1)
        w[lo:hi + 1] += dz[lo:hi + 1]
    else:
        hi = gz if span == "full" else gz - 1
        for i in range(1, hi + 1):
            w[i - 1] += 0.5 * dz[i]
            w[i] += 0.5 * dz[i]
    return dx * dy * np.tensordot(f, w, axes=([-3], [0])).sum(axis=(-1, -2))


def integrator_weights(dz, int_scheme=1, span="full"):
    """Per-plane weights w_i such that integrator(f) = dx dy sum_i w_i f_i."""
    gz = dz.shape[0] - 1
    w = np.zeros(gz + 1)
    if int_scheme == 0:
        lo, hi = (0, gz - 1) if span == "full" else (1, gz - 1)
        w[lo:hi + 1] += dz[lo:hi + 1]
    else:
        hi = gz if span == "full" else gz - 1
        for i in range(1, hi + 1):
            w[i - 1] += 0.5 * dz[i]
            w[i] += 0.5 * dz[i]
    return w


# ----------------------------------------------------------------------------
# 1D Crank-Nicolson step (films and brushes)
# ----------------------------------------------------------------------------
def cn_coefficients(dz, ds, film1d_form=True):
    """z coefficients of Film_1D/.../mod_realspace.f90:34-43 (film1d_form,
    bz = ds (h1+h2)/h1/h2/(h1+h2)) or Film_3D/.../mod_realspace.f90:70-76
    (bz = ds/h1/h2).  Rows 0 and gz are Dirichlet (a = c = 0)."""
    gz = dz.shape[0] - 1
    az = np.zeros(gz + 1)
    cz = np.zeros(gz + 1)
    bz = np.zeros(gz + 1)
    h1 = dz[1:gz]
    h2 = dz[2:gz + 1]
    az[1:gz] = -ds * 1.0 / h1 / (h1 + h2)
    cz[1:gz] = -ds * 1.0 / h2 / (h1 + h2)
    if film1d_form:
        bz[1:gz] = ds * (h1 + h2) / h1 / h2 / (h1 + h2)
    else:
        bz[1:gz] = ds * 1.0 / h1 / h2
    return az, bz, cz


def cn_step_1d(prop, field, dz, ds, solver="nr"):
    """Propagate_Step, Film_1D/.../mod_realspace.f90:24-79 and
    Brush_CK_AD/Geometry_Modules/mod_realspace.f90:26-79 (per-call ds).

    prop, field: [0:gz, ...] (trailing axes are independent lines).
    solver: "inplace" = the Film_1D tridiag (:120-148), "nr" = the Brush /
    Film_3D NR tridiag (equal up to rounding)."""
    gz = dz.shape[0] - 1
    az, bz, cz = cn_coefficients(dz, ds, film1d_form=True)
    ext = (slice(None),) + (None,) * (prop.ndim - 1)
    diag = np.ones_like(prop)
    diag[1:gz] = 1.0 + bz[1:gz][ext] + ds * field[1:gz] / 2.0
    rhs = np.zeros_like(prop)
    rhs[1:gz] = (-az[1:gz][ext] * prop[0:gz - 1]
                 + (1.0 - bz[1:gz][ext] - ds * field[1:gz] / 2.0) * prop[1:gz]
                 - cz[1:gz][ext] * prop[2:gz + 1])
    A = np.broadcast_to(az[ext], prop.shape)
    C = np.broadcast_to(cz[ext], prop.shape)
    if solver == "inplace":
        return tridiag_inplace(A, diag, C, rhs)
    return tridiag_nr(A, diag, C, rhs)


# ----------------------------------------------------------------------------
# 3D Douglas ADI step
# ----------------------------------------------------------------------------
def adi_step_3d(prop, field, dz, dx, dy, ds):
    """Propagate_Step, Film_3D/.../mod_realspace.f90:22-140.

    prop, field: [0:gz][gy][gx]; x and y periodic (ghosts :37-43), z
    Dirichlet on the nonuniform mesh."""
    gz = dz.shape[0] - 1
    gy, gx = prop.shape[1], prop.shape[2]
    p0 = prop.copy()                       # prop_0 (interior part)
    xm = np.roll(p0, 1, axis=2)            # prop_0(x-1) with periodic ghost
    xp = np.roll(p0, -1, axis=2)
    ym = np.roll(p0, 1, axis=1)
    yp = np.roll(p0, -1, axis=1)
    ax = -ds / dx / dx / 2.0               # :46-48
    bx = ds / dx / dx
    cx = -ds / dx / dx / 2.0
    ay = -ds / dy / dy / 2.0               # :58-60
    by = ds / dy / dy
    cy = -ds / dy / dy / 2.0
    az, bz, cz = cn_coefficients(dz, ds, film1d_form=False)   # :70-76
    zb = (slice(1, gz), None, None)
    out = prop.copy()
    # x sweep (:90-102), interior z only
    rhs = (-ax * xm[1:gz] - 2.0 * ay * ym[1:gz] - 2.0 * az[zb] * p0[0:gz - 1]
           - cx * xp[1:gz] - 2.0 * cy * yp[1:gz] - 2.0 * cz[zb] * p0[2:gz + 1]
           + (1.0 - bx - by * 2.0 - bz[zb] * 2.0 - ds * field[1:gz]) * p0[1:gz])
    # lines along x: move x to axis 0
    rl = np.moveaxis(rhs, 2, 0)
    A = np.full(rl.shape, ax)
    B = np.full(rl.shape, 1.0 + bx)
    C = np.full(rl.shape, cx)
    out[1:gz] = np.moveaxis(cyclic_tridiag(A, B, C, rl), 0, 2)
    # y sweep (:108-119)
    rhs = ay * ym[1:gz] + out[1:gz] + by * p0[1:gz] + cy * yp[1:gz]
    rl = np.moveaxis(rhs, 1, 0)
    A = np.full(rl.shape, ay)
    B = np.full(rl.shape, 1.0 + by)
    C = np.full(rl.shape, cy)
    out[1:gz] = np.moveaxis(cyclic_tridiag(A, B, C, rl), 0, 1)
    # z sweep (:125-139)
    rhs = np.zeros_like(prop)
    rhs[1:gz] = (az[zb] * p0[0:gz - 1] + out[1:gz]
                 + (bz[zb] + ds * field[1:gz] / 2.0) * p0[1:gz]
                 + cz[zb] * p0[2:gz + 1])
    diag = np.ones_like(prop)
    diag[1:gz] = 1.0 + bz[zb] + ds * field[1:gz] / 2.0
    A = np.broadcast_to(az[:, None, None], prop.shape)
    C = np.broadcast_to(cz[:, None, None], prop.shape)
    return tridiag_nr(A, diag, C, rhs)


# ----------------------------------------------------------------------------
# contour schemes and chain propagation
# ----------------------------------------------------------------------------
def contour_steps(ns, ds_scheme=0):
    """dss(0:segments), Initialize_Homopolymer, Brush_CK_AD/Polymer_Modules/
    mod_homopolymer.f90:98-115: 0 uniform, 1 half-cosine, 2 quarter-cosine;
    normalised to sum 1, dss(0) = 0."""
    dss = np.zeros(ns + 1)
    i = np.arange(1, ns + 1, dtype=np.float64)
    if ds_scheme == 0:
        dss[1:] = 1.0 / ns
    elif ds_scheme == 1:
        dss[1:] = 1.0 * 0.5 * (np.cos(np.pi * (i - 1) / ns) - np.cos(np.pi * i / ns))
    elif ds_scheme == 2:
        dss[1:] = 1.0 * (np.cos(np.pi * (i - 1) / (2.0 * ns)) - np.cos(np.pi * i / (2.0 * ns)))
    else:
        raise ValueError("ds_scheme")
    dss[1:] /= dss[1:].sum()
    return dss


def contour_weights(dss, lo, hi):
    """Trapezoid weights over contour nodes lo..hi for steps dss (dss[s]
    is the step from node s-1 to s): 1/2 (dss_s + dss_{s+1}) inside, half a
    step at each end.  Uniform dss reproduces mod_diblock.f90:143-154; the
    full range reproduces mod_homopolymer.f90:231-239."""
    w = np.zeros(len(dss))
    for s in range(lo, hi):
        w[s] += 0.5 * dss[s + 1]
        w[s + 1] += 0.5 * dss[s + 1]
    return w


def propagate_chain_1d(field_of_step, q0, dz, dss, stepper):
    """Run q_s = step(q_{s-1}, w(s), dss_s) for s = 1..Ns; returns all nodes."""
    ns = len(dss) - 1
    q = np.empty((ns + 1,) + q0.shape)
    q[0] = q0
    for s in range(1, ns + 1):
        q[s] = stepper(q[s - 1], field_of_step(s), dss[s])
    return q


def film_propagate_diblock(field, dz, dss, n_a, step, rho=1.0, dx=1.0,
                           dy=1.0, int_scheme=1, span="full", ensemble=1,
                           mu=0.0, sizes=None):
    """Propagate_Diblock for films, Film_CK_AD/Film_1D/Polymer_Modules/
    mod_diblock.f90:110-195 (Film_3D :105-182), generalised to a contour step
    array ``dss`` (uniform dss gives the reference; the adaptive form
    follows Brush_CK_AD/Polymer_Modules/mod_homopolymer.f90:209-239).

    field: [2][0:gz][...]; block A covers contour nodes 0..n_a.  ``step`` is
    step(prop, w, ds).  volume = sizes product (default dx*dy*sum(dz))."""
    ns = len(dss) - 1
    shape = field.shape[1:]
    q = np.empty((ns + 1,) + shape)
    qd = np.empty((ns + 1,) + shape)
    q[0] = 1.0
    for s in range(1, ns + 1):
        t = 0 if s <= n_a else 1
        q[s] = step(q[s - 1], field[t], dss[s])
    qd[0] = 1.0
    n_b = ns - n_a
    for s in range(1, ns + 1):
        t = 1 if s <= n_b else 0
        qd[s] = step(qd[s - 1], field[t], dss[ns + 1 - s])
    if q[0].ndim == 1:
        integ = lambda f: float(dx * dy * np.dot(integrator_weights(dz, int_scheme, span), f))
    else:
        integ = lambda f: float(integrator(f, dz, dx, dy, int_scheme, span))
    qsum = integ(q[ns])
    wa = contour_weights(dss, 0, n_a)
    wb = contour_weights(dss, n_a, ns)
    dist = np.zeros((2,) + shape)
    for s in range(ns + 1):
        prod = q[s] * qd[ns - s]
        dist[0] += wa[s] * prod
        dist[1] += wb[s] * prod
    if sizes is None:
        volume = dx * dy * float(np.sum(dz))
    else:
        volume = sizes[0] * sizes[1] * sizes[2]
    out = dict(Qsum=qsum, distribution=dist, qq=q, qqdag=qd, volume=volume)
    if ensemble == 1:
        out["density"] = rho * volume * dist / qsum
        out["mu"] = np.log(rho * volume / qsum)
        out["rho"] = rho
        out["energy"] = rho * volume * (out["mu"] - 1.0)
    else:
        out["density"] = np.exp(mu) * dist
        out["mu"] = mu
        total = integ(out["density"][0] + out["density"][1])
        out["rho"] = total / volume / float(np.sum(dss))
        out["energy"] = -out["rho"] * volume
    return out


def propagate_homopolymer(field, dz, dss, graft, rho, dx=1.0, dy=1.0,
                          int_scheme=1, span="interior", sizes=None):
    """Propagate_Homopolymer, Brush_CK_AD/Polymer_Modules/mod_homopolymer.f90:
    181-259: free end q_0 = 1, grafted q-dagger_0 = graft, reversed dss for
    q-dagger (:220), Q = integral q-dagger_0 q_N (:226), variable-weight
    trapezoid (:231-239), canonical closure with density(z=0) = 0 (:244-248).
    field: [0:gz][...] single species."""
    ns = len(dss) - 1
    q = np.empty((ns + 1,) + field.shape)
    qd = np.empty_like(q)
    q[0] = 1.0
    for s in range(1, ns + 1):
        q[s] = cn_step_1d(q[s - 1], field, dz, dss[s])
    qd[0] = graft
    for s in range(1, ns + 1):
        qd[s] = cn_step_1d(qd[s - 1], field, dz, dss[ns + 1 - s])
    wts = integrator_weights(dz, int_scheme, span)
    ext = (slice(None),) + (None,) * (field.ndim - 1)
    qsum = float(dx * dy * np.sum(wts[ext] * qd[0] * q[ns]))
    dist = dss[0] * q[0] * qd[ns]
    for s in range(1, ns):
        dist = dist + (dss[s] + dss[s + 1]) * q[s] * qd[ns - s]
    dist = dist + dss[ns] * q[ns] * qd[0]
    dist = 0.5 * dist
    if sizes is None:
        volume = dx * dy * float(np.sum(dz))
    else:
        volume = sizes[0] * sizes[1] * sizes[2]
    dens = rho * volume * dist / qsum
    dens[0] = 0.0
    mu = np.log(rho * volume / qsum)
    return dict(Qsum=qsum, distribution=dist, density=dens, mu=mu,
                energy=rho * volume * (mu - 1.0), qq=q, qqdag=qd)
