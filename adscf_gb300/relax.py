"""Unit-cell relaxation with the adjoint cell stress.

The reference finds the equilibrium box by re-running the SCF at
neighbouring box sizes.  Here the SCF is converged once per box, the exact
derivative of the discrete free energy with respect to the side lengths comes
from adscf_forward / adscf_backward at the converged field (at a saddle the
derivative at fixed fields is the derivative of the equilibrium free energy),
and the side lengths move by a secant step per axis until the stress is
below `tol`.
"""
from __future__ import annotations

import numpy as np


def relax_box(ctx, field, axes=(0,), tol=1e-6, scf_tol=1e-16, max_scf=3000, max_steps=25,
              step0=0.02, max_rel_step=0.1):
    """Relax the side lengths `axes` of an FP64 bulk context.

    Returns (size, F, grad, history); history holds (size, F, grad, accuracy)
    per box visited.  Each box restarts the mixing from the last converged
    field."""
    size = [ctx.params.sizex, ctx.params.sizey, ctx.params.sizez]
    w = np.asarray(field, dtype=np.float64).ravel()
    history = []
    prev = None
    F = g = None
    for _ in range(max_steps):
        ctx.set_field(w)
        res = ctx.scf_run(max_scf, tol=scf_tol)
        w = ctx.get_field()
        F = ctx.forward(w)
        g = ctx.backward()
        history.append((tuple(size), F, g.copy(), res.accuracy))
        if max(abs(g[a]) for a in axes) < tol:
            break
        new = list(size)
        for a in axes:
            if prev is None or prev[1][a] == g[a]:
                d = -step0 * size[a] * np.sign(g[a])
            else:
                d = -g[a] * (size[a] - prev[0][a]) / (g[a] - prev[1][a])
            lim = max_rel_step * size[a]
            new[a] = size[a] + float(np.clip(d, -lim, lim))
        prev = (list(size), g.copy())
        size = new
        ctx.set_box(size)
    return tuple(size), F, g, history
