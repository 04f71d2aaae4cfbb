"""Mixed-precision batched basis solves: every electrode basis of a deck in
one batch, FP32 multigrid inside FP64 iterative refinement.

Same inputs and outputs as multigrid3d.solve_bases_mg ({index: mask} ->
{index: phi float64 at v_basis}) but a different stopping rule: each basis
is refined until the applied FP64 change of a refinement step is below
`accuracy` x the electrode span (v_basis), so the potential is within about
that accuracy of the exact solution of the same discrete problem (the
reference's fine operator: theta None, 7-point, even-reflection faces,
Dirichlet metal).  The FP64 drop-in solves the same problem with the
reference's V-cycle and its cycle-delta rule; the two agree to the stated
accuracy (tests/test_gpu_mixed.py).
"""
import ctypes

import numpy as np

from ion_gym_gb300 import _lib
from ion_gym_gb300._lib import ptr, as_mask
from ion_gym_gb300.physics.solver3d import (SolveNotConverged, stencil_code,
                                            _union)


def solve_bases_mixed(masks, v_basis=1e4, accuracy=1e-9,
                      stencil="ghost_linear", only=None, nu1=2, nu2=2,
                      vcycles=2, max_steps=40, return_stats=False):
    """All bases in one batch.  Returns {index: phi}; with return_stats also
    {"steps": refinement steps, "dmax": {index: last applied change}}."""
    code = stencil_code(stencil)
    metal = _union(masks)
    items = [(i, np.asarray(m, bool)) for i, m in sorted(masks.items())
             if only is None or i in only]
    if not items:
        return ({}, {"steps": 0, "dmax": {}}) if return_stats else {}
    shape = metal.shape
    n = metal.size
    B = len(items)
    stack = np.empty((B,) + shape, np.uint8)
    for b, (_, m) in enumerate(items):
        stack[b] = m
    phi = np.empty((B,) + shape)
    steps = ctypes.c_int(0)
    dmax = np.zeros(B)
    acc = float(accuracy) * abs(float(v_basis))
    L = _lib.lib()
    st = L.ig_mixed_bases(ptr(as_mask(metal)), ptr(stack), B, float(v_basis),
                          *shape, code, acc, int(max_steps), int(nu1),
                          int(nu2), int(vcycles), ptr(phi),
                          ctypes.byref(steps), ptr(dmax))
    _lib.check(st, "solve_bases_mixed")
    if st == _lib.IG_NOT_CONVERGED:
        raise SolveNotConverged(
            f"mixed-precision refinement: {steps.value} steps without every "
            f"basis reaching {accuracy:.1e} of the span (worst applied change "
            f"{dmax.max():.3e} V)")
    out = {i: phi[b] for b, (i, _) in enumerate(items)}
    if return_stats:
        return out, {"steps": int(steps.value),
                     "dmax": {i: float(dmax[b]) for b, (i, _) in
                              enumerate(items)}}
    return out
