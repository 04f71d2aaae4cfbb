"""oracle.field -- CPU restatement of the reference's field build from
solved bases: drive superposition (ion_gym physics/build_stl3d.py:547-568)
and the electrode-aware gradient (physics/tracer3d.py:55-117).

TEST INFRASTRUCTURE ONLY.  Only tests/ and __graft_entry__.smoke() use this
module, as the checker.  The library (ion_gym_gb300) never imports it.

Parity is pinned: tests/test_oracle_golden.py replays tests/golden/field.npz,
recorded from the reference itself, and requires identical bits.

The arithmetic is numpy with every rounding written out: a float32
difference divided in float32 by float32(2h) / float32(h) when the spacing
is a Python float, in float64 and rounded to float32 when it is a numpy
float64 (numpy.gradient under NEP 50), and in float64 (rounded to the
potential's dtype) for the metal-node rule, whose spacing the reference
passes as a float64 into compiled code (tracer3d.py:115-116).
"""
import numpy as np


def _div(d, h, h_is_f64):
    """d / h as numpy.gradient computes it for a float32 or float64 d."""
    if d.dtype == np.float64:
        return d / np.float64(h)
    if h_is_f64:
        return (d.astype(np.float64) / np.float64(h)).astype(np.float32)
    return d / np.float32(h)


def _div64(d, h):
    """The metal rule's division: float64, rounded to d's dtype."""
    return (d.astype(np.float64) / np.float64(h)).astype(d.dtype)


def gradient_axis(phi, axis, h, h_is_f64):
    """numpy.gradient(phi, h)[axis] (edge_order 1, uniform spacing): central
    differences inside, first-order differences at the two faces."""
    f = np.moveaxis(phi, axis, 0)
    out = np.empty_like(f)
    out[1:-1] = _div(f[2:] - f[:-2], 2.0 * h, h_is_f64)
    out[0] = _div(f[1] - f[0], h, h_is_f64)
    out[-1] = _div(f[-1] - f[-2], h, h_is_f64)
    return np.moveaxis(out, 0, axis)


def field_aware_3d(phi, ele, h, h_is_f64=False, electrode_aware=True):
    """(Ex, Ey, Ez) of tracer3d.build_field_aware_3d (tracer3d.py:94-117);
    the metal pass of _fa3d_correct (tracer3d.py:55-91) vectorised: at a
    metal node with vacuum on exactly one side along an axis, the one-sided
    difference into the vacuum replaces that axis's derivative."""
    phi = np.asarray(phi)
    if np.issubdtype(phi.dtype, np.integer) or phi.dtype == np.bool_:
        phi = phi.astype(np.float64)
    if min(phi.shape) < 2:
        raise ValueError("Shape of array too small to calculate a numerical "
                         "gradient, at least (edge_order + 1) elements are "
                         "required.")
    d = [gradient_axis(phi, a, h, h_is_f64) for a in range(3)]
    if electrode_aware:
        metal = np.asarray(ele) != 0
        for a in range(3):
            f = np.moveaxis(phi, a, 0)
            m = np.moveaxis(metal, a, 0)
            da = np.moveaxis(d[a], a, 0)
            vp = np.zeros_like(m)
            vm = np.zeros_like(m)
            vp[:-1] = ~m[1:]
            vm[1:] = ~m[:-1]
            fwd = m & vp & ~vm
            bwd = m & vm & ~vp
            up = np.zeros_like(f)
            dn = np.zeros_like(f)
            up[:-1] = _div64(f[1:] - f[:-1], h)
            dn[1:] = _div64(f[1:] - f[:-1], h)
            da[fwd] = up[fwd]
            da[bwd] = dn[bwd]
    return tuple(-x for x in d)


def superpose(stack, rows, weights, mult):
    """Channel potentials of a superposition plan (build_stl3d.py:547-568):
    per channel, from +0 in float32, for each step in order, mult repeats
    of acc = acc + float32(w * basis[row])."""
    stack = np.asarray(stack, np.float32)
    weights = np.asarray(weights, np.float32)
    mult = np.asarray(mult)
    nch, nsteps = weights.shape
    out = np.zeros((nch,) + stack.shape[1:], np.float32)
    for c in range(nch):
        for s in range(nsteps):
            if mult[c, s]:
                t = weights[c, s] * stack[rows[s]]
                for _ in range(int(mult[c, s])):
                    out[c] = out[c] + t
    return out
