"""oracle.port -- CPU restatement of the reference ion_gym 3-D Laplace solve
(drivers in Python, kernels in oracle/igoracle.c).

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use this module, as the checker and as the timed
CPU restatement.  The library (ion_gym_gb300) never imports it.

Parity is pinned: tests/test_oracle_golden.py replays the fixtures that
tests/golden/make_golden.py recorded from the reference itself and requires
identical bits for every kernel and identical (phi, sweeps, delta) for every
driver.

Each driver follows the reference function cited in its docstring statement
for statement: the same order of sweeps, the same stopping rules, the same
host-side float arithmetic for tolerances, so the results are bit-identical.
"""
import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libigoracle.so")

_lib = None
_lock = threading.Lock()

_d = ctypes.c_double
_l = ctypes.c_long
_i = ctypes.c_int
_p = ctypes.c_void_p


def lib():
    """The compiled restatement (built by __graft_entry__.build())."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"oracle library {LIB_PATH} is not built; run "
                    f"__graft_entry__.build() first")
            L = ctypes.CDLL(LIB_PATH)
            sig = {
                "ig_or_sweep": (_d, [_p, _p, _p, _l, _l, _l, _d, _i, _i]),
                "ig_or_residual": (None, [_p, _p, _p, _l, _l, _l, _i, _p]),
                "ig_or_sweep_rhs": (_d, [_p, _p, _p, _l, _l, _l, _d, _i]),
                "ig_or_residual_rhs": (None, [_p, _p, _p, _l, _l, _l, _p]),
                "ig_or_restrict_fw": (None, [_p, _l, _l, _l, _p, _l, _l, _l]),
                "ig_or_prolong_add": (None, [_p, _l, _l, _l, _p, _p, _l, _l,
                                             _l]),
                "ig_or_prolongate": (None, [_p, _l, _l, _l, _p, _l, _l, _l]),
                "ig_or_coarsen_fixed_any": (None, [_p, _l, _l, _l, _p, _l, _l,
                                                   _l]),
                "ig_or_coarsen_mask": (None, [_p, _p, _l, _l, _l, _p, _p, _l,
                                              _l, _l]),
                "ig_or_residual_audit": (None, [_p, _p, _p, _l, _l, _l, _p]),
                "ig_or_err_sweep": (_d, [_p, _p, _p, _p, _l, _l, _l, _d, _i]),
                "ig_or_num_threads": (_i, []),
                "ig_or_set_threads": (None, [_i]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c64(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a


def _u8(a):
    return np.ascontiguousarray(a, dtype=bool).view(np.uint8)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def set_threads(n):
    lib().ig_or_set_threads(int(n))


def num_threads():
    return int(lib().ig_or_num_threads())


# ------------------------------------------------------------------ kernels
def sweep(phi, fixed, th, omega, colour, ghost_linear):
    """solver3d._sweep (solver3d.py:131-198); phi updated in place."""
    nx, ny, nz = phi.shape
    fx = _u8(fixed)
    t = _f32(th)
    return lib().ig_or_sweep(_ptr(_c64(phi)), _ptr(fx), _ptr(t), nx, ny, nz,
                             float(omega), int(colour), int(bool(ghost_linear)))


def residual(phi, fixed, th, ghost_linear, out):
    """multigrid3d._residual (multigrid3d.py:305-354)."""
    nx, ny, nz = phi.shape
    fx = _u8(fixed)
    t = _f32(th)
    lib().ig_or_residual(_ptr(_c64(phi)), _ptr(fx), _ptr(t), nx, ny, nz,
                         int(bool(ghost_linear)), _ptr(_c64(out)))


def sweep_rhs(e, fixed, f, omega, colour):
    """multigrid3d._sweep_rhs (multigrid3d.py:357-391); e updated in place."""
    nx, ny, nz = e.shape
    fx = _u8(fixed)
    fr = np.ascontiguousarray(f, np.float64)
    return lib().ig_or_sweep_rhs(_ptr(_c64(e)), _ptr(fx), _ptr(fr), nx, ny, nz,
                                 float(omega), int(colour))


def residual_rhs(e, fixed, f, out):
    """multigrid3d._residual_rhs (multigrid3d.py:394-417)."""
    nx, ny, nz = e.shape
    fx = _u8(fixed)
    fr = np.ascontiguousarray(f, np.float64)
    lib().ig_or_residual_rhs(_ptr(_c64(e)), _ptr(fx), _ptr(fr), nx, ny, nz,
                             _ptr(_c64(out)))


def restrict_fw(fine, out=None):
    """multigrid3d._restrict_fw_njit (multigrid3d.py:420-455)."""
    nx, ny, nz = fine.shape
    cs = ((nx + 1) // 2, (ny + 1) // 2, (nz + 1) // 2)
    if out is None:
        out = np.empty(cs)
    fr = np.ascontiguousarray(fine, np.float64)
    lib().ig_or_restrict_fw(_ptr(fr), nx, ny, nz, _ptr(_c64(out)), *out.shape)
    return out


def prolong_add(coarse, out, fixed):
    """multigrid3d._prolong_add_njit (multigrid3d.py:458-499)."""
    cr = np.ascontiguousarray(coarse, np.float64)
    fx = _u8(fixed)
    lib().ig_or_prolong_add(_ptr(cr), *cr.shape, _ptr(_c64(out)), _ptr(fx),
                            *out.shape)


def prolongate(coarse, shape_f):
    """multigrid3d._prolongate (multigrid3d.py:138-171)."""
    cr = np.ascontiguousarray(coarse, np.float64)
    out = np.empty(tuple(int(s) for s in shape_f))
    lib().ig_or_prolongate(_ptr(cr), *cr.shape, _ptr(out), *out.shape)
    return out


def coarsen_fixed_any(fixed):
    """multigrid3d._coarsen_fixed_any (multigrid3d.py:507-526)."""
    nx, ny, nz = fixed.shape
    cs = ((nx + 1) // 2, (ny + 1) // 2, (nz + 1) // 2)
    out = np.empty(cs, np.uint8)
    lib().ig_or_coarsen_fixed_any(_ptr(_u8(fixed)), nx, ny, nz, _ptr(out), *cs)
    return out.view(bool)


def coarsen_mask(fixed, val):
    """multigrid3d._coarsen_mask (multigrid3d.py:85-135)."""
    nx, ny, nz = fixed.shape
    cs = ((nx + 1) // 2, (ny + 1) // 2, (nz + 1) // 2)
    fc = np.empty(cs, np.uint8)
    vc = np.empty(cs)
    v = np.ascontiguousarray(val, np.float64)
    lib().ig_or_coarsen_mask(_ptr(_u8(fixed)), _ptr(v), nx, ny, nz, _ptr(fc),
                             _ptr(vc), *cs)
    return fc.view(bool), vc


def residual_audit(u, fixed, th):
    """solver3d._residual_kernel (solver3d.py:366-386)."""
    u = np.ascontiguousarray(u, np.float64)
    out = np.empty_like(u)
    lib().ig_or_residual_audit(_ptr(u), _ptr(_u8(fixed)), _ptr(_f32(th)),
                               *u.shape, _ptr(out))
    return out


def err_sweep(e, fixed, th, rhs, omega, colour):
    """solver3d._err_sweep (solver3d.py:389-417); e updated in place."""
    r = np.ascontiguousarray(rhs, np.float64)
    return lib().ig_or_err_sweep(_ptr(_c64(e)), _ptr(_u8(fixed)),
                                 _ptr(_f32(th)), _ptr(r), *e.shape,
                                 float(omega), int(colour))


# ------------------------------------------------------------------ drivers
class SolveNotConverged(RuntimeError):
    """solver3d.SolveNotConverged (solver3d.py:233)."""


class SolveInterrupted(Exception):
    """multigrid3d.SolveInterrupted (multigrid3d.py:38)."""


STOP = threading.Event()


def optimal_omega(shape, spacing=None):
    """solver3d.optimal_omega (solver3d.py:201-230): Young's optimum from
    the Jacobi radius of the axes with at least two nodes."""
    if spacing is None:
        axes = [(int(n), 1.0) for n in shape if int(n) >= 2]
    else:
        axes = [(int(n), 1.0 / (float(s) * float(s)))
                for n, s in zip(shape, spacing) if int(n) >= 2]
    if not axes:
        return 1.0
    acc = sum(w * np.cos(np.pi / (n + 1)) for n, w in axes)
    rho = acc / sum(w for _, w in axes)
    rho = min(rho, 1.0 - 1e-15)
    return 2.0 / (1.0 + np.sqrt(1.0 - rho * rho))


def _theta_or_ones(theta, shape):
    if theta is None:
        return np.ones((6,) + tuple(shape), np.float32)
    return np.ascontiguousarray(theta, np.float32)


def _check_stencil(stencil):
    if stencil not in ("ghost_linear", "sw"):
        raise ValueError(f"unknown stencil {stencil!r}; known stencils are "
                         f"'ghost_linear' and 'sw'")
    return stencil == "ghost_linear"


def solve3d(fixed, val, theta=None, mirror=(False, False, False), tol=1e-6,
            max_sweeps=60000, omega=None, phi0=None, verbose=False,
            stencil="ghost_linear"):
    """solver3d.solve3d (solver3d.py:250-293)."""
    fixed = np.asarray(fixed, bool)
    shape = fixed.shape
    phi = (np.array(phi0, np.float64) if phi0 is not None
           else np.zeros(shape))
    phi[fixed] = np.asarray(val)[fixed]
    th = _theta_or_ones(theta, shape)
    if omega is None:
        omega = optimal_omega(shape)
    gl = _check_stencil(stencil)
    d = np.inf
    for s in range(max_sweeps):
        d1 = sweep(phi, fixed, th, omega, 0, gl)
        d2 = sweep(phi, fixed, th, omega, 1, gl)
        d = max(d1, d2)
        if d < tol:
            return phi, s + 1, d
    raise SolveNotConverged(
        f"SOR cap of {max_sweeps} sweeps reached: delta {d:.3e} vs tol "
        f"{tol:.3e} ({d / max(tol, 1e-30):.0f}x too loose)")


def solve_bases(masks, scene=None, mirror=(False, False, False), v_basis=1e4,
                tol=1e-6, verbose=False, stencil="ghost_linear", omega=None,
                only=None, theta=None):
    """solver3d.solve_bases (solver3d.py:296-320); theta stands in for the
    scene-derived fractions."""
    metal = np.zeros(next(iter(masks.values())).shape, bool)
    for m in masks.values():
        metal |= m
    out = {}
    for i, m in sorted(masks.items()):
        if only is not None and i not in only:
            continue
        val = np.zeros(metal.shape)
        val[m] = v_basis
        out[i] = solve3d(metal, val, theta=theta, mirror=mirror, tol=tol,
                         stencil=stencil, omega=omega)[0]
    return out


def solve3d_mg(fixed, val, theta=None, mirror=(False, False, False), tol=1e-6,
               max_sweeps=60000, verbose=False, stencil="ghost_linear",
               min_coarse=9, max_levels=8, level_tol_factor=30.0, omega=None):
    """multigrid3d.solve3d_mg (multigrid3d.py:175-230), the cascadic scheme.
    omega (not in the reference signature) fixes the SOR factor on every
    level; None keeps the reference's per-level optimum."""
    levels = cascadic_levels(fixed, val, min_coarse, max_levels)
    fc, vc = levels[-1]
    phic, _, _ = solve3d(fc, vc, theta=None, tol=tol, max_sweeps=max_sweeps,
                         stencil=stencil, omega=omega)
    for lev in range(len(levels) - 2, 0, -1):
        f, v = levels[lev]
        p0 = prolongate(phic, f.shape)
        p0[f] = v[f]
        phic, _, _ = solve3d(f, v, theta=None, tol=tol * level_tol_factor,
                             max_sweeps=max_sweeps, phi0=p0, stencil=stencil,
                             omega=omega)
    f, v = levels[0]
    p0 = prolongate(phic, f.shape) if len(levels) > 1 else None
    if p0 is not None:
        p0[f] = v[f]
    return solve3d(f, v, theta=theta, tol=tol, max_sweeps=max_sweeps,
                   phi0=p0, stencil=stencil, omega=omega)


def cascadic_levels(fixed, val, min_coarse=9, max_levels=8):
    """The cascadic hierarchy of solve3d_mg (multigrid3d.py:188-194): the
    fine (fixed, val) and its _coarsen_mask levels, fine first."""
    levels = [(np.asarray(fixed, bool), np.asarray(val, np.float64))]
    while len(levels) < max(1, max_levels):
        f, v = levels[-1]
        if min(f.shape) <= min_coarse or min((s + 1) // 2 for s in f.shape) < 3:
            break
        levels.append(coarsen_mask(f, v))
    return levels


def solve3d_cascadic_relres(fixed, val, rel_tol=1e-10, omega=1.85,
                            max_levels=4, min_coarse=9, check_every=20,
                            level_tol_factor=30.0, max_sweeps=200000,
                            on_level=None):
    """The residual-stopped cascadic solve of the 257^3 quadrupole workload
    (no reference driver: the reference's cascadic solve3d_mg,
    multigrid3d.py:175-230, stops each level on the max |update| of a sweep
    pair; this rule stops it on a relative residual instead).

    Built from the reference's pieces: the solve3d_mg hierarchy
    (_coarsen_mask, multigrid3d.py:85-135, at most max_levels levels), the
    coarsest level started from its Dirichlet values with zeros elsewhere,
    each finer level from _prolongate (multigrid3d.py:138-171) of the level
    below with its Dirichlet values reset, red-black _sweep pairs
    (solver3d.py:131-198, theta None read as ones) at omega[L] on level L
    (fine = 0), and the relative residual max|r| / max|r(phi_D)| with r from
    multigrid3d._residual (multigrid3d.py:305-354) and phi_D the level's
    Dirichlet values with zeros elsewhere, checked before the first pair and
    after every `check_every` pairs.  The coarsest and fine levels stop below
    rel_tol, intermediate levels below rel_tol * level_tol_factor (the
    reference's level_tol_factor); max_sweeps caps each level's pairs, and a
    coarse level that reaches the cap hands its iterate on (only the fine
    level's cap raises SolveNotConverged).

    Returns (phi, fine pairs, fine relative residual, pairs on all levels,
    per-level pair counts coarsest first).  on_level(L, shape, pairs, rr),
    when given, is called after each level."""
    levels = cascadic_levels(fixed, val, min_coarse, max_levels)
    nl = len(levels)
    om = np.broadcast_to(np.asarray(omega, np.float64), (nl,))
    ones = None
    cur = None
    total = 0
    per_level = []
    phi = rr = pairs = None
    for L in range(nl - 1, -1, -1):
        f, v = levels[L]
        if ones is None or ones.shape[1:] != f.shape:
            ones = np.ones((6,) + f.shape, np.float32)
        r = np.empty(f.shape)
        phid = np.zeros(f.shape)
        phid[f] = v[f]
        residual(phid, f, ones, True, r)
        bnorm = float(np.abs(r).max())
        if L < nl - 1:
            phi = prolongate(cur, f.shape)
            phi[f] = v[f]
        else:
            phi = phid
        ltol = rel_tol if L in (0, nl - 1) else rel_tol * level_tol_factor
        pairs = 0
        while True:
            residual(phi, f, ones, True, r)
            rmax = float(np.abs(r).max())
            rr = rmax / bnorm if bnorm > 0 else rmax
            if rr < ltol or pairs >= max_sweeps:
                break
            chunk = min(check_every, max_sweeps - pairs)
            for _ in range(chunk):
                sweep(phi, f, ones, float(om[L]), 0, True)
                sweep(phi, f, ones, float(om[L]), 1, True)
            pairs += chunk
        total += pairs
        per_level.append(pairs)
        if on_level is not None:
            on_level(L, f.shape, pairs, rr)
        if L == 0 and not rr < ltol:
            raise SolveNotConverged(
                f"cascadic solve stopped at {max_sweeps} sweeps with relative "
                f"residual {rr:.3e} vs {rel_tol:.1e}")
        cur = phi
    return phi, pairs, rr, total, per_level


def _solve_err(fixed, f, rel_tol=0.02, max_cycles=30, nu1=2, nu2=2,
               min_coarse=9, _depth=0):
    """multigrid3d._solve_err (multigrid3d.py:553-599)."""
    e = np.zeros_like(f)
    scale = max(np.abs(f).max(), 1e-300)
    tol = rel_tol * scale / 6.0
    if min(e.shape) <= min_coarse:
        om = optimal_omega(e.shape)
        for _ in range(20000):
            d1 = sweep_rhs(e, fixed, f, om, 0)
            d2 = sweep_rhs(e, fixed, f, om, 1)
            if max(d1, d2) < 0.02 * tol:
                break
        return e
    fc = coarsen_fixed_any(fixed)
    r = np.empty_like(e)
    for _ in range(max_cycles):
        for _s in range(nu1):
            sweep_rhs(e, fixed, f, 1.0, 0)
            sweep_rhs(e, fixed, f, 1.0, 1)
        residual_rhs(e, fixed, f, r)
        rc = restrict_fw(r)
        rc *= 4.0
        ec = _solve_err(fc, -rc, rel_tol, max_cycles, nu1, nu2, min_coarse,
                        _depth + 1)
        prolong_add(ec, e, fixed)
        d = 0.0
        for _s in range(nu2):
            d1 = sweep_rhs(e, fixed, f, 1.0, 0)
            d2 = sweep_rhs(e, fixed, f, 1.0, 1)
            d = max(d1, d2)
        if d < tol:
            break
    return e


def symmetric_axes(fixed, val, theta):
    """The axes along which fixed and val are exactly flip-invariant
    (multigrid3d.py:643-650); none when theta is supplied."""
    axes = []
    if theta is None:
        for a in range(3):
            if fixed.shape[a] < 3:
                continue
            if (np.array_equal(fixed, np.flip(fixed, axis=a))
                    and np.array_equal(val, np.flip(val, axis=a))):
                axes.append(a)
    return axes


def solve3d_vmg(fixed, val, theta=None, mirror=(False, False, False), tol=1e-6,
                max_cycles=60, nu1=3, nu2=3, verbose=False,
                stencil="ghost_linear", phi0=None, accept_stagnation=False):
    """multigrid3d.solve3d_vmg (multigrid3d.py:602-731)."""
    fixed = np.asarray(fixed, bool)
    shape = fixed.shape
    phi = (np.array(phi0, np.float64) if phi0 is not None
           else np.zeros(shape))
    val = np.asarray(val)
    phi[fixed] = val[fixed]
    th = _theta_or_ones(theta, shape)
    gl = _check_stencil(stencil)
    sym = symmetric_axes(fixed, val, theta)
    r = np.empty_like(phi)
    fcm = coarsen_fixed_any(fixed)
    sweeps = 0
    prev = np.inf
    cycle_d = np.inf
    for cyc in range(max_cycles):
        if STOP.is_set():
            raise SolveInterrupted(f"stopped at cycle {cyc}")
        phi_c0 = phi.copy()
        for _ in range(nu1):
            sweep(phi, fixed, th, 1.0, 0, gl)
            sweep(phi, fixed, th, 1.0, 1, gl)
            sweeps += 1
        if STOP.is_set():
            raise SolveInterrupted(f"stopped in cycle {cyc}")
        residual(phi, fixed, th, gl, r)
        r[fixed] = 0.0
        rc = restrict_fw(r)
        rc *= 4.0
        ec = _solve_err(fcm, -rc, rel_tol=0.05, nu1=nu1, nu2=nu2)
        prolong_add(ec, phi, fixed)
        for _ in range(nu2):
            sweep(phi, fixed, th, 1.0, 0, gl)
            sweep(phi, fixed, th, 1.0, 1, gl)
            sweeps += 1
        for a in sym:
            np.add(phi, np.flip(phi, axis=a), out=phi)
            phi *= 0.5
        cycle_d = float(np.abs(phi - phi_c0).max())
        if cycle_d < tol:
            return phi, sweeps, cycle_d
        if cycle_d >= prev:
            if accept_stagnation:
                return phi, sweeps, cycle_d
            raise SolveNotConverged(
                f"V-cycle STAGNATED at cycle {cyc}: {cycle_d:.3e} after "
                f"{prev:.3e}, tol {tol:.1e}")
        prev = cycle_d
    raise SolveNotConverged(
        f"V-cycle exhausted max_cycles={max_cycles} at delta {cycle_d:.3e}, "
        f"tol {tol:.1e}")


def solve_bases_mg(masks, scene=None, mirror=(False, False, False),
                   v_basis=1e4, tol=1e-6, verbose=False, stencil="ghost_linear",
                   theta=None, only=None):
    """multigrid3d.solve_bases_mg (multigrid3d.py:233-291)."""
    metal = np.zeros(next(iter(masks.values())).shape, bool)
    for m in masks.values():
        metal |= m
    out = {}
    for i, m in sorted(masks.items()):
        if only is not None and i not in only:
            continue
        if STOP.is_set():
            raise SolveInterrupted("stopped between electrodes")
        val = np.zeros(metal.shape)
        val[m] = v_basis
        phi, _, d = solve3d_vmg(metal, val, theta=theta, mirror=mirror,
                                tol=tol, stencil=stencil)
        out[i] = phi
    return out
