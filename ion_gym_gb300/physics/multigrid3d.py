"""ion_gym_gb300.physics.multigrid3d -- drop-in for ion_gym.physics.multigrid3d.

Same public names, signatures, defaults, return tuples and exceptions as the
reference module (ion_gym physics/multigrid3d.py): the cascadic solve
(solve3d_mg), the V-cycle (solve3d_vmg) with its recursive error-equation
solve, the basis door (solve_bases_mg), and the cooperative stop
(request_stop / clear_stop / stop_event / SolveInterrupted) with the
process-wide SOLVE_EXCLUSIVE lock.

The solves run in libigsolve.so on the GPU and return the reference's
float64 bits.  The stop flag is shared with the library, which polls it where
the reference polls _STOP: twice per V-cycle and between bases.
"""
import threading
import os
import time

import numpy as np

from ion_gym_gb300 import _lib
from ion_gym_gb300._lib import ptr, as_mask, as_f64, as_f32
from ion_gym_gb300.physics.solver3d import (  # noqa: F401  (re-exported)
    SolveNotConverged, optimal_omega, solve3d, stencil_code, _sweep,
    _grid_args, _union, fractions_from_scene)


class SolveInterrupted(Exception):
    """Raised by a solve when a stop was requested (multigrid3d.py:38)."""


class _StopEvent(threading.Event):
    """The solver's stop event: a threading.Event whose set/clear also arm
    the library's flag, so code that sets the event itself (rather than
    calling request_stop) stops the GPU solve too."""

    def set(self):
        super().set()
        try:
            _lib.lib().ig_request_stop()
        except _lib.LibraryMissing:
            pass

    def clear(self):
        super().clear()
        try:
            _lib.lib().ig_clear_stop()
        except _lib.LibraryMissing:
            pass


_STOP = _StopEvent()

# Process-wide solve exclusivity (multigrid3d.py:44-58): drivers that can run
# builds from several threads hold this for the duration of a build, after
# calling request_stop() so an older solve ends at its next stop check.
SOLVE_EXCLUSIVE = threading.Lock()


def request_stop():
    """Ask any in-flight solve to stop at its next stop check."""
    _STOP.set()


def stop_event():
    """The stop event itself, for code that must stop on the same request."""
    return _STOP


def clear_stop():
    """Re-arm the solver after a stop (hold SOLVE_EXCLUSIVE if solves can
    overlap)."""
    _STOP.clear()


# ------------------------------------------------------------ hierarchy
def cascadic_shapes(shape, min_coarse=9, max_levels=8):
    """Level shapes of the cascadic hierarchy, fine first
    (multigrid3d.py:188-194)."""
    levels = [tuple(int(s) for s in shape)]
    while len(levels) < max_levels:
        s = levels[-1]
        if min(s) <= min_coarse or min((x + 1) // 2 for x in s) < 3:
            break
        levels.append(tuple((x + 1) // 2 for x in s))
    return levels


def bottom_shape(shape, min_coarse=9):
    """Shape of the bottom error level of the V-cycle: the first level of
    the (n+1)//2 chain below the fine grid with min(shape) <= min_coarse
    (multigrid3d.py:570, 675)."""
    s = tuple((int(x) + 1) // 2 for x in shape)
    while min(s) > min_coarse:
        s = tuple((x + 1) // 2 for x in s)
    return s


def solve3d_mg(fixed, val, theta=None, mirror=(False, False, False),
               tol=1e-6, max_sweeps=60000, verbose=False,
               stencil="ghost_linear", min_coarse=9, max_levels=8,
               level_tol_factor=30.0):
    """Cascadic multigrid (multigrid3d.py:175-230): the same Dirichlet
    problem solved on 2x-coarsened grids, coarsest first, each solution
    prolongated as the next level's start; the fine level is the plain SOR
    solve with theta at tol.  Returns (phi, fine sweeps, fine delta)."""
    fixed, th, shape = _grid_args(fixed, theta)
    code = stencil_code(stencil)
    v = as_f64(np.broadcast_to(np.asarray(val, np.float64), shape))
    levels = cascadic_shapes(shape, min_coarse, max_levels)
    omegas = np.array([optimal_omega(s) for s in levels], np.float64)
    phi = np.empty(shape)
    sw = _lib.ctypes.c_long(0)
    d = _lib.ctypes.c_double(0.0)
    L = _lib.lib()
    st = L.ig_solve3d_mg(ptr(as_mask(fixed)), ptr(v), ptr(th), *shape,
                         float(tol), int(max_sweeps), code, int(min_coarse),
                         int(max_levels), float(level_tol_factor),
                         ptr(omegas), len(omegas), ptr(phi),
                         _lib.ctypes.byref(sw), _lib.ctypes.byref(d))
    _lib.check(st, "solve3d_mg")
    if st == _lib.IG_NOT_CONVERGED:
        raise SolveNotConverged(
            f"cascadic solve: SOR stopped at its cap of {max_sweeps} sweeps "
            f"({_lib.last_error()}), delta {d.value:.3e} vs tol {tol:.3e} "
            f"({d.value / max(tol, 1e-30):.0f}x too loose)")
    if verbose:
        print(f"[mg] {len(levels)} levels: "
              + " <- ".join(str(s) for s in levels)
              + f"; fine: {sw.value} sweeps")
    return phi, int(sw.value), float(d.value)


def solve3d_cascadic_relres(fixed, val, rel_tol=1e-10, omega=1.85,
                            max_levels=4, min_coarse=9, check_every=20,
                            level_tol_factor=30.0, max_sweeps=200000,
                            out=None):
    """Cascadic multigrid stopped on a relative residual (no reference
    counterpart; the stopping rule of the quadrupole benchmark).

    The level hierarchy is solve3d_mg's (_coarsen_mask, at most max_levels);
    each level is relaxed by red-black SOR at `omega` (a float, or one value
    per level, fine first) until max|r| / max|r(phi_D)| < rel_tol (times
    level_tol_factor on the intermediate levels), where r is
    multigrid3d._residual with theta None and phi_D holds the Dirichlet values
    with zeros elsewhere; the residual is checked every `check_every` pairs.

    fixed/val: numpy arrays, or CUDA torch tensors (uint8/bool and float64)
    already resident on the device.  out: optional float64 array or CUDA
    tensor for phi.  Returns (phi, fine sweep pairs, fine relative residual,
    pairs on all levels)."""
    shape = tuple(int(s) for s in fixed.shape)
    levels = cascadic_shapes(shape, min_coarse, max_levels)
    om = np.broadcast_to(np.asarray(omega, np.float64), (len(levels),))
    om = np.ascontiguousarray(om)
    dev = type(fixed).__module__.startswith("torch")
    if dev:
        fx, v = fixed, val
        phi = out if out is not None else val.new_empty(shape)
        pf, pv, pp = (_lib.ctypes.c_void_p(fx.data_ptr()),
                      _lib.ctypes.c_void_p(v.data_ptr()),
                      _lib.ctypes.c_void_p(phi.data_ptr()))
    else:
        fx = as_mask(fixed)
        v = as_f64(val)
        phi = out if out is not None else np.empty(shape)
        pf, pv, pp = ptr(fx), ptr(v), ptr(phi)
    sw = _lib.ctypes.c_long(0)
    rr = _lib.ctypes.c_double(0.0)
    tot = _lib.ctypes.c_long(0)
    nl = _lib.ctypes.c_int(0)
    st = _lib.lib().ig_cascadic_relres(
        pf, pv, *shape, float(rel_tol), int(max_sweeps), int(min_coarse),
        int(max_levels), float(level_tol_factor), ptr(om), len(om),
        int(check_every), pp, _lib.ctypes.byref(sw), _lib.ctypes.byref(rr),
        _lib.ctypes.byref(tot), _lib.ctypes.byref(nl))
    _lib.check(st, "solve3d_cascadic_relres")
    if st == _lib.IG_NOT_CONVERGED:
        raise SolveNotConverged(
            f"cascadic solve stopped at {max_sweeps} sweeps with relative "
            f"residual {rr.value:.3e} vs {rel_tol:.1e}")
    return phi, int(sw.value), float(rr.value), int(tot.value)


def _vmg_outcome(st, shape, tol, max_cycles, sw, d, cyc, prev, phi,
                 accept_stagnation):
    if st == _lib.IG_OK:
        return phi, int(sw), float(d)
    if st == _lib.IG_INTERRUPTED:
        raise SolveInterrupted(
            f"stopped mid-solve at cycle {cyc} (delta {prev:.2e} V)")
    if st == _lib.IG_STAGNATED:
        raise SolveNotConverged(
            f"V-cycle STAGNATED at cycle {cyc}: delta {d:.3e} V did not "
            f"improve on the previous cycle's {prev:.3e} before reaching tol "
            f"{tol:.1e}. A stalled iterate is not a converged field: loosen "
            f"tol toward the achieved delta, or pass accept_stagnation=True "
            f"to take the iterate knowingly.")
    if st == _lib.IG_CYCLE_CAP:
        raise SolveNotConverged(
            f"V-cycle exhausted max_cycles={max_cycles} at delta {d:.3e} V "
            f"without reaching tol {tol:.1e}; raise max_cycles or loosen "
            f"tol.")
    raise RuntimeError(f"solve3d_vmg: unexpected status {st}: "
                       f"{_lib.last_error()}")


def solve3d_vmg(fixed, val, theta=None, mirror=(False, False, False),
                tol=1e-6, max_cycles=60, nu1=3, nu2=3, verbose=False,
                stencil="ghost_linear", phi0=None,
                accept_stagnation=False):
    """V-cycle multigrid with the validated fine sweep (multigrid3d.py:
    602-731): per cycle nu1 sweep pairs (omega 1), the coarse error equation
    solved to relative tolerance 0.05 by _solve_err, nu2 sweep pairs, the
    projection onto proven flip symmetries (theta None only), and the
    full-cycle max change as the convergence test.  Returns (phi, fine sweep
    pairs, cycle delta)."""
    fixed, th, shape = _grid_args(fixed, theta)
    v = as_f64(np.broadcast_to(np.asarray(val, np.float64), shape))
    code = stencil_code(stencil)
    p0 = None if phi0 is None else as_f64(np.broadcast_to(
        np.asarray(phi0, np.float64), shape))
    bom = optimal_omega(bottom_shape(shape))
    phi = np.empty(shape)
    sw = _lib.ctypes.c_long(0)
    d = _lib.ctypes.c_double(0.0)
    cyc = _lib.ctypes.c_int(0)
    prev = _lib.ctypes.c_double(0.0)
    L = _lib.lib()
    st = L.ig_solve3d_vmg(ptr(as_mask(fixed)), ptr(v), ptr(th), *shape,
                          float(tol), int(max_cycles), int(nu1), int(nu2),
                          code, ptr(p0), int(bool(accept_stagnation)),
                          float(bom), ptr(phi), _lib.ctypes.byref(sw),
                          _lib.ctypes.byref(d), _lib.ctypes.byref(cyc),
                          _lib.ctypes.byref(prev))
    _lib.check(st, "solve3d_vmg")
    if verbose and st == _lib.IG_OK:
        print(f"[vmg] {cyc.value} cycles, {sw.value} sweeps, cycle delta "
              f"{d.value:.3e}")
    return _vmg_outcome(st, shape, tol, max_cycles, sw.value, d.value,
                        cyc.value, prev.value, phi, accept_stagnation)


def _record_solve(n_nodes, seconds):
    """The reference door records each basis's solve time for its cost
    quote (multigrid3d.py:283-287, physics/sizing.py:159); kept when the
    reference package is importable, skipped otherwise."""
    try:
        from ion_gym.physics.sizing import record_solve
    except ImportError:
        return
    record_solve("mg", n_nodes, basis_s=seconds)


# Bases solved at once by solve_bases_mg: each runs on its own host thread
# and CUDA stream, so the latency-bound coarse levels of one basis overlap
# the others' work.  Independent problems: every basis keeps its bits.
BASIS_CONCURRENCY = int(os.environ.get("IG_BASIS_CONCURRENCY", "8"))


def _basis_workers(n_bases, n_nodes):
    """Concurrent basis solves that fit in free device memory (about 32
    bytes per node each: the potential, its mask and value staging, and the
    V-cycle's error levels)."""
    w = max(1, min(BASIS_CONCURRENCY, n_bases))
    try:
        free = _lib.lib().ig_device_free_bytes()
    except Exception:
        free = 0
    if free > 0:
        w = max(1, min(w, int(free * 0.8) // max(32 * n_nodes, 1)))
    return w


# How the basis door solves when its caller does not say: "fp64", the
# reference's V-cycle with its bits, or "mixed", the batched FP32-multigrid /
# FP64-refinement session (IG_BASIS_PRECISION overrides the default).
PRECISIONS = ("fp64", "mixed")
BASIS_PRECISION = os.environ.get("IG_BASIS_PRECISION", "fp64")


def basis_precision(precision=None):
    """The precision a basis solve runs in: `precision`, else the module's
    BASIS_PRECISION; refuses anything but 'fp64' and 'mixed'."""
    p = BASIS_PRECISION if precision is None else precision
    if p not in PRECISIONS:
        raise ValueError(f"unknown basis precision {p!r}; known precisions "
                         f"are 'fp64' and 'mixed'")
    return p


def _solve_bases_mixed_door(masks, todo, v_basis, tol, stencil, verbose, unit=False):
    """The basis door's mixed-precision form: every requested basis in
    batched mixed-precision sessions, each to tol volts (tol / |v_basis|
    of the electrode span, in the max norm against the converged FP64
    solution of the same discrete problem).  unit: float32 unit bases
    (phi / v_basis) formed on the device instead of float64 potentials."""
    from ion_gym_gb300.physics.mixed import solve_bases_mixed
    n = len(masks)
    want = {i for _, i, _ in todo}

    def progress(done, total, idx):
        if _STOP.is_set():
            raise SolveInterrupted(f"stopped after {done} of {n} electrodes")
        print(f"  [{time.strftime('%H:%M:%S')}] solving electrodes "
              f"{idx[0]}..{idx[-1]} ({done + len(idx)} of {total}) in one "
              f"mixed-precision batch ...", flush=True)

    if _STOP.is_set():
        raise SolveInterrupted(f"stopped after 0 of {n} electrodes")
    t0 = time.time()
    out, st = solve_bases_mixed(masks, v_basis=v_basis,
                                accuracy=float(tol) / abs(float(v_basis)),
                                stencil=stencil, only=want, return_stats=True,
                                on_batch=progress, unit=unit)
    secs = time.time() - t0
    print(f"  {len(out)} bases in {st['batches']} mixed-precision batch(es), "
          f"{st['steps']} refinement steps ({secs:.1f}s)", flush=True)
    shape = next(iter(masks.values())).shape
    for _ in out:
        _record_solve(int(np.prod(shape)), secs / max(len(out), 1))
    return {i: out[i] for _, i, _ in todo}


def solve_unit_bases_mg(masks, v_basis=1e4, tol=1e-6, verbose=False,
                        stencil="ghost_linear", only=None, precision=None):
    """The basis door followed by the field cache's conversion to unit
    bases, {index: (phi / v_basis).astype(float32)} (build_stl3d.py:835-849:
    _solve_stl3d_bases divides the door's potentials by V_BASIS and stores
    float32).  With precision "mixed" the division and the cast run on the
    device after the batched solve (the same two roundings, so the same
    bits as converting solve_bases_mg's result on the host) and half the
    bytes come back; "fp64" converts the bit-exact door's result on the
    host.  Theta None only (the cache's STL route has no scene)."""
    prec = basis_precision(precision)
    if prec == "mixed":
        stencil_code(stencil)
        todo = [(j, i, m) for j, (i, m) in enumerate(sorted(masks.items()), 1)
                if only is None or i in only]
        return _solve_bases_mixed_door(masks, todo, v_basis, tol, stencil,
                                       verbose, unit=True)
    bases = solve_bases_mg(masks, v_basis=v_basis, tol=tol, verbose=verbose,
                           stencil=stencil, only=only, precision=prec)
    return {i: (b / v_basis).astype(np.float32) for i, b in bases.items()}


def solve_bases_mg(masks, scene=None, mirror=(False, False, False),
                   v_basis=1e4, tol=1e-6, verbose=False,
                   stencil="ghost_linear", theta=None, only=None,
                   precision=None):
    """The basis door (multigrid3d.py:233-291): for each electrode, in
    index order, the V-cycle on the metal union with that electrode at
    v_basis and the rest at 0.  Raises SolveInterrupted between bases after
    request_stop(), and refuses to return a basis whose delta is not below
    tol.  Up to BASIS_CONCURRENCY bases run at once (each on its own
    stream); progress lines, refusals and the returned dict follow the
    electrode order exactly as a one-at-a-time loop gives them.

    precision (not in the reference signature; default BASIS_PRECISION,
    "fp64"): "mixed" solves the bases in batches by the mixed-precision
    session instead, each to tol volts of the converged solution (max
    norm); it takes theta None only (no scene, no theta)."""
    from concurrent.futures import ThreadPoolExecutor
    prec = basis_precision(precision)
    metal = _union(masks)
    if prec == "mixed":
        if scene is not None or theta is not None:
            raise ValueError("solve_bases_mg: precision='mixed' solves the "
                             "plain stencil only (theta None); pass no scene "
                             "or theta, or use precision='fp64'")
        stencil_code(stencil)
        todo = [(j, i, m) for j, (i, m) in enumerate(sorted(masks.items()), 1)
                if only is None or i in only]
        return _solve_bases_mixed_door(masks, todo, v_basis, tol, stencil,
                                       verbose)
    th = theta
    if th is None and scene is not None:
        th = fractions_from_scene(scene, metal, mirror=mirror)
    th = None if th is None else as_f32(th)
    code = stencil_code(stencil)
    shape = metal.shape
    bom = optimal_omega(bottom_shape(shape))
    mu = as_mask(metal)
    items = sorted(masks.items())
    n = len(items)
    todo = [(j, i, m) for j, (i, m) in enumerate(items, start=1)
            if only is None or i in only]
    out = {}
    L = _lib.lib()

    def one(i, m):
        t0 = time.time()
        phi = np.empty(shape)
        sw = _lib.ctypes.c_long(0)
        d = _lib.ctypes.c_double(0.0)
        cyc = _lib.ctypes.c_int(0)
        prev = _lib.ctypes.c_double(0.0)
        st = L.ig_solve_basis_vmg(
            ptr(mu), ptr(as_mask(m)), float(v_basis), ptr(th), *shape,
            float(tol), 60, 3, 3, code, float(bom), ptr(phi),
            _lib.ctypes.byref(sw), _lib.ctypes.byref(d),
            _lib.ctypes.byref(cyc), _lib.ctypes.byref(prev))
        return st, phi, sw.value, d.value, cyc.value, prev.value, time.time() - t0

    workers = _basis_workers(len(todo), metal.size)
    pool = ThreadPoolExecutor(max_workers=workers)
    futs = {}
    nxt = 0

    def fill(upto):
        nonlocal nxt
        while nxt < len(todo) and nxt < upto:
            if _STOP.is_set():
                return
            _, i, m = todo[nxt]
            futs[nxt] = pool.submit(one, i, m)
            nxt += 1

    try:
        fill(workers)
        for q, (j, i, m) in enumerate(todo):
            if q not in futs:
                raise SolveInterrupted(f"stopped after {j - 1} of {n} electrodes")
            print(f"  [{time.strftime('%H:%M:%S')}] solving electrode {j} of "
                  f"{n} (basis {i}) ...", flush=True)
            st, phi, swv, dv, cycv, prevv, secs = futs.pop(q).result()
            _lib.check(st, "solve_bases_mg")
            phi, swv, dv = _vmg_outcome(st, shape, tol, 60, swv, dv, cycv, prevv,
                                        phi, False)
            print(f"  electrode {j} of {n}: {swv} sweeps, delta {dv:.2e} V "
                  f"({secs:.0f}s)", flush=True)
            if dv >= tol and not np.isnan(dv):
                raise SolveNotConverged(
                    f"basis {i}: delta {dv:.3e} V >= tol {tol:.1e} came back "
                    f"without a refusal; refusing to cache it.")
            out[i] = phi
            _record_solve(metal.size, secs)
            fill(q + 1 + workers)
    except KeyboardInterrupt:
        raise SolveInterrupted(f"interrupted during electrode solve "
                               f"(completed {len(out)} of {n})")
    finally:
        for f in futs.values():
            f.cancel()
        pool.shutdown(wait=True)
    return out


# ------------------------------------------------------------ kernels
def _residual(phi, fixed, th, ghost_linear_stencil, out):
    """multigrid3d._residual (multigrid3d.py:305-354) into out."""
    from ion_gym_gb300.physics import _device
    _device.residual(phi, fixed, th, ghost_linear_stencil, out)


def _sweep_rhs(e, fixed, f, omega, colour):
    """multigrid3d._sweep_rhs (multigrid3d.py:357-391)."""
    from ion_gym_gb300.physics import _device
    return _device.sweep_rhs(e, fixed, f, omega, colour)


def _residual_rhs(e, fixed, f, out):
    """multigrid3d._residual_rhs (multigrid3d.py:394-417)."""
    from ion_gym_gb300.physics import _device
    _device.residual_rhs(e, fixed, f, out)


def _restrict_fw_njit(fine, out):
    """multigrid3d._restrict_fw_njit (multigrid3d.py:420-455)."""
    from ion_gym_gb300.physics import _device
    _device.restrict_fw(fine, out)


def _prolong_add_njit(coarse, out, fixed):
    """multigrid3d._prolong_add_njit (multigrid3d.py:458-499)."""
    from ion_gym_gb300.physics import _device
    _device.prolong_add(coarse, out, fixed)


def _restrict_fw(fine):
    """Full-weighting restriction returning the coarse array
    (multigrid3d.py:529-550)."""
    shape = tuple((s + 1) // 2 for s in np.shape(fine))
    out = np.empty(shape)
    _restrict_fw_njit(fine, out)
    return out


def _restrict(fine):
    """Injection to the (n+1)//2 grid (multigrid3d.py:502-504)."""
    return np.ascontiguousarray(np.asarray(fine)[::2, ::2, ::2])


def _coarsen_fixed_any(fixed):
    """Block-ANY coarse mask (multigrid3d.py:507-526)."""
    from ion_gym_gb300.physics import _device
    return _device.coarsen_fixed_any(fixed)


def _coarsen_mask(fixed, val):
    """Injection + max-|val| block rescue (multigrid3d.py:85-135)."""
    from ion_gym_gb300.physics import _device
    return _device.coarsen_mask(fixed, val)


def _prolongate(phic, shape_f):
    """Cascadic trilinear prolongation (multigrid3d.py:138-171)."""
    from ion_gym_gb300.physics import _device
    return _device.prolongate(phic, shape_f)


def _solve_err(fixed, f, rel_tol=0.02, max_cycles=30, nu1=2, nu2=2,
               min_coarse=9, _depth=0):
    """The error-equation solve (multigrid3d.py:553-599), recursion on the
    device.  The V-cycle itself runs the same recursion inside the library;
    this module-level form serves callers of the reference's private name."""
    from ion_gym_gb300.physics import _device
    torch = _device._torch()
    fx = _device._mask_dev(fixed)
    fd = _device._to_dev(f, np.float64)
    e = _solve_err_dev(fx, fd, rel_tol, max_cycles, nu1, nu2, min_coarse)
    return e.cpu().numpy() if not _device._is_tensor(f) else e


def _solve_err_dev(fx, fd, rel_tol, max_cycles, nu1, nu2, min_coarse):
    from ion_gym_gb300.physics import _device as D
    torch = D._torch()
    e = torch.zeros_like(fd)
    scale = max(float(fd.abs().max().item()) if fd.numel() else 0.0, 1e-300)
    tol = rel_tol * scale / 6.0
    if min(fd.shape) <= min_coarse:
        om = optimal_omega(tuple(fd.shape))
        for _ in range(20000):
            d1 = D.sweep_rhs(e, fx, fd, om, 0)
            d2 = D.sweep_rhs(e, fx, fd, om, 1)
            if max(d1, d2) < 0.02 * tol:
                break
        return e
    fc = D.coarsen_fixed_any(fx.bool()).to(torch.uint8)
    r = torch.empty_like(e)
    for _ in range(max_cycles):
        for _s in range(nu1):
            D.sweep_rhs(e, fx, fd, 1.0, 0)
            D.sweep_rhs(e, fx, fd, 1.0, 1)
        D.residual_rhs(e, fx, fd, r)
        rc = torch.empty(tuple(fc.shape), dtype=torch.float64, device="cuda")
        D.restrict_fw(r, rc)
        rc *= 4.0
        ec = _solve_err_dev(fc, -rc, rel_tol, max_cycles, nu1, nu2,
                            min_coarse)
        D.prolong_add(ec, e, fx)
        d = 0.0
        for _s in range(nu2):
            d1 = D.sweep_rhs(e, fx, fd, 1.0, 0)
            d2 = D.sweep_rhs(e, fx, fd, 1.0, 1)
            d = max(d1, d2)
        if d < tol:
            break
    return e
