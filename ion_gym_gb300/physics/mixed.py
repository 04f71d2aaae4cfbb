"""Mixed-precision batched basis solves: every electrode basis of a deck in
one batch, FP32 multigrid inside FP64 iterative refinement.

Same inputs and outputs as multigrid3d.solve_bases_mg ({index: mask} ->
{index: phi float64 at v_basis}) but a different stopping rule: each basis
is refined until the error left after a refinement step, estimated from
that step's applied FP64 change and the observed contraction of the
changes, is below `accuracy` x the electrode span (v_basis), so the
potential is within that accuracy of the exact solution of the same
discrete problem (the reference's fine operator: theta None, 7-point,
even-reflection faces, Dirichlet metal).  The FP64 drop-in solves the same problem with the
reference's V-cycle and its cycle-delta rule; the two agree to the stated
accuracy (tests/test_gpu_mixed.py).
"""
import ctypes

import numpy as np

from ion_gym_gb300 import _lib
from ion_gym_gb300._lib import ptr, as_mask
from ion_gym_gb300.physics.solver3d import (SolveNotConverged, stencil_code,
                                            _union)


# Method of the FP32 correction solve: method 1 = flexible CG preconditioned
# by one multigrid cycle, cg_iters iterations per refinement step; method 0
# = defect correction with `vcycles` cycles per step.  Cycle shape:
# nu1/nu2 red-black smoothing pairs before/after the coarse correction,
# gamma 1 (V) or 2 (W; gamma_levels limits the second coarse visit to the
# finest levels, 0 = all), smoother relaxation factor.
#
# The default depends on the batch (from GPU sweeps with the tail stopping
# rule): a session of one to three problems runs V(3,3) with 3 CG
# iterations per step -- its coarse launches are small and latency-bound,
# so a second coarse visit only costs (quadrupole 141 against 98-114
# solves/s with W) --; a batch of four or more runs (2,2) pairs, 3 CG
# iterations and a W-cycle at the top level only, whose better coarse
# correction saves refinement steps once the coarse launches carry the
# whole batch (8 ring-stack bases 131 -> 174 solves/s, 25 board bases
# 651 -> 682).
CYCLE_SINGLE = {"nu1": 3, "nu2": 3, "vcycles": 2, "gamma": 1, "gamma_levels": 0,
                "smooth_omega": 1.0, "method": 1, "cg_iters": 3}
CYCLE_BATCH = {"nu1": 2, "nu2": 2, "vcycles": 2, "gamma": 2, "gamma_levels": 1,
               "smooth_omega": 1.0, "method": 1, "cg_iters": 3}
BATCH_MIN = 4
CYCLE = CYCLE_SINGLE   # the single-problem cycle (kept under its old name)


def cycle_for(max_problems):
    """The default cycle of a session holding max_problems problems."""
    return dict(CYCLE_BATCH if int(max_problems) >= BATCH_MIN else CYCLE_SINGLE)


def session_bytes(shape, max_problems, per_problem=False):
    """Device bytes a MixedSession of this grid and batch holds
    (per_problem: one metal per problem)."""
    fn = _lib.lib().ig_mixed_bytes_multi if per_problem else _lib.lib().ig_mixed_bytes
    return int(fn(*[int(s) for s in shape], int(max_problems)))


class MixedSession:
    """One geometry resident on the GPU: its multigrid hierarchy, the FP64
    potentials of up to `max_problems` problems and the captured CUDA graphs
    stay allocated between solves.  Each session owns a CUDA stream, so
    sessions of different geometries, driven from different host threads,
    run concurrently on the device."""

    def __init__(self, metal, max_problems=None, stencil="ghost_linear", **cycle):
        """metal: the (nx, ny, nz) metal union every problem shares, or a
        (P, nx, ny, nz) stack of one metal per problem (decks of one grid
        shape solved as one batch with solve_values; max_problems is then
        P).  cycle: overrides of the batch-size default (`cycle_for`): nu1,
        nu2, vcycles, gamma, gamma_levels, smooth_omega, method,
        cg_iters."""
        metal = np.ascontiguousarray(np.asarray(metal, bool))
        self.per_problem = metal.ndim == 4
        if self.per_problem:
            self.shape = metal.shape[1:]
            self.max_problems = int(metal.shape[0])
            if max_problems not in (None, self.max_problems):
                raise ValueError("MixedSession: a stack of metals sets max_problems")
        else:
            if max_problems is None:
                raise TypeError("MixedSession: max_problems is required with one metal")
            self.shape = metal.shape
            self.max_problems = int(max_problems)
        unknown = set(cycle) - set(CYCLE_SINGLE)
        if unknown:
            raise TypeError(f"MixedSession: unknown cycle settings {sorted(unknown)}")
        self.cycle = {**cycle_for(self.max_problems), **cycle}
        c = self.cycle
        self.nbytes = session_bytes(self.shape, self.max_problems, self.per_problem)
        self._h = ctypes.c_void_p(None)
        args = (stencil_code(stencil), int(c["nu1"]), int(c["nu2"]),
                int(c["vcycles"]), int(c["gamma"]), int(c["gamma_levels"]),
                float(c["smooth_omega"]), int(c["method"]), int(c["cg_iters"]),
                ctypes.byref(self._h))
        if self.per_problem:
            st = _lib.lib().ig_mixed_open_multi(ptr(as_mask(metal)), self.max_problems,
                                                *self.shape, *args)
        else:
            st = _lib.lib().ig_mixed_open_ex(ptr(as_mask(metal)), *self.shape,
                                             self.max_problems, *args)
        _lib.check(st, "MixedSession")

    def _outcome(self, st, steps, dmax, accuracy, span):
        _lib.check(st, "MixedSession")
        if st == _lib.IG_NOT_CONVERGED:
            raise SolveNotConverged(
                f"mixed-precision refinement: {steps} steps without reaching "
                f"{accuracy:.1e} of the span {span:g} V (worst applied change "
                f"{dmax.max():.3e} V)")

    def solve_bases(self, masks, v_basis=1e4, accuracy=1e-9, max_steps=40,
                    out=None):
        """masks: a sequence of (nx,ny,nz) bool arrays, a (B, nx, ny, nz)
        uint8 / bool numpy array (used in place: pinned host memory makes
        the upload fast), or a CUDA uint8 tensor already on the device ->
        potentials (B, nx, ny, nz) float64: a new numpy array, or `out` (a
        C-contiguous float64 numpy array -- pinned for a fast download -- or
        CUDA tensor) when given."""
        return self._bases(masks, v_basis, accuracy, max_steps, out, np.float64)

    def solve_unit_bases(self, masks, v_basis=1e4, accuracy=1e-9, max_steps=40,
                         out=None):
        """solve_bases returning the unit bases the field cache stores:
        float32 (B, nx, ny, nz), each (phi / v_basis).astype(float32) of the
        float64 potential solve_bases returns, bit for bit, formed on the
        device (half the bytes to download).  `out`: a C-contiguous float32
        numpy array or CUDA tensor to fill."""
        return self._bases(masks, v_basis, accuracy, max_steps, out, np.float32)

    def _bases(self, masks, v_basis, accuracy, max_steps, out, dtype):
        if type(masks).__module__.startswith("torch"):
            B = int(masks.shape[0])
            mptr = ctypes.c_void_p(masks.data_ptr())
        elif (isinstance(masks, np.ndarray) and masks.ndim == 4
              and masks.dtype in (np.uint8, np.bool_) and masks.flags.c_contiguous):
            B = int(masks.shape[0])
            mptr = ptr(masks)
        else:
            # a list of masks is stacked into the session's pinned staging
            # buffer (kept for the next call), so the upload runs at the
            # link's speed
            B = len(masks)
            stack = self._mask_stage(B)
            for b, m in enumerate(masks):
                stack[b] = np.asarray(m, bool)
            mptr = ptr(stack)
        if out is None:
            phi = np.empty((B,) + self.shape, dtype)
            pptr = ptr(phi)
        elif isinstance(out, np.ndarray):
            if out.dtype != dtype or not out.flags.c_contiguous or \
                    out.shape != (B,) + self.shape:
                raise ValueError(f"solve_bases: out must be a C-contiguous "
                                 f"{np.dtype(dtype).name} array of shape "
                                 f"{(B,) + self.shape}")
            phi = out
            pptr = ptr(out)
        else:
            phi = out
            pptr = ctypes.c_void_p(out.data_ptr())
        steps = ctypes.c_int(0)
        dmax = np.zeros(B)
        span = abs(float(v_basis))
        fn = (_lib.lib().ig_mixed_solve_bases if dtype == np.float64
              else _lib.lib().ig_mixed_solve_unit_bases)
        st = fn(self._h, mptr, B, float(v_basis), float(accuracy) * span,
                int(max_steps), pptr, ctypes.byref(steps), ptr(dmax))
        self._outcome(st, steps.value, dmax, accuracy, span)
        self.last_steps = int(steps.value)
        return phi

    def solve_values(self, vals, accuracy=1e-9, max_steps=40, out=None,
                     span=None):
        """vals: (P, nx, ny, nz) Dirichlet values (read at the metal nodes;
        on a session with one metal per problem, problem p's on metal p)
        -> array (P, nx, ny, nz); accuracy is relative to the span of the
        Dirichlet values (max - min of vals, at least 1 V; pass `span` when
        it is known, to skip the host pass over vals; a sequence of P spans
        gives each problem its own accuracy).  `out`: a C-contiguous
        float64 array of that shape to fill (pinned host memory makes the
        download fast)."""
        vals = np.ascontiguousarray(vals, np.float64)
        if vals.ndim == 3:
            vals = vals[None]
        P = vals.shape[0]
        if out is None:
            phi = np.empty_like(vals)
        else:
            if out.dtype != np.float64 or not out.flags.c_contiguous or \
                    out.size != vals.size:
                raise ValueError("solve_values: out must be a C-contiguous float64 "
                                 f"array of {vals.size} values")
            phi = out.reshape(vals.shape)
        steps = ctypes.c_int(0)
        dmax = np.zeros(P)
        if span is not None and np.ndim(span) == 1:
            spans = np.maximum(np.asarray(span, np.float64), 1.0)
            if spans.shape != (P,):
                raise ValueError(f"solve_values: {spans.shape[0]} spans for {P} problems")
            accs = np.ascontiguousarray(float(accuracy) * spans)
            st = _lib.lib().ig_mixed_solve_values_acc(
                self._h, ptr(vals), P, ptr(accs), int(max_steps), ptr(phi),
                ctypes.byref(steps), ptr(dmax))
            span = float(spans.min())
        else:
            span = max(float(np.ptp(vals)) if span is None else float(span), 1.0)
            st = _lib.lib().ig_mixed_solve_values(
                self._h, ptr(vals), P, float(accuracy) * span, int(max_steps),
                ptr(phi), ctypes.byref(steps), ptr(dmax))
        self._outcome(st, steps.value, dmax, accuracy, span)
        self.last_steps = int(steps.value)
        return phi

    def rebind(self, metal):
        """Give the session another geometry of the same shape: the new
        metal union replaces the old on every multigrid level, while the
        device buffers, the tuned smoother and the captured CUDA graphs are
        kept -- a solve after rebind costs no session build.  Results equal
        those of a session opened on the new metal."""
        metal = np.ascontiguousarray(np.asarray(metal, bool))
        want = ((self.max_problems,) + tuple(self.shape) if self.per_problem
                else tuple(self.shape))
        if metal.shape != want:
            raise ValueError(f"rebind: metal of shape {metal.shape}, session "
                             f"shape {want}")
        st = _lib.lib().ig_mixed_rebind(self._h, ptr(as_mask(metal)), *self.shape)
        _lib.check(st, "MixedSession.rebind")
        return self

    def step_bytes(self, n_problems=None):
        """Algorithmic DRAM bytes of one refinement step for n_problems
        problems (default: the session's maximum): every kernel's inputs
        read once and outputs written once, over all levels."""
        b = ctypes.c_double(0.0)
        n = self.max_problems if n_problems is None else int(n_problems)
        st = _lib.lib().ig_mixed_step_bytes(self._h, n, ctypes.byref(b))
        _lib.check(st, "MixedSession.step_bytes")
        return float(b.value)

    def set_cycle(self, nu1, nu2, cg_iters):
        """Change the session's cycle (smoothing pairs before and after the
        coarse correction, CG iterations per refinement step); the next
        solve recaptures its graphs, the buffers stay."""
        st = _lib.lib().ig_mixed_set_cycle(self._h, int(nu1), int(nu2), int(cg_iters))
        _lib.check(st, "MixedSession.set_cycle")
        self.cycle = {**self.cycle, "nu1": int(nu1), "nu2": int(nu2),
                      "cg_iters": int(cg_iters)}

    def solve_bytes(self):
        """Algorithmic DRAM bytes of every refinement step of the last
        solve."""
        b = ctypes.c_double(0.0)
        _lib.check(_lib.lib().ig_mixed_solve_bytes(self._h, ctypes.byref(b)),
                   "MixedSession.solve_bytes")
        return float(b.value)

    def tuning(self, n_problems=None):
        """The smoother shape the session's tuner chose (tuning first if
        needed): {"groups_per_thread", "threads", "temporal_depth" (half-
        sweeps per blocked pass on the finest level, 0 = separate launches),
        "us_per_half_sweep", "best_blocked_depth", "blocked_us_per_half_sweep"
        (the fastest blocked pass timed; 0 and None when none was)}."""
        ng, th = ctypes.c_int(0), ctypes.c_int(0)
        tb = (ctypes.c_int * 2)()
        us = (ctypes.c_double * 2)()
        n = self.max_problems if n_problems is None else int(n_problems)
        st = _lib.lib().ig_mixed_tuning(self._h, n, ctypes.byref(ng), ctypes.byref(th), tb, us)
        _lib.check(st, "MixedSession.tuning")
        return {"groups_per_thread": ng.value, "threads": th.value,
                "temporal_depth": tb[0], "us_per_half_sweep": round(us[0], 2),
                "best_blocked_depth": tb[1],
                "blocked_us_per_half_sweep": round(us[1], 2) if tb[1] else None}

    def _mask_stage(self, B):
        st = getattr(self, "_stage", None)
        if st is None or st.shape[0] < B:
            import torch
            st = torch.empty((B,) + self.shape, dtype=torch.uint8).pin_memory().numpy()
            self._stage = st
        return st[:B]

    def close(self):
        if self._h:
            _lib.lib().ig_mixed_close(self._h)
            self._h = ctypes.c_void_p(None)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def max_batch(shape, n_bases, budget_frac=0.8):
    """How many bases of this grid one MixedSession can hold in the free
    device memory (at least 1)."""
    try:
        free = int(_lib.lib().ig_device_free_bytes())
    except Exception:
        free = 0
    if free <= 0:
        return max(1, n_bases)
    b = max(1, n_bases)
    while b > 1 and session_bytes(shape, b) > budget_frac * free:
        b = (b + 1) // 2
    return b


def solve_bases_mixed(masks, v_basis=1e4, accuracy=1e-9,
                      stencil="ghost_linear", only=None, max_steps=40,
                      return_stats=False, batch=None, on_batch=None, unit=False,
                      **cycle):
    """All bases of a deck by the mixed-precision session: {index: mask} ->
    {index: phi float64 at v_basis} (unit: {index: (phi / v_basis) as
    float32}, formed on the device, MixedSession.solve_unit_bases).  The bases run in batches of `batch`
    (default: as many as free device memory holds, all of them when they
    fit) on one resident session.  on_batch(done, total, indices), when
    given, is called before each batch (and may raise to stop).  With
    return_stats, also {"steps": the largest refinement-step count of any
    batch, "batches": n}.  cycle: overrides of the batch-size default
    cycle (`cycle_for`)."""
    metal = _union(masks)
    items = [(i, np.asarray(m, bool)) for i, m in sorted(masks.items())
             if only is None or i in only]
    if not items:
        return ({}, {"steps": 0, "batches": 0}) if return_stats else {}
    B = int(batch) if batch else max_batch(metal.shape, len(items))
    B = max(1, min(B, len(items)))
    out = {}
    steps = 0
    nb = 0
    with MixedSession(metal, B, stencil=stencil, **cycle) as s:
        for q in range(0, len(items), B):
            part = items[q:q + B]
            if on_batch is not None:
                on_batch(q, len(items), [i for i, _ in part])
            solve = s.solve_unit_bases if unit else s.solve_bases
            phi = solve([m for _, m in part], v_basis, accuracy, max_steps)
            out.update({i: phi[b] for b, (i, _) in enumerate(part)})
            steps = max(steps, s.last_steps)
            nb += 1
    if return_stats:
        return out, {"steps": steps, "batches": nb}
    return out
