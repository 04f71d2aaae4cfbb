"""Small, self-contained launches of one kernel for profiling (ncu) and
timing: the arrays are built, a few launches run, the process exits.

    python -m ion_gym_gb300.profile_case sweep_f64 --n 257 --pairs 4

Cases:
  sweep_f64   FP64 red-black sweep (k_sweep<kPlain>) on the 257^3
              quadrupole, `pairs` red-black pairs, omega 1.85
  mixed_rings the mixed-precision basis batch of the ring stack (8 bases)
  mixed_quad  the mixed-precision solve of the 257^3 quadrupole (one problem)
  mixed_board the mixed-precision bases of a 512x128x96 planar board
"""
import argparse
import ctypes
import time

import numpy as np


def sweep_f64(n, pairs):
    import torch
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.workloads import quadrupole
    fixed, val = quadrupole(n)
    # a mid-solve state: Dirichlet values on the rods and box, a smooth
    # nonzero field elsewhere (a cold start of zeros is not representative)
    x = np.linspace(-1.0, 1.0, n)
    smooth = 0.3 * (x[:, None, None] ** 2 - x[None, :, None] ** 2) \
        + 0.01 * np.cos(3 * x)[None, None, :]
    phi = torch.from_numpy(np.where(fixed, val, smooth)).cuda()
    fx = torch.from_numpy(fixed.view(np.uint8)).cuda()
    L = _lib.lib()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    d = ctypes.c_double(0.0)
    t0 = time.perf_counter()
    for _ in range(pairs):
        for colour in (0, 1):
            st = L.ig_sweep_dev(ctypes.c_void_p(phi.data_ptr()),
                                ctypes.c_void_p(fx.data_ptr()), None,
                                n, n, n, 1.85, colour, 0, ctypes.byref(d), s)
            _lib.check(st, "ig_sweep_dev")
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    print(f"sweep_f64 n={n}: {pairs} pairs in {el * 1e3:.2f} ms "
          f"({n ** 3 * pairs / el / 1e9:.1f} GLUP/s incl. host syncs), "
          f"last max|d| {d.value:.3e}")


def mixed_rings(solves, gs_pairs):
    """One resident session of the 193x193x385 ring stack (8 bases + the
    grounded box as metal): `solves` mixed solves to 1e-9 of the span, then
    `gs_pairs` timed pairs of the fine-level FP32 smoother alone."""
    import torch
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.workloads import ring_stack
    from ion_gym_gb300.physics.mixed import MixedSession
    masks, box = ring_stack(0)
    metal = box.copy()
    for m in masks.values():
        metal |= m
    rings = [masks[i] for i in sorted(masks)]
    with MixedSession(metal, len(rings)) as s:
        for _ in range(solves):
            t0 = time.perf_counter()
            s.solve_bases(rings, 1e4, 1e-9)
            print(f"mixed_rings: 8 bases in {time.perf_counter() - t0:.3f} s, "
                  f"{s.last_steps} refinement steps")
        if gs_pairs:
            ms = ctypes.c_double(0)
            by = ctypes.c_double(0)
            _lib.lib().ig_mixed_time_gs(s._h, len(rings), gs_pairs,
                                        ctypes.byref(ms), ctypes.byref(by))
            print(f"k_gs: {ms.value * 1e3:.1f} us per launch, "
                  f"{by.value / (ms.value * 1e-3) / 1e9:.0f} GB/s algorithmic")
    torch.cuda.synchronize()


def mixed_quad(n, solves):
    """The 257^3 quadrupole (one problem) solved by a resident mixed session
    to 1e-9 of its 2 V span, `solves` times (values already on the
    device)."""
    import torch
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.workloads import quadrupole
    from ion_gym_gb300.physics.mixed import MixedSession
    fixed, val = quadrupole(n)
    v = torch.from_numpy(val[None].copy()).cuda()
    out = torch.empty_like(v)
    L = _lib.lib()
    with MixedSession(fixed, 1) as s:
        for _ in range(solves):
            steps = ctypes.c_int(0)
            dmax = np.zeros(1)
            t0 = time.perf_counter()
            st = L.ig_mixed_solve_values(s._h, ctypes.c_void_p(v.data_ptr()), 1, 1e-9 * 2.0,
                                         40, ctypes.c_void_p(out.data_ptr()),
                                         ctypes.byref(steps),
                                         dmax.ctypes.data_as(ctypes.c_void_p))
            _lib.check(st, "mixed_quad")
            print(f"mixed_quad n={n}: {time.perf_counter() - t0:.4f} s, "
                  f"{steps.value} refinement steps")
    torch.cuda.synchronize()


def mixed_board(solves, n_el=24):
    """A seeded 512x128x96 planar board (n_el extruded electrodes on two
    layers plus the grounded box): its unit bases in one resident session
    to 1e-9 of the span, `solves` times (masks already on the device)."""
    import torch
    from ion_gym_gb300.workloads import planar_board
    from ion_gym_gb300.physics.mixed import MixedSession
    masks, box = planar_board(101, shape=(512, 128, 96), n_electrodes=n_el)
    masks = {k: m for k, m in masks.items() if m.any()}
    metal = box.copy()
    for m in masks.values():
        metal |= m
    stack = torch.from_numpy(
        np.stack([masks[k] for k in sorted(masks)]).view(np.uint8)).cuda()
    out = torch.empty(stack.shape, dtype=torch.float64, device="cuda")
    with MixedSession(metal, len(masks)) as s:
        for _ in range(solves):
            t0 = time.perf_counter()
            s.solve_bases(stack, 1e4, 1e-9, out=out)
            print(f"mixed_board: {len(masks)} bases in {time.perf_counter() - t0:.4f} s, "
                  f"{s.last_steps} refinement steps")
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["sweep_f64", "mixed_rings", "mixed_quad",
                                     "mixed_board"])
    ap.add_argument("--n", type=int, default=257)
    ap.add_argument("--pairs", type=int, default=4)
    ap.add_argument("--solves", type=int, default=1)
    a = ap.parse_args()
    if a.case == "sweep_f64":
        sweep_f64(a.n, a.pairs)
    elif a.case == "mixed_quad":
        mixed_quad(a.n, a.solves)
    elif a.case == "mixed_board":
        mixed_board(a.solves)
    else:
        mixed_rings(a.solves, a.pairs)


if __name__ == "__main__":
    main()
