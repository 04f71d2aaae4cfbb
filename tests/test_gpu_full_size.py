"""Parity at the full sizes of the benchmark workloads, through properties
that do not need a CPU solve of the same size (the oracle would take hours
there; the same kernels are pinned to it bit for bit on smaller grids):

* the 257^3 quadrupole, FP64 cascadic multigrid stopped on relative
  residual 1e-10: the returned relative residual is met when recomputed
  independently with the reference's residual operator, the solution is
  antisymmetric under x <-> y (the rods swap voltages), lies within the
  rods' +-1 V (maximum principle), and the mixed session agrees with it to
  the cascadic's own stopping accuracy;
* the 193 x 193 x 385 ring stack, 8 unit bases plus the grounded box in one
  mixed batch to 1e-9 of the span: the bases superpose to v_basis
  everywhere (all metal at v_basis has the constant solution), each lies in
  [0, v_basis], and one basis matches the bit-exact FP64 drop-in basis door.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

V = 1e4
ACC = 1e-9


def test_quadrupole_257_cascadic_properties():
    import torch
    from ion_gym_gb300.physics import _device as D
    from ion_gym_gb300.physics import multigrid3d as MG
    from ion_gym_gb300.physics.mixed import MixedSession
    from ion_gym_gb300.workloads import quadrupole
    torch.cuda.set_device(0)
    n = 257
    fixed, val = quadrupole(n)
    fx = torch.from_numpy(fixed.view(np.uint8)).cuda()
    vd = torch.from_numpy(val).cuda()
    phi, fine_pairs, relres, total = MG.solve3d_cascadic_relres(fx, vd, 1e-10, 1.85, 4, 9, 20)
    assert relres < 1e-10 and fine_pairs > 0
    # the stop rule recomputed with the reference's residual operator
    r = torch.empty_like(vd)
    D.residual(phi, fx, None, True, r)
    phid = torch.where(fx.bool(), vd, torch.zeros_like(vd))
    r0 = torch.empty_like(vd)
    D.residual(phid, fx, None, True, r0)
    assert float(r.abs().max() / r0.abs().max()) == pytest.approx(relres, rel=1e-12)
    p = phi.cpu().numpy()
    # x <-> y antisymmetry (the sum order of the stencil differs between a
    # node and its mirror, so equality holds to rounding)
    assert np.abs(p + p.transpose(1, 0, 2)).max() < 1e-9
    assert np.abs(p).max() <= 1.0 + 1e-8
    assert np.all(p[fixed] == val[fixed])
    # the mixed session solves the same discrete problem to 1e-9 of the
    # 2 V span; the cascadic stops at relative residual 1e-10, a few 1e-9
    # of the span from the exact solution
    with MixedSession(fixed, 1) as s:
        pm = s.solve_values(val, ACC)[0]
    assert np.abs(pm - p).max() / 2.0 < 1e-8


def test_ring_stack_bases_superpose_and_match_fp64():
    import torch
    from ion_gym_gb300.physics import multigrid3d as MG
    from ion_gym_gb300.physics.mixed import MixedSession
    from ion_gym_gb300.workloads import ring_stack
    torch.cuda.set_device(0)
    masks, box = ring_stack(0)
    metal = box.copy()
    for m in masks.values():
        metal |= m
    rings = sorted(masks)
    with MixedSession(metal, len(rings) + 1) as s:
        stack = [masks[i] for i in rings] + [box]
        out = torch.empty((len(stack),) + metal.shape, dtype=torch.float64, device="cuda")
        s.solve_bases(stack, V, ACC, out=out)
    total = out.sum(0)
    assert float((total - V).abs().max()) <= 9 * ACC * V
    assert float(out.min()) >= -ACC * V and float(out.max()) <= V * (1 + ACC)
    # one basis against the bit-exact FP64 drop-in (the reference's V-cycle
    # basis door at tol 1e-9 of the span)
    decks = dict(masks)
    decks[len(rings) + 1] = box       # the grounded box is metal too
    fp = MG.solve_bases_mg(decks, v_basis=V, tol=ACC * V, only={rings[0]})
    diff = np.abs(out[0].cpu().numpy() - fp[rings[0]]).max() / V
    assert diff < 2e-9
