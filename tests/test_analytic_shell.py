"""Analytic check of the sphere solve: a grounded concentric spherical shell.

Inner sphere r <= a at V0, every node at r >= b held at the exact potential
V(r) = V0 a (b - r) / (r (b - a)) (harmonic everywhere but the centre, so
the outer boundary carries no staircase error), with a = 10 and b = 30 cells
on the 65^3 grid of the sphere workload and scaled with the grid.  The only
discretisation error is the staircase of the inner sphere (node-Dirichlet),
first order in h: the tests bound the error and require it to fall at
least at order 0.7 per grid doubling.  The CPU test runs the oracle, the GPU
test the drop-in SOR, the residual-stopped cascadic driver and the mixed
session."""
import numpy as np
import pytest


def shell_case(n, v0=1.0):
    c = (n - 1) / 2.0
    s = (n - 1) / 64.0
    a, b = 10.0 * s, 30.0 * s
    i, j, k = np.meshgrid(*[np.arange(n, dtype=float)] * 3, indexing="ij")
    r = np.sqrt((i - c) ** 2 + (j - c) ** 2 + (k - c) ** 2)
    rs = np.maximum(r, 1e-300)
    exact = v0 * a * (b - rs) / (rs * (b - a))
    inner = r <= a
    outer = r >= b
    fixed = inner | outer
    val = np.where(inner, v0, 0.0) + np.where(outer, exact, 0.0)
    vac = ~fixed
    far = vac & (r > 1.5 * a)
    return fixed, val, exact, vac, far


def _errors(phi, exact, vac, far):
    d = np.abs(phi - exact)
    return float(d[vac].max()), float(d[far].max())


def test_oracle_concentric_shell_first_order():
    from oracle import port
    errs = []
    for n in (33, 65):
        fixed, val, exact, vac, far = shell_case(n)
        phi, _, _ = port.solve3d(fixed, val, tol=1e-10)
        errs.append(_errors(phi, exact, vac, far))
    assert errs[1][0] < 0.1 and errs[1][1] < 0.03, errs
    assert np.log2(errs[0][1] / errs[1][1]) > 0.7, errs


@pytest.mark.gpu
def test_gpu_solvers_concentric_shell():
    from ion_gym_gb300.physics import solver3d as S
    from ion_gym_gb300.physics import multigrid3d as M
    from ion_gym_gb300.physics.mixed import MixedSession
    errs = {}
    for n in (33, 65):
        fixed, val, exact, vac, far = shell_case(n)
        phi, _, _ = S.solve3d(fixed, val, tol=1e-10)
        errs[n] = _errors(phi, exact, vac, far)
    fixed, val, exact, vac, far = shell_case(129)
    phi, _, rr, _ = M.solve3d_cascadic_relres(fixed, val, rel_tol=1e-12,
                                              omega=1.9, max_levels=4)
    errs[129] = _errors(phi, exact, vac, far)
    with MixedSession(fixed, 1) as s:
        pm = s.solve_values(val, 1e-9)[0]
    # the two 129^3 solutions solve the same discrete problem
    assert np.abs(pm - phi).max() < 1e-8
    em = _errors(pm, exact, vac, far)
    assert abs(em[0] - errs[129][0]) < 1e-8
    assert errs[65][0] < 0.1 and errs[65][1] < 0.03, errs
    assert errs[129][0] < 0.06 and errs[129][1] < 0.016, errs
    assert np.log2(errs[33][1] / errs[65][1]) > 0.7, errs
    assert np.log2(errs[65][1] / errs[129][1]) > 0.8, errs
