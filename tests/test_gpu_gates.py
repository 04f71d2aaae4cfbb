"""The reference's solver gates, run against the GPU drop-in.

Each test restates one gate of the reference test-suite (cited) with the
same geometry, tolerances and thresholds: analytic exactness and order
(tests/test_solver3d_analytic.py), V-cycle vs SOR (tests/test_multigrid.py),
never-silent convergence (tests/test_solver_convergence.py), nz=1 limits
(tests/test_solver3d_nz1.py) and fractional surfaces (tests/test_pasurf.py).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    from ion_gym_gb300.physics import solver3d
    return solver3d


@pytest.fixture(scope="module")
def M():
    from ion_gym_gb300.physics import multigrid3d
    multigrid3d.clear_stop()
    return multigrid3d


def _shell(shape):
    f = np.zeros(shape, bool)
    f[0] = f[-1] = True
    f[:, 0] = f[:, -1] = True
    f[:, :, 0] = f[:, :, -1] = True
    return f


# ---- test_solver3d_analytic.py -------------------------------------------
def test_quadratic_harmonic_is_exact(S):
    """S1-a (:40-49): x^2 + y^2 - 2 z^2 is discretely harmonic."""
    n = 33
    i, j, k = np.meshgrid(*[np.arange(n, dtype=float)] * 3, indexing="ij")
    exact = i * i + j * j - 2 * k * k
    fixed = _shell((n, n, n))
    phi, _, _ = S.solve3d(fixed, np.where(fixed, exact, 0.0), tol=1e-9)
    assert np.abs(phi - exact)[~fixed].max() < 1e-6


def test_second_order_convergence(S):
    """S1-b (:52-69): sin sin sinh error falls ~h^2 (order > 1.8)."""
    errs = []
    for n in (17, 33):
        x = np.arange(n) / (n - 1)
        X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
        a = np.pi
        exact = np.sin(a * X) * np.sin(a * Y) * np.sinh(np.hypot(a, a) * Z)
        fixed = _shell((n, n, n))
        phi, _, _ = S.solve3d(fixed, np.where(fixed, exact, 0.0), tol=1e-10)
        errs.append(np.abs(phi - exact)[~fixed].max())
    assert np.log2(errs[0] / errs[1]) > 1.8


def _coax_rings(N, c, r, nz):
    ii, jj = np.meshgrid(np.arange(N, dtype=float), np.arange(N, dtype=float),
                         indexing="ij")
    rr = np.hypot(ii - c, jj - c)
    inner = (rr <= r)[:, :, None] & np.ones((1, 1, nz), bool)
    ring = (rr >= 32)[:, :, None] & np.ones((1, 1, nz), bool)
    exact = np.log(np.maximum(rr, r) / 32.0) / np.log(r / 32.0) * 100.0
    val = np.where(inner, 100.0, 0.0) + np.where(ring, exact[:, :, None], 0.0)
    return inner, ring, val, rr, exact


def test_fold_matches_full(S):
    """S1-c (:79-106): the x,y-folded quadrant with mirror flags equals the
    full domain's quadrant."""
    n, nz, r = 41, 9, 6.3
    inner, ring, val, _, _ = _coax_rings(2 * n - 1, 40.0, r, nz)
    full, _, _ = S.solve3d(inner | ring, val, tol=1e-8)
    qi, qr, qv, _, _ = _coax_rings(n, 0.0, r, nz)
    fold, _, _ = S.solve3d(qi | qr, qv, mirror=(True, True, False), tol=1e-8)
    assert np.abs(fold - full[40:, 40:, :]).max() < 1e-5


def test_shortley_weller_beats_node_dirichlet(S):
    """S1-d/e (:109-138): fractional legs on a non-lattice inner radius."""
    from ion_gym_gb300.physics.scene3d import (GeomScene, GridSpec, Electrode,
                                               Shape, Cylinder)
    n, nz, r, c = 81, 9, 6.3, 40.0
    inner, ring, val, rr, exact2 = _coax_rings(n, c, r, nz)
    exact = exact2[:, :, None] * np.ones((1, 1, nz))
    fixed = inner | ring
    vac = ~fixed & (rr[:, :, None] > r) & (rr[:, :, None] < 32)
    p0, _, _ = S.solve3d(fixed, val, tol=1e-8)
    e0 = np.abs(p0 - exact)[vac].max()
    sc = GeomScene(grid=GridSpec(n, n, nz), units="gu", electrodes=[
        Electrode(1, "inner", [Shape([Cylinder(c, c, nz + 2.0, r,
                                               nz + 4.0)])])])
    th = S.fractions_from_scene(sc, inner)
    p1, _, _ = S.solve3d(fixed, val, theta=th, tol=1e-8, stencil="sw")
    p2, _, _ = S.solve3d(fixed, val, theta=th, tol=1e-8, stencil="ghost_linear")
    assert np.abs(p1 - exact)[vac].max() * 10 <= e0
    assert np.abs(p2 - exact)[vac].max() * 3 <= e0


# ---- test_multigrid.py -----------------------------------------------------
def _plate(n=65, thin=False):
    fixed = np.zeros((n, n, 33), bool)
    val = np.zeros(fixed.shape)
    w = 1 if thin else 3
    fixed[n // 4:3 * n // 4, n // 2:n // 2 + w, 8:25] = True
    val[fixed] = 1e4
    fixed[:, 0, :] = True
    fixed[:, -1, :] = True
    return fixed, val


@pytest.mark.parametrize("thin", [False, True])
def test_vcycle_same_fixed_point_as_sor(S, M, thin):
    """Gates 1 and 2 (:34-52): plate + walls, thick and one-node plates."""
    fixed, val = _plate(thin=thin)
    ps, _, _ = S.solve3d(fixed, val, tol=1e-6)
    pv, _, d = M.solve3d_vmg(fixed, val, tol=1e-6)
    assert d < 1e-6 and np.abs(pv - ps).max() < 5e-4


def test_vcycle_with_mirror(S, M):
    """Gate 3 (:55-66)."""
    n = 65
    fixed = np.zeros((n, n, 17), bool)
    val = np.zeros(fixed.shape)
    fixed[n // 4:3 * n // 4, n // 4:3 * n // 4, 12:15] = True
    val[fixed] = 1e4
    fixed[0] = True
    ps, _, _ = S.solve3d(fixed, val, mirror=(False, False, True), tol=1e-6)
    pv, _, d = M.solve3d_vmg(fixed, val, mirror=(False, False, True), tol=1e-6)
    assert d < 1e-6 and np.abs(pv - ps).max() < 5e-4


def test_vcycle_accelerates(S, M):
    """Gate 4 (:69-84): fewer than half of SOR's fine sweeps."""
    fixed = np.zeros((129, 65, 33), bool)
    val = np.zeros(fixed.shape)
    fixed[10:119, 30:33, 8:25] = True
    val[fixed] = 1e4
    fixed[:, 0, :] = True
    ps, ss, _ = S.solve3d(fixed, val, tol=1e-6)
    pv, sv, d = M.solve3d_vmg(fixed, val, tol=1e-6)
    assert d < 1e-6 and np.abs(pv - ps).max() < 5e-4
    assert sv < 0.5 * ss


# ---- test_solver_convergence.py -------------------------------------------
def test_stalled_sor_refuses(S):
    """SC-1 (:50-63): a 520x80 thin domain at 200 sweeps raises."""
    metal = np.zeros((520, 80, 1), bool)
    metal[100:110, 30:50] = True
    metal[250:260, 30:50] = True
    metal[400:410, 30:50] = True
    val = np.zeros(metal.shape)
    val[400:410, 30:50] = 1e4
    with pytest.raises(S.SolveNotConverged, match="too loose"):
        S.solve3d(metal, val, tol=1e-4, max_sweeps=200)


def test_tolerance_controls_and_plates_exact(S, M):
    """SC-2/SC-3 (:65-91): tol moves the answer; SOR and the V-cycle are
    exact on parallel plates and agree."""
    m1 = np.zeros((48, 24, 1), bool)
    m1[0] = True
    m2 = np.zeros((48, 24, 1), bool)
    m2[-1] = True
    masks = {1: m1, 2: m2}
    a = S.solve_bases(masks, v_basis=1e4, tol=1e-4)
    b = S.solve_bases(masks, v_basis=1e4, tol=1e-10)
    assert np.abs(a[1] - b[1]).max() > 0.0
    i = np.arange(48)[:, None, None]
    exact = 1e4 * (1.0 - i / 47.0) * np.ones((48, 24, 1))
    g = M.solve_bases_mg(masks, v_basis=1e4, tol=1e-8)
    assert np.abs(b[1] - exact).max() / 1e4 < 1e-6
    assert np.abs(g[1] - exact).max() / 1e4 < 1e-6
    assert np.abs(b[1] - g[1]).max() / 1e4 < 1e-6


# ---- test_solver3d_nz1.py --------------------------------------------------
def _axis_potential(S, ex, ey, nz, N=51, C=25):
    metal = np.zeros((N, N, nz), bool)
    metal[0] = metal[-1] = True
    metal[:, 0] = metal[:, -1] = True
    metal[ex - 2:ex + 3, ey - 2:ey + 3] = True
    val = np.zeros(metal.shape)
    val[ex - 2:ex + 3, ey - 2:ey + 3] = 1e4
    phi, _, _ = S.solve3d(metal, val, tol=1e-8, max_sweeps=20000, omega=1.0)
    return phi[C, C, nz // 2], phi


def test_nz1_limits(S):
    """Z-1..Z-3 (:48-74): x/y symmetry, nz invariance, 2-D 5-point mean."""
    vx, phi = _axis_potential(S, 40, 25, 1)
    vy, _ = _axis_potential(S, 25, 40, 1)
    assert abs(vx - vy) < 1e-4
    v3, _ = _axis_potential(S, 40, 25, 3)
    v5, _ = _axis_potential(S, 40, 25, 5)
    assert abs(vx - v3) < 1e-3 and abs(vx - v5) < 1e-3
    i, j = 15, 30
    mean4 = 0.25 * (phi[i - 1, j, 0] + phi[i + 1, j, 0] + phi[i, j - 1, 0]
                    + phi[i, j + 1, 0])
    assert abs(phi[i, j, 0] - mean4) < 1e-3


# ---- test_pasurf.py ----------------------------------------------------------
def _cyl_problem(n=176, a=20.0, b=80.0):
    from ion_gym_gb300.physics.scene3d import (GeomScene, GridSpec, Electrode,
                                               Shape, Cylinder)
    c = (n - 1) / 2
    X, Y = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    R = np.hypot(X - c, Y - c)
    fixed = ((R <= a) | (R >= b))[:, :, None]
    val = np.zeros((n, n, 1))
    val[(R >= b)[:, :, None]] = 100.0
    sc = GeomScene(grid=GridSpec(nx=n, ny=n, nz=1), units="gu", electrodes=[
        Electrode(1, "i", [Shape(within=[Cylinder(c, c, 5, a, 10)])]),
        Electrode(2, "o", [Shape(within=[Cylinder(c, c, 5, b + 40, 10)],
                                 notin=[Cylinder(c, c, 5, b, 10)])])])
    Vex = 100 * np.log(np.maximum(R, 1e-9) / a) / np.log(b / a)
    return fixed, val, sc, Vex, (R > a) & (R < b), R - a


def test_fractional_surface_collapses_error(S):
    """(:29-42): thetas shrink the curved-surface error > 20x."""
    fixed, val, sc, Vex, m, d = _cyl_problem()
    Vi, _, _ = S.solve3d(fixed, val, tol=1e-5)
    th = S.fractions_from_scene(sc, fixed)
    assert (th < 0.999).sum() > 500
    Vf, _, _ = S.solve3d(fixed, val, theta=th, tol=1e-5)
    surf = m & (d >= 0) & (d < 1)
    ei = np.abs(Vi[:, :, 0] - Vex)[surf].max()
    ef = np.abs(Vf[:, :, 0] - Vex)[surf].max()
    assert ei > 1.0 and ef < 0.1 and ef < ei / 20


def test_vcycle_carries_theta(S, M):
    """(:45-52): V-cycle with theta matches SOR with theta."""
    fixed, val, sc, *_ = _cyl_problem()
    th = S.fractions_from_scene(sc, fixed)
    Vs, _, _ = S.solve3d(fixed, val, theta=th, tol=1e-6)
    Vm, _, _ = M.solve3d_vmg(fixed, val, theta=th, tol=1e-5)
    assert np.abs(Vm - Vs).max() < 5e-3
