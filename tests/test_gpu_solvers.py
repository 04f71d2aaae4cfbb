"""The drop-in solvers on the GPU return the reference's results bit for bit:
(phi, sweeps, delta) of solve3d, solve3d_mg, solve3d_vmg, solve_bases and
solve_bases_mg against the golden fixtures recorded from the reference, and
against the oracle on larger seeded problems.  Refusals raise the
reference's exceptions with its key phrases."""
import numpy as np
import pytest

from conftest import same_bits
from oracle import port

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


def _opt(c, key):
    return c[key] if bool(c[f"has_{key}"]) else None


def test_solve3d_golden(S, drivers_golden):
    for c in drivers_golden.cases("solve3d"):
        shape = c["fixed"].shape
        om = float(c["omega"])
        if not bool(c["omega_given"]):
            assert S.optimal_omega(shape) == om
        phi, sw, d = S.solve3d(c["fixed"].astype(bool), c["val"],
                               theta=_opt(c, "theta"), tol=float(c["tol"]),
                               omega=om, phi0=_opt(c, "phi0"),
                               stencil=str(c["stencil"]))
        assert (sw, d) == (int(c["sweeps"]), float(c["delta"]))
        assert same_bits(phi, c["phi"])


def test_solve3d_refuses(S, drivers_golden):
    c = drivers_golden.cases("solve3d")[0]
    with pytest.raises(S.SolveNotConverged, match="too loose"):
        S.solve3d(c["fixed"].astype(bool), c["val"], tol=1e-12, max_sweeps=7)
    with pytest.raises(ValueError, match="known stencils are"):
        S.solve3d(c["fixed"].astype(bool), c["val"], stencil="node")


def test_cascadic_golden(M, drivers_golden):
    for c in drivers_golden.cases("mg"):
        phi, sw, d = M.solve3d_mg(c["fixed"].astype(bool), c["val"],
                                  theta=_opt(c, "theta"), tol=float(c["tol"]),
                                  max_levels=int(c["max_levels"]),
                                  stencil=str(c["stencil"]))
        assert (sw, d) == (int(c["sweeps"]), float(c["delta"]))
        assert same_bits(phi, c["phi"])


def test_vcycle_golden(M, drivers_golden):
    for c in drivers_golden.cases("vmg"):
        phi, sw, d = M.solve3d_vmg(c["fixed"].astype(bool), c["val"],
                                   theta=_opt(c, "theta"), tol=float(c["tol"]),
                                   stencil=str(c["stencil"]),
                                   phi0=_opt(c, "phi0"))
        assert (sw, d) == (int(c["sweeps"]), float(c["delta"]))
        assert same_bits(phi, c["phi"])


def test_vcycle_refusals(M, S, drivers_golden):
    acc = drivers_golden.cases("vmg_refuse")[2]
    fp = np.zeros((20, 20, 20), bool)
    vp = np.zeros((20, 20, 20))
    fp[0] = fp[-1] = True
    vp[0] = 100.0
    with pytest.raises(S.SolveNotConverged, match="exhausted max_cycles"):
        M.solve3d_vmg(fp, vp, tol=1e-30, max_cycles=1)
    with pytest.raises(S.SolveNotConverged, match="STAGNATED"):
        M.solve3d_vmg(fp, vp, tol=1e-14, max_cycles=200)
    phi, sw, d = M.solve3d_vmg(fp, vp, tol=1e-14, max_cycles=200,
                               accept_stagnation=True)
    assert (sw, d) == (int(acc["sweeps"]), float(acc["delta"]))
    assert same_bits(phi, acc["phi"])


def test_basis_doors_golden(S, M, drivers_golden):
    (b,) = drivers_golden.cases("bases")
    masks = {1: b["m1"].astype(bool), 2: b["m2"].astype(bool),
             4: b["m4"].astype(bool)}
    out = S.solve_bases(masks, tol=1e-6)
    assert sorted(out) == [1, 2, 4]
    for i in (1, 2, 4):
        assert same_bits(out[i], b[f"b{i}"])
    (m,) = drivers_golden.cases("bases_mg")
    masks = {1: m["m1"].astype(bool), 2: m["m2"].astype(bool),
             3: m["m3"].astype(bool)}
    out = M.solve_bases_mg(masks, tol=float(m["tol"]), only={1, 2})
    assert sorted(out) == list(m["keys"])
    for i in (1, 2):
        assert same_bits(out[i], m[f"b{i}"])


def test_stop_interrupts_between_bases(M):
    masks = {1: np.zeros((12, 12, 12), bool), 2: np.zeros((12, 12, 12), bool)}
    masks[1][0] = True
    masks[2][-1] = True
    M.request_stop()
    try:
        with pytest.raises(M.SolveInterrupted, match="stopped after 0 of 2"):
            M.solve_bases_mg(masks, tol=1e-4)
        fixed = masks[1] | masks[2]
        with pytest.raises(M.SolveInterrupted, match="cycle 0"):
            M.solve3d_vmg(fixed, np.where(masks[1], 1e4, 0.0), tol=1e-4)
    finally:
        M.clear_stop()
    out = M.solve_bases_mg(masks, tol=1e-4)
    assert sorted(out) == [1, 2]


# ---------------------------------------------------------------- oracle
def _sphere_box(n, r, v=1.0):
    i, j, k = np.meshgrid(*[np.arange(n, dtype=float)] * 3, indexing="ij")
    c = (n - 1) / 2
    fixed = np.zeros((n, n, n), bool)
    fixed[0] = fixed[-1] = True
    fixed[:, 0] = fixed[:, -1] = True
    fixed[:, :, 0] = fixed[:, :, -1] = True
    s = (i - c) ** 2 + (j - c) ** 2 + (k - c) ** 2 <= r * r
    return fixed | s, np.where(s, v, 0.0)


def test_sphere_in_box_65_matches_oracle(S):
    """The plain FP64 SOR case: 65^3 box, r=10 sphere at 1 V, omega 1.9,
    tol 1e-8 -- identical sweeps, delta and potential."""
    fixed, val = _sphere_box(65, 10.0)
    phi, sw, d = S.solve3d(fixed, val, tol=1e-8, omega=1.9)
    po, swo, do = port.solve3d(fixed, val, tol=1e-8, omega=1.9)
    assert (sw, d) == (swo, do)
    assert same_bits(phi, po)


def test_vcycle_and_cascadic_match_oracle_49(M):
    rng = np.random.default_rng(11)
    shape = (49, 37, 45)
    fixed = np.zeros(shape, bool)
    fixed[:, 0] = fixed[:, -1] = True
    fixed[10:20, 15:18, 5:40] = True
    fixed[30:33, 5:30, 20:25] = True
    val = np.where(fixed, rng.choice([0.0, 1e4, -3e3], shape), 0.0)
    a = M.solve3d_vmg(fixed, val, tol=1e-6)
    b = port.solve3d_vmg(fixed, val, tol=1e-6)
    assert a[1:] == b[1:] and same_bits(a[0], b[0])
    a = M.solve3d_mg(fixed, val, tol=1e-7)
    b = port.solve3d_mg(fixed, val, tol=1e-7)
    assert a[1:] == b[1:] and same_bits(a[0], b[0])


def test_shortley_weller_vcycle_matches_oracle(M):
    rng = np.random.default_rng(12)
    shape = (33, 34, 21)
    fixed = np.zeros(shape, bool)
    fixed[0] = True
    fixed[12:20, 10:24, 8:13] = True
    val = np.where(fixed[:, :, :] & (np.arange(33)[:, None, None] > 0), 1e4, 0.0)
    th = rng.uniform(0.3, 1.0, (6,) + shape).astype(np.float32)
    th[rng.random(th.shape) < 0.9] = 1.0
    for stencil in ("sw", "ghost_linear"):
        a = M.solve3d_vmg(fixed, val, theta=th, tol=1e-5, stencil=stencil)
        b = port.solve3d_vmg(fixed, val, theta=th, tol=1e-5, stencil=stencil)
        assert a[1:] == b[1:] and same_bits(a[0], b[0])
    # theta None with the Shortley-Weller residual (halved correction)
    a = M.solve3d_vmg(fixed, val, tol=1e-5, stencil="sw")
    b = port.solve3d_vmg(fixed, val, tol=1e-5, stencil="sw")
    assert a[1:] == b[1:] and same_bits(a[0], b[0])


def test_solve_stl3d_bases_golden_and_mixed(M, drivers_golden):
    """build_stl3d._solve_stl3d_bases (build_stl3d.py:835-849): the basis
    door at tol 1e-4 V, v_basis 1e4, as float32 unit bases -- the golden
    deck's bases 1 and 2 are the reference's own (b / 1e4) rounded to
    float32 bit for bit, basis 3 the oracle's; the mixed-precision form of
    the same call lands within the tolerance of the two solves (1e-4 V of
    1e4 V each) plus one float32 rounding."""
    from ion_gym_gb300.io import fa_cache
    (m,) = drivers_golden.cases("bases_mg")
    masks = {1: m["m1"].astype(bool), 2: m["m2"].astype(bool),
             3: m["m3"].astype(bool)}
    got = fa_cache.solve_stl3d_bases(masks)
    assert sorted(got) == [1, 2, 3]
    for i in (1, 2):
        want = (m[f"b{i}"] / 1e4).astype(np.float32)
        assert got[i].dtype == np.float32
        assert np.array_equal(got[i].view(np.uint32), want.view(np.uint32))
    o3 = port.solve_bases_mg(masks, v_basis=1e4, tol=1e-4, only={3})[3]
    assert np.array_equal(got[3].view(np.uint32),
                          (o3 / 1e4).astype(np.float32).view(np.uint32))
    mixed = fa_cache.solve_stl3d_bases(masks, precision="mixed")
    for i in (1, 2, 3):
        assert mixed[i].dtype == np.float32
        assert np.abs(mixed[i].astype(np.float64) - got[i]).max() <= 2e-8 + 2.0 ** -23
    # the mixed route forms the unit bases on the device: the bits of the
    # host conversion of the same session's float64 potentials
    phi = M.solve_bases_mg(masks, v_basis=1e4, tol=1e-4, precision="mixed")
    for i in (1, 2, 3):
        want = (phi[i] / 1e4).astype(np.float32)
        assert np.array_equal(mixed[i].view(np.uint32), want.view(np.uint32))


def test_basis_door_mixed_precision_batches(M):
    """solve_bases_mg(precision='mixed'): the requested bases, in index
    order, within 1e-9 of the span of the FP64 door's result at a tight
    tolerance, the same with several small batches as with one, and the
    stop flag honoured before the first batch."""
    rng = np.random.default_rng(21)
    shape = (37, 41, 33)
    box = np.zeros(shape, bool)
    box[0] = box[-1] = True
    box[:, 0] = box[:, -1] = True
    box[:, :, 0] = box[:, :, -1] = True
    masks = {9: box}
    i, j, k = np.ogrid[:37, :41, :33]
    for e in (2, 3, 5, 7):
        c = rng.uniform(8, 28, 3)
        masks[e] = ((i - c[0]) ** 2 + (j - c[1]) ** 2 + (k - c[2]) ** 2
                    <= rng.uniform(9, 25)) & ~box
    ref = M.solve_bases_mg(masks, tol=1e-9, only={2, 5, 7})
    got = M.solve_bases_mg(masks, tol=1e-5, only={2, 5, 7}, precision="mixed")
    assert list(got) == [2, 5, 7]
    for e in got:
        assert np.abs(got[e] - ref[e]).max() <= 1e-9 * 1e4 + 1e-9 * 1e4
    from ion_gym_gb300.physics.mixed import solve_bases_mixed
    small = solve_bases_mixed(masks, v_basis=1e4, accuracy=1e-9,
                              only={2, 5, 7}, batch=2)
    for e in got:
        assert np.abs(small[e] - got[e]).max() <= 2e-9 * 1e4
    M.request_stop()
    try:
        with pytest.raises(M.SolveInterrupted, match="stopped after 0"):
            M.solve_bases_mg(masks, tol=1e-5, precision="mixed")
    finally:
        M.clear_stop()
