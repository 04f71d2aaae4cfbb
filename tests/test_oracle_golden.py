"""Pins the oracle (oracle/igoracle.c + oracle/port.py) to the reference.

Every fixture in tests/golden/ was produced by running the reference ion_gym
solver itself (tests/golden/make_golden.py).  The oracle must reproduce each
output bit for bit; only then is it trusted as the checker of the CUDA path.
"""
import numpy as np
import pytest

from conftest import same_bits
from oracle import port


def _th(c):
    return np.ascontiguousarray(c["th"], np.float32)


def test_sweep_kernel(kernels_golden):
    cases = kernels_golden.cases("sweep")
    assert len(cases) >= 30
    for c in cases:
        phi = c["phi"].copy()
        d = port.sweep(phi, c["fixed"].astype(bool), _th(c), float(c["omega"]),
                       int(c["colour"]), bool(c["ghost_linear"]))
        assert same_bits(phi, c["out"]), c["phi"].shape
        assert d == float(c["d"])


def test_residual_kernel(kernels_golden):
    for c in kernels_golden.cases("residual"):
        out = np.full(c["phi"].shape, np.nan)
        port.residual(c["phi"], c["fixed"].astype(bool), _th(c),
                      bool(c["ghost_linear"]), out)
        assert same_bits(out, c["out"])


def test_sweep_rhs_and_residual_rhs(kernels_golden):
    for c in kernels_golden.cases("sweep_rhs"):
        e = c["e"].copy()
        d = port.sweep_rhs(e, c["fixed"].astype(bool), c["f"],
                           float(c["omega"]), int(c["colour"]))
        assert same_bits(e, c["out"])
        assert d == float(c["d"])
        r = np.full(c["e"].shape, np.nan)
        port.residual_rhs(c["e"], c["fixed"].astype(bool), c["f"], r)
        assert same_bits(r, c["res"])


def test_restriction_and_coarse_masks(kernels_golden):
    for c in kernels_golden.cases("restrict"):
        assert same_bits(port.restrict_fw(c["fine"]), c["out"])
        fixed = c["fixed"].astype(bool)
        assert np.array_equal(port.coarsen_fixed_any(fixed),
                              c["any"].astype(bool))
        fc, vc = port.coarsen_mask(fixed, c["val"])
        assert np.array_equal(fc, c["fc"].astype(bool))
        assert same_bits(vc, c["vc"])


def test_prolongations(kernels_golden):
    for c in kernels_golden.cases("prolong"):
        o = c["base"].copy()
        port.prolong_add(c["coarse"], o, c["fixed"].astype(bool))
        assert same_bits(o, c["out"])
        assert same_bits(port.prolongate(c["coarse"], c["base"].shape),
                         c["prolongate"])


def test_audit_kernels(kernels_golden):
    for c in kernels_golden.cases("audit"):
        fixed = c["fixed"].astype(bool)
        assert same_bits(port.residual_audit(c["u"], fixed, _th(c)), c["res"])
        e = c["e"].copy()
        d = port.err_sweep(e, fixed, _th(c), c["rhs"], float(c["omega"]),
                           int(c["colour"]))
        assert same_bits(e, c["out"])
        assert d == float(c["d"])


def _opt(c, key):
    return c[key] if bool(c[f"has_{key}"]) else None


def test_solve3d_driver(drivers_golden):
    for c in drivers_golden.cases("solve3d"):
        theta = c["theta"] if bool(c["has_theta"]) else None
        omega = float(c["omega"]) if bool(c["omega_given"]) else None
        phi, sw, d = port.solve3d(c["fixed"].astype(bool), c["val"],
                                  theta=theta, tol=float(c["tol"]),
                                  omega=omega, phi0=_opt(c, "phi0"),
                                  stencil=str(c["stencil"]))
        assert sw == int(c["sweeps"]) and d == float(c["delta"])
        assert same_bits(phi, c["phi"])


def test_solve3d_refusal(drivers_golden):
    (c,) = drivers_golden.cases("solve3d_refuse")
    assert "too loose" in str(c["message"])
    (s,) = drivers_golden.cases("solve3d")[:1]
    with pytest.raises(port.SolveNotConverged, match="too loose"):
        port.solve3d(s["fixed"].astype(bool), s["val"], tol=1e-12,
                     max_sweeps=7)


def test_cascadic_driver(drivers_golden):
    for c in drivers_golden.cases("mg"):
        theta = c["theta"] if bool(c["has_theta"]) else None
        phi, sw, d = port.solve3d_mg(c["fixed"].astype(bool), c["val"],
                                     theta=theta, tol=float(c["tol"]),
                                     max_levels=int(c["max_levels"]),
                                     stencil=str(c["stencil"]))
        assert sw == int(c["sweeps"]) and d == float(c["delta"])
        assert same_bits(phi, c["phi"])


def test_vcycle_driver(drivers_golden):
    for c in drivers_golden.cases("vmg"):
        theta = c["theta"] if bool(c["has_theta"]) else None
        phi, sw, d = port.solve3d_vmg(c["fixed"].astype(bool), c["val"],
                                      theta=theta, tol=float(c["tol"]),
                                      stencil=str(c["stencil"]),
                                      phi0=_opt(c, "phi0"))
        assert sw == int(c["sweeps"]) and d == float(c["delta"])
        assert same_bits(phi, c["phi"])


def test_vcycle_refusals(drivers_golden):
    cap, stag, acc = drivers_golden.cases("vmg_refuse")
    assert "exhausted max_cycles" in str(cap["message"])
    assert "STAGNATED" in str(stag["message"])
    fp = np.zeros((20, 20, 20), bool)
    vp = np.zeros((20, 20, 20))
    fp[0] = fp[-1] = True
    vp[0] = 100.0
    with pytest.raises(port.SolveNotConverged, match="exhausted max_cycles"):
        port.solve3d_vmg(fp, vp, tol=1e-30, max_cycles=1)
    with pytest.raises(port.SolveNotConverged, match="STAGNATED"):
        port.solve3d_vmg(fp, vp, tol=1e-14, max_cycles=200)
    phi, sw, d = port.solve3d_vmg(fp, vp, tol=1e-14, max_cycles=200,
                                  accept_stagnation=True)
    assert sw == int(acc["sweeps"]) and d == float(acc["delta"])
    assert same_bits(phi, acc["phi"])


def test_basis_doors(drivers_golden):
    (b,) = drivers_golden.cases("bases")
    masks = {1: b["m1"].astype(bool), 2: b["m2"].astype(bool),
             4: b["m4"].astype(bool)}
    out = port.solve_bases(masks, tol=1e-6)
    for i in (1, 2, 4):
        assert same_bits(out[i], b[f"b{i}"])
    (m,) = drivers_golden.cases("bases_mg")
    masks = {1: m["m1"].astype(bool), 2: m["m2"].astype(bool),
             3: m["m3"].astype(bool)}
    out = port.solve_bases_mg(masks, tol=float(m["tol"]), only={1, 2})
    assert sorted(out) == list(m["keys"])
    for i in (1, 2):
        assert same_bits(out[i], m[f"b{i}"])


def test_relres_driver_restates_its_rule():
    """The oracle's residual-stopped cascadic driver (the quadrupole
    workload's rule; no reference driver to replay) is built from the pinned
    kernels above and the hierarchy of the pinned solve3d_mg; its own rule
    is checked here: the returned relative residual is max|r| / max|r(phi_D)|
    of the returned potential, every level's pairs are whole residual-check
    chunks, the level shapes are solve3d_mg's, and a tolerance already met
    runs no pair at all."""
    from ion_gym_gb300.physics.multigrid3d import cascadic_shapes
    n = 33
    i, j, k = np.meshgrid(*[np.arange(n, dtype=float)] * 3, indexing="ij")
    fixed = np.zeros((n, n, n), bool)
    fixed[0] = fixed[-1] = True
    fixed[:, 0] = fixed[:, -1] = True
    fixed[:, :, 0] = fixed[:, :, -1] = True
    s = (i - 16) ** 2 + (j - 16) ** 2 + (k - 16) ** 2 <= 25
    fixed |= s
    val = np.where(s, 1.0, 0.0)
    seen = []
    phi, fine, rr, tot, per = port.solve3d_cascadic_relres(
        fixed, val, rel_tol=1e-9, omega=1.8, max_levels=3, check_every=6,
        on_level=lambda L, shape, p, r: seen.append(shape))
    assert [tuple(x) for x in seen[::-1]] == cascadic_shapes((n,) * 3, 9, 3)
    assert all(p % 6 == 0 for p in per) and sum(per) == tot and per[-1] == fine
    ones = np.ones((6, n, n, n), np.float32)
    r = np.empty_like(phi)
    port.residual(phi, fixed, ones, True, r)
    phid = np.where(fixed, val, 0.0)
    r0 = np.empty_like(phi)
    port.residual(phid, fixed, ones, True, r0)
    assert rr == float(np.abs(r).max()) / float(np.abs(r0).max()) and rr < 1e-9
    assert np.array_equal(phi[fixed], val[fixed])
    _, fine0, _, tot0, _ = port.solve3d_cascadic_relres(fixed, val, rel_tol=2.0)
    assert fine0 == 0 and tot0 == 0
