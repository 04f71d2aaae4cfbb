"""The residual-stopped cascadic solve of the quadrupole workload
(multigrid3d.solve3d_cascadic_relres, ig_cascadic_relres) against the
oracle's restatement of the same driver (oracle.port.solve3d_cascadic_relres):
identical fine pairs, pairs on all levels, fine relative residual and
potential, bit for bit -- quadrupoles at 65^3 and 97^3, an odd/even
non-cubic random deck, per-level SOR factors, a one-level hierarchy and a
level cap of two; the device-array and host-array forms of the call alike.
FP64 integer-exact parity: the tolerance of these tests is bit equality."""
import numpy as np
import pytest

from conftest import same_bits
from oracle import port

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    from ion_gym_gb300.physics import multigrid3d
    multigrid3d.clear_stop()
    return multigrid3d


def _crop_deck(seed, side, n_el, shape):
    """A random deck cut to `shape`, its cut faces grounded again."""
    from ion_gym_gb300.workloads import random_deck
    f, v = random_deck(seed, side, n_el)
    f = np.ascontiguousarray(f[:shape[0], :shape[1], :shape[2]])
    v = np.ascontiguousarray(v[:shape[0], :shape[1], :shape[2]])
    for a in range(3):
        sl = [slice(None)] * 3
        sl[a] = -1
        f[tuple(sl)] = True
        v[tuple(sl)] = 0.0
    return f, v


def _check(M, fixed, val, device, **kw):
    import torch
    o_phi, o_fine, o_rr, o_tot, _ = port.solve3d_cascadic_relres(fixed, val, **kw)
    if device:
        fx = torch.from_numpy(np.ascontiguousarray(fixed).view(np.uint8)).cuda()
        vd = torch.from_numpy(np.ascontiguousarray(val)).cuda()
        phi, fine, rr, tot = M.solve3d_cascadic_relres(fx, vd, **kw)
        phi = phi.cpu().numpy()
    else:
        phi, fine, rr, tot = M.solve3d_cascadic_relres(fixed, val, **kw)
    assert (fine, tot) == (o_fine, o_tot)
    assert rr == o_rr
    assert same_bits(phi, o_phi)
    return fine, tot


@pytest.mark.parametrize("n,r0", [(65, 8.0), (97, 12.0)])
def test_quadrupole_relres_matches_oracle(M, n, r0):
    from ion_gym_gb300.workloads import quadrupole
    fixed, val = quadrupole(n, r0)
    fine, tot = _check(M, fixed, val, True, rel_tol=1e-10, omega=1.85,
                       max_levels=4, min_coarse=9, check_every=20)
    assert fine > 0 and tot > fine


def test_noncubic_deck_relres_matches_oracle(M):
    """Odd and even extents on different axes; five levels, per-level SOR
    factors, a residual check every 7 pairs; host arrays in and out."""
    fixed, val = _crop_deck(31, 97, 7, (97, 74, 83))
    _check(M, fixed, val, False, rel_tol=1e-9,
           omega=[1.9, 1.85, 1.8, 1.7, 1.6], max_levels=5, min_coarse=9,
           check_every=7)


@pytest.mark.parametrize("max_levels", [1, 2])
def test_short_hierarchies_match_oracle(M, max_levels):
    """One level (the fine grid alone, from its Dirichlet values) and two."""
    fixed, val = _crop_deck(5, 49, 4, (41, 49, 36))
    _check(M, fixed, val, True, rel_tol=1e-8, omega=1.8,
           max_levels=max_levels, min_coarse=9, check_every=10)


def test_relres_cap_refuses_like_the_oracle(M):
    """A pair cap below what the stop needs raises SolveNotConverged on both
    sides."""
    from ion_gym_gb300.workloads import quadrupole
    fixed, val = quadrupole(65, 8.0)
    with pytest.raises(port.SolveNotConverged, match="relative residual"):
        port.solve3d_cascadic_relres(fixed, val, max_sweeps=30)
    with pytest.raises(M.SolveNotConverged, match="relative residual"):
        M.solve3d_cascadic_relres(fixed, val, max_sweeps=30)
