"""Mixed-precision batched bases reach the FP64 solution of the same
discrete problem to the stated accuracy (1e-9 of the electrode span).

The FP64 reference solution is the drop-in V-cycle (bit-identical to the
reference's solve3d_vmg) run to a cycle delta of 1e-13 of the span."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ACC = 1e-9
V = 1e4


def _deck(shape, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    box = np.zeros(shape, bool)
    box[0] = box[-1] = True
    box[:, 0] = box[:, -1] = True
    if nz > 2:
        box[:, :, 0] = box[:, :, -1] = True
    masks = {1: box}
    i, j, k = np.ogrid[:nx, :ny, :nz]
    for e in range(2, 5):
        c = rng.uniform(0.3, 0.7, 3) * np.array(shape)
        r = rng.uniform(0.08, 0.16) * min(nx, ny)
        m = (i - c[0]) ** 2 + (j - c[1]) ** 2 <= r * r
        if nz > 2:
            m = m & (np.abs(k - c[2]) <= rng.uniform(0.1, 0.3) * nz)
        masks[e] = np.broadcast_to(m, shape) & ~box
    return masks


def _fp64_bases(masks):
    from ion_gym_gb300.physics import multigrid3d as M
    metal = np.zeros(next(iter(masks.values())).shape, bool)
    for m in masks.values():
        metal |= m
    out = {}
    for i, m in masks.items():
        out[i] = M.solve3d_vmg(metal, np.where(m, V, 0.0), tol=1e-13 * V,
                               max_cycles=200, accept_stagnation=True)[0]
    return out


@pytest.mark.parametrize("shape,seed", [((41, 37, 45), 1), ((33, 20, 17), 2),
                                        ((64, 48, 1), 3)])
def test_mixed_bases_reach_fp64_accuracy(shape, seed):
    from ion_gym_gb300.physics.mixed import solve_bases_mixed
    masks = _deck(shape, seed)
    ref = _fp64_bases(masks)
    got, stats = solve_bases_mixed(masks, v_basis=V, accuracy=ACC,
                                   return_stats=True)
    assert sorted(got) == sorted(masks)
    for i in masks:
        err = np.abs(got[i] - ref[i]).max() / V
        assert err <= ACC, (i, err, stats)
        assert np.all(got[i][masks[i]] == V)
    assert stats["steps"] >= 2


def test_mixed_only_and_superposition():
    """Unit bases superpose: the sum of all bases (box included) is v_basis
    everywhere, since the sum solves the problem with all metal at v_basis."""
    from ion_gym_gb300.physics.mixed import solve_bases_mixed
    masks = _deck((40, 44, 36), 7)
    got = solve_bases_mixed(masks, v_basis=V, accuracy=ACC)
    total = sum(got.values())
    assert np.abs(total - V).max() <= 4 * ACC * V
    part = solve_bases_mixed(masks, v_basis=V, accuracy=ACC, only={2, 3})
    assert sorted(part) == [2, 3]
    assert np.abs(part[2] - got[2]).max() <= 2 * ACC * V


@pytest.mark.parametrize("shape,seed", [((41, 37, 45), 1), ((33, 20, 18), 2),
                                        ((20, 19, 2), 4)])
def test_fused_kernels_are_bit_identical(shape, seed):
    """Each fused kernel of the mixed path writes the bits of the separate
    launches it replaces, on every multigrid level, for odd and even z
    extents (both row parities at the z faces) and a grid whose coarse
    levels reach size-1 axes (the per-node prolongation takes over there):
    the first Gauss-Seidel pair from a zero correction, the float4 colour-0
    residual, the windowed prolongation, the direction update fused into
    the operator apply (direction, L p and the inner-product partials), the
    four-node restriction of the colour-0 residual, the first CG update of a
    refinement step written without reading x, and the last one folded
    into the FP64 update."""
    import ctypes
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.physics.mixed import MixedSession
    masks = _deck(shape, seed)
    metal = np.zeros(shape, bool)
    for m in masks.values():
        metal |= m
    rings = [masks[i] for i in sorted(masks)]
    with MixedSession(metal, len(rings)) as s:
        s.solve_bases(rings, V, ACC)
        bad = (ctypes.c_longlong * 8)(*([-1] * 8))
        st = _lib.lib().ig_mixed_check_fused(s._h, len(rings), bad)
        _lib.check(st, "ig_mixed_check_fused")
    assert list(bad) == [0] * 8


def test_tuner_times_launch_shapes_and_temporal_depths():
    """The session's tuner reports the separate half-sweep shape it chose
    and the temporal-block depths it timed (2, 4 or 6 half-sweeps per pass
    on the finest level); whichever it takes, the potentials are those of a
    session whose blocking is fixed off."""
    import os
    from ion_gym_gb300.physics.mixed import MixedSession
    masks = _deck((41, 37, 45), 1)
    metal = np.zeros((41, 37, 45), bool)
    for m in masks.values():
        metal |= m
    rings = [masks[i] for i in sorted(masks)]
    with MixedSession(metal, len(rings)) as s:
        t = s.tuning()
        got = s.solve_bases(rings, V, ACC)
        assert s.solve_bytes() == s.last_steps * s.step_bytes(len(rings)) > 0
    assert t["groups_per_thread"] in (1, 2, 4, 8) and t["threads"] in (128, 256, 512)
    assert t["best_blocked_depth"] in (2, 4, 6) and t["temporal_depth"] in (0, 2, 4, 6)
    assert t["us_per_half_sweep"] > 0 and t["blocked_us_per_half_sweep"] > 0
    os.environ["IG_MIXED_TB_LEVELS"] = "0"
    try:
        with MixedSession(metal, len(rings)) as s:
            assert s.tuning()["best_blocked_depth"] == 0
            ref = s.solve_bases(rings, V, ACC)
    finally:
        del os.environ["IG_MIXED_TB_LEVELS"]
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("shape", [(41, 37, 45), (30, 20, 200)])
def test_row_and_flat_residual_update_give_the_same_bits(shape):
    """The FP64 residual and update run one natural row per warp or several
    rows per warp (short rows); both forms give the same potentials, bit
    for bit (a short-row grid and one past the switch)."""
    import os
    from ion_gym_gb300.physics.mixed import MixedSession
    masks = _deck(shape, 3)
    metal = np.zeros(shape, bool)
    for m in masks.values():
        metal |= m
    rings = [masks[i] for i in sorted(masks)]
    got = {}
    for force in ("0", "1"):
        os.environ["IG_MIXED_FLAT"] = force
        try:
            with MixedSession(metal, len(rings)) as s:
                got[force] = s.solve_bases(rings, V, ACC)
        finally:
            del os.environ["IG_MIXED_FLAT"]
    assert np.array_equal(got["0"].view(np.uint64), got["1"].view(np.uint64))


@pytest.mark.parametrize("shape,n_b", [((41, 37, 45), 4), ((64, 48, 40), 1),
                                       ((70, 66, 34), 3)])
def test_tail_cycle_gives_the_separate_launches_bits(shape, n_b):
    """The cycle of the level above the bottom in one CTA per problem
    (k_tail_cycle) gives the potentials of the separate launches, bit for
    bit: odd and even extents, one problem and batches."""
    import os
    from ion_gym_gb300.physics.mixed import MixedSession
    masks = _deck(shape, 4)
    metal = np.zeros(shape, bool)
    for m in masks.values():
        metal |= m
    rings = [masks[i] for i in sorted(masks)][:n_b]
    got = {}
    for tail in ("0", "1"):
        os.environ["IG_MIXED_TAIL"] = tail
        try:
            with MixedSession(metal, len(rings)) as s:
                got[tail] = s.solve_bases(rings, V, ACC)
        finally:
            del os.environ["IG_MIXED_TAIL"]
    assert np.array_equal(got["0"].view(np.uint64), got["1"].view(np.uint64))


@pytest.mark.parametrize("shape,n_b", [((41, 37, 45), 4), ((64, 48, 40), 1)])
def test_folded_cg_updates_give_the_separate_launches_bits(shape, n_b):
    """The flexible CG's updates folded into the next iteration's zero-start
    pair (g += alpha q) and direction update (x += alpha p) give the
    potentials of the separate k_cg_update launches, bit for bit, over
    several refinement steps."""
    import os
    from ion_gym_gb300.physics.mixed import MixedSession
    masks = _deck(shape, 6)
    metal = np.zeros(shape, bool)
    for m in masks.values():
        metal |= m
    rings = [masks[i] for i in sorted(masks)][:n_b]
    got = {}
    for fold in ("0", "1"):
        os.environ["IG_MIXED_FOLD"] = fold
        try:
            with MixedSession(metal, len(rings)) as s:
                got[fold] = s.solve_bases(rings, V, ACC)
                got[fold + "steps"] = s.last_steps
        finally:
            del os.environ["IG_MIXED_FOLD"]
    assert got["1steps"] == got["0steps"] >= 2
    assert np.array_equal(got["0"].view(np.uint64), got["1"].view(np.uint64))


def test_set_cycle_matches_a_session_opened_with_it():
    """A session whose cycle is changed after a solve (its graphs dropped
    and recaptured) gives the bits of a session opened with that cycle."""
    from ion_gym_gb300.physics.mixed import MixedSession
    shape = (41, 37, 45)
    masks = _deck(shape, 8)
    metal = np.zeros(shape, bool)
    for m in masks.values():
        metal |= m
    rings = [masks[i] for i in sorted(masks)]
    with MixedSession(metal, len(rings)) as s:
        s.solve_bases(rings, V, ACC)
        s.set_cycle(3, 3, 3)
        got = s.solve_bases(rings, V, ACC)
        assert s.cycle["nu1"] == 3 and s.cycle["nu2"] == 3
    with MixedSession(metal, len(rings), nu1=3, nu2=3, cg_iters=3) as s:
        ref = s.solve_bases(rings, V, ACC)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("shape,n_b", [((41, 37, 45), 4), ((64, 48, 40), 1)])
def test_fused_inner_product_keeps_the_accuracy(shape, n_b):
    """<z, q> formed by the last half-sweep of the finest level (k_gs4_dot)
    instead of its own kernel sums in another order; the solves take the
    same refinement steps and agree within the stated accuracy."""
    import os
    from ion_gym_gb300.physics.mixed import MixedSession
    masks = _deck(shape, 9)
    metal = np.zeros(shape, bool)
    for m in masks.values():
        metal |= m
    rings = [masks[i] for i in sorted(masks)][:n_b]
    got = {}
    for dot in ("0", "1"):
        os.environ["IG_MIXED_DOT"] = dot
        try:
            with MixedSession(metal, len(rings)) as s:
                got[dot] = s.solve_bases(rings, V, ACC)
                got[dot + "steps"] = s.last_steps
        finally:
            del os.environ["IG_MIXED_DOT"]
    assert got["0steps"] == got["1steps"]
    assert np.abs(got["0"] - got["1"]).max() <= 2 * ACC * V


def test_fixed_point_update_conversion_matches_the_hardware():
    """The integer-pipe float -> int64 conversion with which the update adds
    a correction to the fixed-point potential gives the GPU conversion
    instruction's bits on floats of every exponent: zeros, subnormals,
    values around one half and the halfway points of every integer step
    (ties to even both ways), every float with a fraction bit just above or
    below a half, values at and past 2^63, infinities and NaN."""
    import ctypes
    from ion_gym_gb300 import _lib
    rng = np.random.default_rng(7)
    random = rng.integers(0, 2 ** 32, 2_000_000, dtype=np.uint64).astype(np.uint32)
    halves = np.arange(-5000, 5000) + 0.5
    near = np.concatenate([np.nextafter(halves, np.inf), np.nextafter(halves, -np.inf)])
    ties = rng.integers(0, 1 << 23, 20_000) + 0.5   # exact in float32
    special = [0.0, -0.0, 0.5, -0.5, 1.5, 2.5, -2.5, 0.49999997, 2.0 ** 62,
               2.0 ** 63, -2.0 ** 63, 2.0 ** 64, 1e-45, -1e-45, np.inf, -np.inf,
               np.nan]
    floats = np.ascontiguousarray(np.concatenate([
        np.array(special), halves, near, ties, -ties]).astype(np.float32))
    floats = np.concatenate([floats, random.view(np.float32)])
    bad = ctypes.c_longlong(-1)
    st = _lib.lib().ig_mixed_check_convert(
        floats.ctypes.data_as(ctypes.c_void_p), floats.size, ctypes.byref(bad))
    _lib.check(st, "ig_mixed_check_convert")
    assert bad.value == 0


@pytest.mark.parametrize("seed,side,n_el", [(1000, 33, 5), (1001, 65, 12),
                                            (1002, 97, 3), (1003, 65, 16)])
def test_uneven_batch_decks_reach_fp64_accuracy(seed, side, n_el):
    """Decks of the uneven-batch workload (random spheres, cylinders and
    plates in a grounded box, voltages U(-100, 100) V) solved by a mixed
    session as the batch solves them: within 1e-9 of each deck's voltage
    span of the FP64 drop-in V-cycle run to 1e-13 of the span."""
    from ion_gym_gb300.physics import multigrid3d as M
    from ion_gym_gb300.physics.mixed import MixedSession
    from ion_gym_gb300.workloads import random_deck
    fixed, val = random_deck(seed, side, n_el)
    span = max(float(val.max() - val.min()), 1.0)
    ref = M.solve3d_vmg(fixed, val, tol=1e-13 * span, max_cycles=400,
                        accept_stagnation=True)[0]
    with MixedSession(fixed, 1) as s:
        got = s.solve_values(val, ACC, span=span)[0]
        steps = s.last_steps
    err = np.abs(got - ref).max() / span
    assert err <= ACC, (err, steps)
    assert np.array_equal(got[fixed], val[fixed])


def test_fixed_point_units_refuse_out_of_range_values():
    """The refined potential is held in 64-bit fixed point in units of 2^-56
    of the problem's largest Dirichlet magnitude: values of 2^60 or more
    (or not finite) are refused before any refinement, small and large
    voltages within range solve to the same relative accuracy, and the
    metal keeps its Dirichlet values exactly."""
    from ion_gym_gb300.physics.mixed import MixedSession
    masks = _deck((33, 29, 31), 5)
    metal = np.zeros((33, 29, 31), bool)
    for m in masks.values():
        metal |= m
    rng = np.random.default_rng(3)
    base = np.where(metal, rng.uniform(-1.0, 1.0, metal.shape), 0.0)
    with MixedSession(metal, 1) as s:
        ref = s.solve_values(base, ACC, span=2.0)[0]
        for scale in (1e-12, 1e12):
            got = s.solve_values(base * scale, ACC, span=2.0 * scale)[0]
            assert np.array_equal(got[metal], (base * scale)[metal])
            # the accuracy is relative to the span, taken as at least 1 V
            tol = 2 * ACC * max(2.0 * scale, 1.0) + 2 * ACC * 2.0 * scale
            assert np.abs(got - scale * ref).max() <= tol
        with pytest.raises(ValueError, match="2\\^60"):
            s.solve_values(np.where(metal, 2.0 ** 61, 0.0), ACC)


def test_rebound_session_matches_a_fresh_one():
    """A session rebound to another geometry of its shape returns the bits
    of a session opened on that geometry (the same kernels, launch shapes
    and captured graphs, the new masks on every level); a rebind to another
    shape is refused."""
    from ion_gym_gb300.physics.mixed import MixedSession
    a = _deck((41, 37, 45), 1)
    b = _deck((41, 37, 45), 8)
    stack_b = [b[i] for i in sorted(b)]
    metal_a = np.zeros((41, 37, 45), bool)
    for m in a.values():
        metal_a |= m
    metal_b = np.zeros((41, 37, 45), bool)
    for m in b.values():
        metal_b |= m
    with MixedSession(metal_b, len(stack_b)) as s:
        fresh = s.solve_bases(stack_b, V, ACC).copy()
    with MixedSession(metal_a, len(stack_b)) as s:
        s.solve_bases([a[i] for i in sorted(a)][:len(stack_b)] +
                      [a[sorted(a)[0]]] * (len(stack_b) - len(a)), V, ACC)
        s.rebind(metal_b)
        again = s.solve_bases(stack_b, V, ACC)
        with pytest.raises(ValueError, match="shape"):
            s.rebind(np.zeros((41, 37, 44), bool))
    assert np.array_equal(again.view(np.uint64), fresh.view(np.uint64))


@pytest.mark.parametrize("n_decks", [3, 5])
def test_decks_of_one_shape_batch_with_one_metal_each(n_decks):
    """Decks of one grid shape with different electrodes and voltages as one
    batch (a session with one metal per problem, every launch covering all
    of them; 3 decks run the single-problem cycle, 5 the batch cycle): each
    deck within 1e-9 of its own span of the FP64 V-cycle run to 1e-13, the
    metal at its exact values, per-problem accuracies honoured, the fused
    kernels bit-identical with per-problem masks, and a rebind to other
    decks of the shape gives the same results as a session opened on
    them."""
    import ctypes
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.physics import multigrid3d as M
    from ion_gym_gb300.physics.mixed import MixedSession
    from ion_gym_gb300.workloads import random_deck
    decks = [random_deck(300 + q, 49, 2 + 3 * q) for q in range(2 * n_decks)]
    first, second = decks[:n_decks], decks[n_decks:]

    def stacks(ds):
        return (np.stack([f for f, _ in ds]), np.stack([v for _, v in ds]),
                np.array([max(float(v.max() - v.min()), 1.0) for _, v in ds]))

    fx, vx, sp = stacks(first)
    with MixedSession(fx) as s:
        assert s.per_problem and s.max_problems == n_decks
        got = s.solve_values(vx, ACC, span=sp).copy()
        bad = (ctypes.c_longlong * 8)(*([-1] * 8))
        _lib.check(_lib.lib().ig_mixed_check_fused(s._h, n_decks, bad), "check")
        assert list(bad) == [0] * 8
        fy, vy, sq = stacks(second)
        s.rebind(fy)
        again = s.solve_values(vy, ACC, span=sq).copy()
        with pytest.raises(ValueError, match="bases"):
            s.solve_bases(fy, 1e4, ACC)
    for q, (f, v) in enumerate(first):
        ref = M.solve3d_vmg(f, v, tol=1e-13 * sp[q], max_cycles=400,
                            accept_stagnation=True)[0]
        assert np.abs(got[q] - ref).max() <= ACC * sp[q], q
        assert np.array_equal(got[q][f], v[f])
    with MixedSession(fy) as s2:
        fresh = s2.solve_values(vy, ACC, span=sq)
    assert np.array_equal(again.view(np.uint64), fresh.view(np.uint64))
