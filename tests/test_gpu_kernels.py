"""Bit-exact parity of every CUDA kernel with the reference.

Two checks per kernel: the golden fixtures recorded from the reference
(tests/golden/kernels.npz), and the oracle on larger seeded inputs (odd,
even and size-1 axes, theta None and given, both stencils).  All calls go
through the C-ABI (libigsolve.so) via the drop-in module functions.
"""
import numpy as np
import pytest

from conftest import same_bits
from oracle import port

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    from ion_gym_gb300.physics import _device
    _device._torch()
    return _device


def _th(c):
    return np.ascontiguousarray(c["th"], np.float32)


def test_div6_is_correctly_rounded():
    """The integer-pipe division by 6 of the theta-free sweep equals x/6
    for values across the whole exponent range, the significands on either
    side of 1.5 (where the quotient's scaling changes) and the exponents
    where the hardware division takes over."""
    from ion_gym_gb300.physics import _device as D
    torch = D._torch()
    rng = np.random.default_rng(5)
    bits = rng.integers(0, 2 ** 63, 2_000_000, dtype=np.uint64)
    expo = rng.integers(1, 2046, bits.size).astype(np.uint64)
    bits = (bits & np.uint64(0x800FFFFFFFFFFFFF)) | (expo << np.uint64(52))
    x = bits.view(np.float64)
    x = x[np.isfinite(x) & (np.abs(x) < 1e300)]
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 1e-310, -2.2e-308, 6.0,
                        -6.0, 3.0, 1e-300, 1e300, 0.5, 1.0 / 3.0])
    mant = np.array([0, 1, 2, (1 << 51) - 1, 1 << 51, (1 << 51) + 1,
                     (1 << 52) - 2, (1 << 52) - 1], dtype=np.uint64)
    ex = np.concatenate([np.arange(1, 9), np.arange(1020, 1030),
                         np.arange(2040, 2047)]).astype(np.uint64)
    edge = ((ex[:, None] << np.uint64(52)) | mant[None, :]).ravel()
    edge = np.concatenate([edge, edge | np.uint64(1 << 63)]).view(np.float64)
    x = np.concatenate([special, special, edge, x])
    # a 1 x 1 x n grid with every node free: the sweep on colour c reads
    # its two z-neighbours; put x/2 on the neighbours so num = 6 * (x/2) *...
    # Instead drive the residual-free identity directly: sweep_rhs with
    # e = 0, f = -x gives e_new = (0 - (-x)) / 6 = x / 6 at omega 1.
    n = x.size
    e = torch.zeros((1, 1, n), dtype=torch.float64, device="cuda")
    f = torch.from_numpy(-x.reshape(1, 1, n)).to("cuda")
    fixed = torch.zeros((1, 1, n), dtype=torch.uint8, device="cuda")
    D.sweep_rhs(e, fixed, f, 1.0, 0)
    got = e.cpu().numpy().ravel()
    # the reference update with zero neighbours: e = 0 + 1*((0 - f)/6 - 0);
    # (0 - f) is x except that x = -0.0 gives +0.0
    fn = -x
    want = 0.0 + 1.0 * ((0.0 - fn) / 6.0 - 0.0)
    even = np.arange(n) % 2 == 0  # colour 0 nodes of a 1x1xn grid
    assert np.array_equal(got[even].view(np.uint64), want[even].view(np.uint64))


def test_sor_step_is_exact():
    """The integer-pipe SOR step RN(omega * RN(nv - old)) equals the FP64
    expression: old and nv in one binade or adjacent ones, far apart,
    opposite signs, equal, tiny and huge, for several omegas.  A 1 x 1 x n
    grid: a colour-0 node sees itself on the four flat-axis legs and its two
    z-neighbours."""
    from ion_gym_gb300.physics import _device as D
    torch = D._torch()
    rng = np.random.default_rng(17)
    n = 1_200_001
    mag = 2.0 ** rng.integers(-900, 900, n)
    e = rng.uniform(0.5, 2.0, n) * mag * rng.choice([-1.0, 1.0], n)
    mode = rng.integers(0, 6, n)
    rel = 10.0 ** rng.uniform(-16, 0, n) * rng.choice([-1.0, 1.0], n)
    target = e * (1 + rel)
    target = np.where(mode == 1, e, target)                       # nv == old
    target = np.where(mode == 2, -e * rng.uniform(0.3, 3, n), target)
    target = np.where(mode == 3, np.nextafter(e, 2 * e), target)  # one ulp
    target = np.where(mode == 4, e * 2.0 ** rng.integers(-3, 4, n), target)
    k = np.arange(n)
    zm = e[np.where(k > 0, k - 1, 1)]
    zp = e[np.where(k < n - 1, k + 1, n - 2)]
    s6 = ((((e + e) + e) + e) + zm) + zp
    with np.errstate(over="ignore", invalid="ignore"):
        f = s6 - 6.0 * target
    f = np.where(np.isfinite(f), f, 0.0)
    fixed = torch.zeros((1, 1, n), dtype=torch.uint8, device="cuda")
    even = k % 2 == 0
    for omega in (1.0, 1.85, 1.2345678901234567, 0.7):
        et = torch.from_numpy(e.reshape(1, 1, n).copy()).to("cuda")
        ft = torch.from_numpy(f.reshape(1, 1, n)).to("cuda")
        D.sweep_rhs(et, fixed, ft, omega, 0)
        got = et.cpu().numpy().ravel()
        with np.errstate(over="ignore", invalid="ignore"):
            want = e + omega * ((s6 - f) / 6.0 - e)
        assert np.array_equal(got[even].view(np.uint64), want[even].view(np.uint64)), omega
        assert np.array_equal(got[~even].view(np.uint64), e[~even].view(np.uint64))


def test_sweep(dev, kernels_golden):
    for c in kernels_golden.cases("sweep"):
        phi = c["phi"].copy()
        d = dev.sweep(phi, c["fixed"].astype(bool), _th(c), float(c["omega"]),
                      int(c["colour"]), bool(c["ghost_linear"]))
        assert same_bits(phi, c["out"]), c["phi"].shape
        assert d == float(c["d"])


def test_residual(dev, kernels_golden):
    for c in kernels_golden.cases("residual"):
        out = np.full(c["phi"].shape, np.nan)
        dev.residual(c["phi"], c["fixed"].astype(bool), _th(c),
                     bool(c["ghost_linear"]), out)
        assert same_bits(out, c["out"])


def test_sweep_rhs_residual_rhs(dev, kernels_golden):
    for c in kernels_golden.cases("sweep_rhs"):
        e = c["e"].copy()
        d = dev.sweep_rhs(e, c["fixed"].astype(bool), c["f"],
                          float(c["omega"]), int(c["colour"]))
        assert same_bits(e, c["out"]) and d == float(c["d"])
        r = np.full(c["e"].shape, np.nan)
        dev.residual_rhs(c["e"], c["fixed"].astype(bool), c["f"], r)
        assert same_bits(r, c["res"])


def test_restrict_and_masks(dev, kernels_golden):
    for c in kernels_golden.cases("restrict"):
        cs = c["out"].shape
        out = np.empty(cs)
        dev.restrict_fw(c["fine"], out)
        assert same_bits(out, c["out"])
        fixed = c["fixed"].astype(bool)
        assert np.array_equal(dev.coarsen_fixed_any(fixed), c["any"].astype(bool))
        fc, vc = dev.coarsen_mask(fixed, c["val"])
        assert np.array_equal(fc, c["fc"].astype(bool))
        assert same_bits(vc, c["vc"])


def test_prolongations(dev, kernels_golden):
    for c in kernels_golden.cases("prolong"):
        o = c["base"].copy()
        dev.prolong_add(c["coarse"], o, c["fixed"].astype(bool))
        assert same_bits(o, c["out"])
        assert same_bits(dev.prolongate(c["coarse"], c["base"].shape),
                         c["prolongate"])


def test_audit(dev, kernels_golden):
    for c in kernels_golden.cases("audit"):
        fixed = c["fixed"].astype(bool)
        assert same_bits(dev.residual_audit(c["u"], fixed, _th(c)), c["res"])
        e = c["e"].copy()
        d = dev.err_sweep(e, fixed, _th(c), c["rhs"], float(c["omega"]),
                          int(c["colour"]))
        assert same_bits(e, c["out"]) and d == float(c["d"])


SHAPES = [(65, 47, 33), (33, 1, 40), (1, 1, 70), (2, 64, 3), (31, 30, 1),
          (40, 41, 42)]


def _rand_case(rng, shape, theta):
    phi = rng.uniform(-3, 3, shape)
    fixed = rng.random(shape) < 0.2
    th = None
    if theta:
        th = rng.uniform(1e-3, 1, (6,) + shape).astype(np.float32)
        th[rng.random(th.shape) < 0.7] = 1.0
    return phi, fixed, th


@pytest.mark.parametrize("shape", SHAPES)
def test_kernels_vs_oracle_random(dev, shape):
    rng = np.random.default_rng(hash(shape) % (2 ** 32))
    for theta in (False, True):
        for gl in (True, False):
            phi, fixed, th = _rand_case(rng, shape, theta)
            tho = th if th is not None else np.ones((6,) + shape, np.float32)
            for colour, omega in ((0, 1.93), (1, 1.0)):
                a, b = phi.copy(), phi.copy()
                da = dev.sweep(a, fixed, th, omega, colour, gl)
                db = port.sweep(b, fixed, tho, omega, colour, gl)
                assert same_bits(a, b) and da == db
            ra = np.empty(shape)
            rb = np.empty(shape)
            dev.residual(phi, fixed, th, gl, ra)
            port.residual(phi, fixed, tho, gl, rb)
            assert same_bits(ra, rb)
    e, fixed, _ = _rand_case(rng, shape, False)
    f = rng.uniform(-1, 1, shape)
    for colour, omega in ((0, 1.0), (1, 1.77)):
        a, b = e.copy(), e.copy()
        assert dev.sweep_rhs(a, fixed, f, omega, colour) == \
            port.sweep_rhs(b, fixed, f, omega, colour)
        assert same_bits(a, b)
    ra, rb = np.empty(shape), np.empty(shape)
    dev.residual_rhs(e, fixed, f, ra)
    port.residual_rhs(e, fixed, f, rb)
    assert same_bits(ra, rb)
    cs = tuple((s + 1) // 2 for s in shape)
    out = np.empty(cs)
    dev.restrict_fw(e, out)
    assert same_bits(out, port.restrict_fw(e))
    coarse = rng.uniform(-1, 1, cs)
    a, b = e.copy(), e.copy()
    dev.prolong_add(coarse, a, fixed)
    port.prolong_add(coarse, b, fixed)
    assert same_bits(a, b)
    assert same_bits(dev.prolongate(coarse, shape), port.prolongate(coarse, shape))
    val = rng.uniform(-5, 5, shape)
    assert np.array_equal(dev.coarsen_fixed_any(fixed), port.coarsen_fixed_any(fixed))
    fa, va = dev.coarsen_mask(fixed, val)
    fb, vb = port.coarsen_mask(fixed, val)
    assert np.array_equal(fa, fb) and same_bits(va, vb)


def test_torch_tensors_in_place(dev):
    """CUDA tensors are updated in place on the device (no round trip)."""
    import torch
    rng = np.random.default_rng(3)
    phi, fixed, _ = _rand_case(rng, (20, 21, 22), False)
    t = torch.from_numpy(phi.copy()).cuda()
    ptr = t.data_ptr()
    d = dev.sweep(t, torch.from_numpy(fixed).cuda(), None, 1.5, 0, True)
    b = phi.copy()
    db = port.sweep(b, fixed, np.ones((6, 20, 21, 22), np.float32), 1.5, 0, True)
    assert t.data_ptr() == ptr and d == db
    assert same_bits(t.cpu().numpy(), b)


def test_residual_field_and_attribute_difference_match_oracle():
    """solver3d.residual_field and attribute_difference (solver3d.py:420-444)
    against the oracle's restatement of the same audit and error-equation
    loop, bit for bit, with theta given."""
    from ion_gym_gb300.physics import solver3d as S
    rng = np.random.default_rng(31)
    shape = (14, 11, 9)
    fixed = np.zeros(shape, bool)
    fixed[0] = fixed[-1] = True
    fixed[:, 0] = fixed[:, -1] = True
    fixed[:, :, 0] = fixed[:, :, -1] = True
    fixed[5:8, 4:7, 3:6] = True
    val = np.where(fixed, rng.uniform(-1.0, 1.0, shape), 0.0)
    theta = np.where(rng.random((6,) + shape) < 0.7, 1.0,
                     rng.uniform(0.2, 1.0, (6,) + shape)).astype(np.float32)
    ref = np.where(fixed, val, rng.uniform(-1.0, 1.0, shape))
    phi = np.where(fixed, val, ref + rng.normal(0.0, 1e-6, shape))
    r = S.residual_field(ref, fixed, theta)
    ro = port.residual_audit(ref, fixed, theta)
    assert same_bits(r, ro)
    e, rest = S.attribute_difference(ref, phi, fixed, theta, tol=1e-9,
                                     max_sweeps=400)
    eo = np.zeros_like(ref)
    om = 2.0 / (1.0 + np.sin(np.pi / (max(shape) + 1)))
    for _ in range(400):
        d = max(port.err_sweep(eo, fixed, theta, -ro, om, 0),
                port.err_sweep(eo, fixed, theta, -ro, om, 1))
        if d < 1e-9:
            break
    assert same_bits(e, eo)
    assert same_bits(rest, (ref - phi) - eo)
