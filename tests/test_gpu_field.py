"""Fields from solved bases on the GPU against the reference and the
oracle, bit for bit: the electrode-aware gradient
(tracer3d.build_field_aware_3d), the drive superposition and channel pack
(build_stl3d.compose_drive_channels), the unit-basis conversion, and the
C-ABI one-call compose."""
import ctypes
import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest

from conftest import GOLDEN, same_bits
from oracle import field as F

sys.path.insert(0, GOLDEN)
import make_golden as MG  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fz():
    return np.load(os.path.join(GOLDEN, "field.npz"), allow_pickle=False)


def _grad_cases(z):
    idx = sorted({int(k.split("/")[1]) for k in z.files if k.startswith("grad/")})
    return [{f: z[f"grad/{i}/{f}"] for f in ("phi", "ele", "h", "h_is_f64",
                                              "aware", "ex", "ey", "ez")}
            for i in idx]


def _h(c):
    return np.float64(float(c["h"])) if bool(c["h_is_f64"]) else float(c["h"])


def test_gradient_matches_reference(fz):
    from ion_gym_gb300.physics.field3d import build_field_aware_3d
    for c in _grad_cases(fz):
        got = build_field_aware_3d(c["phi"], c["ele"], _h(c),
                                   electrode_aware=bool(c["aware"]))
        for g, k in zip(got, ("ex", "ey", "ez")):
            assert g.dtype == c[k].dtype and same_bits(g, c[k]), c["phi"].shape


def test_gradient_resident_matches_reference(fz):
    import torch
    from ion_gym_gb300.physics.field3d import build_field_aware_3d
    for c in _grad_cases(fz):
        phi = torch.from_numpy(c["phi"]).cuda()
        ele = torch.from_numpy(c["ele"].astype(np.int16)).cuda()
        got = build_field_aware_3d(phi, ele, _h(c), electrode_aware=bool(c["aware"]))
        for g, k in zip(got, ("ex", "ey", "ez")):
            assert same_bits(g.cpu().numpy(), c[k])


@pytest.mark.parametrize("shape,dt,h", [
    ((67, 45, 130), np.float32, 0.1),
    ((67, 45, 130), np.float32, np.float64(0.07)),
    ((33, 40, 21), np.float64, 0.3),
    ((17, 2, 9), np.float32, 1.7),
])
def test_gradient_matches_oracle(shape, dt, h):
    from ion_gym_gb300.physics.field3d import build_field_aware_3d
    rng = np.random.default_rng(hash(shape) % 2**32)
    phi = (rng.standard_normal(shape) * 100).astype(dt)
    ele = (rng.random(shape) < 0.3).astype(np.int16) * 2
    ele[:, :, : shape[2] // 3] = 1
    h64 = isinstance(h, np.float64)
    for aware in (True, False):
        got = build_field_aware_3d(phi, ele, h, electrode_aware=aware)
        want = F.field_aware_3d(phi, ele, float(h), h64, aware)
        for g, w in zip(got, want):
            assert g.dtype == w.dtype and same_bits(g, w)


def test_gradient_refuses_a_flat_axis():
    from ion_gym_gb300.physics.field3d import build_field_aware_3d
    with pytest.raises(ValueError, match="too small to calculate a numerical"):
        build_field_aware_3d(np.zeros((4, 1, 4), np.float32),
                             np.zeros((4, 1, 4), np.int16), 0.1)


def _spec(groups, els, **gkw):
    return MG._Spec(SimpleNamespace(rf_groups=groups, electrodes=els, **gkw))


def _check_compose(ch, fz, k, to_np=lambda a: a):
    for key in ("EAx", "EAy", "EAz", "ExK", "EyK", "EzK", "ch_kind", "ch_om",
                "ch_ph", "ch_amp", "ch_off", "ch_duty", "tab_t", "tab_v",
                "tab_off"):
        got, want = to_np(ch[key]), fz[f"{k}/{key}"]
        assert got.dtype == want.dtype and same_bits(got, want), (k, key)
    cp = [to_np(a) for a in ch["chan_phi"]]
    want = fz[k + "/chan_phi"]
    assert len(cp) == want.shape[0]
    for a, w in zip(cp, want):
        assert same_bits(a, w), k
    assert list(ch["ch_name"]) == [str(s) for s in fz[k + "/ch_name"]]


def test_compose_matches_reference(fz):
    from ion_gym_gb300.physics.field3d import compose_drive_channels
    for name, gkw, groups, els in MG.field_specs():
        k = f"compose/{name}"
        stack = fz[k + "/bases"]
        bases = {i + 1: stack[i] for i in range(stack.shape[0])}
        ch = compose_drive_channels(_spec(groups, els, **gkw), bases, fz[k + "/ele"])
        _check_compose(ch, fz, k)


def test_compose_resident_matches_reference(fz):
    import torch
    from ion_gym_gb300.physics.field3d import compose_drive_channels
    for name, gkw, groups, els in MG.field_specs():
        k = f"compose/{name}"
        stack = torch.from_numpy(fz[k + "/bases"]).cuda()
        bases = {i + 1: stack[i] for i in range(stack.shape[0])}
        ele = torch.from_numpy(fz[k + "/ele"]).cuda()
        ch = compose_drive_channels(_spec(groups, els, **gkw), bases, ele)
        assert ch["EAx"].is_cuda
        _check_compose(ch, fz, k, to_np=lambda a: a.cpu().numpy()
                       if hasattr(a, "cpu") else a)


def test_compose_fields_c_abi(fz):
    """ig_compose_fields on host buffers: the channel potentials and float32
    fields of the reference's aware case."""
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.physics.field3d import drive_plan
    name, gkw, groups, els = MG.field_specs()[0]
    k = f"compose/{name}"
    stack = np.ascontiguousarray(fz[k + "/bases"])
    bases = {i + 1: stack[i] for i in range(stack.shape[0])}
    plan, _ = drive_plan(_spec(groups, els, **gkw), bases)
    sub = np.ascontiguousarray(np.stack([bases[i] for i in plan["keys"]]))
    nch = plan["weights"].shape[0]
    shape = stack.shape[1:]
    metal = np.ascontiguousarray(fz[k + "/ele"] != 0).view(np.uint8)
    P = np.empty((nch,) + shape, np.float32)
    E = [np.empty((nch,) + shape, np.float32) for _ in range(3)]
    rows = np.ascontiguousarray(plan["rows"], np.int32)
    w = np.ascontiguousarray(plan["weights"], np.float32)
    m = np.ascontiguousarray(plan["mult"], np.uint8)
    st = _lib.lib().ig_compose_fields(
        _lib.ptr(sub), sub.shape[0], rows.size, _lib.ptr(rows), nch,
        _lib.ptr(w), _lib.ptr(m), _lib.ptr(metal), *shape,
        float(gkw["mm_per_gu"]), 0, _lib.ptr(P), *(_lib.ptr(e) for e in E))
    assert st == 0, _lib.last_error()
    assert same_bits(P[1:], fz[k + "/chan_phi"])
    for ax, (a, b) in enumerate((("EAx", "ExK"), ("EAy", "EyK"), ("EAz", "EzK"))):
        assert same_bits(E[ax][0].astype(np.float64), fz[f"{k}/{a}"])
        assert same_bits(E[ax][1:].astype(np.float64), fz[f"{k}/{b}"])


@pytest.mark.parametrize("shape", [(21, 17, 19), (16, 12, 20)])
def test_superpose_long_plans_match_oracle(shape):
    """More steps and channels than one launch holds (64 x 8): the device
    continues the float32 sums across launches exactly as one long loop."""
    import torch
    from ion_gym_gb300.physics.field3d import superpose_device
    rng = np.random.default_rng(7)
    nrows, nsteps, nch = 40, 70, 11
    stack = rng.standard_normal((nrows,) + shape).astype(np.float32)
    rows = rng.integers(0, nrows, nsteps).astype(np.int32)
    w = rng.standard_normal((nch, nsteps)).astype(np.float32)
    m = rng.integers(0, 3, (nch, nsteps)).astype(np.uint8)
    got = superpose_device(torch.from_numpy(stack).cuda(), rows, w, m)
    want = F.superpose(stack, rows, w, m)
    assert same_bits(got.cpu().numpy(), want)
    # bases as separate tensors, one of them not 16-byte aligned
    n = int(np.prod(shape))
    big = torch.from_numpy(np.concatenate([[0.0], stack[0].ravel()])
                           .astype(np.float32)).cuda()
    lst = [big[1:1 + n].view(shape)] + [torch.from_numpy(stack[r]).cuda()
                                        for r in range(1, nrows)]
    got = superpose_device(lst, rows, w, m)
    assert same_bits(got.cpu().numpy(), want)


def test_unit_bases_match_numpy():
    import torch
    from ion_gym_gb300.physics.field3d import unit_bases_device
    rng = np.random.default_rng(3)
    phi = rng.random((3, 19, 23, 29)) * 1e4
    got = unit_bases_device(torch.from_numpy(phi).cuda(), 1e4).cpu().numpy()
    assert same_bits(got, (phi / 1e4).astype(np.float32))


@pytest.mark.parametrize("h", [0.1, 0.2, 0.35, 1.7, 1e-3, 0.0123456789, 0.15])
def test_division_emulation_is_exact(h):
    """The kernels' fast divisions equal the IEEE ones: every float32
    numerator over float32(h) and float32(2h), and 2^24 hashed numerators
    over the float64 h and 2h."""
    from ion_gym_gb300 import _lib
    bad = ctypes.c_ulonglong(99)
    st = _lib.lib().ig_field_check_division(float(h), 1 << 24, 12345,
                                            ctypes.byref(bad))
    assert st == 0, _lib.last_error()
    assert bad.value == 0


@pytest.mark.parametrize("nch", [1, 2, 3, 4, 5, 7])
def test_field_channel_groups_match_oracle(nch):
    """Channels are fused four to a thread; every group size and remainder
    gives the oracle's bits, including exact zeros and signed zeros in
    flat (metal) regions."""
    import torch
    from ion_gym_gb300.physics.field3d import _field_device
    rng = np.random.default_rng(nch)
    shape = (23, 18, 37)
    phi = (rng.standard_normal((nch,) + shape) * 3).astype(np.float32)
    phi[:, :6] = 0.0
    phi[:, 6:8, :, :5] = -0.0
    phi[:, 10:14, 4:9, 10:20] = 2.5
    ele = np.zeros(shape, np.int16)
    ele[:7] = 1
    ele[10:14, 4:9, 10:20] = 2
    ele[(rng.random(shape) < 0.05)] = 3
    for h in (0.1, np.float64(0.3)):
        out = _field_device(torch.from_numpy(phi).cuda(), ele, h, True)
        got = [o.cpu().numpy() for o in out]
        if nch == 1:
            got = [g[None] for g in got]
        for c in range(nch):
            want = F.field_aware_3d(phi[c], ele, float(h),
                                    isinstance(h, np.float64), True)
            for ax in range(3):
                assert same_bits(got[ax][c], want[ax]), (nch, c, ax, h)


def test_bundle_to_device_to_fields(tmp_path):
    """A field bundle read straight into 16-byte-aligned device rows gives
    the same composed fields as the host arrays, and device bases written
    back as an entry export to the same bundle members."""
    import torch
    from ion_gym_gb300.io import field_io
    from ion_gym_gb300.physics.field3d import compose_drive_channels
    from ion_gym_gb300.workloads import DriveElectrode, DriveGeometry, DriveGroup, DriveSpec
    rng = np.random.default_rng(5)
    shape = (17, 13, 11)                       # odd node count
    lab = np.zeros(shape, np.uint8)
    lab[0], lab[-1], lab[5:8, 4:9, 3:7] = 3, 3, 1
    lab[10:12, 2:5, 6:10] = 2
    bases = {i: rng.random(shape).astype(np.float32) for i in (1, 2, 3)}
    stack = torch.stack([torch.from_numpy(bases[i]) for i in (1, 2, 3)]).cuda()
    key = field_io.store_device_bases({"name": "t", "geometry": {"g": 1}}, stack,
                                      [1, 2, 3], torch.from_numpy(lab).cuda(),
                                      root=str(tmp_path / "c"), name="t",
                                      spec_json={"name": "t", "geometry": {"g": 1}})
    npz, _ = field_io.export_field_bundle(key, str(tmp_path / "o"), root=str(tmp_path / "c"))
    dstack, dlab, keys, meta = field_io.load_field_device(npz)
    assert keys == [1, 2, 3] and meta["spec_name"] == "t"
    for r in range(3):
        assert dstack[r].data_ptr() % 16 == 0
        assert same_bits(dstack[r].cpu().numpy(), bases[r + 1])
    assert same_bits(dlab.cpu().numpy(), lab)
    spec = DriveSpec(DriveGeometry(
        [DriveGroup("rf", amplitude_v=10.0)],
        [DriveElectrode("a", ["rf"], 1.5), DriveElectrode("b", [], -2.0),
         DriveElectrode("box", [], 0.0)], 0.1))
    host = compose_drive_channels(spec, bases, lab)
    dev = compose_drive_channels(spec, {k: dstack[r] for r, k in enumerate(keys)}, dlab)
    for name in ("EAx", "EAy", "EAz", "ExK", "EyK", "EzK"):
        assert same_bits(dev[name].cpu().numpy(), host[name]), name
