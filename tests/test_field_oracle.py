"""Pins the field-build oracle (oracle/field.py) and the host half of the
composer (ion_gym_gb300.physics.field3d.drive_plan) to the reference.

tests/golden/field.npz was recorded from the reference's own
tracer3d.build_field_aware_3d and build_stl3d.compose_drive_channels
(tests/golden/make_golden.py); the oracle and the plan must reproduce every
array and scalar bit for bit, and every refusal's message.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, same_bits
from oracle import field as F
from ion_gym_gb300.physics import field3d

sys.path.insert(0, GOLDEN)
import make_golden as MG  # noqa: E402  (the stand-in specs of the fixtures)


@pytest.fixture(scope="module")
def fz():
    return np.load(os.path.join(GOLDEN, "field.npz"), allow_pickle=False)


def grad_cases(z):
    idx = sorted({int(k.split("/")[1]) for k in z.files if k.startswith("grad/")})
    return [{f: z[f"grad/{i}/{f}"] for f in ("phi", "ele", "h", "h_is_f64",
                                              "aware", "ex", "ey", "ez")}
            for i in idx]


def spacing(c):
    h = float(c["h"])
    return np.float64(h) if bool(c["h_is_f64"]) else h


def test_gradient_oracle_matches_reference(fz):
    cases = grad_cases(fz)
    assert len(cases) == 7
    for c in cases:
        ex, ey, ez = F.field_aware_3d(c["phi"], c["ele"], float(c["h"]),
                                      bool(c["h_is_f64"]), bool(c["aware"]))
        for got, want in ((ex, c["ex"]), (ey, c["ey"]), (ez, c["ez"])):
            assert got.dtype == want.dtype
            assert same_bits(got, want), c["phi"].shape


def test_gradient_oracle_metal_rule_changes_values(fz):
    """The aware cases differ from the plain gradient somewhere, so the
    metal rule is exercised by the fixtures."""
    c = grad_cases(fz)[0]
    plain = F.field_aware_3d(c["phi"], c["ele"], float(c["h"]), False, False)
    assert any(not same_bits(p, c[k]) for p, k in zip(plain, ("ex", "ey", "ez")))


def compose_oracle(spec, bases):
    plan, pack = field3d.drive_plan(spec, bases)
    g = spec.geometry
    shape = next(iter(bases.values())).shape
    stack = (np.stack([bases[k] for k in plan["keys"]]) if plan["keys"]
             else np.zeros((0,) + shape, np.float32))
    P = F.superpose(stack, plan["rows"], plan["weights"], plan["mult"])
    return plan, pack, P


def test_compose_plan_and_oracle_match_reference(fz):
    names = [n for n, *_ in MG.field_specs()]
    assert len(names) == 4
    for name, gkw, groups, els in MG.field_specs():
        from types import SimpleNamespace
        k = f"compose/{name}"
        stack = fz[k + "/bases"]
        bases = {i + 1: stack[i] for i in range(stack.shape[0])}
        ele = fz[k + "/ele"]
        spec = MG._Spec(SimpleNamespace(rf_groups=groups, electrodes=els, **gkw))
        plan, pack, P = compose_oracle(spec, bases)
        aware = gkw.get("field_method", "electrode_aware") == "electrode_aware"
        f32 = gkw.get("channel_dtype", "float64") == "float32"
        h = gkw["mm_per_gu"]
        h64 = isinstance(h, np.float64)
        E = [F.field_aware_3d(P[c], ele, float(h), h64, aware)
             for c in range(P.shape[0])]
        cv = (lambda a: a) if f32 else (lambda a: a.astype(np.float64))
        for ax, key in enumerate(("EAx", "EAy", "EAz")):
            assert same_bits(cv(E[0][ax]), fz[f"{k}/{key}"]), (name, key)
        for ax, key in enumerate(("ExK", "EyK", "EzK")):
            want = fz[f"{k}/{key}"]
            got = (np.stack([cv(e[ax]) for e in E[1:]]) if len(E) > 1
                   else np.zeros(want.shape, want.dtype))
            assert got.dtype == want.dtype and same_bits(got, want), (name, key)
        assert same_bits(P[1:], fz[k + "/chan_phi"]), name
        arr = field3d._pack_arrays(pack)
        assert list(arr.pop("ch_name")) == [str(s) for s in fz[k + "/ch_name"]]
        for key, v in arr.items():
            want = fz[f"{k}/{key}"]
            assert v.dtype == want.dtype and same_bits(v, want), (name, key)


def test_compose_refusals_match_reference(fz):
    from types import SimpleNamespace
    shape = (6, 5, 4)
    bases = {1: np.zeros(shape, np.float32), 2: np.zeros(shape, np.float32)}
    ele = np.zeros(shape, np.int16)
    for name, groups, els in MG.field_error_specs():
        geom = SimpleNamespace(rf_groups=groups, electrodes=els, mm_per_gu=0.1)
        with pytest.raises(ValueError) as ei:
            field3d.compose_drive_channels(MG._Spec(geom), bases, ele)
        assert str(ei.value) == str(fz[f"compose_err/{name}/message"]), name
    geom = SimpleNamespace(rf_groups=[], electrodes=[MG._El("e1", [], 1.0)],
                           mm_per_gu=0.1)
    with pytest.raises(ValueError) as ei:
        field3d.compose_drive_channels(MG._Spec(geom), bases, np.zeros((6, 5, 3)))
    assert str(ei.value) == str(fz["compose_err/shape/message"])


def test_plan_chunks_and_repeats():
    """An electrode naming a group twice adds its basis twice; a zero DC
    drops the static term; the plan lists each needed basis once."""
    from types import SimpleNamespace
    els = [MG._El("a", ["p", "p"], 0.0), MG._El("b", [], 2.0),
           MG._El("c", [], 0.0)]
    geom = SimpleNamespace(rf_groups=[MG._group("p", amplitude_v=1.0)],
                           electrodes=els, mm_per_gu=0.1)
    bases = {i: np.zeros((2, 2, 2), np.float32) for i in (1, 2, 3)}
    plan, _ = field3d.drive_plan(MG._Spec(geom), bases)
    assert plan["keys"] == [1, 2]
    assert list(plan["rows"]) == [0, 1]
    assert plan["mult"].tolist() == [[0, 1], [2, 0]]
    assert plan["weights"].tolist() == [[0.0, 2.0], [1.0, 0.0]]
