"""Extruded 2-D shapes to 3-D masks on the GPU against the reference's
build_shapes3d.shapes_masks_3d (tests/golden/shapes.npz, recorded from the
reference on decks of rotated rects, ellipses, polygons and cutouts along
x, y and z, with an origin and a mirror plane): identical label grids, and
every refusal with the reference's message."""
import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
import make_golden as MG  # noqa: E402

pytestmark = pytest.mark.gpu


class _Shape:
    def __init__(self, d):
        d = dict(d)
        self.type = d.pop("type")
        self.children = [_Shape(c) for c in d.pop("children", [])]
        self.params = d

    def extrude(self):
        e = self.params.get("extrude")
        if e is None:
            return None
        return {"axis": e["axis"], "lo_mm": float(e["lo_mm"]), "hi_mm": float(e["hi_mm"])}


def _spec(deck):
    g = dict(deck["geometry"])
    els = [SimpleNamespace(name=e["name"], stl=e.get("stl"),
                           shapes=[_Shape(s) for s in e.get("shapes", [])])
           for e in g.pop("electrodes")]
    sym = g.pop("symmetry", {})
    return SimpleNamespace(geometry=SimpleNamespace(
        electrodes=els, symmetry=SimpleNamespace(planes=sym.get("planes", {})),
        origin_mm=g.pop("origin_mm", None), **g))


@pytest.fixture(scope="module")
def sz():
    return np.load(os.path.join(GOLDEN, "shapes.npz"), allow_pickle=False)


def test_labels_match_reference(sz):
    from ion_gym_gb300.physics.shapes3d import shapes_masks_3d
    ok, _ = MG.shapes_decks()
    for name, deck in ok:
        masks = shapes_masks_3d(_spec(deck))
        want = sz[f"shapes/{name}/lab"]
        lab = np.zeros(want.shape, np.int16)
        for i, m in masks.items():
            assert m.shape == want.shape
            lab[m] = i
        assert np.array_equal(lab, want), name


def test_refusals_match_reference(sz):
    from ion_gym_gb300.physics.shapes3d import shapes_masks_3d
    _, bad = MG.shapes_decks()
    for name, deck in bad:
        with pytest.raises(ValueError) as e:
            shapes_masks_3d(_spec(deck))
        assert str(e.value) == str(sz[f"shapes_err/{name}/message"]), name


def test_cross_sections_against_numpy():
    """The device cross-section of each shape kind equals a numpy
    evaluation of the same float64 expressions on a finer, shifted grid."""
    import math
    from ion_gym_gb300.physics.shapes3d import cross_section
    A = np.arange(161) * 0.0371 - 0.8
    B = np.arange(97) * 0.0413 - 0.3
    X = A[:, None] * np.ones((1, len(B)))
    Y = np.ones((len(A), 1)) * B[None, :]
    T = 1e-9
    p = {"x_mm": 0.4, "y_mm": 0.2, "width_mm": 2.1, "height_mm": 1.3,
         "rotation_deg": 17.0}
    cx, cy = p["x_mm"] + p["width_mm"] / 2, p["y_mm"] + p["height_mm"] / 2
    a = math.radians(-17.0)
    ca, sa = math.cos(a), math.sin(a)
    xr = cx + (X - cx) * ca - (Y - cy) * sa
    yr = cy + (X - cx) * sa + (Y - cy) * ca
    want = ((xr >= p["x_mm"] - T) & (xr <= p["x_mm"] + p["width_mm"] + T)
            & (yr >= p["y_mm"] - T) & (yr <= p["y_mm"] + p["height_mm"] + T))
    assert np.array_equal(cross_section(_Shape({"type": "rect", **p}), A, B), want)
    q = {"cx_mm": 1.9, "cy_mm": 1.1, "rx_mm": 1.3, "ry_mm": 0.7}
    want = (((X - 1.9) / (1.3 + T)) ** 2 + ((Y - 1.1) / (0.7 + T)) ** 2 <= 1.0)
    assert np.array_equal(cross_section(_Shape({"type": "ellipse", **q}), A, B), want)
    pts = np.array([[0.0, 0.0], [3.0, 0.5], [2.0, 2.5], [1.0, 1.0], [-0.5, 2.0]])
    x, y = X.ravel(), Y.ravel()
    x0, y0 = pts[:, 0], pts[:, 1]
    x1, y1 = np.roll(x0, -1), np.roll(y0, -1)
    inside = np.zeros(x.shape, bool)
    for j in range(len(pts)):
        if y0[j] == y1[j]:
            continue
        st = (y0[j] > y) != (y1[j] > y)
        xint = x0[j] + (y - y0[j]) * (x1[j] - x0[j]) / (y1[j] - y0[j])
        inside ^= st & (x < xint)
    ex, ey = x1 - x0, y1 - y0
    seg2 = ex * ex + ey * ey
    d2 = np.full(x.shape, np.inf)
    for j in range(len(pts)):
        t = np.clip(((x - x0[j]) * ex[j] + (y - y0[j]) * ey[j]) / seg2[j], 0.0, 1.0)
        d2 = np.minimum(d2, (x - (x0[j] + t * ex[j])) ** 2 + (y - (y0[j] + t * ey[j])) ** 2)
    want = (inside | (d2 <= T ** 2)).reshape(X.shape)
    got = cross_section(_Shape({"type": "polygon", "points_mm": pts.tolist()}), A, B)
    assert np.array_equal(got, want)
