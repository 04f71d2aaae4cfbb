"""Analytic scenes on the GPU: the labelled node raster and the
fractional-surface legs theta.

rasterize(scene) is ion_gym physics/rasterize3d.rasterize (:45-109): an
int16 grid with the electrode index at every node inside one of its shapes
(within minus notin, surfaces inclusive with EPS = 1e-9 grid units), 0 for
vacuum; a node claimed by two electrodes and an electrode with no node are
refused.  fractions_from_scene_device(scene, metal, mirror) is
solver3d.fractions_from_scene (:75-127) evaluated on the device.  Both
return the reference's bits: the scene's bounds are combined with EPS on the
host exactly as the reference writes them, and the kernels evaluate
(x - cx)**2 + (y - cy)**2 in round-to-nearest float64.
"""
import ctypes

import numpy as np

from ion_gym_gb300 import _lib
from ion_gym_gb300._lib import ptr, as_mask

EPS = 1e-9


def _is_cyl(p):
    k = getattr(p, "kind", None)
    if k is not None:
        return k == "cylinder"
    return hasattr(p, "r")


def _bounds(p, e):
    """The six compared bounds of one primitive with tolerance e (the
    reference's expressions, evaluated in float64 here)."""
    if _is_cyl(p):
        zlo = p.z - p.length
        return [float(p.cx), float(p.cy), p.r ** 2 + e, zlo - e, p.z + e, 0.0]
    return [p.x1 - e, p.x2 + e, p.y1 - e, p.y2 + e, p.z1 - e, p.z2 + e]


def primitive_table(scene):
    """(table float64 (n, 16), electrode indices, names) of a scene in grid
    units: rows kind, electrode slot, shape id, role (0 within, 1 notin),
    inclusive bounds (+EPS), strict bounds (-EPS); electrodes in scene order,
    each shape's within primitives before its notin primitives."""
    sc = scene.in_gu()
    rows, idx, names = [], [], []
    for slot, el in enumerate(sc.electrodes):
        idx.append(int(el.index))
        names.append(getattr(el, "name", str(el.index)))
        for sid, sh in enumerate(el.shapes):
            for role, prims in ((0, sh.within), (1, sh.notin)):
                for p in prims:
                    rows.append([0.0 if _is_cyl(p) else 1.0, float(slot),
                                 float(sid), float(role)]
                                + _bounds(p, EPS) + _bounds(p, -EPS))
    table = np.array(rows, np.float64).reshape(-1, 16)
    return np.ascontiguousarray(table), idx, names


def _grid_shape(scene):
    g = scene.grid
    return int(g.nx), int(g.ny), int(g.nz)


def _node_owner(table, idx, node, upto):
    """Label the raster holds at `node` after electrodes [0, upto)."""
    x, y, z = (float(v) for v in node)
    owner = 0
    for slot in range(upto):
        rows = table[table[:, 1] == slot]
        m = False
        for sid in np.unique(rows[:, 2]):
            w = False
            for r in rows[rows[:, 2] == sid]:
                b = r[4:10]
                if r[0] == 0.0:
                    dx, dy = x - b[0], y - b[1]
                    hit = dx * dx + dy * dy <= b[2] and b[3] <= z <= b[4]
                else:
                    hit = (b[0] <= x <= b[1] and b[2] <= y <= b[3]
                           and b[4] <= z <= b[5])
                w = (w or hit) if r[3] == 0.0 else (w and not hit)
            m = m or w
        if m:
            owner = idx[slot]
    return owner


def rasterize(scene):
    """Labelled occupancy grid (nx, ny, nz) int16 of the stored-frame nodes
    (rasterize3d.py:45-109)."""
    if hasattr(scene, "check"):
        scene = scene.check()
    table, idx, names = primitive_table(scene)
    shape = _grid_shape(scene)
    ne = len(idx)
    lab = np.empty(shape, np.int16)
    counts = np.zeros(ne, np.uint64)
    ccount = np.zeros(ne, np.uint64)
    cfirst = np.zeros(ne, np.uint64)
    eidx = np.array(idx, np.int32)
    st = _lib.lib().ig_rasterize(ptr(table), len(table), ptr(eidx), ne,
                                 *shape, ptr(lab), ptr(counts), ptr(ccount),
                                 ptr(cfirst))
    _lib.check(st, "rasterize")
    for e in range(ne):
        if ccount[e]:
            node = np.unravel_index(int(cfirst[e]), shape)
            other = _node_owner(table, idx, node, e)
            at = ",".join(str(int(v)) for v in node)
            raise ValueError(
                f"electrode {idx[e]} ({names[e]}) overlaps electrode {other} "
                f"at node ({at}) (+{int(ccount[e])} more). Two electrodes may "
                f"not claim the same node: separate them or merge them into "
                f"one electrode.")
        if not counts[e]:
            g = scene.grid
            raise ValueError(
                f"electrode {idx[e]} ({names[e]}) rasterises EMPTY: no node "
                f"of the {g.nx}x{g.ny}x{g.nz} stored grid falls inside it. A "
                f"Dirichlet electrode with zero nodes would solve as if "
                f"absent; fix the geometry or the grid.")
    return lab


def fractions_from_scene_device(scene, metal, mirror=(False, False, False),
                                iters=45):
    """solver3d.fractions_from_scene on the GPU: theta (6, nx, ny, nz)
    float32, the same bits."""
    table, _, _ = primitive_table(scene)
    metal = np.asarray(metal, bool)
    th = np.empty((6,) + metal.shape, np.float32)
    bits = sum(1 << a for a in range(3) if mirror[a])
    st = _lib.lib().ig_theta_scene(ptr(table), len(table), ptr(as_mask(metal)),
                                   *metal.shape, int(bits), int(iters),
                                   ptr(th))
    _lib.check(st, "fractions_from_scene_device")
    return th


def masks_from_labels(lab):
    """{electrode index: bool mask} of a labelled raster."""
    return {int(i): lab == i for i in np.unique(lab) if i != 0}
