"""Extruded 2-D shapes to 3-D electrode masks on the GPU.

``shapes_masks_3d(spec)`` is ion_gym physics/build_shapes3d.shapes_masks_3d
(build_shapes3d.py:167-243) with electrode_mask_3d (:113-164) and
_shape_volume (:71-110): each electrode's shapes, in order, are 2-D
cross-sections (rect, optionally rotated; ellipse; polygon as a closed
solid -- raster2d.py:113-230) swept along an axis between lo_mm and hi_mm
(default: z through the whole stored depth); additive shapes union their
volumes in and cutouts subtract theirs.  The cross-sections are evaluated on
the GPU with the reference's float64 expressions (``ig_shape_xsection``),
and one 3-D kernel (``ig_shapes_label``) assembles every electrode's volume,
labels the nodes and counts clashes, so the refusals (empty electrode,
overlapping electrodes, a shape or cutout with no node, extrusion ranges
off the domain or below a mirror plane, STL references, electrodes without
shapes) are raised in the reference's order with its messages.  Returns
{electrode index (1-based position): bool mask}.
"""
import math

import numpy as np

from ion_gym_gb300 import _lib
from ion_gym_gb300._lib import ptr

POLY_EDGE_TOL = 1e-9
DEFAULT_EXTRUDE_AXIS = "z"
_AXIS_INDEX = {"x": 0, "y": 1, "z": 2}
SHARED_NODE_HINT = ("To drive one conductor with several drive groups, "
                    "list them all in that electrode's rf_groups instead "
                    "of stacking copies of it.")


def _inplane_axes(ai):
    """Cyclic in-plane axes of an extrusion axis: x->(y,z), y->(z,x),
    z->(x,y)."""
    return (ai + 1) % 3, (ai + 2) % 3


def _params(shape):
    return getattr(shape, "params", shape)


def _type(shape):
    return shape.type if hasattr(shape, "type") else shape["type"]


def _extrude(shape):
    if hasattr(shape, "extrude") and callable(shape.extrude):
        return shape.extrude()
    d = _params(shape).get("extrude")
    if d is None:
        return None
    return {"axis": d["axis"], "lo_mm": float(d["lo_mm"]), "hi_mm": float(d["hi_mm"])}


def _children(shape):
    return list(getattr(shape, "children", None) or
                (shape.get("children", []) if isinstance(shape, dict) else []))


def cross_section(shape, A, B):
    """(len(A), len(B)) bool cross-section of one shape on in-plane node
    coordinates A, B (raster2d._shape_mask), evaluated on the GPU."""
    t = _type(shape)
    p = _params(shape)
    T = POLY_EDGE_TOL
    poly = None
    if t == "rect":
        x0, y0 = p["x_mm"], p["y_mm"]
        w, h = p["width_mm"], p["height_mm"]
        rot = p.get("rotation_deg", 0.0)
        cx, cy = x0 + w / 2, y0 + h / 2
        ca = sa = 0.0
        if rot:
            a = math.radians(-rot)
            ca, sa = math.cos(a), math.sin(a)
        vals = [cx, cy, ca, sa, x0 - T, x0 + w + T, y0 - T, y0 + h + T,
                1.0 if rot else 0.0]
        code = 0
    elif t == "ellipse":
        vals = [p["cx_mm"], p["cy_mm"], p["rx_mm"] + T, p["ry_mm"] + T]
        code = 1
    elif t == "polygon":
        pts = np.asarray(p["points_mm"], float)
        if pts.ndim != 2 or pts.shape[0] < 3 or pts.shape[1] != 2:
            raise ValueError(f"polygon needs >=3 (x,y) points_mm, got "
                             f"shape {pts.shape}")
        x0, y0 = pts[:, 0], pts[:, 1]
        x1, y1 = np.roll(x0, -1), np.roll(y0, -1)
        ex, ey = x1 - x0, y1 - y0
        seg2 = ex * ex + ey * ey
        poly = np.ascontiguousarray(np.stack([x0, y0, x1, y1, ex, ey, seg2]))
        vals = [T ** 2]
        code = 2
    else:
        raise ValueError(f"planar rasterizer: unsupported shape {t!r}")
    A = np.ascontiguousarray(A, np.float64)
    B = np.ascontiguousarray(B, np.float64)
    prm = np.asarray(vals, np.float64)
    out = np.empty((len(A), len(B)), np.uint8)
    st = _lib.lib().ig_shape_xsection(code, ptr(prm), len(prm),
                                      ptr(poly) if poly is not None else None,
                                      0 if poly is None else poly.shape[1],
                                      ptr(A), len(A), ptr(B), len(B), ptr(out))
    _lib.check(st, "cross_section")
    return out.view(bool)


def _shape_piece(shape, coords, mirror_axes, extents_mm, el_name, shape_pos):
    """(axis, cross-section, range) of one shape (build_shapes3d.py:71-110)
    with the extrusion refusals."""
    ext = _extrude(shape)
    typ = _type(shape)
    if ext is None:
        ai = _AXIS_INDEX[DEFAULT_EXTRUDE_AXIS]
        lo, hi = 0.0, extents_mm[ai]
    else:
        ai = _AXIS_INDEX[ext["axis"]]
        lo, hi = ext["lo_mm"], ext["hi_mm"]
        if mirror_axes[ai] and lo < 0.0:
            raise ValueError(
                f"electrode {el_name!r} shape #{shape_pos} "
                f"({typ!r}): extrude {ext['axis']}=[{lo:g},{hi:g}] "
                f"mm has lo_mm < 0 on the declared mirror axis "
                f"{ext['axis']!r}. The stored frame on a mirrored axis is "
                f"the non-negative half with the plane at 0 supplying the "
                f"image; author the [0,+] half (a symmetric-through-plane "
                f"shape is [0, hi]).")
        if hi < 0.0 or lo > extents_mm[ai]:
            raise ValueError(
                f"electrode {el_name!r} shape #{shape_pos} "
                f"({typ!r}): extrude {ext['axis']}=[{lo:g},{hi:g}] "
                f"mm lies entirely outside the stored domain "
                f"[0, {extents_mm[ai]:g}] mm on that axis — the shape "
                f"would rasterize empty. Fix the range or the domain.")
    a1, a2 = _inplane_axes(ai)
    xs = cross_section(shape, coords[a1], coords[a2])
    rng = ((coords[ai] >= lo - POLY_EDGE_TOL) & (coords[ai] <= hi + POLY_EDGE_TOL))
    return ai, xs, rng


def _electrode_pieces(el, coords, mirror_axes, extents_mm):
    """[(axis, xs, rng, cutout)] of an electrode with electrode_mask_3d's
    zero-node refusals (build_shapes3d.py:113-164)."""
    out = []
    for pos, s in enumerate(el.shapes):
        if _type(s) == "cutout":
            ch = _children(s)
            inner = ch[0] if ch else None
            if inner is not None:
                ai, xs, rng = _shape_piece(inner, coords, mirror_axes, extents_mm,
                                           el.name, pos)
                if not (xs.any() and rng.any()):
                    raise ValueError(
                        f"shapes3d: electrode {el.name!r} cutout #{pos} "
                        f"rasterises to ZERO nodes — the declared "
                        f"subtraction removes nothing on this grid. A "
                        f"no-op cutout is a silent declaration failure: "
                        f"either its coordinates miss the stored frame "
                        f"(shapes are authored in the STORED frame, "
                        f"non-negative; world coordinates must be "
                        f"shifted by the origin before authoring) or "
                        f"the pitch is too coarse to resolve it.")
                out.append((ai, xs, rng, True))
        else:
            ai, xs, rng = _shape_piece(s, coords, mirror_axes, extents_mm,
                                       el.name, pos)
            if not (xs.any() and rng.any()):
                raise ValueError(
                    f"shapes3d: electrode {el.name!r} shape #{pos} "
                    f"({_type(s)}) rasterises to ZERO nodes on the stored "
                    f"grid — it would be silently absent from the solve "
                    f"while its siblings keep the electrode alive. "
                    f"Shapes are authored in the STORED frame "
                    f"(non-negative; a world coordinate below the origin "
                    f"must be shifted by the origin before authoring), "
                    f"or the pitch may be too coarse to resolve this "
                    f"shape.")
            out.append((ai, xs, rng, False))
    return out


def electrode_labels_3d(electrodes, coords, mirror_axes, extents_mm, pitch_mm=None):
    """Labelled int16 grid (0 vacuum, i for the i-th electrode) of the
    electrodes' extruded shapes, with shapes_masks_3d's refusals in its
    order.  coords: the three stored-frame node coordinate vectors (mm)."""
    n = tuple(len(c) for c in coords)
    els = list(electrodes)
    pieces, fail = [], None
    for el in els:
        try:
            if getattr(el, "stl", None):
                raise ValueError(
                    f"shapes3d: electrode {el.name!r} references an STL "
                    f"({el.stl!r}) — this route is inline-shapes-only. Use "
                    f"the STL route, or drop the reference.")
            if not el.shapes:
                raise ValueError(
                    f"shapes3d: electrode {el.name!r} has no shapes — a "
                    f"Dirichlet electrode with zero volume would solve "
                    f"silently as if absent.")
            pieces.append(_electrode_pieces(el, coords, mirror_axes, extents_mm))
        except ValueError as e:
            fail = e
            break
    lab = np.zeros(n, np.int16)
    built = len(pieces)
    if built:
        table, xs_parts, rng_parts = [], [], []
        xs_off = rng_off = 0
        for slot, pc in enumerate(pieces):
            for ai, xs, rng, cut in pc:
                table.append([slot, ai, int(cut), xs_off, rng_off, xs.shape[0], xs.shape[1]])
                xs_parts.append(xs.view(np.uint8).ravel())
                rng_parts.append(rng.astype(np.uint8))
                xs_off += xs.size
                rng_off += rng.size
        tab = np.ascontiguousarray(np.asarray(table, np.int64).reshape(-1, 7))
        xs_all = np.ascontiguousarray(np.concatenate(xs_parts) if xs_parts
                                      else np.zeros(1, np.uint8))
        rng_all = np.ascontiguousarray(np.concatenate(rng_parts) if rng_parts
                                       else np.zeros(1, np.uint8))
        eidx = np.arange(1, built + 1, dtype=np.int32)
        counts = np.zeros(built, np.uint64)
        ccount = np.zeros(built, np.uint64)
        cfirst = np.zeros(built, np.uint64)
        st = _lib.lib().ig_shapes_label(ptr(tab), len(tab), ptr(xs_all), xs_all.size,
                                        ptr(rng_all), rng_all.size, ptr(eidx), built,
                                        *n, ptr(lab), ptr(counts), ptr(ccount), ptr(cfirst))
        _lib.check(st, "shapes_masks_3d")
        for e in range(built):
            el = els[e]
            if not counts[e]:
                h = pitch_mm
                raise ValueError(
                    f"shapes3d: electrode {el.name!r} rasterises EMPTY on the "
                    f"{n[0]}x{n[1]}x{n[2]} stored grid @ {h} mm/gu (stored extents "
                    f"{tuple(extents_mm)} mm, mirror "
                    f"{''.join(a for a, on in zip('xyz', mirror_axes) if on) or 'none'}). "
                    f"A conductor with zero nodes cannot hold a boundary "
                    f"condition and the solve would silently proceed without "
                    f"it — check the shape coordinates against the stored "
                    f"frame, or use a finer pitch.")
            if ccount[e]:
                i, j, k = np.unravel_index(int(cfirst[e]), n)
                other = _owner_before(pieces, e, (i, j, k))
                raise ValueError(
                    f"shapes3d: electrode {e + 1} ({el.name!r}) overlaps "
                    f"electrode {other} at node ({i},{j},{k}) "
                    f"(+{int(ccount[e]) - 1} more) — two conductors cannot "
                    f"own one voxel. {SHARED_NODE_HINT}")
    if fail is not None:
        raise fail
    return lab


def _owner_before(pieces, e, node):
    """Label the grid holds at `node` after electrodes [0, e)."""
    owner = 0
    for slot in range(e):
        m = False
        for ai, xs, rng, cut in pieces[slot]:
            a1, a2 = _inplane_axes(ai)
            v = bool(rng[node[ai]] and xs[node[a1], node[a2]])
            m = (m and not v) if cut else (m or v)
        if m:
            owner = slot + 1
    return owner


def _grid(g, grid):
    if grid is not None:
        nx, ny, nz, h = grid
        return int(nx), int(ny), int(nz), h
    h = g.mm_per_gu
    return (int(round(float(g.width_mm) / float(h))) + 1,
            int(round(float(g.height_mm) / float(h))) + 1,
            int(round(float(g.depth_mm) / float(h))) + 1, h)


def _mirror_axes(spec):
    sc = getattr(spec, "scene", None)
    if sc:
        m = (sc.get("grid", {}) or {}).get("mirror", "") or ""
        return tuple(a in m for a in ("x", "y", "z"))
    sym = getattr(spec.geometry, "symmetry", None)
    pl = (getattr(sym, "planes", None) if sym is not None else None) or {}
    return tuple(pl.get(a) == "mirror" for a in ("x", "y", "z"))


def shapes_masks_3d(spec, verbose=False, grid=None):
    """{electrode index: (nx, ny, nz) bool} of a spec's inline shapes on the
    stored grid (build_shapes3d.py:167-243).  The grid is
    floor(extent / pitch) + 1 nodes per axis (the reference's loader has
    already refused non-conforming extents), or `grid` = (nx, ny, nz, h)."""
    g = spec.geometry
    nx, ny, nz, h = _grid(g, grid)
    org = getattr(g, "origin_mm", None) or (0.0, 0.0)
    mirror_axes = _mirror_axes(spec)
    for a in (0, 1):
        if mirror_axes[a] and float(org[a]) != 0.0:
            raise ValueError(
                f"shapes3d: origin_mm[{a}] = {org[a]!r} on a declared "
                f"{'xy'[a]}-mirror axis. On a mirrored axis coordinates "
                f"mean 'distance from the mirror plane' and the plane "
                f"sits at 0 by construction -- a nonzero origin there "
                f"has no defined meaning. Drop the origin on that axis "
                f"or the mirror declaration.")
    coords = (np.arange(nx) * h + float(org[0]), np.arange(ny) * h + float(org[1]),
              np.arange(nz) * h)
    extents_mm = (float(g.width_mm), float(g.height_mm), float(g.depth_mm))
    lab = electrode_labels_3d(g.electrodes, coords, mirror_axes, extents_mm,
                              pitch_mm=g.mm_per_gu if grid is None else h)
    if verbose:
        print(f"[shapes3d] rasterized {len(g.electrodes)} conductors on "
              f"{nx}x{ny}x{nz} @ {h} mm/gu on the GPU")
    return {i: lab == i for i in range(1, len(g.electrodes) + 1)}
