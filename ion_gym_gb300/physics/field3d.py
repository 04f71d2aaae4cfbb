"""From solved bases to the flight's fields, on the GPU.

Drop-ins for the reference's field build, with the same bits:

* ``build_field_aware_3d(phi, ele, h_mm, electrode_aware=True)`` is
  ion_gym physics/tracer3d.build_field_aware_3d (tracer3d.py:94-117) with
  its metal-node pass _fa3d_correct (tracer3d.py:55-91): E = -grad(phi) in
  V/mm, numpy.gradient everywhere and, at metal nodes with vacuum on exactly
  one side along an axis, the one-sided difference into the vacuum.
* ``compose_drive_channels(spec, bases, ele, verbose=False)`` is
  physics/build_stl3d.compose_drive_channels (build_stl3d.py:493-709): the
  static drive A = sum float32(dc_i) * b_i, one potential per active drive
  group (the plain sum of its members' bases), the electrode-aware field of
  each, and the channel pack (ch_kind, ch_om, ch_ph, ch_amp, ch_off,
  ch_duty, tab_t, tab_v, tab_off).
* ``unit_bases_device(phis, v_basis)`` is the basis door's output
  conversion (build_stl3d.py:849): float32(phi / v_basis).

The superposition and the gradients run in libigsolve.so (two launches for
all channels); host work is the packing of scalars and the copies.  Arrays
may be numpy (host) or CUDA torch tensors (resident; results stay on the
device).  The reference caches group gradients between drive-only changes
(build_stl3d.py:420-478); here a compose costs two bandwidth-bound launches,
so nothing is cached and ``clear_memory_cache`` drops nothing.
"""
import ctypes
import math

import numpy as np

from ion_gym_gb300 import _lib
from ion_gym_gb300.physics._device import _torch, _is_tensor, _p, _stream

WAVE_KIND = {"sin": 0, "cos": 1, "square": 2, "table": 3}
MAX_CHANNELS_PER_LAUNCH = 8
MAX_STEPS_PER_LAUNCH = 64


def padded(rows, shape, dtype=None, device="cuda"):
    """(rows, *shape) CUDA tensor whose rows start 16 bytes apart or more on
    16-byte boundaries (row stride rounded up to 4 elements), so the
    superposition reads and writes them as float4 whatever the node count.
    Each row is contiguous; the stack as a whole is not when padding was
    needed."""
    torch = _torch()
    dtype = dtype or torch.float32
    n = int(np.prod(shape))
    ns = (n + 3) // 4 * 4
    buf = torch.empty((rows, ns), dtype=dtype, device=device)
    return buf[:, :n].view((rows,) + tuple(shape))


def _rows_ok(t):
    """A (rows, nx, ny, nz) tensor whose rows are each contiguous."""
    return t.dim() == 4 and (t.shape[0] <= 1 or t[0].is_contiguous()) and \
        t.stride(3) == 1 and t.stride(2) == t.shape[3] and \
        t.stride(1) == t.shape[2] * t.shape[3]


def _h_is_f64(h):
    """numpy.gradient divides a float32 array by a numpy float64 spacing in
    float64 (NEP 50: numpy scalars are strongly typed) and by a Python
    float, int or float32 spacing in float32."""
    return isinstance(h, np.generic) and np.dtype(type(h)) == np.float64


def _phi_dtype(a):
    dt = a.dtype if not _is_tensor(a) else np.dtype(str(a.dtype).split(".")[1])
    if dt == np.float32:
        return np.float32, 0
    if dt == np.float64:
        return np.float64, 1
    if np.issubdtype(dt, np.integer) or dt == np.bool_:
        return np.float64, 1       # numpy.gradient converts integers to float64
    raise TypeError(f"build_field_aware_3d: unsupported potential dtype {dt}")


def _metal_u8(ele):
    """uint8 0/1 of the label grid's truth value (``not ele[...]`` is the
    vacuum test of the reference's metal pass)."""
    if _is_tensor(ele):
        return (ele != 0).to(_torch().uint8).contiguous()
    return np.ascontiguousarray(np.asarray(ele) != 0).view(np.uint8)


def build_field_aware_3d(phi, ele, h_mm, electrode_aware=True):
    """(Ex, Ey, Ez) = -grad(phi) in V/mm (tracer3d.py:94-117), the dtype of
    phi (float32 stays float32, integers become float64)."""
    if _is_tensor(phi):
        return _field_device(phi, ele, h_mm, electrode_aware)
    phi = np.asarray(phi)
    dt, code = _phi_dtype(phi)
    phi = np.ascontiguousarray(phi, dtype=dt)
    if phi.ndim != 3:
        raise ValueError("build_field_aware_3d: phi must be a 3-D node grid")
    if electrode_aware and np.asarray(ele).shape != phi.shape:
        raise ValueError(f"build_field_aware_3d: label grid shape "
                         f"{np.asarray(ele).shape} does not match phi {phi.shape}")
    metal = _metal_u8(ele) if electrode_aware else None
    out = [np.empty_like(phi) for _ in range(3)]
    st = _lib.lib().ig_field_aware_3d(
        _lib.ptr(phi), code, _lib.ptr(metal) if metal is not None else None,
        *phi.shape, float(h_mm), int(_h_is_f64(h_mm)), *(_lib.ptr(o) for o in out))
    _lib.check(st, "build_field_aware_3d")
    return tuple(out)


def _field_device(phi, ele, h_mm, electrode_aware, out=None):
    torch = _torch()
    if phi.dim() == 3:
        phi = phi.unsqueeze(0)
    nch, nx, ny, nz = phi.shape
    _, code = _phi_dtype(phi)
    if code == 1 and phi.dtype != torch.float64:
        phi = phi.to(torch.float64)
    if not _rows_ok(phi):
        phi = phi.contiguous()
    metal = None
    if electrode_aware:
        metal = _metal_u8(ele if _is_tensor(ele) else torch.from_numpy(
            np.ascontiguousarray(np.asarray(ele) != 0).view(np.uint8)).to(phi.device))
        if tuple(metal.shape) != (nx, ny, nz):
            raise ValueError(f"build_field_aware_3d: label grid shape "
                             f"{tuple(metal.shape)} does not match phi {(nx, ny, nz)}")
    if out is None:
        out = torch.empty((3, nch, nx, ny, nz), dtype=phi.dtype, device=phi.device)
    n = nx * ny * nz
    pstride = phi.stride(0) if nch > 1 else n
    ostride = out.stride(1) if nch > 1 else n
    st = _lib.lib().ig_field_aware_dev(
        _p(phi), code, pstride, nch, _p(metal), nx, ny, nz, float(h_mm),
        int(_h_is_f64(h_mm)), _p(out[0]), _p(out[1]), _p(out[2]), ostride,
        _stream())
    _lib.check(st, "build_field_aware_3d")
    if nch == 1:
        return out[0, 0], out[1, 0], out[2, 0]
    return out[0], out[1], out[2]


def unit_bases_device(phis, v_basis=1e4):
    """float32(phi / v_basis) of a CUDA float64 stack (..., nx, ny, nz), as
    the basis door returns its bases (build_stl3d.py:849)."""
    torch = _torch()
    phis = phis.contiguous()
    if phis.dtype != torch.float64 or phis.device.type != "cuda":
        raise TypeError("unit_bases_device: a CUDA float64 tensor is required")
    if phis.dim() == 4:
        out = padded(phis.shape[0], phis.shape[1:], torch.float32, phis.device)
        for r in range(phis.shape[0]):
            st = _lib.lib().ig_unit_bases_dev(_p(phis[r]), phis[r].numel(),
                                              float(v_basis), _p(out[r]), _stream())
            _lib.check(st, "unit_bases_device")
        return out
    out = torch.empty(phis.shape, dtype=torch.float32, device=phis.device)
    st = _lib.lib().ig_unit_bases_dev(_p(phis), phis.numel(), float(v_basis),
                                      _p(out), _stream())
    _lib.check(st, "unit_bases_device")
    return out


def superpose_device(bases, plan_rows, weights, mult, shape=None):
    """Channel potentials (n_channels, nx, ny, nz) float32 from CUDA
    float32 bases (a stack (n_rows, nx, ny, nz) or a list of (nx, ny, nz)
    tensors, used in place) and a plan: the basis row of each step in
    electrode order, weights and repeat counts per channel and step."""
    torch = _torch()
    rows = np.ascontiguousarray(plan_rows, np.int64)
    w = np.ascontiguousarray(weights, np.float32)
    m = np.ascontiguousarray(mult, np.uint8)
    nch, nsteps = w.shape
    if m.shape != w.shape or rows.shape != (nsteps,):
        raise ValueError("superpose_device: weights, repeats and rows disagree")
    nrows = len(bases)
    if nsteps and (rows.min() < 0 or rows.max() >= nrows):
        raise ValueError("superpose_device: a plan row is outside the bases")
    if shape is None:
        shape = tuple(bases[0].shape)
    shape = tuple(shape)
    n = int(np.prod(shape))
    used = {}
    for r in rows.tolist():
        if r not in used:
            b = bases[r]
            if (b.dtype != torch.float32 or not b.is_cuda or not b.is_contiguous()
                    or tuple(b.shape) != shape):
                raise ValueError("superpose_device: bases must be contiguous CUDA "
                                 f"float32 tensors of shape {shape}")
            used[r] = b.data_ptr()
    ptrs = (ctypes.c_void_p * max(nsteps, 1))(*[used[r] for r in rows.tolist()])
    dev = bases[0].device if nrows else torch.device("cuda")
    out = padded(nch, shape, torch.float32, dev)
    ostride = out.stride(0) if nch > 1 else (n + 3) // 4 * 4
    st = _lib.lib().ig_superpose_dev(ptrs, nsteps, nch, _lib.ptr(w), _lib.ptr(m),
                                     n, _p(out), ostride, _stream())
    _lib.check(st, "superpose_device")
    return out


# ---------------------------------------------------------------- compose
def _group_names(el):
    gn = getattr(el, "group_names", None)
    return list(gn()) if callable(gn) else list(gn or [])


def drive_plan(spec, bases):
    """Host half of compose_drive_channels: validation in the reference's
    order, the scalar channel pack and the superposition plan.

    Returns (plan, pack): plan = dict(keys = basis keys in stack order,
    rows, weights, mult, names) with channel 0 the static drive A and
    channel 1 + g the g-th active group; pack = the ch_* / tab_* entries."""
    g = spec.geometry
    groups = {gr.name: gr for gr in g.rf_groups}
    els = list(g.electrodes)
    dc = []
    for i, el in enumerate(els, start=1):
        dc.append(spec.dc_effective(el))
        if dc[-1] and i not in bases:
            raise KeyError(i)
    member = []
    used = set()
    for i, el in enumerate(els, start=1):
        names = _group_names(el)
        for gname in names:
            if gname not in groups:
                raise ValueError(
                    f"electrode {el.name!r} names drive group "
                    f"{gname!r}, which is not defined in geometry."
                    f"rf_groups ({sorted(groups)})")
            if i not in bases:
                raise KeyError(i)
            used.add(gname)
        member.append(names)
    unused = [n for n in groups if n not in used
              and (groups[n].amplitude_v or getattr(groups[n], "offset_v", 0.0))]
    if unused:
        raise ValueError(
            f"drive groups {unused} are defined and non-zero but no "
            f"electrode belongs to them (nothing to drive) — assign "
            f"members or remove the group")
    active = [(nm, gr) for nm, gr in groups.items()
              if nm in used and (gr.amplitude_v or getattr(gr, "offset_v", 0.0))]
    pack = dict(ch_name=[], ch_kind=[], ch_om=[], ch_ph=[], ch_amp=[],
                ch_off=[], ch_duty=[], tab_t=[], tab_v=[], tab_off=[0])
    for name, gr in active:
        kind = WAVE_KIND.get(getattr(gr, "waveform", "sin"))
        if kind is None:
            raise ValueError(
                f"group {name!r} waveform {gr.waveform!r} unsupported; "
                f"one of {sorted(WAVE_KIND)}")
        if kind == 3 and getattr(gr, "interp", "hold") != "hold":
            kind = 4
        pack["ch_name"].append(str(name))
        pack["ch_kind"].append(kind)
        pack["ch_om"].append(2.0 * math.pi * float(gr.frequency_hz) * 1e-6)
        pack["ch_ph"].append(math.radians(float(gr.phase_deg)))
        pack["ch_amp"].append(float(gr.amplitude_v))
        pack["ch_off"].append(float(getattr(gr, "offset_v", 0.0)))
        d = float(getattr(gr, "duty", 0.5))
        if not (0.0 < d < 1.0):
            raise ValueError(f"group {name!r}: duty {d} outside (0, 1)")
        pack["ch_duty"].append(d)
        if kind == 3:
            t = list(getattr(gr, "table_t_us", []) or [])
            v = list(getattr(gr, "table_v", []) or [])
            if len(t) != len(v) or len(t) < 2:
                raise ValueError(f"group {name!r} table waveform needs "
                                 f"matching table_t_us/table_v (>=2 pts)")
            pack["tab_t"].extend(t)
            pack["tab_v"].extend(v)
        pack["tab_off"].append(len(pack["tab_t"]))

    # superposition plan: one step per electrode that contributes anywhere
    gidx = {nm: 1 + c for c, (nm, _) in enumerate(active)}
    nch = 1 + len(active)
    keys, rows, wcols, mcols = [], [], [], []
    for i, el in enumerate(els, start=1):
        w = np.zeros(nch, np.float32)
        m = np.zeros(nch, np.uint8)
        if dc[i - 1]:
            w[0] = np.float32(dc[i - 1])
            m[0] = 1
        for gname in member[i - 1]:
            if gname in gidx:
                w[gidx[gname]] = 1.0
                m[gidx[gname]] += 1
        if not m.any():
            continue
        if i not in keys:
            keys.append(i)
        rows.append(keys.index(i))
        wcols.append(w)
        mcols.append(m)
    if rows:
        weights = np.stack(wcols, axis=1)
        mult = np.stack(mcols, axis=1)
    else:
        weights = np.zeros((nch, 0), np.float32)
        mult = np.zeros((nch, 0), np.uint8)
    plan = dict(keys=keys, rows=np.array(rows, np.int32), weights=weights,
                mult=mult, names=["static"] + [nm for nm, _ in active])
    return plan, pack


def _pack_arrays(pack):
    return dict(
        ch_name=list(pack["ch_name"]),
        ch_kind=np.array(pack["ch_kind"], np.int64),
        ch_om=np.array(pack["ch_om"], np.float64),
        ch_ph=np.array(pack["ch_ph"], np.float64),
        ch_amp=np.array(pack["ch_amp"], np.float64),
        ch_off=np.array(pack["ch_off"], np.float64),
        ch_duty=np.array(pack["ch_duty"], np.float64),
        tab_t=np.array(pack["tab_t"], np.float64),
        tab_v=np.array(pack["tab_v"], np.float64),
        tab_off=np.array(pack["tab_off"], np.int64))


def compose_drive_channels(spec, bases, ele, verbose=False):
    """(static field + one affine channel per active drive group) as the
    reference's dict (build_stl3d.py:493-709).  bases: {electrode position
    (1-based): unit basis float32 (nx, ny, nz)}, numpy or CUDA tensors; ele:
    the label grid the solve rastered.  With CUDA tensors every array of
    the result is a CUDA tensor (float32 or float64 per channel_dtype)."""
    g = spec.geometry
    first = next(iter(bases.values()))
    shape = tuple(first.shape)
    resident = _is_tensor(first)
    if tuple(np.shape(ele) if not _is_tensor(ele) else ele.shape) != shape:
        raise ValueError(
            f"compose_drive_channels: label grid shape "
            f"{tuple(np.shape(ele) if not _is_tensor(ele) else ele.shape)} does not "
            f"match the bases {shape}; pass the label grid the solve "
            f"rastered (after any mirror unfold).")
    eaware = getattr(g, "field_method", "electrode_aware") == "electrode_aware"
    f32_out = getattr(g, "channel_dtype", "float64") == "float32"
    h = g.mm_per_gu
    plan, pack = drive_plan(spec, bases)
    torch = _torch()
    nch = len(plan["names"])
    dev = first.device if resident else torch.device("cuda")
    src = []
    for key in plan["keys"]:
        b = bases[key]
        if resident:
            b = b.to(dtype=torch.float32).contiguous()
        else:
            b = torch.from_numpy(np.ascontiguousarray(b, np.float32)).to(dev)
        src.append(b)
    P = superpose_device(src, plan["rows"], plan["weights"], plan["mult"],
                         shape=shape)
    del src
    E = torch.empty((3, nch) + shape, dtype=torch.float32, device=dev)
    _field_device(P, ele if eaware else None, h, eaware, out=E)
    if verbose:
        print(f"[compose] {nch} channel(s) composed on the GPU", flush=True)
    if not resident:
        torch.cuda.current_stream().synchronize()
    conv = (lambda t: t) if f32_out else (lambda t: t.to(torch.float64))
    host = (lambda t: t.cpu().numpy()) if not resident else (lambda t: t)
    K = nch - 1
    out = dict(
        EAx=host(conv(E[0, 0])), EAy=host(conv(E[1, 0])), EAz=host(conv(E[2, 0])),
        ExK=host(conv(E[0, 1:])), EyK=host(conv(E[1, 1:])), EzK=host(conv(E[2, 1:])),
        chan_phi=[host(P[c]) for c in range(1, 1 + K)])
    res = dict(EAx=out["EAx"], EAy=out["EAy"], EAz=out["EAz"],
               ExK=out["ExK"], EyK=out["EyK"], EzK=out["EzK"])
    arr = _pack_arrays(pack)
    res["ch_name"] = arr.pop("ch_name")
    res["chan_phi"] = out["chan_phi"]
    res.update(arr)
    return res


def clear_memory_cache():
    """build_stl3d.clear_memory_cache: no gradient cache is kept (a compose
    is two bandwidth-bound launches), so nothing is dropped."""
    return 0
