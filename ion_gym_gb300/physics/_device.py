"""Single-kernel entry points of libigsolve.so on numpy arrays or CUDA torch
tensors.

These back the reference's module-level kernel names (_sweep, _residual,
_sweep_rhs, _restrict_fw_njit, ...).  A numpy argument makes one round trip
through device memory; a CUDA tensor is used in place on torch's current
stream.  torch supplies device memory and the stream handle only; all
arithmetic is in the library's kernels.
"""
import ctypes

import numpy as np

from ion_gym_gb300 import _lib


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("ion_gym_gb300: no CUDA device is visible; the "
                           "field solve runs only on the GPU")
    return torch


def _is_tensor(a):
    return type(a).__module__.startswith("torch")


_TD = {np.float64: "float64", np.float32: "float32", np.uint8: "uint8"}


def _to_dev(a, np_dtype):
    torch = _torch()
    tdt = getattr(torch, _TD[np_dtype])
    if _is_tensor(a):
        if a.device.type != "cuda":
            a = a.to("cuda")
        if a.dtype == torch.bool and np_dtype == np.uint8:
            a = a.to(torch.uint8)
        return a.to(tdt).contiguous()
    arr = np.ascontiguousarray(np.asarray(a), dtype=np_dtype)
    return torch.from_numpy(arr).to("cuda")


def _mask_dev(a):
    if _is_tensor(a):
        return _to_dev(a, np.uint8)
    return _to_dev(np.asarray(a, bool).view(np.uint8)
                   if np.asarray(a).dtype == bool else
                   (np.asarray(a) != 0).view(np.uint8), np.uint8)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(_torch().cuda.current_stream().cuda_stream)


def _all_ones(th):
    if th is None:
        return True
    if _is_tensor(th):
        return bool((th == 1).all().item())
    return bool(np.all(np.asarray(th) == 1.0))


def _writeback(orig, dev):
    """Copy a device result into the caller's array (numpy in place, or the
    tensor if it was not already the device buffer)."""
    if _is_tensor(orig):
        if orig.data_ptr() != dev.data_ptr():
            orig.copy_(dev.to(orig.dtype))
    else:
        orig[...] = dev.cpu().numpy()


def _check(st, what):
    _lib.check(st, what)


def sweep(phi, fixed, th, omega, colour, ghost_linear):
    """solver3d._sweep: one colour, phi in place, returns max |update|."""
    L = _lib.lib()
    shape = tuple(phi.shape)
    p = _to_dev(phi, np.float64)
    f = _mask_dev(fixed)
    t = None if _all_ones(th) else _to_dev(th, np.float32)
    out = ctypes.c_double(0.0)
    st = L.ig_sweep_dev(_p(p), _p(f), _p(t), *shape, float(omega),
                        int(colour), 0 if ghost_linear else 1,
                        ctypes.byref(out), _stream())
    _check(st, "_sweep")
    _writeback(phi, p)
    return float(out.value)


def residual(phi, fixed, th, ghost_linear, out):
    """multigrid3d._residual into `out`."""
    L = _lib.lib()
    shape = tuple(phi.shape)
    p = _to_dev(phi, np.float64)
    f = _mask_dev(fixed)
    t = None if _all_ones(th) else _to_dev(th, np.float32)
    o = _to_dev(np.empty(shape), np.float64) if not _is_tensor(out) else out
    st = L.ig_residual_dev(_p(p), _p(f), _p(t), *shape,
                           0 if ghost_linear else 1, _p(o), _stream())
    _check(st, "_residual")
    _writeback(out, o)


def sweep_rhs(e, fixed, f, omega, colour):
    L = _lib.lib()
    shape = tuple(e.shape)
    ed = _to_dev(e, np.float64)
    fx = _mask_dev(fixed)
    fd = _to_dev(f, np.float64)
    out = ctypes.c_double(0.0)
    st = L.ig_sweep_rhs_dev(_p(ed), _p(fx), _p(fd), *shape, float(omega),
                            int(colour), ctypes.byref(out), _stream())
    _check(st, "_sweep_rhs")
    _writeback(e, ed)
    return float(out.value)


def residual_rhs(e, fixed, f, out):
    L = _lib.lib()
    shape = tuple(e.shape)
    ed = _to_dev(e, np.float64)
    fx = _mask_dev(fixed)
    fd = _to_dev(f, np.float64)
    o = _to_dev(np.empty(shape), np.float64) if not _is_tensor(out) else out
    st = L.ig_residual_rhs_dev(_p(ed), _p(fx), _p(fd), *shape, _p(o),
                               _stream())
    _check(st, "_residual_rhs")
    _writeback(out, o)


def restrict_fw(fine, out):
    L = _lib.lib()
    shape = tuple(fine.shape)
    fd = _to_dev(fine, np.float64)
    cs = tuple((s + 1) // 2 for s in shape)
    if tuple(out.shape) != cs:
        raise ValueError(f"restriction output must have shape {cs}")
    o = _to_dev(np.empty(cs), np.float64) if not _is_tensor(out) else out
    st = L.ig_restrict_fw_dev(_p(fd), *shape, _p(o), _stream())
    _check(st, "_restrict_fw_njit")
    _writeback(out, o)


def prolong_add(coarse, out, fixed):
    L = _lib.lib()
    cd = _to_dev(coarse, np.float64)
    od = _to_dev(out, np.float64)
    fx = _mask_dev(fixed)
    st = L.ig_prolong_add_dev(_p(cd), *tuple(coarse.shape), _p(od), _p(fx),
                              *tuple(out.shape), _stream())
    _check(st, "_prolong_add_njit")
    _writeback(out, od)


def prolongate(coarse, shape_f):
    L = _lib.lib()
    torch = _torch()
    cd = _to_dev(coarse, np.float64)
    shape_f = tuple(int(s) for s in shape_f)
    od = torch.empty(shape_f, dtype=torch.float64, device="cuda")
    st = L.ig_prolongate_dev(_p(cd), *tuple(coarse.shape), _p(od), *shape_f,
                             _stream())
    _check(st, "_prolongate")
    return od if _is_tensor(coarse) else od.cpu().numpy()


def coarsen_fixed_any(fixed):
    L = _lib.lib()
    torch = _torch()
    shape = tuple(fixed.shape)
    fx = _mask_dev(fixed)
    cs = tuple((s + 1) // 2 for s in shape)
    od = torch.empty(cs, dtype=torch.uint8, device="cuda")
    st = L.ig_coarsen_fixed_any_dev(_p(fx), *shape, _p(od), _stream())
    _check(st, "_coarsen_fixed_any")
    return od.bool() if _is_tensor(fixed) else od.cpu().numpy().astype(bool)


def coarsen_mask(fixed, val):
    L = _lib.lib()
    torch = _torch()
    shape = tuple(fixed.shape)
    fx = _mask_dev(fixed)
    vd = _to_dev(val, np.float64)
    cs = tuple((s + 1) // 2 for s in shape)
    fc = torch.empty(cs, dtype=torch.uint8, device="cuda")
    vc = torch.empty(cs, dtype=torch.float64, device="cuda")
    st = L.ig_coarsen_mask_dev(_p(fx), _p(vd), *shape, _p(fc), _p(vc),
                               _stream())
    _check(st, "_coarsen_mask")
    if _is_tensor(fixed):
        return fc.bool(), vc
    return fc.cpu().numpy().astype(bool), vc.cpu().numpy()


def residual_audit(u, fixed, theta):
    L = _lib.lib()
    torch = _torch()
    shape = tuple(u.shape)
    ud = _to_dev(u, np.float64)
    fx = _mask_dev(fixed)
    td = _to_dev(theta, np.float32)
    od = torch.empty(shape, dtype=torch.float64, device="cuda")
    st = L.ig_residual_audit_dev(_p(ud), _p(fx), _p(td), *shape, _p(od),
                                 _stream())
    _check(st, "residual_field")
    return od if _is_tensor(u) else od.cpu().numpy()


def err_sweep(e, fixed, theta, rhs, omega, colour):
    L = _lib.lib()
    shape = tuple(e.shape)
    ed = _to_dev(e, np.float64)
    fx = _mask_dev(fixed)
    td = _to_dev(theta, np.float32)
    rd = _to_dev(rhs, np.float64)
    out = ctypes.c_double(0.0)
    st = L.ig_err_sweep_dev(_p(ed), _p(fx), _p(td), _p(rd), *shape,
                            float(omega), int(colour), ctypes.byref(out),
                            _stream())
    _check(st, "_err_sweep")
    _writeback(e, ed)
    return float(out.value)


def explain_residual(ref, fixed, theta, tol, max_sweeps):
    """The error-equation solve of attribute_difference (solver3d.py:435-443)
    with the arrays resident on the device."""
    torch = _torch()
    r = residual_audit(_to_dev(ref, np.float64), _mask_dev(fixed), theta)
    neg = -r
    e = torch.zeros_like(r)
    fx = _mask_dev(fixed)
    th = _to_dev(theta, np.float32)
    shape = tuple(r.shape)
    om = 2.0 / (1.0 + np.sin(np.pi / (max(shape) + 1)))
    for _ in range(max_sweeps):
        d = max(err_sweep(e, fx, th, neg, om, 0),
                err_sweep(e, fx, th, neg, om, 1))
        if d < tol:
            break
    return e.cpu().numpy()
