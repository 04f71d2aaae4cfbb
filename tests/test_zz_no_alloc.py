"""ig_cascadic_relres_noalloc: the residual-stopped cascadic solve for
callers that cannot allocate device memory while they run (a process whose
HBM budget is reserved up front, a framework custom call that only lends its
own buffers).  It must give the same result as ig_cascadic_relres, the
allocating entry point, on two calls in a row (the static scratch keeps the
previous call's contents), allocate nothing, and refuse a grid whose coarse
levels do not fit its scratch.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(L, fx, val, out, shape, stream, omega):
    sw = ctypes.c_long(0)
    rr = ctypes.c_double(0.0)
    tot = ctypes.c_long(0)
    nl = ctypes.c_int(0)
    st = L.ig_cascadic_relres_noalloc(
        ctypes.c_void_p(fx.data_ptr()), ctypes.c_void_p(val.data_ptr()),
        *shape, 1e-10, 200000, 9, 4, 30.0, omega.ctypes.data_as(ctypes.c_void_p),
        len(omega), 20, ctypes.c_void_p(out.data_ptr()), ctypes.byref(sw),
        ctypes.byref(rr), ctypes.byref(tot), ctypes.byref(nl), stream)
    return st, sw.value, rr.value, tot.value, nl.value


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.physics import multigrid3d as MG
    from ion_gym_gb300.workloads import quadrupole, random_deck
    torch.cuda.set_device(0)
    L = _lib.lib()
    n = 97
    fixed, val = quadrupole(n, r0=12.0)
    fx = torch.from_numpy(fixed.view(np.uint8)).cuda()
    vd = torch.from_numpy(val).cuda()
    ref, ref_sw, ref_rr, ref_tot = MG.solve3d_cascadic_relres(
        fx, vd, 1e-10, 1.85, 4, 9, 20)
    # a second deck of another shape and other Dirichlet values, solved
    # between the two compared calls: it overwrites the shared scratch with
    # coarse levels of other sizes and values, so the last call shows that
    # every coarse array is written before it is read
    f2, v2 = random_deck(77, 81, 6)
    f2 = np.ascontiguousarray(f2[:, :65, :73])
    v2 = np.ascontiguousarray(v2[:, :65, :73])
    f2[:, -1] = True
    f2[:, :, -1] = True
    v2[:, -1] = 0.0
    v2[:, :, -1] = 0.0
    fx2 = torch.from_numpy(f2.view(np.uint8)).cuda()
    vd2 = torch.from_numpy(v2).cuda()
    ref2, ref2_sw, ref2_rr, ref2_tot = MG.solve3d_cascadic_relres(
        fx2, vd2, 1e-10, 1.85, 4, 9, 20)
    omega = np.full(4, 1.85)
    outs = [torch.empty_like(vd) for _ in range(2)]
    out2 = torch.empty_like(vd2)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    first = _call(L, fx, vd, outs[0], (n, n, n), stream, omega)
    other = _call(L, fx2, vd2, out2, f2.shape, stream, omega)
    torch.cuda.synchronize()
    # the last call must not touch the allocator at all
    free_before = torch.cuda.mem_get_info()[0]
    second = _call(L, fx, vd, outs[1], (n, n, n), stream, omega)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    for st, sw, rr, tot, nl in (first, second):
        assert st == _lib.IG_OK, _lib.last_error()
        assert (sw, rr, tot, nl) == (ref_sw, ref_rr, ref_tot, 4)
    assert other[0] == _lib.IG_OK, _lib.last_error()
    assert other[1:4] == (ref2_sw, ref2_rr, ref2_tot)
    # FP64 path: the tolerance of these tests is bit equality
    for o in outs:
        assert torch.equal(o.view(torch.int64), ref.view(torch.int64))
    assert torch.equal(out2.view(torch.int64), ref2.view(torch.int64))
    assert free_after == free_before


def test_noalloc_refuses_grids_beyond_its_scratch():
    import torch
    from ion_gym_gb300 import _lib
    L = _lib.lib()
    shape = (257, 257, 513)        # coarse levels need ~83 MB > 48 MiB
    fx = torch.zeros(shape, dtype=torch.uint8, device="cuda")
    vd = torch.zeros(shape, dtype=torch.float64, device="cuda")
    out = torch.empty_like(vd)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st, *_ = _call(L, fx, vd, out, shape, stream, np.full(4, 1.85))
    assert st == _lib.IG_BAD_ARG
    assert "static scratch holds" in _lib.last_error()
