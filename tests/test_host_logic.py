"""Host-side logic of the drop-in, on the CPU: the theta builder and the
cache layout against fixtures recorded from the reference, the SOR factor,
the multigrid level shapes, the stop flag shared with the library, and the
refusals that happen before any GPU work."""
import json
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, Golden
from oracle import port


def test_fractions_from_scene_matches_reference():
    from ion_gym_gb300.physics import solver3d as S
    from ion_gym_gb300.physics.scene3d import (GeomScene, GridSpec, Electrode,
                                               Shape, Cylinder, Box3D)
    g = Golden("theta.npz")
    cases = g.cases("theta")
    n, nz, c = 23, 5, 11.0
    sc0 = GeomScene(grid=GridSpec(n, n, nz), units="gu", electrodes=[
        Electrode(1, "inner", [Shape([Cylinder(c, c, nz + 2.0, 4.3,
                                               nz + 4.0)])]),
        Electrode(2, "outer", [Shape(within=[Cylinder(c, c, nz + 2.0, 40.0,
                                                      nz + 4.0)],
                                     notin=[Cylinder(c, c, nz + 2.0, 9.6,
                                                     nz + 4.0)])])])
    sc1 = GeomScene(grid=GridSpec(17, 15, 13, mm_per_gu=0.5), units="mm",
                    electrodes=[Electrode(1, "plate", [Shape(
                        within=[Box3D(1.3, 0.65, 2.6, 6.6, 6.35, 3.7)],
                        notin=[Cylinder(4.0, 3.5, 4.0, 1.55, 3.0)])])])
    sc2 = GeomScene(grid=GridSpec(15, 15, 3), units="gu", electrodes=[
        Electrode(1, "rod", [Shape([Cylinder(0.0, 0.0, 9.0, 3.7, 20.0)])]),
        Electrode(2, "can", [Shape(within=[Cylinder(0.0, 0.0, 9.0, 40.0,
                                                    20.0)],
                                   notin=[Cylinder(0.0, 0.0, 9.0, 12.2,
                                                   20.0)])])])
    for sc, case in zip((sc0, sc1, sc2), cases):
        th = S.fractions_from_scene(sc, case["metal"].astype(bool),
                                    mirror=tuple(bool(x) for x in
                                                 case["mirror"]))
        assert th.dtype == np.float32
        assert np.array_equal(th, case["th"])
        assert (th < 1).sum() > 0


def test_cache_layout_matches_reference():
    from ion_gym_gb300.io import fa_cache
    g = Golden("cache.npz")
    for c in g.cases("cache"):
        spec = json.loads(str(c["spec"]))
        assert fa_cache.spec_key(spec) == str(c["key"])
        arrays = {k[4:]: c[k] for k in c if k.startswith("arr_")}
        with tempfile.TemporaryDirectory() as root:
            key = fa_cache.store(spec, arrays, root=root)
            assert key == str(c["key"])
            meta = json.load(open(os.path.join(root, key, "meta.json")))
            assert meta == json.loads(str(c["meta"]))
            for name in arrays:
                raw = open(os.path.join(root, key, name + ".npy"), "rb").read()
                assert raw == c[f"npy_{name}"].tobytes()
            back, m2 = fa_cache.load(key, root=root)
            for name, a in arrays.items():
                assert np.array_equal(back[name], a)
            # a tampered array is refused loudly, a missing entry is a miss
            p = os.path.join(root, key, "basis_1.npy")
            a = np.load(p)
            a.flat[0] += 1
            np.save(p, a)
            with pytest.raises(IOError, match="head hash"):
                fa_cache.load(key, root=root)
            assert fa_cache.load("0" * 16, root=root) == (None, None)


def test_store_bases_layout():
    from ion_gym_gb300.io import fa_cache
    m1 = np.zeros((4, 3, 2), bool)
    m1[0] = True
    m2 = np.zeros((4, 3, 2), bool)
    m2[-1] = True
    bases = {1: np.full((4, 3, 2), 0.5), 2: np.full((4, 3, 2), 0.25)}
    with tempfile.TemporaryDirectory() as root:
        key = fa_cache.store_bases({"k": 1}, bases, {1: m1, 2: m2}, root=root)
        b, masks = fa_cache.load_bases(key, root=root)
        assert b[1].dtype == np.float32 and np.all(b[1] == 0.5)
        assert np.array_equal(masks[2], m2)
        arrs, meta = fa_cache.load(key, root=root)
        assert arrs["labels"].dtype == np.uint8
        assert sorted(meta["arrays"]) == ["basis_1", "basis_2", "labels"]


def test_optimal_omega_matches_restatement(drivers_golden):
    from ion_gym_gb300.physics.solver3d import optimal_omega
    for shape in [(65, 65, 65), (257,) * 3, (520, 80, 1), (1, 1, 1), (9, 10, 9),
                  (193, 193, 385), (2, 2, 2)]:
        assert optimal_omega(shape) == port.optimal_omega(shape)
    assert optimal_omega((10, 20), spacing=(0.5, 1.0)) == \
        port.optimal_omega((10, 20), spacing=(0.5, 1.0))
    for c in drivers_golden.cases("solve3d"):
        if not bool(c["omega_given"]):
            assert optimal_omega(c["fixed"].shape) == float(c["omega"])


def test_level_shapes():
    from ion_gym_gb300.physics.multigrid3d import cascadic_shapes, bottom_shape
    assert cascadic_shapes((257,) * 3, 9, 4) == [(257,) * 3, (129,) * 3,
                                                 (65,) * 3, (33,) * 3]
    assert cascadic_shapes((257,) * 3) == [(257,) * 3, (129,) * 3, (65,) * 3,
                                           (33,) * 3, (17,) * 3, (9,) * 3]
    assert cascadic_shapes((21, 19, 23)) == [(21, 19, 23), (11, 10, 12),
                                             (6, 5, 6)]
    assert cascadic_shapes((9, 50, 50)) == [(9, 50, 50)]
    assert bottom_shape((193, 193, 385)) == (7, 7, 13)
    assert bottom_shape((19, 21, 17)) == (10, 11, 9)
    assert bottom_shape((5, 6, 1)) == (3, 3, 1)


def test_stencil_refused_before_any_work():
    from ion_gym_gb300.physics import solver3d as S, multigrid3d as M
    f = np.zeros((4, 4, 4), bool)
    for fn in (S.solve3d, M.solve3d_vmg, M.solve3d_mg):
        with pytest.raises(ValueError, match="known stencils are"):
            fn(f, np.zeros((4, 4, 4)), stencil="node")


def test_stop_event_arms_the_library():
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.physics import multigrid3d as M
    L = _lib.lib()
    M.clear_stop()
    assert L.ig_stop_requested() == 0 and not M.stop_event().is_set()
    M.request_stop()
    assert L.ig_stop_requested() == 1 and M.stop_event().is_set()
    M.stop_event().clear()
    assert L.ig_stop_requested() == 0
    M.stop_event().set()        # setting the event itself also arms it
    assert L.ig_stop_requested() == 1
    M.clear_stop()
    assert isinstance(M.SOLVE_EXCLUSIVE, type(__import__("threading").Lock()))


def test_no_gpu_means_a_loud_error():
    """Without a device the solvers raise; nothing computes on the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from ion_gym_gb300.physics import solver3d as S
    f = np.zeros((5, 5, 5), bool)
    f[0] = True
    with pytest.raises(RuntimeError, match="no CUDA device"):
        S.solve3d(f, np.where(f, 1.0, 0.0))


def test_concurrent_basis_door_keeps_the_serial_order(monkeypatch, capsys):
    """The basis door runs bases on several threads; with a fake library
    whose solves finish out of order, the progress lines, the returned dict
    and the first refusal (in electrode order) are those of a serial loop."""
    import ctypes
    import random
    import time as _t
    from ion_gym_gb300 import _lib
    from ion_gym_gb300.physics import multigrid3d as M

    shape = (5, 6, 7)
    masks = {k: np.zeros(shape, bool) for k in (1, 2, 3, 4, 5)}
    for k, m in masks.items():
        m[k - 1, 0, 0] = True
    rnd = random.Random(3)
    bad = {4}

    class FakeLib:
        def ig_solve_basis_vmg(self, mu, mk, v, th, nx, ny, nz, tol, mc, n1, n2,
                               code, bom, phi_p, sw, d, cyc, prev):
            m = np.ctypeslib.as_array(ctypes.cast(mk, ctypes.POINTER(ctypes.c_uint8)),
                                      shape=(nx * ny * nz,))
            k = int(np.argmax(m) // (ny * nz)) + 1
            _t.sleep(rnd.random() * 0.05)
            vals = np.full(nx * ny * nz, float(k))
            ctypes.memmove(phi_p, vals.ctypes.data, vals.nbytes)
            sw._obj.value = 10 * k
            d._obj.value = (2 * tol) if k in bad else tol / 2
            cyc._obj.value = 3
            prev._obj.value = 0.0
            return _lib.IG_OK

        def ig_device_free_bytes(self):
            return 1 << 34

        def ig_clear_stop(self):
            pass

        def ig_request_stop(self):
            pass

    M.clear_stop()
    monkeypatch.setattr(_lib, "lib", lambda: FakeLib())
    monkeypatch.setattr(M, "BASIS_CONCURRENCY", 3)
    with pytest.raises(M.SolveNotConverged, match="basis 4"):
        M.solve_bases_mg(masks, tol=1e-3)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if "electrode" in ln]
    assert [ln.split("electrode ")[1].split(" ")[0] for ln in lines] == \
        ["1", "1", "2", "2", "3", "3", "4", "4"]
    bad.clear()
    out = M.solve_bases_mg(masks, tol=1e-3, only={2, 3, 5})
    assert list(out) == [2, 3, 5]
    for k, phi in out.items():
        assert phi.shape == shape and np.all(phi == k)


def test_empty_basis_deck_fails_like_the_reference():
    """An empty {index: mask} deck: the reference's basis doors take the
    first mask's shape with next(iter(...)) and raise StopIteration before
    any solve (solver3d.py:296-320, multigrid3d.py:233-246); the drop-ins
    do the same, before touching the GPU."""
    from ion_gym_gb300.physics import solver3d, multigrid3d
    with pytest.raises(StopIteration):
        solver3d.solve_bases({})
    with pytest.raises(StopIteration):
        multigrid3d.solve_bases_mg({})


def test_pa_surf_sidecar_matches_reference(tmp_path):
    """fractions_from_pa_surf (solver3d.py:323-363) decodes the reference's
    theta, bit for bit, from synthetic sidecars recorded with the
    reference's reader (tests/golden/pasurf.npz): vacuum and metal records,
    clamped fractions, records past the grid, terminators, an empty chunk."""
    import os
    from ion_gym_gb300.physics import solver3d
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "pasurf.npz"))
    cases = sorted({k.split("/")[1] for k in z.files})
    assert len(cases) == 3
    for c in cases:
        path = tmp_path / f"case{c}.surf"
        path.write_bytes(z[f"pasurf/{c}/raw"].tobytes())
        shape = tuple(int(s) for s in z[f"pasurf/{c}/shape"])
        th = solver3d.fractions_from_pa_surf(str(path), shape,
                                             z[f"pasurf/{c}/metal"].astype(bool))
        want = z[f"pasurf/{c}/th"]
        assert th.dtype == want.dtype and th.shape == want.shape
        assert np.array_equal(th.view(np.uint32), want.view(np.uint32))
        assert (want < 1).sum() > 5


def test_unit_basis_door_routes_by_precision(monkeypatch):
    """solve_unit_bases_mg (the field cache's fill, build_stl3d.py:835-849):
    "fp64" converts the bit-exact door's float64 potentials on the host,
    (phi / v_basis).astype(float32); "mixed" asks the mixed door for unit
    bases formed on the device; fa_cache.solve_stl3d_bases passes the
    cache's V_BASIS and tolerance through."""
    from ion_gym_gb300.physics import multigrid3d as M
    from ion_gym_gb300.io import fa_cache
    shape = (3, 4, 5)
    masks = {1: np.zeros(shape, bool), 2: np.zeros(shape, bool)}
    masks[1][0, 0, 0] = masks[2][1, 1, 1] = True
    seen = {}

    def fake_door(masks_, v_basis=1e4, tol=1e-6, verbose=False,
                  stencil="ghost_linear", only=None, precision=None, **kw):
        seen["fp64"] = (v_basis, tol, precision)
        return {i: np.full(shape, 1234.5678901 * i) for i in masks_}

    def fake_mixed(masks_, todo, v_basis, tol, stencil, verbose, unit=False):
        seen["mixed"] = (v_basis, tol, unit, [i for _, i, _ in todo])
        return {i: np.full(shape, 0.5, np.float32) for _, i, _ in todo}

    monkeypatch.setattr(M, "solve_bases_mg", fake_door)
    monkeypatch.setattr(M, "_solve_bases_mixed_door", fake_mixed)
    got = M.solve_unit_bases_mg(masks, v_basis=1e4, tol=1e-4, precision="fp64")
    assert seen["fp64"] == (1e4, 1e-4, "fp64")
    for i in (1, 2):
        want = (np.full(shape, 1234.5678901 * i) / 1e4).astype(np.float32)
        assert got[i].dtype == np.float32 and np.array_equal(got[i], want)
    got = fa_cache.solve_stl3d_bases(masks, precision="mixed")
    assert seen["mixed"] == (fa_cache.V_BASIS, fa_cache.STL3D_SOLVE_TOL, True, [1, 2])
    assert sorted(got) == [1, 2] and got[1].dtype == np.float32
