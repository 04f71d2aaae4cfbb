"""Generate the golden fixtures under tests/golden/ by running the reference
ion_gym solver itself (unmodified, from a checkout given by --ref) under the
pure-Python numba stand-in in tests/golden/numba_stub.

    PYTHONPATH=tests/golden/numba_stub:<ion_gym checkout> \
        NUMBA_CACHE_DIR=/tmp/nbc ION_GYM_CACHE=/tmp/igc \
        python tests/golden/make_golden.py

Nothing in the test-suite or the library imports the reference at run time:
the fixtures written here are the only thing carried forward.  Every case
stores its inputs, the exact call, and the reference's outputs, so a test can
replay the call through the oracle or the CUDA path and compare bits.

Fixture files:
  kernels.npz  single calls of the reference's numba kernels
               (solver3d._sweep, multigrid3d._residual, _sweep_rhs,
               _residual_rhs, _restrict_fw_njit, _prolong_add_njit,
               _coarsen_fixed_any, _coarsen_mask, _prolongate,
               solver3d._residual_kernel, _err_sweep)
  drivers.npz  whole solves (solve3d, solve3d_mg, solve3d_vmg, solve_bases,
               solve_bases_mg) with their returned (phi, sweeps, delta) and
               the messages of the refusals.
  field.npz    tracer3d.build_field_aware_3d and
               build_stl3d.compose_drive_channels on small grids, with the
               messages of the composer's refusals.
  shapes.npz   physics/build_shapes3d.shapes_masks_3d on decks of rotated
               rects, ellipses, polygons and cutouts extruded along x, y and
               z (origin, mirror), as label grids, and its refusals.
  bundle.npz   io/fa_cache.store + annotate and io/field_io
               export_field_bundle / import_field_bundle /
               read_field_arrays on a small 3-D entry: the key, every bundle
               member, the spec JSON written beside it and the refusals.
  pasurf.npz   solver3d.fractions_from_pa_surf on synthetic surface-fraction
               sidecars (the sidecar bytes, grid, metal and theta).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

SHAPES = [(9, 10, 11), (8, 8, 8), (5, 6, 1), (1, 7, 9), (2, 3, 4),
          (1, 1, 5), (3, 1, 1), (6, 5, 7)]


def _theta(rng, shape, frac_ones=0.6, lo=1e-3):
    th = rng.uniform(lo, 1.0, (6,) + shape).astype(np.float32)
    th[rng.random(th.shape) < frac_ones] = 1.0
    return th


def kernel_cases(rng, S, M):
    out = {}

    def put(kind, idx, **arrs):
        for k, v in arrs.items():
            out[f"{kind}/{idx}/{k}"] = np.asarray(v)

    # _sweep ---------------------------------------------------------------
    variants = [(False, True, 0, 1.83), (False, False, 1, 1.0),
                (True, True, 1, 1.5), (True, False, 0, 1.2)]
    idx = 0
    for shape in SHAPES:
        for use_th, gl, colour, omega in variants:
            phi = rng.uniform(-2.0, 2.0, shape)
            fixed = rng.random(shape) < 0.25
            th = _theta(rng, shape) if use_th else np.ones((6,) + shape,
                                                           np.float32)
            p = phi.copy()
            d = S._sweep(p, fixed, th, False, False, False, omega, colour, gl)
            put("sweep", idx, phi=phi, fixed=fixed.astype(np.uint8), th=th,
                has_theta=use_th, omega=omega, colour=colour, ghost_linear=gl,
                out=p, d=float(d))
            idx += 1

    # multigrid _residual --------------------------------------------------
    idx = 0
    for shape in SHAPES:
        for use_th, gl in [(False, True), (True, True), (True, False)]:
            phi = rng.uniform(-2.0, 2.0, shape)
            fixed = rng.random(shape) < 0.25
            th = _theta(rng, shape) if use_th else np.ones((6,) + shape,
                                                           np.float32)
            r = np.full(shape, np.nan)
            M._residual(phi, fixed, th, gl, r)
            put("residual", idx, phi=phi, fixed=fixed.astype(np.uint8), th=th,
                has_theta=use_th, ghost_linear=gl, out=r)
            idx += 1

    # _sweep_rhs / _residual_rhs -------------------------------------------
    idx = 0
    for shape in SHAPES:
        for colour, omega in [(0, 1.0), (1, 1.0), (0, 1.71), (1, 1.71)]:
            e = rng.uniform(-1.0, 1.0, shape)
            f = rng.uniform(-3.0, 3.0, shape)
            fixed = rng.random(shape) < 0.25
            e[fixed] = 0.0
            p = e.copy()
            d = M._sweep_rhs(p, fixed, f, omega, colour)
            r = np.full(shape, np.nan)
            M._residual_rhs(e, fixed, f, r)
            put("sweep_rhs", idx, e=e, f=f, fixed=fixed.astype(np.uint8),
                omega=omega, colour=colour, out=p, d=float(d), res=r)
            idx += 1

    # _restrict_fw_njit, _coarsen_fixed_any, _coarsen_mask ------------------
    idx = 0
    for shape in SHAPES + [(3, 3, 3), (4, 5, 6)]:
        fine = rng.uniform(-1.0, 1.0, shape)
        cs = tuple((s + 1) // 2 for s in shape)
        rc = np.full(cs, np.nan)
        M._restrict_fw_njit(fine, rc)
        fixed = rng.random(shape) < 0.15
        val = np.where(fixed, rng.uniform(-5, 5, shape), rng.uniform(-1, 1, shape))
        fa = M._coarsen_fixed_any(fixed)
        fc, vc = M._coarsen_mask(fixed, val)
        put("restrict", idx, fine=fine, out=rc, fixed=fixed.astype(np.uint8),
            val=val, any=fa.astype(np.uint8), fc=fc.astype(np.uint8), vc=vc)
        idx += 1

    # _prolong_add_njit and cascadic _prolongate ---------------------------
    idx = 0
    for shape in SHAPES + [(3, 3, 3), (4, 5, 6)]:
        cs = tuple((s + 1) // 2 for s in shape)
        coarse = rng.uniform(-1.0, 1.0, cs)
        base = rng.uniform(-1.0, 1.0, shape)
        fixed = rng.random(shape) < 0.2
        o = base.copy()
        M._prolong_add_njit(coarse, o, fixed)
        pl = M._prolongate(coarse, shape)
        put("prolong", idx, coarse=coarse, base=base,
            fixed=fixed.astype(np.uint8), out=o, prolongate=pl)
        idx += 1

    # solver3d audit kernels (_residual_kernel, _err_sweep) -----------------
    idx = 0
    for shape in [(9, 10, 11), (8, 8, 8), (6, 5, 7), (4, 5, 6)]:
        u = rng.uniform(-2.0, 2.0, shape)
        fixed = rng.random(shape) < 0.2
        th = _theta(rng, shape)
        r = S._residual_kernel(u, fixed, th)
        e = rng.uniform(-0.1, 0.1, shape)
        rhs = rng.uniform(-0.1, 0.1, shape)
        p = e.copy()
        d = S._err_sweep(p, fixed, th, rhs, 1.6, idx & 1)
        put("audit", idx, u=u, fixed=fixed.astype(np.uint8), th=th, res=r,
            e=e, rhs=rhs, omega=1.6, colour=idx & 1, out=p, d=float(d))
        idx += 1
    return out


# ---------------------------------------------------------------- drivers
def _sphere_box(shape, c, r, v=1.0):
    i, j, k = np.meshgrid(*[np.arange(s, dtype=float) for s in shape],
                          indexing="ij")
    fixed = np.zeros(shape, bool)
    fixed[0] = fixed[-1] = True
    fixed[:, 0] = fixed[:, -1] = True
    fixed[:, :, 0] = fixed[:, :, -1] = True
    sph = (i - c[0]) ** 2 + (j - c[1]) ** 2 + (k - c[2]) ** 2 <= r * r
    fixed |= sph
    val = np.where(sph, v, 0.0)
    return fixed, val


def _plate(shape, thin=False):
    nx, ny, nz = shape
    fixed = np.zeros(shape, bool)
    val = np.zeros(shape)
    w = 1 if thin else 3
    fixed[nx // 4:3 * nx // 4, ny // 2:ny // 2 + w, nz // 4:3 * nz // 4] = True
    val[fixed] = 1e4
    fixed[:, 0, :] = True
    fixed[:, -1, :] = True
    return fixed, val


def driver_cases(rng, S, M):
    out = {}

    def put(kind, idx, **arrs):
        for k, v in arrs.items():
            out[f"{kind}/{idx}/{k}"] = np.asarray(v)

    def timed(label, fn):
        t = time.time()
        r = fn()
        print(f"  {label}: {time.time() - t:.1f}s", flush=True)
        return r

    # solve3d ---------------------------------------------------------------
    cases = []
    f, v = _sphere_box((12, 13, 11), (6, 6.5, 5), 2.6)
    cases.append(dict(fixed=f, val=v, tol=1e-8, omega=None, phi0=None,
                      theta=None, stencil="ghost_linear"))
    phi0 = rng.uniform(0, 1, f.shape)
    cases.append(dict(fixed=f, val=v, tol=1e-7, omega=1.7, phi0=phi0,
                      theta=None, stencil="ghost_linear"))
    th = _theta(rng, f.shape, 0.8)
    cases.append(dict(fixed=f, val=v, tol=1e-7, omega=None, phi0=None,
                      theta=th, stencil="sw"))
    cases.append(dict(fixed=f, val=v, tol=1e-7, omega=None, phi0=None,
                      theta=th, stencil="ghost_linear"))
    f1 = np.zeros((20, 17, 1), bool)
    f1[0] = f1[-1] = True
    f1[:, 0] = f1[:, -1] = True
    f1[12:15, 5:8] = True
    v1 = np.where(f1, 0.0, 0.0)
    v1[12:15, 5:8] = 1e4
    cases.append(dict(fixed=f1, val=v1, tol=1e-8, omega=1.0, phi0=None,
                      theta=None, stencil="ghost_linear"))
    for idx, c in enumerate(cases):
        phi, sw, d = timed(f"solve3d {idx}", lambda: S.solve3d(
            c["fixed"], c["val"], theta=c["theta"], tol=c["tol"],
            omega=c["omega"], phi0=c["phi0"], stencil=c["stencil"]))
        om = c["omega"] if c["omega"] is not None else S.optimal_omega(
            c["fixed"].shape)
        put("solve3d", idx, fixed=c["fixed"].astype(np.uint8), val=c["val"],
            tol=c["tol"], omega=om, omega_given=c["omega"] is not None,
            has_phi0=c["phi0"] is not None,
            phi0=c["phi0"] if c["phi0"] is not None else np.zeros(0),
            has_theta=c["theta"] is not None,
            theta=c["theta"] if c["theta"] is not None else np.zeros(0,
                                                                 np.float32),
            stencil=c["stencil"], phi=phi, sweeps=sw, delta=d)
    # the refusal
    try:
        S.solve3d(cases[0]["fixed"], cases[0]["val"], tol=1e-12,
                  max_sweeps=7)
        raise AssertionError("reference did not refuse")
    except S.SolveNotConverged as e:
        put("solve3d_refuse", 0, message=str(e))

    # cascadic solve3d_mg ----------------------------------------------------
    f, v = _sphere_box((21, 19, 23), (10, 9, 11), 4.2)
    phi, sw, d = timed("solve3d_mg 0", lambda: M.solve3d_mg(f, v, tol=1e-8))
    put("mg", 0, fixed=f.astype(np.uint8), val=v, tol=1e-8, max_levels=8,
        has_theta=False, theta=np.zeros(0, np.float32), stencil="ghost_linear",
        phi=phi, sweeps=sw, delta=d)
    th = _theta(rng, f.shape, 0.85)
    phi, sw, d = timed("solve3d_mg 1", lambda: M.solve3d_mg(
        f, v, theta=th, tol=1e-7, max_levels=2, stencil="sw"))
    put("mg", 1, fixed=f.astype(np.uint8), val=v, tol=1e-7, max_levels=2,
        has_theta=True, theta=th, stencil="sw", phi=phi, sweeps=sw, delta=d)

    # V-cycle solve3d_vmg -----------------------------------------------------
    vcases = []
    f, v = _plate((19, 21, 17))
    vcases.append(dict(fixed=f, val=v, tol=1e-5, theta=None,
                       stencil="ghost_linear", phi0=None))
    f2, v2 = _plate((25, 27, 23), thin=True)
    vcases.append(dict(fixed=f2, val=v2, tol=1e-5, theta=None,
                       stencil="ghost_linear", phi0=None))
    # x- and y-symmetric: exercises the symmetric-subspace projection
    fs = np.zeros((21, 21, 15), bool)
    fs[0] = fs[-1] = True
    fs[:, 0] = fs[:, -1] = True
    fs[7:14, 7:14, 5:10] = True
    vs = np.where(fs, 0.0, 0.0)
    vs[7:14, 7:14, 5:10] = 100.0
    vcases.append(dict(fixed=fs, val=vs, tol=1e-7, theta=None,
                       stencil="ghost_linear", phi0=None))
    th = _theta(rng, f.shape, 0.95, lo=0.3)
    vcases.append(dict(fixed=f, val=v, tol=1e-5, theta=th, stencil="sw",
                       phi0=rng.uniform(0, 1e3, f.shape)))
    for idx, c in enumerate(vcases):
        phi, sw, d = timed(f"solve3d_vmg {idx}", lambda: M.solve3d_vmg(
            c["fixed"], c["val"], theta=c["theta"], tol=c["tol"],
            stencil=c["stencil"], phi0=c["phi0"]))
        put("vmg", idx, fixed=c["fixed"].astype(np.uint8), val=c["val"],
            tol=c["tol"], has_theta=c["theta"] is not None,
            theta=c["theta"] if c["theta"] is not None else np.zeros(
                0, np.float32),
            stencil=c["stencil"], has_phi0=c["phi0"] is not None,
            phi0=c["phi0"] if c["phi0"] is not None else np.zeros(0),
            phi=phi, sweeps=sw, delta=d)
    # refusals: cycle cap and stagnation (reference test_multigrid_refusal)
    fp = np.zeros((20, 20, 20), bool)
    vp = np.zeros((20, 20, 20))
    fp[0] = fp[-1] = True
    vp[0] = 100.0
    try:
        M.solve3d_vmg(fp, vp, tol=1e-30, max_cycles=1)
        raise AssertionError("no cap refusal")
    except S.SolveNotConverged as e:
        put("vmg_refuse", 0, message=str(e))
    try:
        timed("stagnation", lambda: M.solve3d_vmg(fp, vp, tol=1e-14,
                                                  max_cycles=200))
        raise AssertionError("no stagnation refusal")
    except S.SolveNotConverged as e:
        put("vmg_refuse", 1, message=str(e))
    phi, sw, d = M.solve3d_vmg(fp, vp, tol=1e-14, max_cycles=200,
                               accept_stagnation=True)
    put("vmg_refuse", 2, phi=phi, sweeps=sw, delta=d)

    # solve_bases (SOR) and solve_bases_mg (V-cycle) --------------------------
    shape = (14, 12, 10)
    m1 = np.zeros(shape, bool)
    m1[0] = True
    m2 = np.zeros(shape, bool)
    m2[-1] = True
    m3 = np.zeros(shape, bool)
    m3[5:8, 4:7, 3:6] = True
    masks = {1: m1, 2: m2, 4: m3}
    b = timed("solve_bases", lambda: S.solve_bases(masks, tol=1e-6))
    put("bases", 0, m1=m1.astype(np.uint8), m2=m2.astype(np.uint8),
        m4=m3.astype(np.uint8), b1=b[1], b2=b[2], b4=b[4])
    shape = (19, 17, 21)
    mm1 = np.zeros(shape, bool)
    mm1[:, 0, :] = True
    mm2 = np.zeros(shape, bool)
    mm2[6:12, 8:10, 5:16] = True
    mm3 = np.zeros(shape, bool)
    mm3[:, -1, :] = True
    masks = {1: mm1, 2: mm2, 3: mm3}
    bm = timed("solve_bases_mg", lambda: M.solve_bases_mg(masks, tol=1e-4,
                                                         only={1, 2}))
    put("bases_mg", 0, m1=mm1.astype(np.uint8), m2=mm2.astype(np.uint8),
        m3=mm3.astype(np.uint8), tol=1e-4, b1=bm[1], b2=bm[2],
        keys=np.array(sorted(bm)))
    return out


def theta_cases(S):
    """solver3d.fractions_from_scene on small analytic scenes: a coax
    (cylinder inside a ring), a box with a cylindrical hole, and a folded
    (mirror x, y) quadrant."""
    from ion_gym.physics.scene3d import (GeomScene, GridSpec, Electrode,
                                         Shape, Cylinder, Box3D)
    out = {}
    n, nz = 23, 5
    c = 11.0
    ii, jj = np.meshgrid(np.arange(n, dtype=float), np.arange(n, dtype=float),
                         indexing="ij")
    rr = np.hypot(ii - c, jj - c)
    metal = ((rr <= 4.3) | (rr >= 9.6))[:, :, None] & np.ones((1, 1, nz), bool)
    sc = GeomScene(grid=GridSpec(n, n, nz), units="gu", electrodes=[
        Electrode(1, "inner", [Shape([Cylinder(c, c, nz + 2.0, 4.3,
                                               nz + 4.0)])]),
        Electrode(2, "outer", [Shape(within=[Cylinder(c, c, nz + 2.0, 40.0,
                                                      nz + 4.0)],
                                     notin=[Cylinder(c, c, nz + 2.0, 9.6,
                                                     nz + 4.0)])])])
    out["theta/0/metal"] = metal.astype(np.uint8)
    out["theta/0/mirror"] = np.array([False, False, False])
    out["theta/0/th"] = S.fractions_from_scene(sc, metal)
    # a box plate with a hole, in mm (scaled to gu by the scene)
    shape = (17, 15, 13)
    i, j, k = np.meshgrid(*[np.arange(s, dtype=float) for s in shape],
                          indexing="ij")
    plate = ((i >= 2.6) & (i <= 13.2) & (j >= 1.3) & (j <= 12.7)
             & (k >= 5.2) & (k <= 7.4)
             & ~((i - 8.0) ** 2 + (j - 7.0) ** 2 < 3.1 ** 2))
    sc2 = GeomScene(grid=GridSpec(*shape, mm_per_gu=0.5), units="mm",
                    electrodes=[Electrode(1, "plate", [Shape(
                        within=[Box3D(1.3, 0.65, 2.6, 6.6, 6.35, 3.7)],
                        notin=[Cylinder(4.0, 3.5, 4.0, 1.55, 3.0)])])])
    out["theta/1/metal"] = plate.astype(np.uint8)
    out["theta/1/mirror"] = np.array([False, False, False])
    out["theta/1/th"] = S.fractions_from_scene(sc2, plate)
    # folded quadrant with mirror planes at x = 0 and y = 0
    q = 15
    qi, qj = np.meshgrid(np.arange(q, dtype=float), np.arange(q, dtype=float),
                         indexing="ij")
    rq = np.hypot(qi, qj)
    mq = ((rq <= 3.7) | (rq >= 12.2))[:, :, None] & np.ones((1, 1, 3), bool)
    sc3 = GeomScene(grid=GridSpec(q, q, 3), units="gu", electrodes=[
        Electrode(1, "rod", [Shape([Cylinder(0.0, 0.0, 9.0, 3.7, 20.0)])]),
        Electrode(2, "can", [Shape(within=[Cylinder(0.0, 0.0, 9.0, 40.0,
                                                    20.0)],
                                   notin=[Cylinder(0.0, 0.0, 9.0, 12.2,
                                                   20.0)])])])
    out["theta/2/metal"] = mq.astype(np.uint8)
    out["theta/2/mirror"] = np.array([True, True, False])
    out["theta/2/th"] = S.fractions_from_scene(sc3, mq,
                                               mirror=(True, True, False))
    return out


def pasurf_cases(S):
    """solver3d.fractions_from_pa_surf on synthetic surface-fraction
    sidecars: a header, XOFF / YOFF / ZOFF chunks of (u64 flat index with x
    fastest, f64 fraction) records at vacuum and metal nodes (metal records
    set the -leg of the vacuum node above; records whose node above is metal
    or off the grid are dropped), fractions below the 1e-3 clamp, indices
    past the grid, terminator records, and an empty chunk."""
    import tempfile
    out = {}
    rng = np.random.default_rng(4242)
    for case, shape in enumerate([(9, 7, 6), (5, 8, 1), (12, 4, 5)]):
        nx, ny, nz = shape
        n = nx * ny * nz
        metal = rng.random(shape) < 0.3
        chunks = [b"SIMEXP\x00\x01" + bytes(8)]
        for tag in (b"XOFF", b"YOFF", b"ZOFF"):
            if tag == b"ZOFF" and case == 1:
                chunks.append(tag)              # empty chunk
                continue
            m = int(rng.integers(10, 40))
            idx = rng.integers(0, n, m).astype("<u8")
            f = rng.random(m)
            f[:3] = [0.0, 5e-4, 1.0]            # clamp and edge fractions
            rec = np.empty(m + 2, dtype=[("idx", "<u8"), ("f", "<f8")])
            rec["idx"][:m] = idx
            rec["f"][:m] = f
            rec["idx"][m] = n + 7                # past the grid
            rec["f"][m] = 0.5
            rec["idx"][m + 1] = 0xFFFFFFFF00000000  # terminator record
            rec["f"][m + 1] = 0.0
            chunks.append(tag + rec.tobytes())
        raw = b"".join(chunks)
        with tempfile.NamedTemporaryFile(suffix=".surf", delete=False) as fh:
            fh.write(raw)
            path = fh.name
        try:
            th = S.fractions_from_pa_surf(path, shape, metal)
        finally:
            os.unlink(path)
        out[f"pasurf/{case}/raw"] = np.frombuffer(raw, np.uint8).copy()
        out[f"pasurf/{case}/shape"] = np.array(shape)
        out[f"pasurf/{case}/metal"] = metal.astype(np.uint8)
        out[f"pasurf/{case}/th"] = th
    return out


def cache_cases():
    """io/fa_cache.store of a small basis set (the entry layout of
    build_stl3d.py:919-924) into a scratch root: the key, meta.json and the
    .npy bytes the reference writes."""
    import json
    import tempfile
    from ion_gym.io import fa_cache
    out = {}
    rng = np.random.default_rng(4)
    specs = [{"stl3d-v1_bases": "0123456789abcdef" * 4},
             {"geometry": {"h": 0.1, "name": "einzel"}, "v": [1.5, 2.25e-7],
              "n": 3}]
    lab = np.zeros((6, 5, 4), np.uint8)
    lab[1:3, 2:4, :] = 1
    lab[4:, :, 1:3] = 2
    arrays = {"basis_1": rng.random((6, 5, 4)).astype(np.float32),
              "basis_2": rng.random((6, 5, 4)).astype(np.float32),
              "labels": lab}
    for idx, spec in enumerate(specs):
        with tempfile.TemporaryDirectory() as root:
            key = fa_cache.store(spec, arrays, root=root)
            meta = open(os.path.join(root, key, "meta.json")).read()
            out[f"cache/{idx}/spec"] = np.array(json.dumps(spec))
            out[f"cache/{idx}/key"] = np.array(key)
            out[f"cache/{idx}/meta"] = np.array(meta)
            for name in arrays:
                raw = open(os.path.join(root, key, name + ".npy"), "rb").read()
                out[f"cache/{idx}/npy_{name}"] = np.frombuffer(raw, np.uint8)
                out[f"cache/{idx}/arr_{name}"] = arrays[name]
    return out


def raster_cases():
    """physics/rasterize3d.rasterize on small analytic scenes, and the
    messages of its two refusals (overlapping electrodes, an electrode with
    no node)."""
    from ion_gym.physics.scene3d import (GeomScene, GridSpec, Electrode,
                                         Shape, Cylinder, Box3D)
    from ion_gym.physics.rasterize3d import rasterize
    out = {}
    g = GridSpec(31, 29, 27, mm_per_gu=0.5, overhang="allow")
    scenes = [
        GeomScene(grid=g, units="mm", electrodes=[
            Electrode(1, "rod", [Shape([Cylinder(7.5, 7.0, 12.0, 2.35, 9.0)])]),
            Electrode(3, "plate", [Shape(
                within=[Box3D(1.0, 1.0, 1.2, 14.0, 3.3, 2.1)],
                notin=[Cylinder(7.5, 2.0, 3.0, 1.1, 4.0)])]),
            Electrode(2, "cup", [Shape(
                within=[Cylinder(7.5, 7.0, 13.0, 6.4, 2.0)],
                notin=[Cylinder(7.5, 7.0, 13.0, 5.2, 2.0)])])]),
        GeomScene(grid=GridSpec(25, 23, 9, overhang="allow"), units="gu",
                  electrodes=[
            Electrode(1, "a", [Shape([Box3D(2.0, 2.0, 0.0, 10.0, 20.0, 8.0)]),
                               Shape([Cylinder(18.0, 11.0, 8.0, 4.5, 8.0)])]),
            Electrode(2, "b", [Shape([Box3D(12.5, 0.0, 0.0, 13.5, 22.0,
                                            8.0)])])]),
    ]
    for idx, sc in enumerate(scenes):
        out[f"raster/{idx}/lab"] = rasterize(sc)
    clash = GeomScene(grid=GridSpec(20, 20, 5, overhang="allow"), units="gu",
                      electrodes=[
        Electrode(1, "a", [Shape([Box3D(2.0, 2.0, 0.0, 10.0, 10.0, 4.0)])]),
        Electrode(2, "b", [Shape([Box3D(8.0, 8.0, 0.0, 15.0, 15.0, 4.0)])])])
    empty = GeomScene(grid=GridSpec(20, 20, 5, overhang="allow"), units="gu",
                      electrodes=[
        Electrode(1, "a", [Shape([Box3D(2.0, 2.0, 0.0, 10.0, 10.0, 4.0)])]),
        Electrode(2, "tiny", [Shape([Cylinder(15.5, 15.5, 2.5, 0.2, 0.3)])])])
    for name, sc in (("clash", clash), ("empty", empty)):
        try:
            rasterize(sc)
            raise AssertionError(f"{name}: no refusal")
        except ValueError as e:
            out[f"raster_err/{name}/message"] = np.array(str(e))
    return out


class _El:
    """Electrode stand-in with the two attributes the composer reads."""

    def __init__(self, name, groups, dc):
        self.name, self._groups, self.dc = name, list(groups), dc

    def group_names(self):
        return list(self._groups)


class _Spec:
    """SimSpec stand-in: .geometry and dc_effective(el)."""

    def __init__(self, geometry):
        self.geometry = geometry

    def dc_effective(self, el):
        return el.dc


def _group(name, **kw):
    from types import SimpleNamespace
    d = dict(name=name, amplitude_v=0.0, offset_v=0.0, waveform="sin",
             frequency_hz=1.0e6, phase_deg=0.0, duty=0.5)
    d.update(kw)
    return SimpleNamespace(**d)


def _smooth(rng, shape, scale=1.0):
    x = rng.standard_normal(shape)
    for ax in range(3):
        x = (x + np.roll(x, 1, ax) + np.roll(x, -1, ax)) / 3.0
    return (scale * x).astype(np.float32)


def _labels(rng, shape, boxes):
    lab = np.zeros(shape, np.int16)
    for idx, (lo, hi) in enumerate(boxes, start=1):
        lab[tuple(slice(a, b) for a, b in zip(lo, hi))] = idx
    return lab


def field_specs():
    """(name, geometry kwargs, electrodes) of the composer cases."""
    from types import SimpleNamespace
    ga = [_group("rf_a", amplitude_v=150.0, frequency_hz=1.1e6),
          _group("rf_b", amplitude_v=150.0, waveform="cos", phase_deg=180.0,
                 frequency_hz=1.1e6),
          _group("sq", amplitude_v=0.0, offset_v=5.0, waveform="square",
                 duty=0.3, frequency_hz=2.5e5),
          _group("tab", amplitude_v=20.0, waveform="table", interp="linear",
                 table_t_us=[0.0, 1.5, 3.0], table_v=[0.0, 1.0, -0.5]),
          _group("idle", amplitude_v=0.0)]
    ea = [_El("e1", ["rf_a"], 10.0), _El("e2", ["rf_b"], 0.0),
          _El("e3", ["rf_a"], -3.25), _El("e4", ["sq", "tab"], 0.1),
          _El("e5", ["tab", "idle"], 7e-3)]
    gb = [_group("p", amplitude_v=75.5, phase_deg=33.0, frequency_hz=7.7e5),
          _group("hold", amplitude_v=3.0, waveform="table",
                 table_t_us=[0.0, 2.0], table_v=[1.0, 1.0])]
    eb = [_El("a", ["p", "p"], 0.0), _El("b", [], 12.5),
          _El("c", ["hold"], -1.0), _El("d", ["p"], 0.0)]
    return [
        ("aware_f64", dict(mm_per_gu=0.2), ga, ea),
        ("plain_f32", dict(mm_per_gu=np.float64(0.15), field_method="plain",
                           channel_dtype="float32"), ga, ea),
        ("repeat_f64", dict(mm_per_gu=0.35), gb, eb),
        ("static_only", dict(mm_per_gu=0.5), [], [_El("x", [], 2.0),
                                                  _El("y", [], 0.0)]),
    ]


def field_error_specs():
    ok = [_El("e1", ["g"], 1.0), _El("e2", [], 0.0)]
    return [
        ("undefined", [_group("g", amplitude_v=1.0)],
         [_El("e1", ["nope"], 0.0), _El("e2", [], 0.0)]),
        ("unused", [_group("g", amplitude_v=1.0), _group("h", offset_v=2.0)],
         ok),
        ("waveform", [_group("g", amplitude_v=1.0, waveform="saw")], ok),
        ("duty", [_group("g", amplitude_v=1.0, waveform="square", duty=1.0)],
         ok),
        ("table", [_group("g", amplitude_v=1.0, waveform="table",
                          table_t_us=[0.0], table_v=[1.0])], ok),
    ]


def field_cases():
    """tracer3d.build_field_aware_3d (float32 and float64 potentials, Python
    and numpy float64 spacings, with and without the metal rule) and
    build_stl3d.compose_drive_channels on stand-in specs."""
    from types import SimpleNamespace
    from ion_gym.physics.tracer3d import build_field_aware_3d
    from ion_gym.physics.build_stl3d import compose_drive_channels
    rng = np.random.default_rng(4242)
    out = {}
    grads = [((13, 11, 9), np.float32, 0.1, True),
             ((13, 11, 9), np.float32, np.float64(0.05), True),
             ((13, 11, 9), np.float32, 0.3, False),
             ((10, 7, 12), np.float64, 0.25, True),
             ((2, 3, 4), np.float32, 0.7, True),
             ((2, 2, 2), np.float32, np.float64(1.3), True),
             ((5, 9, 2), np.float32, 1, True)]
    for idx, (shape, dt, h, aware) in enumerate(grads):
        phi = _smooth(rng, shape, 40.0).astype(dt)
        boxes = [((0, 0, 0), (max(1, shape[0] // 3), shape[1], 1)),
                 ((shape[0] // 2, 1, shape[2] // 2),
                  (shape[0], max(2, shape[1] // 2), shape[2]))]
        ele = _labels(rng, shape, boxes)
        if idx == 3:
            ele = (ele * 3).astype(np.uint8)
        ex, ey, ez = build_field_aware_3d(phi, ele, h, electrode_aware=aware)
        k = f"grad/{idx}"
        out[k + "/phi"] = phi
        out[k + "/ele"] = ele
        out[k + "/h"] = np.array(float(h))
        out[k + "/h_is_f64"] = np.array(isinstance(h, np.float64))
        out[k + "/aware"] = np.array(aware)
        out[k + "/ex"], out[k + "/ey"], out[k + "/ez"] = ex, ey, ez
    for name, gkw, groups, els in field_specs():
        shape = (12, 10, 9)
        bases = {i: np.abs(_smooth(rng, shape, 0.4)) for i in
                 range(1, len(els) + 1)}
        ele = _labels(rng, shape, [((0, 0, 0), (3, 10, 2)),
                                   ((8, 3, 4), (12, 7, 9))])
        geom = SimpleNamespace(rf_groups=groups, electrodes=els, **gkw)
        ch = compose_drive_channels(_Spec(geom), bases, ele)
        k = f"compose/{name}"
        out[k + "/bases"] = np.stack([bases[i] for i in sorted(bases)])
        out[k + "/ele"] = ele
        for key, v in ch.items():
            if key == "chan_phi":
                out[k + "/chan_phi"] = (np.stack(v) if v else
                                        np.zeros((0,) + shape, np.float32))
            elif key == "ch_name":
                out[k + "/ch_name"] = np.array(v, dtype=str)
            else:
                out[k + "/" + key] = np.asarray(v)
    shape = (6, 5, 4)
    bases = {1: _smooth(rng, shape), 2: _smooth(rng, shape)}
    ele = np.zeros(shape, np.int16)
    for name, groups, els in field_error_specs():
        geom = SimpleNamespace(rf_groups=groups, electrodes=els, mm_per_gu=0.1)
        try:
            compose_drive_channels(_Spec(geom), bases, ele)
            raise AssertionError(f"{name}: no refusal")
        except ValueError as e:
            out[f"compose_err/{name}/message"] = np.array(str(e))
    try:
        geom = SimpleNamespace(rf_groups=[], electrodes=[_El("e1", [], 1.0)],
                               mm_per_gu=0.1)
        compose_drive_channels(_Spec(geom), bases, np.zeros((6, 5, 3)))
        raise AssertionError("shape: no refusal")
    except ValueError as e:
        out["compose_err/shape/message"] = np.array(str(e))
    return out


def _deck(electrodes, width=4.0, height=3.0, depth=3.0, pitch=0.25,
          mirror=None, origin=None):
    g = {"width_mm": width, "height_mm": height, "depth_mm": depth,
         "mm_per_gu": pitch,
         "symmetry": {"coords": "xyz", "planes": mirror or {}},
         "electrodes": electrodes}
    if origin is not None:
        g["origin_mm"] = origin
    return {"name": "shapes_deck",
            "source": {"seed": 0, "distribution": "disc", "n_ions": 100,
                       "x0_mm": 1.0, "y0_mm": 0.0, "z0_mm": 0.0, "r_mm": 4.0,
                       "ke_lo": 0.1, "ke_hi": 1.9, "mz_list": [556.0],
                       "tob_span_us": 2.0},
            "integration": {"dt_ns": 1.0, "t_max_us": 400.0},
            "geometry": g}


def shapes_decks():
    """(name, deck dict) of the shapes fixture: labelled decks first, then
    the refusals."""
    ez = {"axis": "z", "lo_mm": 0.5, "hi_mm": 1.0}
    tri = [[1.9, 1.8], [2.4, 2.3], [1.7, 2.6]]
    ok = [
        ("mixed", _deck([
            {"name": "E1", "shapes": [{"type": "rect", "x_mm": 1.0, "y_mm": 0.5,
                                       "width_mm": 2.0, "height_mm": 1.5,
                                       "extrude": ez}]},
            {"name": "E2", "shapes": [
                {"type": "ellipse", "cx_mm": 2.0, "cy_mm": 2.2, "rx_mm": 1.1,
                 "ry_mm": 0.55,
                 "extrude": {"axis": "x", "lo_mm": 1.5, "hi_mm": 3.5}},
                {"type": "cutout", "children": [{"type": "polygon",
                                                  "points_mm": tri}]}]},
            {"name": "E3", "shapes": [
                {"type": "rect", "x_mm": 0.25, "y_mm": 2.0, "width_mm": 1.0,
                 "height_mm": 0.5, "rotation_deg": 30.0,
                 "extrude": {"axis": "y", "lo_mm": 2.25, "hi_mm": 3.0}},
                {"type": "polygon", "points_mm": [[0.0, 0.0], [0.75, 0.0],
                                                  [0.75, 0.5], [0.25, 1.0]]}]},
        ])),
        ("origin", _deck([
            {"name": "A", "shapes": [{"type": "rect", "x_mm": -1.0, "y_mm": -0.5,
                                      "width_mm": 1.5, "height_mm": 1.0}]},
            {"name": "B", "shapes": [{"type": "ellipse", "cx_mm": 1.5,
                                      "cy_mm": 0.75, "rx_mm": 0.6, "ry_mm": 0.9,
                                      "extrude": {"axis": "z", "lo_mm": 1.0,
                                                  "hi_mm": 2.5}}]},
        ], origin=[-1.5, -1.0])),
        ("mirror", _deck([
            {"name": "M", "shapes": [{"type": "polygon",
                                      "points_mm": [[0.5, 0.5], [3.0, 0.75],
                                                    [2.0, 2.5]],
                                      "extrude": {"axis": "z", "lo_mm": 0.0,
                                                  "hi_mm": 0.5}}]},
        ], mirror={"z": "mirror"})),
    ]
    bad = [
        ("empty", _deck([
            {"name": "A", "shapes": [{"type": "rect", "x_mm": 1.0, "y_mm": 1.0,
                                      "width_mm": 1.0, "height_mm": 1.0}]},
            {"name": "tiny", "shapes": [
                {"type": "rect", "x_mm": 3.0, "y_mm": 2.0, "width_mm": 0.5,
                 "height_mm": 0.5},
                {"type": "cutout", "children": [{"type": "rect", "x_mm": 2.9,
                                                  "y_mm": 1.9, "width_mm": 0.7,
                                                  "height_mm": 0.7}]}]}])),
        ("clash", _deck([
            {"name": "A", "shapes": [{"type": "rect", "x_mm": 1.0, "y_mm": 1.0,
                                      "width_mm": 1.0, "height_mm": 1.0}]},
            {"name": "B", "shapes": [{"type": "ellipse", "cx_mm": 2.0,
                                      "cy_mm": 1.5, "rx_mm": 0.5,
                                      "ry_mm": 0.5}]}])),
        ("zero_shape", _deck([
            {"name": "A", "shapes": [
                {"type": "rect", "x_mm": 1.0, "y_mm": 1.0, "width_mm": 1.0,
                 "height_mm": 1.0},
                {"type": "rect", "x_mm": 1.01, "y_mm": 1.01, "width_mm": 0.1,
                 "height_mm": 0.1}]}])),
        ("zero_cutout", _deck([
            {"name": "A", "shapes": [
                {"type": "rect", "x_mm": 1.0, "y_mm": 1.0, "width_mm": 1.0,
                 "height_mm": 1.0},
                {"type": "cutout", "children": [{"type": "ellipse",
                                                  "cx_mm": 3.1, "cy_mm": 0.1,
                                                  "rx_mm": 0.05,
                                                  "ry_mm": 0.05}]}]}])),
        ("outside", _deck([
            {"name": "A", "shapes": [{"type": "rect", "x_mm": 1.0, "y_mm": 1.0,
                                      "width_mm": 1.0, "height_mm": 1.0,
                                      "extrude": {"axis": "z", "lo_mm": 5.0,
                                                  "hi_mm": 6.0}}]}])),
        ("mirror_lo", _deck([
            {"name": "A", "shapes": [{"type": "rect", "x_mm": 1.0, "y_mm": 1.0,
                                      "width_mm": 1.0, "height_mm": 1.0,
                                      "extrude": {"axis": "z", "lo_mm": -0.5,
                                                  "hi_mm": 1.0}}]}],
            mirror={"z": "mirror"})),
        ("no_shapes", _deck([
            {"name": "A", "shapes": [{"type": "rect", "x_mm": 1.0, "y_mm": 1.0,
                                      "width_mm": 1.0, "height_mm": 1.0}]},
            {"name": "B", "shapes": []}])),
    ]
    return ok, bad


def shapes_cases():
    from ion_gym.io.sim_spec import SimSpec
    from ion_gym.physics.build_shapes3d import shapes_masks_3d
    out = {}
    ok, bad = shapes_decks()
    for name, d in ok:
        masks = shapes_masks_3d(SimSpec.from_dict(d))
        shape = next(iter(masks.values())).shape
        lab = np.zeros(shape, np.int16)
        for i, m in masks.items():
            lab[m] = i
        out[f"shapes/{name}/lab"] = lab
    for name, d in bad:
        try:
            shapes_masks_3d(SimSpec.from_dict(d))
            raise AssertionError(f"{name}: no refusal")
        except ValueError as e:
            out[f"shapes_err/{name}/message"] = np.array(str(e))
    return out


def bundle_spec():
    """The small 3-D entry of the bundle fixture: (spec, arrays, spec_json)."""
    rng = np.random.default_rng(99)
    spec = {"name": "ring deck", "route": "stl3d", "grid": [4, 5, 6],
            "geometry": {"mm_per_gu": 0.25, "electrodes": [
                {"name": "e1", "v": 10.0}, {"name": "e2", "v": -3.5}]}}
    lab = np.zeros((4, 5, 6), np.uint8)
    lab[0] = 1
    lab[-1, :, :2] = 2
    arrays = {"basis_1": rng.random((4, 5, 6)).astype(np.float32),
              "basis_2": rng.random((4, 5, 6)).astype(np.float32),
              "labels": lab}
    spec_json = {"name": "ring deck", "geometry": spec["geometry"]}
    return spec, arrays, spec_json


def bundle_cases():
    """A cache entry written by the reference, exported as a bundle and
    imported back under a fresh root."""
    import tempfile
    from ion_gym.io import fa_cache
    from ion_gym.io import field_io
    out = {}
    spec, arrays, spec_json = bundle_spec()
    with tempfile.TemporaryDirectory() as td:
        root = os.path.join(td, "cache")
        key = fa_cache.store(spec, arrays, root=root)
        fa_cache.annotate(key, "ring deck", label="first", root=root,
                          spec_json=spec_json)
        npz, deck = field_io.export_field_bundle(key, os.path.join(td, "out"),
                                                 root=root)
        out["bundle/0/key"] = np.array(key)
        out["bundle/0/npz_name"] = np.array(os.path.basename(npz))
        out["bundle/0/deck_name"] = np.array(os.path.basename(deck))
        with open(deck, encoding="utf-8") as f:
            out["bundle/0/deck_text"] = np.array(f.read())
        with np.load(npz) as z:
            out["bundle/0/members"] = np.array(sorted(z.files))
            for m in z.files:
                out[f"member/{m}/value"] = z[m]
        bases, labels, meta = field_io.read_field_arrays(npz)
        out["bundle/0/read_keys"] = np.array(sorted(bases))
        for k, b in bases.items():
            out[f"read/{k}/basis"] = b
        out["bundle/0/read_labels"] = labels
        out["bundle/0/meta_json"] = np.array(json.dumps(meta, sort_keys=True))
        root2 = os.path.join(td, "cache2")
        k2 = field_io.import_field_bundle(npz, root=root2)
        out["bundle/0/import_key"] = np.array(k2)
        files = sorted(os.listdir(os.path.join(root2, k2)))
        out["bundle/0/import_files"] = np.array(files)
        with open(os.path.join(root2, k2, "meta.json"), "rb") as f:
            out["bundle/0/import_meta_bytes"] = np.frombuffer(f.read(), np.uint8)
        bad = dict(spec_json, geometry=dict(spec_json["geometry"], mm_per_gu=0.5))

        class _S:
            def to_dict(self):
                return bad
        try:
            field_io.import_field_bundle(npz, spec=_S(), root=root2)
            raise AssertionError("no refusal")
        except ValueError as e:
            out["bundle_err/geometry/message"] = np.array(str(e))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.dirname(os.path.abspath(__file__)))
    ap.add_argument("--only", choices=["kernels", "drivers", "theta", "cache",
                                       "raster", "field", "bundle", "shapes",
                                       "pasurf"],
                    default=None)
    a = ap.parse_args()
    import ion_gym.physics.solver3d as S
    import ion_gym.physics.multigrid3d as M
    assert "stub" in sys.modules["numba"].__version__, "run under the stub"
    if a.only in (None, "kernels"):
        rng = np.random.default_rng(20261203)
        np.savez_compressed(os.path.join(a.out, "kernels.npz"),
                            **kernel_cases(rng, S, M))
        print("kernels.npz written")
    if a.only in (None, "drivers"):
        rng = np.random.default_rng(777)
        np.savez_compressed(os.path.join(a.out, "drivers.npz"),
                            **driver_cases(rng, S, M))
        print("drivers.npz written")
    if a.only in (None, "theta"):
        np.savez_compressed(os.path.join(a.out, "theta.npz"), **theta_cases(S))
        print("theta.npz written")
    if a.only in (None, "cache"):
        np.savez_compressed(os.path.join(a.out, "cache.npz"), **cache_cases())
        print("cache.npz written")
    if a.only in (None, "raster"):
        np.savez_compressed(os.path.join(a.out, "raster.npz"),
                            **raster_cases())
        print("raster.npz written")
    if a.only in (None, "field"):
        np.savez_compressed(os.path.join(a.out, "field.npz"), **field_cases())
        print("field.npz written")
    if a.only in (None, "shapes"):
        np.savez_compressed(os.path.join(a.out, "shapes.npz"), **shapes_cases())
        print("shapes.npz written")
    if a.only in (None, "bundle"):
        np.savez_compressed(os.path.join(a.out, "bundle.npz"), **bundle_cases())
        print("bundle.npz written")
    if a.only in (None, "pasurf"):
        np.savez_compressed(os.path.join(a.out, "pasurf.npz"), **pasurf_cases(S))
        print("pasurf.npz written")


if __name__ == "__main__":
    main()
