"""ion_gym_gb300.physics.solver3d -- drop-in for ion_gym.physics.solver3d.

Same public names, signatures, defaults, return tuples and exceptions as the
reference module (ion_gym physics/solver3d.py).  The sweeps run on the GPU
through libigsolve.so and return the reference's float64 bits: the same
sweep count, the same final delta and the same potential.

Conventions kept from the reference:
  * every outer face is an even reflection (the ghost at -1 is node 1); a
    size-1 axis uses the node itself, so nz=1 is the exact 2-D problem;
  * the `mirror` flags are accepted and, as in the reference kernel, do not
    change the sweep (even reflection already puts a zero-gradient plane on
    the edge node);
  * theta (6, nx, ny, nz) float32, order (-x, +x, -y, +y, -z, +z), None for
    node-Dirichlet; stencil "ghost_linear" (default) or "sw".
"""
import numpy as np

from ion_gym_gb300 import _lib
from ion_gym_gb300._lib import ptr, as_mask, as_f64, as_f32

EPS = 1e-9
KNOWN_STENCILS = ("ghost_linear", "sw")


class SolveNotConverged(RuntimeError):
    """The iteration stopped without meeting its tolerance (a sweep cap, a
    stagnating V-cycle or an exhausted cycle budget).  A solver that cannot
    meet its tolerance raises this instead of returning the iterate
    (solver3d.py:233-247)."""


def stencil_code(stencil):
    """0 for 'ghost_linear', 1 for 'sw'; anything else is refused and quoted
    back (solver3d.py:271-277)."""
    if stencil not in KNOWN_STENCILS:
        raise ValueError(
            f"unknown stencil {stencil!r}; known stencils are "
            f"'ghost_linear' (linear ghost-value fractional surface) and "
            f"'sw' (Shortley-Weller).")
    return 0 if stencil == "ghost_linear" else 1


def optimal_omega(shape, spacing=None):
    """Young's optimal SOR factor for the 7-point Laplacian on a rectangular
    grid (solver3d.py:201-230): rho = sum_a w_a cos(pi/(n_a+1)) / sum_a w_a
    over the axes with at least two nodes (w_a = 1/h_a^2), and
    omega = 2 / (1 + sqrt(1 - rho^2)); 1.0 when no axis couples."""
    if spacing is None:
        axes = [(int(n), 1.0) for n in shape if int(n) >= 2]
    else:
        axes = [(int(n), 1.0 / (float(h) * float(h)))
                for n, h in zip(shape, spacing) if int(n) >= 2]
    if not axes:
        return 1.0
    acc = sum(w * np.cos(np.pi / (n + 1)) for n, w in axes)
    rho = acc / sum(w for _, w in axes)
    rho = min(rho, 1.0 - 1e-15)
    return 2.0 / (1.0 + np.sqrt(1.0 - rho * rho))


def _grid_args(fixed, theta):
    fixed = np.asarray(fixed, bool)
    if fixed.ndim != 3:
        raise ValueError(f"fixed must be a 3-D mask, got shape {fixed.shape}")
    nx, ny, nz = fixed.shape
    th = None
    if theta is not None:
        th = as_f32(theta)
        if th.shape != (6, nx, ny, nz):
            raise ValueError(f"theta must have shape (6, {nx}, {ny}, {nz}), "
                             f"got {th.shape}")
    return fixed, th, (nx, ny, nz)


def _sor_refusal(shape, max_sweeps, d, tol):
    nx, ny, nz = shape
    return SolveNotConverged(
        f"SOR stopped at its cap of {max_sweeps} sweeps on a {nx}x{ny}x{nz} "
        f"grid with the last sweep delta {d:.3e} against tol {tol:.3e} "
        f"({d / max(tol, 1e-30):.0f}x too loose). An unconverged field is "
        f"not returned. SOR stalls on long thin domains: solve with "
        f"multigrid3d.solve_bases_mg / solve3d_vmg, or raise max_sweeps.")


def solve3d(fixed, val, theta=None, mirror=(False, False, False),
            tol=1e-6, max_sweeps=60000, omega=None, phi0=None,
            verbose=False, stencil="ghost_linear"):
    """Red-black SOR solve of Laplace with Dirichlet `fixed` nodes at `val`
    (solver3d.py:250-293).  Returns (phi float64 (nx,ny,nz), sweep pairs,
    final max |update|); raises SolveNotConverged at max_sweeps."""
    fixed, th, shape = _grid_args(fixed, theta)
    code = stencil_code(stencil)
    v = as_f64(np.broadcast_to(np.asarray(val, np.float64), shape))
    if omega is None:
        omega = optimal_omega(shape)
    p0 = None if phi0 is None else as_f64(np.broadcast_to(
        np.asarray(phi0, np.float64), shape))
    phi = np.empty(shape)
    sw = _lib.ctypes.c_long(0)
    d = _lib.ctypes.c_double(0.0)
    L = _lib.lib()
    st = L.ig_solve3d(ptr(as_mask(fixed)), ptr(v), ptr(th), *shape,
                      float(tol), int(max_sweeps), float(omega), ptr(p0),
                      code, ptr(phi), _lib.ctypes.byref(sw),
                      _lib.ctypes.byref(d))
    _lib.check(st, "solve3d")
    if st == _lib.IG_NOT_CONVERGED:
        raise _sor_refusal(shape, max_sweeps, d.value, tol)
    if verbose:
        print(f"  solve3d: {sw.value} sweeps, max|d| {d.value:.3e}")
    return phi, int(sw.value), float(d.value)


def _union(masks):
    metal = np.zeros(np.asarray(next(iter(masks.values()))).shape, bool)
    for m in masks.values():
        metal |= np.asarray(m, bool)
    return metal


def solve_bases(masks, scene=None, mirror=(False, False, False),
                v_basis=1e4, tol=1e-6, verbose=False, stencil="ghost_linear",
                omega=None, only=None):
    """Per-electrode unit-basis SOR solves (solver3d.py:296-320):
    {index: mask} -> {index: phi} with electrode i at v_basis and every other
    electrode at 0.  With a scene, theta comes once from its exact solids."""
    metal = _union(masks)
    th = (fractions_from_scene(scene, metal, mirror=mirror)
          if scene is not None else None)
    code = stencil_code(stencil)
    shape = metal.shape
    if omega is None:
        omega = optimal_omega(shape)
    th = None if th is None else as_f32(th)
    mu = as_mask(metal)
    out = {}
    L = _lib.lib()
    for i, m in sorted(masks.items()):
        if only is not None and i not in only:
            continue
        phi = np.empty(shape)
        sw = _lib.ctypes.c_long(0)
        d = _lib.ctypes.c_double(0.0)
        st = L.ig_solve_basis_sor(ptr(mu), ptr(as_mask(m)), float(v_basis),
                                  ptr(th), *shape, float(tol), 60000,
                                  float(omega), code, ptr(phi),
                                  _lib.ctypes.byref(sw), _lib.ctypes.byref(d))
        _lib.check(st, "solve_bases")
        if st == _lib.IG_NOT_CONVERGED:
            raise _sor_refusal(shape, 60000, d.value, tol)
        if verbose:
            print(f"basis {i}: {sw.value} sweeps, final delta {d.value:.2e} V")
        out[i] = phi
    return out


# ------------------------------------------------------------ kernels
def _sweep(phi, fixed, th, mirror_x, mirror_y, mirror_z, omega, colour,
           ghost_linear_stencil):
    """One colour of the SOR sweep (solver3d.py:131-198), phi updated in
    place; returns the max |update|.  Accepts numpy arrays (one device round
    trip) or CUDA torch tensors (in place on the device)."""
    from ion_gym_gb300.physics import _device
    return _device.sweep(phi, fixed, th, omega, colour, ghost_linear_stencil)


def residual_field(u, fixed, theta):
    """Audit residual num/den - u of u under the ghost_linear stencil
    (solver3d.py:366-386, 420-424); 0 at fixed nodes."""
    from ion_gym_gb300.physics import _device
    return _device.residual_audit(u, fixed, theta)


def attribute_difference(ref, phi, fixed, theta, tol=1e-7, max_sweeps=30000):
    """Split ref - phi into the part explained by ref's own residual and the
    rest (solver3d.py:427-444): SOR on (I - M) e = -r, then
    (e, (ref - phi) - e)."""
    from ion_gym_gb300.physics import _device
    e = _device.explain_residual(ref, fixed, theta, tol, max_sweeps)
    return e, (np.asarray(ref) - np.asarray(phi)) - e


# ------------------------------------------------------------ theta builders
def _prim_kind(p):
    k = getattr(p, "kind", None)
    if k is None:
        k = "cylinder" if hasattr(p, "r") else "box3d"
    return k


def inside_scene_pts(scene, pts):
    """Exact solid test of points (N,3) in grid units (solver3d.py:46-72):
    the union over electrode shapes of (any `within` primitive) minus (any
    `notin` primitive, strictly inside); points on a hole surface stay
    metal."""
    sc = scene.in_gu()
    x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
    total = np.zeros(len(pts), bool)

    def inside(p, strict):
        e = -EPS if strict else EPS
        if _prim_kind(p) == "cylinder":
            return (((x - p.cx) ** 2 + (y - p.cy) ** 2 <= p.r ** 2 + e)
                    & (z >= p.z - p.length - e) & (z <= p.z + e))
        return ((x >= p.x1 - e) & (x <= p.x2 + e)
                & (y >= p.y1 - e) & (y <= p.y2 + e)
                & (z >= p.z1 - e) & (z <= p.z2 + e))

    for el in sc.electrodes:
        for sh in el.shapes:
            w = np.zeros(len(pts), bool)
            for p in sh.within:
                w |= inside(p, False)
            for p in sh.notin:
                w &= ~inside(p, True)
            total |= w
    return total


_DIRS = ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1))


def _metal_neighbour(metal, d, mirror):
    """Mask of nodes whose d-neighbour is metal; a low mirror plane sees the
    reflected node 1 from node 0."""
    dx, dy, dz = _DIRS[d]
    ax = 0 if dx else (1 if dy else 2)
    step = dx + dy + dz
    nb = np.zeros_like(metal)
    dst = [slice(None)] * 3
    src = [slice(None)] * 3
    if step < 0:
        dst[ax], src[ax] = slice(1, None), slice(0, -1)
    else:
        dst[ax], src[ax] = slice(0, -1), slice(1, None)
    nb[tuple(dst)] = metal[tuple(src)]
    if step < 0 and mirror[ax]:
        e0 = [slice(None)] * 3
        e1 = [slice(None)] * 3
        e0[ax], e1[ax] = 0, 1
        nb[tuple(e0)] = metal[tuple(e1)]
    return nb, ax, step


def fractions_from_scene(scene, metal, mirror=(False, False, False),
                         iters=45):
    """theta (6,nx,ny,nz) float32 (solver3d.py:75-127): for every vacuum
    node whose d-neighbour is metal, the fraction of the leg to the exact
    surface by `iters` bisections on inside_scene_pts, clamped to
    [1e-3, 1]; a probe across a low mirror plane is reflected."""
    metal = np.asarray(metal, bool)
    th = np.ones((6,) + metal.shape, np.float32)
    for d in range(6):
        nb, ax, step = _metal_neighbour(metal, d, mirror)
        legs = np.argwhere(~metal & nb)
        if len(legs) == 0:
            continue
        origin = legs.astype(np.float64)
        dvec = np.array(_DIRS[d], float)
        lo = np.zeros(len(origin))
        hi = np.ones(len(origin))
        for _ in range(iters):
            mid = 0.5 * (lo + hi)
            probe = origin + mid[:, None] * dvec
            if mirror[ax] and step < 0:
                probe[:, ax] = np.abs(probe[:, ax])
            hit = inside_scene_pts(scene, probe)
            hi = np.where(hit, mid, hi)
            lo = np.where(hit, lo, mid)
        th[d][legs[:, 0], legs[:, 1], legs[:, 2]] = np.clip(
            0.5 * (lo + hi), 1e-3, 1.0).astype(np.float32)
    return th


def fractions_from_pa_surf(path, shape, metal):
    """theta decoded from a surface-fraction sidecar (solver3d.py:323-363):
    chunks tagged XOFF/YOFF/ZOFF of (u64 flat index with x fastest, f64
    fraction along +axis) records; a record at a vacuum node sets its +leg,
    at a metal node the -leg of the vacuum node above it (1 - fraction);
    clamped below at 1e-3."""
    import re
    nx, ny, nz = shape
    metal = np.asarray(metal, bool)
    th = np.ones((6, nx, ny, nz), np.float32)
    raw = open(path, "rb").read()
    tags = [(m.start(), m.group().decode())
            for m in re.finditer(rb"XOFF|YOFF|ZOFF", raw)]
    axis_of = {"XOFF": 0, "YOFF": 1, "ZOFF": 2}
    for n, (pos, tag) in enumerate(tags):
        end = tags[n + 1][0] if n + 1 < len(tags) else len(raw)
        body = raw[pos + 4:pos + 4 + ((end - pos - 4) // 16) * 16]
        rec = np.frombuffer(body, dtype=[("idx", "<u8"), ("f", "<f8")])
        rec = rec[rec["idx"] < nx * ny * nz]
        ax = axis_of[tag]
        i = (rec["idx"] % nx).astype(int)
        j = ((rec["idx"] // nx) % ny).astype(int)
        k = (rec["idx"] // (nx * ny)).astype(int)
        for ii, jj, kk, f in zip(i, j, k, rec["f"]):
            if not metal[ii, jj, kk]:
                th[2 * ax + 1, ii, jj, kk] = max(f, 1e-3)
            else:
                up = [ii, jj, kk]
                up[ax] += 1
                if up[ax] < shape[ax] and not metal[up[0], up[1], up[2]]:
                    th[2 * ax, up[0], up[1], up[2]] = max(1.0 - f, 1e-3)
    return th


def fractions_from_mesh(meshes, metal, mirror=(False, False, False),
                        slack=0.05):
    """theta from watertight electrode meshes in grid units
    (solver3d.py:447-514): a ray along each metal-facing leg, the first hit
    within 1 + slack of the node sets the leg, clamped to [1e-3, 1].  Needs
    trimesh, as the reference does."""
    import trimesh  # the reference's dependency for this builder
    mesh = trimesh.util.concatenate(list(meshes.values()))
    ray = mesh.ray
    metal = np.asarray(metal, bool)
    th = np.ones((6,) + metal.shape, np.float32)
    for d in range(6):
        nb, ax, _ = _metal_neighbour(metal, d, mirror)
        legs = np.argwhere(~metal & nb)
        if len(legs) == 0:
            continue
        origin = legs.astype(np.float64)
        dirs = np.tile(np.array(_DIRS[d], float), (len(legs), 1))
        loc, iray, _ = ray.intersects_location(origin, dirs,
                                               multiple_hits=False)
        if len(iray) == 0:
            continue
        t = np.abs(loc[:, ax] - origin[iray, ax])
        ok = t <= 1.0 + slack
        hit = legs[iray[ok]]
        th[d][hit[:, 0], hit[:, 1], hit[:, 2]] = np.clip(
            t[ok], 1e-3, 1.0).astype(np.float32)
    return th
