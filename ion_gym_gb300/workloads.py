"""Seeded synthetic geometries of the benchmark workloads (masks and
Dirichlet values on regular grids, 1-cell spacing).

  sphere_box       65^3 grounded box, sphere of radius 10 at 1 V
  quadrupole       257^3 grounded box, four z-rods of radius 1.148 r0
  ring_stack       193x193x385 coaxial ring electrodes (einzel/funnel-like)
  random_deck      a cubic grid with random spheres, cylinders and plates
  planar_board     extruded polygon electrodes on two layers
"""
import numpy as np


def _box_faces(fixed):
    fixed[0] = fixed[-1] = True
    fixed[:, 0] = fixed[:, -1] = True
    fixed[:, :, 0] = fixed[:, :, -1] = True


def sphere_box(n=65, radius=10.0, v=1.0):
    """Grounded n^3 box with a sphere of `radius` cells about the centre
    node held at v."""
    c = (n - 1) / 2.0
    i, j, k = np.ogrid[:n, :n, :n]
    s = (i - c) ** 2 + (j - c) ** 2 + (k - c) ** 2 <= radius * radius
    fixed = np.zeros((n, n, n), bool)
    _box_faces(fixed)
    fixed |= s
    return fixed, np.where(s, v, 0.0)


def quadrupole(n=257, r0=32.0, v=1.0):
    """Grounded n^3 box with four rods along z of radius 1.148 r0 whose axes
    lie r0 + radius from the box axis (so each rod's face is r0 from the
    axis): rods on +-x at +v, on +-y at -v."""
    c = (n - 1) / 2.0
    rad = 1.148 * r0
    off = r0 + rad
    ii, jj = np.meshgrid(np.arange(n, dtype=float), np.arange(n, dtype=float),
                         indexing="ij")
    fixed2 = np.zeros((n, n), bool)
    val2 = np.zeros((n, n))
    for dx, dy, s in ((off, 0, v), (-off, 0, v), (0, off, -v), (0, -off, -v)):
        rod = (ii - c - dx) ** 2 + (jj - c - dy) ** 2 <= rad * rad
        fixed2 |= rod
        val2[rod] = s
    fixed = np.repeat(fixed2[:, :, None], n, axis=2)
    val = np.repeat(val2[:, :, None], n, axis=2)
    _box_faces(fixed)
    val[0] = val[-1] = 0.0
    val[:, 0] = val[:, -1] = 0.0
    val[:, :, 0] = val[:, :, -1] = 0.0
    return fixed, val


def ring_stack(seed=0, shape=(193, 193, 385), n_rings=8, thickness=4,
               r_lo=20.0, r_hi=60.0, gap_lo=8, gap_hi=24):
    """Coaxial ring electrodes along z in a grounded box: inner radius
    U(r_lo, r_hi), radial and axial thickness `thickness` cells, axial gaps
    U(gap_lo, gap_hi); the stack is centred in z.  Returns
    (masks {1..n: bool}, box mask) -- the box faces are grounded metal that
    belongs to no basis."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    cx, cy = (nx - 1) / 2.0, (ny - 1) / 2.0
    radii = rng.uniform(r_lo, r_hi, n_rings)
    gaps = rng.integers(gap_lo, gap_hi + 1, n_rings - 1)
    length = n_rings * thickness + int(gaps.sum())
    z0 = max(1, (nz - length) // 2)
    ii, jj = np.meshgrid(np.arange(nx, dtype=float), np.arange(ny, dtype=float),
                         indexing="ij")
    rr = np.hypot(ii - cx, jj - cy)
    masks = {}
    z = z0
    for e in range(n_rings):
        ring2 = (rr >= radii[e]) & (rr < radii[e] + thickness)
        m = np.zeros(shape, bool)
        m[:, :, z:z + thickness] = ring2[:, :, None]
        masks[e + 1] = m
        if e < n_rings - 1:
            z += thickness + int(gaps[e])
    box = np.zeros(shape, bool)
    _box_faces(box)
    return masks, box


def random_deck(seed, side, n_electrodes, v_range=(-100.0, 100.0)):
    """A cubic grid with n_electrodes random spheres, z-cylinders and plates
    inside a grounded box, voltages U(v_range).  Returns (fixed, val)."""
    rng = np.random.default_rng(seed)
    n = side
    fixed = np.zeros((n, n, n), bool)
    val = np.zeros((n, n, n))
    i, j, k = np.ogrid[:n, :n, :n]
    for _ in range(n_electrodes):
        kind = rng.integers(0, 3)
        v = rng.uniform(*v_range)
        c = rng.uniform(0.2 * n, 0.8 * n, 3)
        if kind == 0:
            r = rng.uniform(0.03, 0.12) * n
            m = (i - c[0]) ** 2 + (j - c[1]) ** 2 + (k - c[2]) ** 2 <= r * r
        elif kind == 1:
            r = rng.uniform(0.02, 0.08) * n
            h = rng.uniform(0.1, 0.5) * n
            m = (((i - c[0]) ** 2 + (j - c[1]) ** 2 <= r * r)
                 & (np.abs(k - c[2]) <= h / 2))
        else:
            w = rng.uniform(0.1, 0.4, 2) * n
            t = max(1.0, rng.uniform(0.01, 0.03) * n)
            m = ((np.abs(i - c[0]) <= w[0] / 2) & (np.abs(j - c[1]) <= w[1] / 2)
                 & (np.abs(k - c[2]) <= t / 2))
        m = np.broadcast_to(m, (n, n, n))
        fixed |= m
        val[m] = v
    _box_faces(fixed)
    val[0] = val[-1] = 0.0
    val[:, 0] = val[:, -1] = 0.0
    val[:, :, 0] = val[:, :, -1] = 0.0
    return fixed, val


def planar_board(seed, shape=(512, 128, 96), n_electrodes=16, layers=2,
                 extrude=4):
    """Extruded polygon electrodes on `layers` board layers: each electrode
    a random convex polygon in x-y, `extrude` cells thick in z, on one of
    the layers.  Returns (masks {1..n}, box mask)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    ii, jj = np.meshgrid(np.arange(nx, dtype=float), np.arange(ny, dtype=float),
                         indexing="ij")
    zs = [int(nz * (L + 1) / (layers + 1)) - extrude // 2
          for L in range(layers)]
    masks = {}
    for e in range(n_electrodes):
        cx = rng.uniform(0.05, 0.95) * nx
        cy = rng.uniform(0.1, 0.9) * ny
        rad = rng.uniform(0.02, 0.08) * min(nx, ny) + 2
        nv = int(rng.integers(3, 8))
        ang = np.sort(rng.uniform(0, 2 * np.pi, nv))
        px = cx + rad * np.cos(ang)
        py = cy + rad * np.sin(ang)
        inside = np.ones((nx, ny), bool)
        for a in range(nv):
            b = (a + 1) % nv
            cross = (px[b] - px[a]) * (jj - py[a]) - (py[b] - py[a]) * (ii - px[a])
            inside &= cross >= 0
        m = np.zeros(shape, bool)
        z = zs[e % layers]
        m[:, :, z:z + extrude] = inside[:, :, None]
        masks[e + 1] = m
    box = np.zeros(shape, bool)
    _box_faces(box)
    return masks, box


class DriveGroup:
    """One declared drive group (the attributes the composer reads)."""

    def __init__(self, name, amplitude_v=0.0, offset_v=0.0, waveform="sin",
                 frequency_hz=1.0e6, phase_deg=0.0, duty=0.5, interp="hold",
                 table_t_us=(), table_v=()):
        self.name, self.amplitude_v, self.offset_v = name, amplitude_v, offset_v
        self.waveform, self.frequency_hz, self.phase_deg = (waveform,
                                                            frequency_hz,
                                                            phase_deg)
        self.duty, self.interp = duty, interp
        self.table_t_us, self.table_v = list(table_t_us), list(table_v)


class DriveElectrode:
    def __init__(self, name, groups=(), dc=0.0):
        self.name, self._groups, self.dc = name, list(groups), dc

    def group_names(self):
        return list(self._groups)


class DriveGeometry:
    def __init__(self, rf_groups, electrodes, mm_per_gu, field_method=
                 "electrode_aware", channel_dtype="float64"):
        self.rf_groups, self.electrodes = rf_groups, electrodes
        self.mm_per_gu, self.field_method = mm_per_gu, field_method
        self.channel_dtype = channel_dtype


class DriveSpec:
    """The spec surface compose_drive_channels reads: .geometry and
    dc_effective(electrode)."""

    def __init__(self, geometry):
        self.geometry = geometry

    def dc_effective(self, el):
        return el.dc


def ring_stack_drive(n_rings=8, mm_per_gu=0.1, seed=0):
    """Drive of a ring stack: alternate rings on two RF groups 180 degrees
    apart (1.1 MHz, 150 V), a DC ladder on every ring and a table-waveform
    gate on ring 1 -- three drive channels plus the static field."""
    rng = np.random.default_rng(seed)
    groups = [DriveGroup("rf_a", amplitude_v=150.0, frequency_hz=1.1e6),
              DriveGroup("rf_b", amplitude_v=150.0, frequency_hz=1.1e6,
                         phase_deg=180.0),
              DriveGroup("gate", amplitude_v=40.0, waveform="table",
                         table_t_us=(0.0, 2.0, 2.5, 10.0),
                         table_v=(0.0, 0.0, 1.0, 1.0))]
    els = []
    for e in range(n_rings):
        gr = ["rf_a" if e % 2 == 0 else "rf_b"] + (["gate"] if e == 0 else [])
        els.append(DriveElectrode(f"ring{e + 1}", gr,
                                  float(np.round(rng.uniform(-20, 20), 3))))
    return DriveSpec(DriveGeometry(groups, els, mm_per_gu))
