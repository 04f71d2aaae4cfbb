"""The analytic-solid scene model the theta builder reads (the data part of
ion_gym physics/scene3d.py: GridSpec, Cylinder, Box3D, Shape, Electrode,
GeomScene with its grid-unit view).  fractions_from_scene accepts these or the
reference's own scene objects: it reads only the field names below.

Conventions: a Cylinder runs along z and spans [z - length, z] (z is its
HIGH face); a Shape is the union of its `within` primitives minus the union
of its `notin` primitives; coordinates are in grid units ("gu") or
millimetres ("mm", scaled by 1/mm_per_gu for the grid view).
"""
from dataclasses import dataclass, field, replace
from typing import List, Union


@dataclass
class GridSpec:
    nx: int
    ny: int
    nz: int
    mm_per_gu: float = 1.0
    symmetry: str = "planar"
    mirror: str = ""
    surface: str = "fractional"
    overhang: str = "refuse"


@dataclass
class Cylinder:
    cx: float
    cy: float
    z: float
    r: float
    length: float
    kind: str = "cylinder"


@dataclass
class Box3D:
    x1: float
    y1: float
    z1: float
    x2: float
    y2: float
    z2: float
    kind: str = "box3d"

    def __post_init__(self):
        if self.x2 < self.x1 or self.y2 < self.y1 or self.z2 < self.z1:
            raise ValueError("Box3D requires x1<=x2, y1<=y2, z1<=z2")


Primitive = Union[Cylinder, Box3D]


@dataclass
class Shape:
    within: List[Primitive] = field(default_factory=list)
    notin: List[Primitive] = field(default_factory=list)


@dataclass
class Electrode:
    index: int
    name: str
    shapes: List[Shape] = field(default_factory=list)
    voltage: Union[float, str] = 0.0

    def __post_init__(self):
        if self.index < 1:
            raise ValueError("electrode index must be >= 1 (0 is vacuum)")


def _scale_prim(p, s):
    if isinstance(p, Cylinder):
        return replace(p, cx=p.cx * s, cy=p.cy * s, z=p.z * s, r=p.r * s,
                       length=p.length * s)
    return replace(p, x1=p.x1 * s, y1=p.y1 * s, z1=p.z1 * s, x2=p.x2 * s,
                   y2=p.y2 * s, z2=p.z2 * s)


@dataclass
class GeomScene:
    grid: GridSpec
    electrodes: List[Electrode] = field(default_factory=list)
    units: str = "gu"
    name: str = "scene"
    notes: str = ""

    def in_gu(self):
        """The scene with every coordinate in grid units."""
        if self.units == "gu":
            return self
        s = 1.0 / self.grid.mm_per_gu
        els = [replace(e, shapes=[Shape(within=[_scale_prim(p, s)
                                                for p in sh.within],
                                        notin=[_scale_prim(p, s)
                                               for p in sh.notin])
                                  for sh in e.shapes])
               for e in self.electrodes]
        return replace(self, electrodes=els, units="gu")
