"""Analytic scenes on the GPU against the reference: the labelled raster
(rasterize3d.rasterize) and the fractional-surface legs
(solver3d.fractions_from_scene), bit for bit, and the raster's refusals."""
import numpy as np
import pytest

from conftest import Golden

pytestmark = pytest.mark.gpu


def _raster_scenes():
    from ion_gym_gb300.physics.scene3d import (GeomScene, GridSpec, Electrode,
                                               Shape, Cylinder, Box3D)
    g = GridSpec(31, 29, 27, mm_per_gu=0.5, overhang="allow")
    return [
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


def test_rasterize_matches_reference():
    from ion_gym_gb300.physics.rasterize3d import rasterize
    g = Golden("raster.npz")
    for sc, case in zip(_raster_scenes(), g.cases("raster")):
        lab = rasterize(sc)
        assert lab.dtype == np.int16 and np.array_equal(lab, case["lab"])


def test_rasterize_refusals():
    from ion_gym_gb300.physics.rasterize3d import rasterize
    from ion_gym_gb300.physics.scene3d import (GeomScene, GridSpec, Electrode,
                                               Shape, Cylinder, Box3D)
    g = Golden("raster.npz")
    ref = {k.split("/")[1]: str(g.z[k]) for k in g.z.files
           if k.startswith("raster_err")}
    clash = GeomScene(grid=GridSpec(20, 20, 5), units="gu", electrodes=[
        Electrode(1, "a", [Shape([Box3D(2.0, 2.0, 0.0, 10.0, 10.0, 4.0)])]),
        Electrode(2, "b", [Shape([Box3D(8.0, 8.0, 0.0, 15.0, 15.0, 4.0)])])])
    with pytest.raises(ValueError) as e:
        rasterize(clash)
    head = ref["clash"].split(". ")[0]
    assert str(e.value).startswith(head)          # same node, count, owner
    empty = GeomScene(grid=GridSpec(20, 20, 5), units="gu", electrodes=[
        Electrode(1, "a", [Shape([Box3D(2.0, 2.0, 0.0, 10.0, 10.0, 4.0)])]),
        Electrode(2, "tiny", [Shape([Cylinder(15.5, 15.5, 2.5, 0.2, 0.3)])])])
    with pytest.raises(ValueError, match="rasterises EMPTY"):
        rasterize(empty)
    assert "rasterises EMPTY" in ref["empty"]


def test_theta_on_device_matches_reference():
    from ion_gym_gb300.physics.rasterize3d import fractions_from_scene_device
    from ion_gym_gb300.physics.scene3d import (GeomScene, GridSpec, Electrode,
                                               Shape, Cylinder, Box3D)
    n, nz, c = 23, 5, 11.0
    scenes = [
        GeomScene(grid=GridSpec(n, n, nz), units="gu", electrodes=[
            Electrode(1, "inner", [Shape([Cylinder(c, c, nz + 2.0, 4.3,
                                                   nz + 4.0)])]),
            Electrode(2, "outer", [Shape(
                within=[Cylinder(c, c, nz + 2.0, 40.0, nz + 4.0)],
                notin=[Cylinder(c, c, nz + 2.0, 9.6, nz + 4.0)])])]),
        GeomScene(grid=GridSpec(17, 15, 13, mm_per_gu=0.5), units="mm",
                  electrodes=[Electrode(1, "plate", [Shape(
                      within=[Box3D(1.3, 0.65, 2.6, 6.6, 6.35, 3.7)],
                      notin=[Cylinder(4.0, 3.5, 4.0, 1.55, 3.0)])])]),
        GeomScene(grid=GridSpec(15, 15, 3), units="gu", electrodes=[
            Electrode(1, "rod", [Shape([Cylinder(0.0, 0.0, 9.0, 3.7, 20.0)])]),
            Electrode(2, "can", [Shape(
                within=[Cylinder(0.0, 0.0, 9.0, 40.0, 20.0)],
                notin=[Cylinder(0.0, 0.0, 9.0, 12.2, 20.0)])])]),
    ]
    g = Golden("theta.npz")
    for sc, case in zip(scenes, g.cases("theta")):
        th = fractions_from_scene_device(
            sc, case["metal"].astype(bool),
            mirror=tuple(bool(x) for x in case["mirror"]))
        assert np.array_equal(th, case["th"])


def test_raster_feeds_the_solver():
    """The device raster's masks drive a basis solve end to end."""
    from ion_gym_gb300.physics.rasterize3d import rasterize, masks_from_labels
    from ion_gym_gb300.physics import multigrid3d as M
    lab = rasterize(_raster_scenes()[0])
    masks = masks_from_labels(lab)
    assert sorted(masks) == [1, 2, 3]
    out = M.solve_bases_mg(masks, tol=1e-3)
    assert np.all(out[1][masks[1]] == 1e4) and np.all(out[2][masks[1]] == 0)
