"""Piston source objects (objectType 1).

The reference stores objects of type 1 (src/Model.cpp:33-35) but never
radiates from them.  Here ProjectSrcPointsToObjects lets every fragment of a
source object radiate a unit surface pressure through the facet -> facet
projection of src/OptiX.cu:192-406 (area, cos_scat at the piston, cos_inc at
a target destination or 1 at a field object, the r < delta regularisation and
0.9 factor, shadowed by the targets, destinations gated by their area) into
the targets and, with projectFieldObjects, the field objects.  GPU vs the FP64
oracle's restatement at 1e-5 relative L2, and the piston hop's interaction
mask bit for bit outside grazing pairs.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _scene(scenes, occluder):
    f = 8e3
    target = scenes.plate_1x05()                                  # z = 0, normal +z
    piston = scenes.translate(scenes.rectangle(0.24, 0.16, z=0.0, normal_up=False), (0.1, 0.05, 1.2))
    field = scenes.rotate(scenes.rectangle(1.6, 1.6, z=0.0), "x", 90.0)  # a vertical plane through the origin
    field = scenes.translate(field, (0.0, 0.9, 0.6))
    targets = [target]
    if occluder:
        targets.append(scenes.box(0.3, 0.3, 0.05, center=(0.25, 0.0, 0.6)))
    fp = np.concatenate([scenes.grid_xy(8, 0.8, 2.5), scenes.arc_xz(3.0, np.linspace(-40, 40, 16))])
    src = np.array([[0.0, 0.0, 4.0]], np.float32)
    return f, targets, piston, field, fp, src


def _run(api, scenes, occluder):
    f, targets, piston, field, fp, src = _scene(scenes, occluder)
    d = scenes.delta_for(f)
    api.TearDownCuda()
    api.set_initial_conditions(1480.0, f, 0.0)
    for t in targets:
        api.load_stl_mesh_to_cuda(t, api.TARGET, d)
    api.load_stl_mesh_to_cuda(piston, api.SOURCE, d)
    api.load_stl_mesh_to_cuda(field, api.FIELD, 1.6 / 64)
    api.load_points_to_cuda(src, isSource=True)
    api.load_points_to_cuda(fp, isSource=False)
    api.render_cuda()
    api.project_source_points_to_objects(True)
    P = [api.get_object_pressures(api.TARGET, i) for i in range(len(targets))]
    F = api.get_object_pressures(api.FIELD, 0)
    api.project_target_to_field_points()
    Q = api.get_field_point_pressures(len(fp))
    return (f, targets, piston, field, fp, src, d), P, F, Q


def _oracle(oracle_mod, sc):
    f, targets, piston, field, fp, src, d = sc
    o = oracle_mod.Oracle()
    o.set_initial_conditions(1480.0, f, 0.0)
    for t in targets:
        o.load_geometry(t, 0, d)
    o.load_geometry(piston, 1, d)
    o.load_geometry(field, 2, 1.6 / 64)
    o.load_source_points(src)
    o.load_field_points(fp)
    o.render()
    return o


@pytest.mark.parametrize("occluder", [False, True])
def test_piston_source_object(api, oracle_mod, scenes, occluder):
    sc, P, F, Q = _run(api, scenes, occluder)
    o = _oracle(oracle_mod, sc)
    o.project_sources(True)
    Po = [o.pressures(0, i) for i in range(len(P))]
    Fo = o.pressures(2, 0)
    o.project_field_points()
    Qo = o.field_points()
    errs = [rel_l2(a, b) for a, b in zip(P, Po)] + [rel_l2(F, Fo), rel_l2(Q, Qo)]
    print("piston (occluder %s): targets %s, field object %.2e, field points %.2e"
          % (occluder, " ".join("%.2e" % e for e in errs[:-2]), errs[-2], errs[-1]))
    assert max(errs) < 1e-5
    assert np.abs(F).max() > 0
    # the piston hop's masks against the oracle's, outside grazing pairs
    checked = 0
    for hop, dst_type, b in [(5, 0, i) for i in range(len(P))] + [(6, 2, 0)]:
        n_dst, n_src = o.nact(dst_type, b), o.nact(1, 0)
        gm = api.get_mask(hop, 0, b).reshape(n_dst, n_src)
        _, om = o.hop_subset(hop, 0, b, np.arange(n_dst), want_mask=True, nsrc=n_src)
        graze = (om & 2) != 0
        diff = (gm != (om & 1)) & ~graze
        print("hop %d -> object %d: pairs %d interacting %d grazing %d mismatches %d"
              % (hop, b, gm.size, int(gm.sum()), int(graze.sum()), int(diff.sum())))
        assert diff.sum() == 0
        checked += int(gm.sum())
    o.close()
    api.TearDownCuda()
    assert checked > 0


def test_piston_alone_without_point_sources(api, oracle_mod, scenes):
    """No source points: the pistons alone excite the target."""
    f, targets, piston, field, fp, src, = _scene(scenes, False)
    d = scenes.delta_for(f)
    api.TearDownCuda()
    api.set_initial_conditions(1480.0, f, 0.0)
    api.load_stl_mesh_to_cuda(targets[0], api.TARGET, d)
    api.load_stl_mesh_to_cuda(piston, api.SOURCE, d)
    api.render_cuda()
    api.project_source_points_to_objects(False)
    P = api.get_object_pressures(api.TARGET, 0)
    api.TearDownCuda()
    o = oracle_mod.Oracle()
    o.set_initial_conditions(1480.0, f, 0.0)
    o.load_geometry(targets[0], 0, d)
    o.load_geometry(piston, 1, d)
    o.render()
    o.project_sources(False)
    Po = o.pressures(0, 0)
    o.close()
    e = rel_l2(P, Po)
    print("piston alone: %.2e" % e)
    assert np.abs(Po).max() > 0 and e < 1e-5
