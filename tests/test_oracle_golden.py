"""The oracle against the golden fixtures written by the reference's own code
(tests/golden/make_golden.py): fragmentation bit for bit, pressures to FP64
round-off."""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES, golden_scene, load_golden, rel_l2


def test_fragmentation_bit_exact(oracle_mod):
    g = load_golden("fragmentation")
    for k, (t, d) in enumerate(zip(g["tris"], g["deltas"])):
        (nx, ny, neg), fr, a = oracle_mod.fragment_triangle(t, float(d))
        assert (nx, ny, neg) == tuple(int(v) for v in g["ints"][k])
        assert np.array_equal(fr.view(np.uint32), g["frames"][k].view(np.uint32)), k
        ref = g["areas"][g["offsets"][k]:g["offsets"][k + 1]]
        assert np.array_equal(a.ravel().view(np.uint32), ref.view(np.uint32)), k


def run_oracle_scene(oracle_mod, sc):
    o = oracle_mod.Oracle()
    o.set_initial_conditions(sc["cp"], sc["f"], sc["att"])
    for t, d in sc["targets"]:
        o.load_geometry(t, 0, d)
    for t, d in sc["fields"]:
        o.load_geometry(t, 2, d)
    o.load_source_points(sc["sources"])
    o.load_field_points(sc["field_points"])
    o.render()
    o.project_sources(False)
    if sc["bounces"]:
        o.project_bounces(sc["bounces"])
    if sc["field_objects"]:
        o.project_field_objects()
    o.project_field_points()
    return o


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_scene_pressures(oracle_mod, name):
    g = load_golden(name)
    sc = golden_scene(g)
    o = run_oracle_scene(oracle_mod, sc)
    for i in range(len(sc["targets"])):
        ref = g["P_target%d" % i]
        assert np.abs(ref).max() > 0
        assert rel_l2(o.pressures(0, i), ref) < 1e-12
    for i in range(len(sc["fields"])):
        assert rel_l2(o.pressures(2, i), g["P_field%d" % i]) < 1e-12
    ref = g["P_points"]
    assert np.abs(ref).max() > 0
    assert rel_l2(o.field_points(), ref) < 1e-12


def test_occluder_casts_a_shadow():
    """The occluded-plates fixture really has shadowed cells: cells of the big
    plate right under the small plate receive nothing from the source."""
    g = load_golden("occluded_plates")
    P = g["P_target0"]
    assert (np.abs(P) == 0).sum() > 20 and (np.abs(P) > 0).sum() > 1000
