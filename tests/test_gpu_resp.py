"""GPU parity of the cross-object bounces (FACET_RESP, option cross_objects).

Scene: two plates facing each other across 0.45 m and a box between them
(three target objects, none of which sees itself), lit from the side.  With
cross_objects every bounce carries the FACET_RESP terms between every pair
of objects (src/OptiX.cu:192-406 with useReciprocity and not isSelf); the
oracle restates the same sequence in FP64.

Tolerances: relative L2 1e-5 per object against FP64 (the single-object
bounce tolerance on small scenes); masks equal to the oracle's on every pair
the oracle does not classify as grazing.
"""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import load_scene, oracle_scene

pytestmark = pytest.mark.gpu


def three_objects(scenes, f=12e3):
    A = scenes.rectangle(0.6, 0.4, z=0.0)
    B = scenes.translate(scenes.rectangle(0.6, 0.4, z=0.0, normal_up=False), (0.15, 0.05, 0.45))
    C = scenes.box(0.12, 0.10, 0.12, center=(0.05, 0.0, 0.2))
    d = scenes.delta_for(f)
    return dict(cp=1480.0, f=f, att=0.0, bounces=2, field_objects=False,
                sources=np.array([[2.0, 0.3, 0.25]], np.float32),
                field_points=scenes.hemisphere(3, 3, 2.0), targets=[(A, d), (B, d), (C, d)], fields=[])


def run_bounces(api, sc, cross):
    api.set_option("cross_objects", 1 if cross else 0)
    load_scene(api, sc)
    api.project_source_points_to_objects(False)
    P0 = [api.get_object_pressures(api.TARGET, i) for i in range(3)]
    api.set_option("reset_stats", 1)
    api.project_target_to_target_objects(sc["bounces"])
    P = [api.get_object_pressures(api.TARGET, i) for i in range(3)]
    st = api.stats()
    api.set_option("cross_objects", 0)
    api.TearDownCuda()
    return P0, P, st


def test_cross_object_bounces_match_oracle(api, oracle_mod, scenes):
    sc = three_objects(scenes)
    P0, P, st = run_bounces(api, sc, True)
    o = oracle_scene(oracle_mod, sc)
    o.project_sources(False)
    o.project_bounces(2, cross_objects=True)
    resp = [h for h in st["hops"] if h["hop"] == 4]
    print("FACET_RESP hop records: %d, pairs per bounce %d" % (len(resp), sum(h["pairs"] for h in resp) // 2))
    assert len(resp) == 2 * 6  # 2 bounces x 3 object pairs x 2 directions
    for i in range(3):
        ref = o.pressures(0, i)
        e_all = rel_l2(P[i], ref)
        e_bounce = rel_l2(P[i] - P0[i], ref - o_incident(oracle_mod, sc, i))
        print("object %d: total rel L2 %.3e, bounce part %.3e" % (i, e_all, e_bounce))
        assert np.linalg.norm(ref) > 0
        assert e_all < 1e-5
        assert e_bounce < 1e-5
    o.close()


_incident = {}


def o_incident(oracle_mod, sc, i):
    """The oracle's source-hop pressures of object i (cached per scene)."""
    key = id(sc)
    if key not in _incident:
        o = oracle_scene(oracle_mod, sc)
        o.project_sources(False)
        _incident[key] = [o.pressures(0, k) for k in range(3)]
        o.close()
    return _incident[key][i]


def test_cross_objects_off_is_the_reference_sequence(api, oracle_mod, scenes):
    """Without the option the objects never interact (the reference): flat
    plates do not see themselves, so their bounces add nothing; the box sees
    itself a little (the reference's patch-corner reference points of cells
    cut by a triangle edge lie outside the face)."""
    sc = three_objects(scenes)
    P0, P, _ = run_bounces(api, sc, False)
    o = oracle_scene(oracle_mod, sc)
    o.project_sources(False)
    o.project_bounces(2)
    for i in range(3):
        if i < 2:
            assert np.array_equal(P[i], P0[i])
        assert rel_l2(P[i], o.pressures(0, i)) < 1e-5
    o.close()


def test_resp_masks_match_oracle(api, oracle_mod, scenes):
    sc = three_objects(scenes)
    load_scene(api, sc)
    o = oracle_scene(oracle_mod, sc)
    checked = 0
    for a in range(3):
        for b in range(3):
            if a == b:
                continue
            ns, nd = o.nact(0, a), o.nact(0, b)
            gm = api.get_mask(4, a, b).reshape(nd, ns)
            _, om = o.hop_subset(4, a, b, np.arange(nd), want_mask=True, nsrc=ns)
            graze = (om & 2) != 0
            diff = (gm != (om & 1)) & ~graze
            print("FACET_RESP %d -> %d: pairs %d interacting %d grazing %d mismatches %d"
                  % (a, b, gm.size, int(gm.sum()), int(graze.sum()), int(diff.sum())))
            assert diff.sum() == 0
            checked += int(gm.sum())
    api.TearDownCuda()
    o.close()
    assert checked > 0
    with pytest.raises(api.SonarError):
        load_scene(api, sc)
        try:
            api.get_mask(4, 1, 1)
        finally:
            api.TearDownCuda()
