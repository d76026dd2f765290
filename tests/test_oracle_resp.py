"""Cross-object bounces (FACET_RESP) in the FP64 oracle, on the CPU.

FACET_RESP is the reference's target -> other-target projection with
reciprocity (src/OptiX.cu:192-406 with useReciprocity and not isSelf,
:427-429); the reference's host never calls it.  The oracle restates it
destination-owned: forward terms into the second object, reciprocal terms
into the first.  Its known answers:
  * reciprocity: with u = area_A * P_in,A and w = area_B * P_in,B, the forward
    field F_B = T u and the reciprocal field R_A = T^T w satisfy
    w . F_B == u . R_A (one operator T, applied both ways);
  * the zero-input skip: a cell of the first object with P_in = 0 receives no
    reciprocal term;
  * the cross-object bounce sequence reduces to the reference's self-only
    sequence on a single target.
"""
import numpy as np


def two_plates(scenes):
    """Plate A at z = 0 (normal +z) and plate B at z = 0.3 facing down, shifted
    so that they see each other at an angle; one source between them at the
    side, lighting both."""
    A = scenes.rectangle(0.30, 0.20, z=0.0)
    B = scenes.translate(scenes.rectangle(0.30, 0.20, z=0.0, normal_up=False), (0.1, 0.05, 0.3))
    return A, B


def load(oracle_mod, tris, f=6e3, src=(1.5, 0.0, 0.15)):
    o = oracle_mod.Oracle()
    o.set_initial_conditions(1480.0, f, 0.0)
    d = float(np.float32(1480.0) / np.float32(f) / np.float32(7.5))
    for t in tris:
        o.load_geometry(t, 0, d)
    o.load_source_points(np.array([src], np.float32))
    o.load_field_points(np.zeros((1, 3), np.float32))
    o.render()
    return o


def test_resp_reciprocity_and_zero_input(oracle_mod, scenes):
    A, B = two_plates(scenes)
    o = load(oracle_mod, [A, B])
    rng = np.random.default_rng(11)
    nA, nB = o.ncells(0, 0), o.ncells(0, 1)
    actA, actB = o.active(0, 0), o.active(0, 1)
    pA = rng.standard_normal(nA) + 1j * rng.standard_normal(nA)
    pB = rng.standard_normal(nB) + 1j * rng.standard_normal(nB)
    o.set_pressures(0, 0, pA, which=1)
    o.set_pressures(0, 1, pB, which=1)
    F_B, mf = o.hop_subset(4, 0, 1, np.arange(len(actB)), want_mask=True, nsrc=len(actA))
    R_A, mr = o.hop_subset(4, 1, 0, np.arange(len(actA)), want_mask=True, nsrc=len(actB))
    u = o.areas(0, 0)[actA] * pA[actA]
    w = o.areas(0, 1)[actB] * pB[actB]
    lhs, rhs = np.dot(w, F_B), np.dot(u, R_A)
    print("plates: %d x %d active cells, interacting pairs %d; w.F_B %s, u.R_A %s"
          % (len(actA), len(actB), int((mf & 1).sum()), lhs, rhs))
    assert (mf & 1).sum() > 0
    # the same pairs interact in both directions (one ray per pair)
    assert np.array_equal(mf & 1, (mr & 1).T)
    # the weights (area cos_scat) cos_inc are FP32 products, as in the reference
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)
    # zero input on half of A: those cells get no reciprocal term; the others keep theirs
    pA0 = pA.copy()
    pA0[actA[::2]] = 0.0
    o.set_pressures(0, 0, pA0, which=1)
    R0, _ = o.hop_subset(4, 1, 0, np.arange(len(actA)))
    assert np.all(R0[::2] == 0.0)
    assert np.array_equal(R0[1::2], R_A[1::2])
    o.close()


def test_cross_sequence_reduces_to_self_on_one_target(oracle_mod, scenes):
    tri = scenes.trihedral(0.4)
    o1 = load(oracle_mod, [tri], src=(3.0, 2.5, 2.0))
    o2 = load(oracle_mod, [tri], src=(3.0, 2.5, 2.0))
    for o in (o1, o2):
        o.project_sources(False)
    o1.project_bounces(2)
    o2.project_bounces(2, cross_objects=True)
    a, b = o1.pressures(0, 0), o2.pressures(0, 0)
    assert np.abs(a).max() > 0
    assert np.array_equal(a, b)
    o1.close()
    o2.close()


def test_cross_terms_change_two_object_bounces(oracle_mod, scenes):
    A, B = two_plates(scenes)
    o1 = load(oracle_mod, [A, B])
    o2 = load(oracle_mod, [A, B])
    for o in (o1, o2):
        o.project_sources(False)
    P0 = o1.pressures(0, 1)
    o1.project_bounces(1)
    o2.project_bounces(1, cross_objects=True)
    # flat plates do not see themselves: without cross terms nothing changes
    assert np.array_equal(o1.pressures(0, 1), P0)
    d = o2.pressures(0, 1) - P0
    print("plate B after one cross bounce: |dP| max %.3e" % np.abs(d).max())
    assert np.abs(d).max() > 1e-3 * np.abs(P0).max()
    o1.close()
    o2.close()
