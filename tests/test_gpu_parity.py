"""GPU parity: the CUDA path through the C ABI against the CPU oracle and the
golden fixtures from the reference's own code.

Tolerances (relative L2 over complex outputs, FP32 kernels vs FP64):
  * single-hop scenes (source hop, field points, field objects): 1e-5
  * fragment -> fragment bounces: 1e-5 per bounce on small scenes, 1e-4 on the
    full-size trihedral subset
Interaction masks must equal the oracle's bit for bit on every pair the
oracle does not classify as grazing.
"""
import numpy as np
import pytest

from conftest import GOLDEN_SCENES, golden_scene, load_golden, rel_l2

pytestmark = pytest.mark.gpu


def load_scene(api, sc):
    api.TearDownCuda()
    api.set_initial_conditions(sc["cp"], sc["f"], sc["att"])
    for t, d in sc["targets"]:
        api.load_stl_mesh_to_cuda(t, api.TARGET, d)
    for t, d in sc["fields"]:
        api.load_stl_mesh_to_cuda(t, api.FIELD, d)
    api.load_points_to_cuda(sc["sources"], isSource=True)
    api.load_points_to_cuda(sc["field_points"], isSource=False)
    api.render_cuda()


def run_gpu(api, sc):
    load_scene(api, sc)
    api.project_source_points_to_objects(False)
    if sc["bounces"]:
        api.project_target_to_target_objects(sc["bounces"])
    if sc["field_objects"]:
        api.project_target_to_field_objects()
    api.project_target_to_field_points()
    out = {}
    for i in range(len(sc["targets"])):
        out["P_target%d" % i] = api.get_object_pressures(api.TARGET, i)
    for i in range(len(sc["fields"])):
        out["P_field%d" % i] = api.get_object_pressures(api.FIELD, i)
    out["P_points"] = api.get_field_point_pressures(len(sc["field_points"]))
    return out


def oracle_scene(oracle_mod, sc, render=True):
    o = oracle_mod.Oracle()
    o.set_initial_conditions(sc["cp"], sc["f"], sc["att"])
    for t, d in sc["targets"]:
        o.load_geometry(t, 0, d)
    for t, d in sc["fields"]:
        o.load_geometry(t, 2, d)
    o.load_source_points(sc["sources"])
    o.load_field_points(sc["field_points"])
    if render:
        o.render()
    return o


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_golden_scene(api, name):
    g = load_golden(name)
    sc = golden_scene(g)
    got = run_gpu(api, sc)
    api.TearDownCuda()
    for k, v in got.items():
        ref = g[k]
        err = rel_l2(v, ref)
        print(name, k, "rel L2 %.3e" % err)
        assert err < 1e-5, (k, err)


def _mask_pairs(api, o, hop, a, b, ndst, nsrc, dst_idx):
    gm = api.get_mask(hop, a, b).reshape(ndst, nsrc)[dst_idx]
    _, om = o.hop_subset(hop, a, b, dst_idx, want_mask=True, nsrc=nsrc)
    return gm, om


@pytest.mark.parametrize("name", GOLDEN_SCENES)
def test_masks_match_oracle_outside_grazing(api, oracle_mod, name):
    g = load_golden(name)
    sc = golden_scene(g)
    load_scene(api, sc)
    o = oracle_scene(oracle_mod, sc)
    checked = 0
    for ti in range(len(sc["targets"])):
        hops = [(0, 0, ti, o.ncells(0, ti), len(sc["sources"])),
                (1, ti, 0, len(sc["field_points"]), o.nact(0, ti)),
                (2, ti, 0, o.nact(0, ti), o.nact(0, ti))]
        for fi in range(len(sc["fields"])):
            hops.append((3, ti, fi, o.nact(2, fi), o.nact(0, ti)))
        for hop, a, b, ndst, nsrc in hops:
            if ndst == 0 or nsrc == 0:
                continue
            dst = np.arange(ndst)
            gm, om = _mask_pairs(api, o, hop, a, b, ndst, nsrc, dst)
            graze = (om & 2) != 0
            diff = (gm != (om & 1)) & ~graze
            print(name, "hop", hop, "pairs", gm.size, "interacting", int(gm.sum()), "grazing", int(graze.sum()),
                  "mismatch", int(diff.sum()))
            assert diff.sum() == 0, (hop, np.argwhere(diff)[:5])
            checked += gm.size
    api.TearDownCuda()
    assert checked > 0


def test_plate_config1_full(api, oracle_mod, scenes):
    """Plain method, small: 1.0 x 0.5 m plate at 10 kHz, 64 x 64 field grid;
    the FP32 kernels within 1e-5 of FP64."""
    cfg = scenes.plate_config()
    sc = dict(cp=cfg["cp"], f=cfg["frequency"], att=0.0, bounces=0, field_objects=False, sources=cfg["sources"],
              field_points=cfg["field_points"], targets=cfg["targets"], fields=[])
    got = run_gpu(api, sc)
    stats = api.stats()
    api.TearDownCuda()
    o = oracle_scene(oracle_mod, sc)
    o.project_sources(False)
    o.project_field_points()
    e_surf = rel_l2(got["P_target0"], o.pressures(0, 0))
    e_pts = rel_l2(got["P_points"], o.field_points())
    print("config1: surface %.3e field %.3e" % (e_surf, e_pts), stats)
    assert e_surf < 1e-5 and e_pts < 1e-5
    assert o.nact(0, 0) > 1200


def test_deterministic(api, scenes):
    g = load_golden("trihedral_bounces")
    sc = golden_scene(g)
    a = run_gpu(api, sc)
    b = run_gpu(api, sc)
    api.TearDownCuda()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_split_count_does_not_change_results_beyond_roundoff(api):
    g = load_golden("trihedral_bounces")
    sc = golden_scene(g)
    api.set_option("split", 1)
    a = run_gpu(api, sc)
    api.set_option("split", 3)
    b = run_gpu(api, sc)
    api.set_option("split", 0)
    api.TearDownCuda()
    for k in a:
        assert rel_l2(a[k], b[k]) < 1e-12, k


def test_frequency_change_reuses_geometry(api, oracle_mod):
    """set_initial_conditions between projections changes k only (masks are
    reused); results follow the oracle at the new frequency."""
    g = load_golden("plate_10khz")
    sc = golden_scene(g)
    load_scene(api, sc)
    api.set_initial_conditions(sc["cp"], 7000.0, 0.0)
    api.project_source_points_to_objects(False)
    api.project_target_to_field_points()
    got = api.get_field_point_pressures(len(sc["field_points"]))
    api.TearDownCuda()
    sc2 = dict(sc, f=7000.0)
    o = oracle_scene(oracle_mod, sc2)
    o.project_sources(False)
    o.project_field_points()
    assert rel_l2(got, o.field_points()) < 1e-5


def test_trihedral_bounces_full_size_subset(api, oracle_mod, scenes):
    """Trihedral, 1 m legs, 40 kHz (~62k fragments), 2 bounces: each bounce's
    output checked on 96 seeded destinations against the oracle run with the
    GPU's own input of that bounce."""
    cfg = scenes.trihedral_config(40e3, bounces=2, n_theta=4, n_phi=4)
    sc = dict(cp=cfg["cp"], f=cfg["frequency"], att=0.0, bounces=0, field_objects=False, sources=cfg["sources"],
              field_points=cfg["field_points"], targets=cfg["targets"], fields=[])
    load_scene(api, sc)
    api.project_source_points_to_objects(False)
    P0 = api.get_object_pressures(api.TARGET, 0)
    api.project_target_to_target_objects(1)
    P1 = api.get_object_pressures(api.TARGET, 0)
    out1 = P1 - P0
    api.project_target_to_target_objects(1)  # prime with P1: input = P1 (P_out <- P)
    P2 = api.get_object_pressures(api.TARGET, 0)
    out2 = P2 - P1
    api.TearDownCuda()
    o = oracle_scene(oracle_mod, sc)
    act = o.active(0, 0)
    assert len(act) > 55000
    rng = np.random.default_rng(1234)
    q = np.sort(rng.choice(len(act), 96, replace=False))
    # source hop on the same cells
    v0, _ = o.hop_subset(0, 0, 0, act[q])
    assert rel_l2(P0[act[q]], v0) < 1e-5
    # bounce 1: input P0 ; bounce 2: the second call re-primes P_out <- P = P1
    v1, _ = o.hop_subset(2, 0, 0, q, pin=P0)
    v2, _ = o.hop_subset(2, 0, 0, q, pin=P1)
    e1, e2 = rel_l2(out1[act[q]], v1), rel_l2(out2[act[q]], v2)
    print("trihedral 40 kHz bounce errors %.3e %.3e" % (e1, e2))
    assert e1 < 1e-4 and e2 < 1e-4


def test_sphere_shadowed_hops(api, oracle_mod, scenes):
    """Icosphere (subdivision 2) at 4 kHz: shadowed source hop and readout to
    field points around it, full oracle comparison and mask parity."""
    sph = scenes.icosphere(2, 1.0)
    fp = np.concatenate([scenes.grid_xy(10, 2.0, 1.6), scenes.grid_xy(10, 2.0, -1.6)])
    sc = dict(cp=1480.0, f=4000.0, att=0.0, bounces=0, field_objects=False,
              sources=np.array([[0.3, 0.2, 6.0]], np.float32), field_points=fp,
              targets=[(sph, 0.05)], fields=[])
    got = run_gpu(api, sc)
    o = oracle_scene(oracle_mod, sc)
    o.project_sources(False)
    o.project_field_points()
    e_surf = rel_l2(got["P_target0"], o.pressures(0, 0))
    e_pts = rel_l2(got["P_points"], o.field_points())
    load_scene(api, sc)
    gm, om = _mask_pairs(api, o, 1, 0, 0, len(fp), o.nact(0, 0), np.arange(len(fp)))
    api.TearDownCuda()
    graze = (om & 2) != 0
    diff = (gm != (om & 1)) & ~graze
    print("sphere: surface %.3e points %.3e grazing %d mismatches %d" % (e_surf, e_pts, graze.sum(), diff.sum()))
    assert diff.sum() == 0
    # field points below the sphere are shadowed from parts of it
    assert e_surf < 1e-5 and e_pts < 1e-4


def test_symmetric_bounce_sum_matches_ordered(api, scenes):
    """The reciprocity form of the bounce sum (one Green's function per
    unordered pair, the default) and the ordered form agree to FP32 round-off,
    on a scene with multiple tiles per facet and a zero-input region."""
    cfg = scenes.trihedral_config(12e3, bounces=2, n_theta=2, n_phi=2)
    sc = dict(cp=cfg["cp"], f=cfg["frequency"], att=0.0, bounces=2, field_objects=False,
              sources=np.array([[3.0, 0.4, 0.5]], np.float32),  # face y = 0 partly unlit: zero inputs
              field_points=cfg["field_points"], targets=cfg["targets"], fields=[])
    out = {}
    for sym in (1, 0):
        api.set_option("f2f_symmetric", sym)
        out[sym] = run_gpu(api, sc)
    api.set_option("f2f_symmetric", 1)
    api.TearDownCuda()
    P1, P0 = out[1]["P_target0"], out[0]["P_target0"]
    assert np.abs(P1).max() > 0
    err = rel_l2(P1, P0)
    print("symmetric vs ordered bounce sums: rel L2 %.3e" % err)
    assert err < 1e-6


@pytest.mark.parametrize("extra", ["none", "box", "sphere"])
def test_bounce_mask_classification_pass_identical(api, oracle_mod, scenes, extra):
    """The bounce mask built by the warp-per-block classification pass (pair
    kernel on the listed blocks only) and by the pair kernel over every block
    give the same block classes and bit-identical bounces: the trihedral
    alone (3 triangles), with a box in the corner (15 triangles, occluded
    pairs) and with an icosphere in the corner (83 triangles: occluder
    candidates from the BVH walk)."""
    tri = scenes.trihedral(1.0)
    if extra == "box":
        tri = np.concatenate([tri, scenes.box(0.2, 0.15, 0.25, center=(0.35, 0.3, 0.2))])
    elif extra == "sphere":
        tri = np.concatenate([tri, scenes.icosphere(1, 0.18, center=(0.35, 0.35, 0.3))])
    f = 15e3
    sc = dict(cp=1480.0, f=f, att=0.0, bounces=2, field_objects=False,
              sources=np.array([[6.0, 5.0, 4.0]], np.float32),
              field_points=scenes.hemisphere(3, 3, 2.0), targets=[(tri, scenes.delta_for(f))], fields=[])
    out, classes = {}, {}
    for mode in (1, 0):
        api.set_option("mask_classify", mode)
        api.set_option("class_stats", 1)
        out[mode] = run_gpu(api, sc)
        classes[mode] = [c for c in api.stats()["mask_classes"] if c["hop"] == 2]
        api.set_option("class_stats", 0)
    api.set_option("mask_classify", 1)
    api.TearDownCuda()
    print(extra, "bounce mask classes", classes[1])
    assert classes[1] == classes[0]
    c = classes[1][0]
    # the bare corner has blocks proved free of occluders; an object in the
    # corner may occlude almost every block's rays
    assert (c["clear"] + c["all"] > 0) if extra == "none" else (c["bits"] > 0)
    for k in out[1]:
        assert np.array_equal(out[1][k], out[0][k]), k
    assert np.abs(out[1]["P_target0"]).max() > 0
    # the exported bounce mask (every pair) with the gates decided from the
    # per-point projections where certain, and always per pair: identical,
    # and equal to the oracle's outside grazing pairs on seeded destinations
    load_scene(api, sc)
    masks = {}
    for gp in (1, 0):
        api.set_option("mask_gate_proj", gp)
        masks[gp] = api.get_mask(2, 0, 0)
    api.set_option("mask_gate_proj", 1)
    api.TearDownCuda()
    assert np.array_equal(masks[1], masks[0])
    o = oracle_scene(oracle_mod, sc)
    n = o.nact(0, 0)
    dst = np.sort(np.random.default_rng(5).choice(n, 96, replace=False))
    gm = masks[1].reshape(n, n)[dst]
    _, om = o.hop_subset(2, 0, 0, dst, want_mask=True, nsrc=n)
    o.close()
    graze = (om & 2) != 0
    diff = (gm != (om & 1)) & ~graze
    print(extra, "bounce mask vs oracle: pairs %d interacting %d grazing %d mismatches %d"
          % (gm.size, int(gm.sum()), int(graze.sum()), int(diff.sum())))
    assert diff.sum() == 0


def test_convex_target_masks_identical(api, scenes):
    """A convex target (icosphere): the masks' shadow tests search only the
    part of each ray where a crossing is possible; the masks of the source
    hop, the readout to field points and the target -> field-object hop are
    bit-identical to those of the full BVH walk."""
    sph = scenes.icosphere(3, 0.5)
    plane = scenes.rotate(scenes.rectangle(2.0, 2.0, z=0.0), "y", 90.0)  # x = 0 plane through the centre
    fp = np.concatenate([scenes.grid_xy(12, 1.5, 1.2), scenes.grid_xy(12, 1.5, -1.2)])
    f = 6e3
    sc = dict(cp=1480.0, f=f, att=0.0, bounces=0, field_objects=True,
              sources=np.array([[0.2, 0.1, 5.0]], np.float32), field_points=fp,
              targets=[(sph, scenes.delta_for(f))], fields=[(plane, 2.0 / 96)])
    load_scene(api, sc)
    masks = {}
    for cv in (1, 0):
        api.set_option("convex_masks", cv)
        masks[cv] = [api.get_mask(0, 0, 0), api.get_mask(1, 0, 0), api.get_mask(3, 0, 0)]
    api.set_option("convex_masks", 1)
    st = api.stats()
    api.TearDownCuda()
    for k, (m1, m0) in enumerate(zip(masks[1], masks[0])):
        print("hop %d: pairs %d interacting %d" % ((0, 1, 3)[k], m1.size, int(m1.sum())))
        assert m1.sum() > 0
        assert np.array_equal(m1, m0)
