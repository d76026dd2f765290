"""Full-size GPU parity of the benchmark configurations that the bench does
not check itself: the shadowed icosphere onto its field surface and the
three-bounce trihedral with its hemisphere readout.

Each hop is checked against the FP64 oracle on seeded destinations, the
oracle given the GPU's own input of that hop (so each error is the hop's
own); interaction masks must equal the oracle's bit for bit on every pair the
oracle does not classify as grazing, and the grazing counts are printed.

Tolerances (relative L2 over complex outputs, FP32 kernels vs FP64): 1e-5
for the source hop, 1e-4 for the full-size readouts and bounces (sums of
10^5 terms with phases k r up to a few hundred radians).
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _load(api, cfg):
    api.TearDownCuda()
    api.set_initial_conditions(cfg["cp"], cfg["frequency"], cfg.get("attenuation", 0.0))
    for t, d in cfg["targets"]:
        api.load_stl_mesh_to_cuda(t, api.TARGET, d)
    for t, d in cfg.get("fields", []):
        api.load_stl_mesh_to_cuda(t, api.FIELD, d)
    api.load_points_to_cuda(cfg["sources"], isSource=True)
    if cfg.get("field_points") is not None:
        api.load_points_to_cuda(cfg["field_points"], isSource=False)
    api.render_cuda()


def _oracle(oracle_mod, cfg):
    o = oracle_mod.Oracle()
    o.set_initial_conditions(cfg["cp"], cfg["frequency"], cfg.get("attenuation", 0.0))
    for t, d in cfg["targets"]:
        o.load_geometry(t, 0, d)
    for t, d in cfg.get("fields", []):
        o.load_geometry(t, 2, d)
    o.load_source_points(cfg["sources"])
    if cfg.get("field_points") is not None:
        o.load_field_points(cfg["field_points"])
    o.render()
    return o


def _mask_check(gm, om, what):
    graze = (om & 2) != 0
    diff = (gm != (om & 1)) & ~graze
    print("%s: pairs %d interacting %d grazing %d mismatches %d"
          % (what, gm.size, int(gm.sum()), int(graze.sum()), int(diff.sum())))
    assert diff.sum() == 0, np.argwhere(diff)[:5]
    return int(graze.sum())


def test_config2_icosphere_onto_field_surface(api, oracle_mod, scenes):
    """r = 1 m icosphere (subdivision 4, 5,120 triangles) at 20 kHz, source at
    10 m: the shadowed source hop, then FACET_NO_RESP onto the 512 x 512 cell
    field plane x = 0 through the centre (~4.6e10 candidate pairs); FP32 vs
    FP64 on 4,096 seeded field cells, masks of both hops on seeded rows."""
    cfg = scenes.sphere_config(512, field_surface=True)
    _load(api, cfg)
    api.project_source_points_to_objects(False)
    P = api.get_object_pressures(api.TARGET, 0)
    api.project_target_to_field_objects()
    F = api.get_object_pressures(api.FIELD, 0)
    o = _oracle(oracle_mod, cfg)
    act_t, act_f = o.active(0, 0), o.active(2, 0)
    nt, nf = len(act_t), len(act_f)
    assert nt > 150000 and nf > 250000
    rng = np.random.default_rng(20)
    # source hop on 4,096 seeded sphere cells (every cell receives pressure)
    cs = np.sort(rng.choice(o.ncells(0, 0), 4096, replace=False))
    v0, m0 = o.hop_subset(0, 0, 0, cs, want_mask=True, nsrc=1)
    e0 = rel_l2(P[cs], v0)
    g0 = _mask_check(api.get_mask_rows(0, 0, 0, cs), m0, "config 2 source hop mask")
    # field-surface hop on 4,096 seeded field cells, given the GPU's sphere pressures
    q = np.sort(rng.choice(nf, 4096, replace=False))
    o.set_pressures(0, 0, P)
    v3, m3 = o.hop_subset(3, 0, 0, q, want_mask=True, nsrc=nt)
    c3 = o.counters()
    gm = api.get_mask_rows(3, 0, 0, q)
    api.TearDownCuda()
    o.close()
    e3 = rel_l2(F[act_f[q]], v3)
    g3 = _mask_check(gm, m3, "config 2 field-surface hop mask")
    print("config 2: source hop rel L2 %.3e (grazing %d); field surface rel L2 %.3e on %d cells, %d pairs, "
          "grazing %d" % (e0, g0, e3, len(q), c3["pairs"], g3))
    assert e0 < 1e-5
    assert e3 < 1e-4
    assert np.abs(F[act_f[q]]).max() > 0


def test_config3_trihedral_three_bounces_hemisphere(api, oracle_mod, scenes):
    """Trihedral (1 m legs) at 40 kHz (~62k fragments), source at 20 m on the
    diagonal, ProjectTargetToTargetObjects(3), readout to 256 x 256 points on
    a 2 m hemisphere.  Bounce k's output is the difference of the totals
    after k and k - 1 bounces (fresh runs; the sums are deterministic), its
    input bounce k - 1's output; each is checked on 96 seeded destinations,
    the readout on 512 seeded field points given the GPU's final pressures."""
    cfg = scenes.trihedral_config(40e3, bounces=3, n_theta=256, n_phi=256)
    totals = []
    for nb in range(4):
        _load(api, cfg)
        api.project_source_points_to_objects(False)
        if nb:
            api.project_target_to_target_objects(nb)
        totals.append(api.get_object_pressures(api.TARGET, 0))
    api.project_target_to_field_points()
    fp = api.get_field_point_pressures(len(cfg["field_points"]))
    o = _oracle(oracle_mod, cfg)
    act = o.active(0, 0)
    n = len(act)
    assert n > 55000
    rng = np.random.default_rng(33)
    outs = [totals[0]] + [totals[k] - totals[k - 1] for k in range(1, 4)]
    errs = []
    q = np.sort(rng.choice(n, 96, replace=False))
    gm = api.get_mask_rows(2, 0, 0, q)
    for k in range(1, 4):
        v, m = o.hop_subset(2, 0, 0, q, pin=outs[k - 1], want_mask=(k == 1), nsrc=n)
        if k == 1:
            _mask_check(gm, m, "config 3 bounce mask")
        errs.append(rel_l2(outs[k][act[q]], v))
        assert np.abs(v).max() > 0
    jj = np.sort(rng.choice(len(cfg["field_points"]), 1024, replace=False))
    o.set_pressures(0, 0, totals[3])
    vf, mf = o.hop_subset(1, 0, 0, jj, want_mask=True, nsrc=n)
    gf = api.get_mask_rows(1, 0, 0, jj)
    api.TearDownCuda()
    o.close()
    _mask_check(gf, mf, "config 3 readout mask")
    # A grazing pair's visibility may be decided either way (the reference's
    # own answer there depends on OptiX's rounding), and at a field point
    # whose sum cancels strongly one such term moves the result by ~1e-3;
    # the tolerance applies to the field points without grazing pairs.
    clean = ~((mf & 2) != 0).any(axis=1)
    ef_all = rel_l2(fp[jj], vf)
    ef = rel_l2(fp[jj][clean], vf[clean])
    print("config 3: bounce errors %s, readout %.3e on %d field points without grazing pairs (%.3e on all %d)"
          % (" ".join("%.3e" % e for e in errs), ef, int(clean.sum()), ef_all, len(jj)))
    assert max(errs) < 1e-4
    assert clean.sum() >= 256
    assert ef < 1e-4
