"""Interpolated bounce blocks: far blocks of class ALL between planar tiles
(one facet's fragment grid, a box of at most 32 x 16 cells) approximated by
directional Chebyshev interpolation instead of cross approximation, judged
on an 8 x 8 grid of exact entries (src/OptiX.cu:340-390 as the dense path
evaluates them).

On the 40 kHz trihedral (1 m legs, ~62k fragments) the compressed bounces
with interpolated blocks must stay within 1e-3 relative L2 of the plain path
and of the FP64 oracle, agree with the cross-approximation-only path to the
same tolerance, be bit-for-bit deterministic, hold the attenuating medium's
(k_a != 0) entries, and pass the full-tile audit.
"""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import load_scene, oracle_scene

pytestmark = pytest.mark.gpu


def _trihedral(scenes, f, att=0.0):
    cfg = scenes.trihedral_config(f, bounces=2, n_theta=4, n_phi=4)
    return dict(cp=cfg["cp"], f=cfg["frequency"], att=att, bounces=2, field_objects=False, sources=cfg["sources"],
                field_points=cfg["field_points"], targets=cfg["targets"], fields=[])


def _run(api, sc, compress, interp=1, bounces=2, tol=5e-4):
    api.set_option("compress", compress)
    api.set_option("compress_select", 0)
    api.set_option("compress_interp", interp)
    api.set_option("compress_tol", tol)
    api.set_option("compress_judge", 3.0 * tol)
    try:
        load_scene(api, sc)
        api.project_source_points_to_objects(False)
        P0 = api.get_object_pressures(api.TARGET, 0)
        api.set_option("reset_stats", 1)
        api.project_target_to_target_objects(bounces)
        P = api.get_object_pressures(api.TARGET, 0)
        st = api.stats()
    finally:
        api.set_option("compress", 0)
        api.set_option("compress_interp", 1)
        api.set_option("compress_tol", 1e-4)
        api.set_option("compress_judge", 3e-4)
        api.TearDownCuda()
    hop = [h for h in st["hops"] if h["hop"] == 2][0] if compress else None
    return P0, P, hop


def _one_bounce_vs_oracle(oracle_mod, sc, P0, P1, seed):
    o = oracle_scene(oracle_mod, sc)
    act = o.active(0, 0)
    q = np.sort(np.random.default_rng(seed).choice(len(act), 64, replace=False))
    v1, _ = o.hop_subset(2, 0, 0, q, pin=P0)
    o.close()
    return rel_l2((P1 - P0)[act[q]], v1)


def test_interpolated_bounces_match_plain_and_cross_approximation(api, scenes):
    sc = _trihedral(scenes, 40e3)
    P0, P_plain, _ = _run(api, sc, 0)
    _, P_ip, hop = _run(api, sc, 1, interp=1)
    _, P_aca, hop0 = _run(api, sc, 1, interp=0)
    print("interpolated blocks %d (mean nodes %.1f) of %d accepted; cross-approximated mean rank %.1f; "
          "build %.2f ms (interpolation %.2f, cross approximation %.2f)"
          % (hop["cmp_ip_blocks"], hop["cmp_ip_nodes"], hop["cmp_accepted"], hop["cmp_mean_rank"],
             hop["cmp_build_ms"], hop["cmp_ip_ms"], hop["cmp_aca_ms"]))
    assert hop["cmp_ip_blocks"] > 1000 and hop0["cmp_ip_blocks"] == 0
    e_plain = rel_l2(P_ip - P0, P_plain - P0)
    e_aca = rel_l2(P_ip - P0, P_aca - P0)
    print("interpolated vs plain bounce contributions %.3e, vs cross approximation only %.3e" % (e_plain, e_aca))
    assert e_plain < 1e-3 and e_aca < 1e-3


def test_interpolated_bounce_vs_oracle(api, oracle_mod, scenes):
    sc = _trihedral(scenes, 40e3)
    P0, P1, hop = _run(api, sc, 1, bounces=1)
    assert hop["cmp_ip_blocks"] > 1000
    e = _one_bounce_vs_oracle(oracle_mod, sc, P0, P1, 91)
    print("one bounce with %d interpolated blocks vs FP64 oracle (64 seeded destinations): rel L2 %.3e"
          % (hop["cmp_ip_blocks"], e))
    assert e < 1e-3


def test_interpolated_attenuating_medium(api, oracle_mod, scenes):
    """k_a != 0: the node entries carry e^{-k_a r} and (k_a - i k_r)."""
    sc = _trihedral(scenes, 40e3, att=0.5)
    P0, P1, hop = _run(api, sc, 1, bounces=1)
    assert hop["cmp_ip_blocks"] > 1000
    e = _one_bounce_vs_oracle(oracle_mod, sc, P0, P1, 92)
    print("attenuating medium: %d interpolated blocks, one bounce vs FP64 oracle rel L2 %.3e"
          % (hop["cmp_ip_blocks"], e))
    assert e < 1e-3


def test_interpolated_deterministic(api, scenes):
    sc = _trihedral(scenes, 40e3)
    _, a, _ = _run(api, sc, 1)
    _, b, _ = _run(api, sc, 1)
    assert np.array_equal(a, b)


def test_interpolated_audit_full_tiles(api, scenes):
    """Every entry of sampled accepted blocks (interpolated and
    cross-approximated) against the exact ones at the library default
    tolerance 1e-4: none may exceed 3x the judge's limit."""
    sc = _trihedral(scenes, 40e3)
    tol = 1e-4
    api.set_option("compress", 1)
    api.set_option("compress_select", 0)
    api.set_option("compress_tol", tol)
    api.set_option("compress_judge", 3.0 * tol)
    try:
        load_scene(api, sc)
        api.project_source_points_to_objects(False)
        api.set_option("reset_stats", 1)
        api.project_target_to_target_objects(1)
        hop = [h for h in api.stats()["hops"] if h["hop"] == 2][0]
        full, judged = api.audit_compression(256, seed=5)
    finally:
        api.set_option("compress", 0)
        api.TearDownCuda()
    limit = 3.0 * tol
    print("audit at tol 1e-4 (%d interpolated of %d accepted): %d blocks, full-tile error median %.2e max %.2e, "
          "judged median %.2e, above the limit %.3f" % (hop["cmp_ip_blocks"], hop["cmp_accepted"], len(full),
                                                       np.median(full), full.max(), np.median(judged),
                                                       float(np.mean(full > limit))))
    assert hop["cmp_ip_blocks"] > 0
    assert len(full) == 256 and np.all(np.isfinite(full))
    assert full.max() < 3 * limit


def _scene(targets, f, sources):
    cp = 1480.0
    return dict(cp=cp, f=f, att=0.0, bounces=2, field_objects=False, sources=np.asarray(sources, np.float32),
                field_points=np.array([[0.0, 0.0, 5.0]], np.float32), targets=targets, fields=[])


def test_interpolation_between_facing_plates(api, oracle_mod, scenes):
    """Two parallel 1 x 1 m plates facing each other 0.8 m apart at 40 kHz,
    the source between them: tiles are whole 16 x 16 patches or two half
    patches of a triangle; the interpolated bounce matches the plain one and
    the FP64 oracle."""
    d = scenes.delta_for(40e3)
    lower = scenes.rectangle(1.0, 1.0, z=0.0, normal_up=True)
    upper = scenes.rectangle(1.0, 1.0, z=0.8, normal_up=False)
    sc = _scene([(np.concatenate([lower, upper]), d)], 40e3, [[0.1, -0.05, 0.4]])
    P0, P_plain, _ = _run(api, sc, 0)
    _, P_ip, hop = _run(api, sc, 1)
    e_plain = rel_l2(P_ip - P0, P_plain - P0)
    print("facing plates: %d interpolated blocks (mean nodes %.1f) of %d accepted; vs plain %.3e"
          % (hop["cmp_ip_blocks"], hop["cmp_ip_nodes"], hop["cmp_accepted"], e_plain))
    # the tiles across the rectangles' diagonals (two facets) stay with the cross approximation
    assert 500 < hop["cmp_ip_blocks"] < hop["cmp_accepted"]
    assert e_plain < 1e-3
    Q0, Q1, _ = _run(api, sc, 1, bounces=1)
    e = _one_bounce_vs_oracle(oracle_mod, sc, Q0, Q1, 93)
    print("facing plates, one bounce vs FP64 oracle: rel L2 %.3e" % e)
    assert e < 1e-3
