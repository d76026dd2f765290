"""Device memory from the stream-ordered pool: repeated TearDownCuda / load /
render cycles (the reference's own calling pattern, src/python_interface.cpp)
reuse the pool's blocks, give bit-identical pressures every cycle, and keep
the pool's footprint flat; a pool that keeps nothing (memory_cache_mb 0) and
an explicit release give the same pressures.  A batch plan created and
destroyed twice gives the same outputs twice."""
import numpy as np
import pytest

from test_gpu_parity import load_scene

pytestmark = pytest.mark.gpu


def _trihedral(scenes, f):
    cfg = scenes.trihedral_config(f, bounces=2, n_theta=4, n_phi=4)
    return dict(cp=cfg["cp"], f=cfg["frequency"], att=0.0, bounces=2, field_objects=False, sources=cfg["sources"],
                field_points=cfg["field_points"], targets=cfg["targets"], fields=[])


def _cycle(api, sc, compress):
    api.set_option("compress", compress)
    load_scene(api, sc)
    api.project_source_points_to_objects(False)
    api.project_target_to_target_objects(2)
    api.project_target_to_field_points()
    P = api.get_object_pressures(api.TARGET, 0)
    F = api.get_field_point_pressures(len(sc["field_points"]))
    reserved = api.stats()["pool_reserved_bytes"]
    api.set_option("compress", 0)
    api.TearDownCuda()
    return P, F, reserved


@pytest.mark.parametrize("compress", [0, 1])
def test_cycles_identical_and_pool_flat(api, scenes, compress):
    sc = _trihedral(scenes, 20e3)
    runs = [_cycle(api, sc, compress) for _ in range(3)]
    P0, F0, r0 = runs[0]
    assert np.abs(P0).max() > 0 and np.abs(F0).max() > 0
    for P, F, r in runs[1:]:
        np.testing.assert_array_equal(P, P0)
        np.testing.assert_array_equal(F, F0)
    print("pool reserved per cycle (MB):", [round(r / 2**20, 1) for _, _, r in runs])
    assert r0 > 0
    assert runs[2][2] <= runs[1][2]  # the third cycle maps nothing new


def test_no_cache_and_release_same_results(api, scenes):
    sc = _trihedral(scenes, 15e3)
    P0, F0, _ = _cycle(api, sc, 0)
    api.set_option("memory_cache_mb", 0)
    try:
        P1, F1, _ = _cycle(api, sc, 0)
    finally:
        api.set_option("memory_cache_mb", 32768)
    api.set_option("release_memory", 1)
    P2, F2, _ = _cycle(api, sc, 0)
    for P, F in ((P1, F1), (P2, F2)):
        np.testing.assert_array_equal(P, P0)
        np.testing.assert_array_equal(F, F0)
    with pytest.raises(Exception):
        api.set_option("memory_cache_mb", -1)


def test_batch_plans_reuse_pool(api, scenes):
    from conftest import rel_l2
    from sonar_render_gb300 import batch
    tris = [scenes.rotate(scenes.rectangle(0.25, 0.25), "x", -10.0), scenes.icosphere(2, 0.07)]
    pos = scenes.arc_xz(8.0, np.linspace(-60.0, 60.0, 16))
    freqs = np.array([15e3, 20e3], np.float32)
    outs, tunings = [], []
    for _ in range(2):
        plan = batch.Plan(tris, pos, pos, freqs)
        outs.append(plan.run())
        tunings.append(plan.stats()["tuning"])
        plan.close()
    assert np.abs(outs[0]).max() > 0
    if tunings[0] == tunings[1]:
        np.testing.assert_array_equal(outs[1], outs[0])
    else:  # another tile shape sums in another order
        assert rel_l2(outs[1], outs[0]) < 1e-6


def test_staged_copies_multi_chunk(api, oracle_mod, scenes):
    """A 1.0 x 1.2 m plate at 1 mm fragments: ~2.4M cells, so the cell
    positions going up (38 MB) and the pressures coming back (38 MB) each take
    several pinned chunks; every cell's source-hop pressure must follow the
    oracle's."""
    from conftest import rel_l2
    from test_gpu_parity import oracle_scene
    plate = scenes.rotate(scenes.rectangle(1.0, 1.2), "x", 20.0)
    sc = dict(cp=1480.0, f=20e3, att=0.0, bounces=0, field_objects=False,
              sources=np.array([[0.3, -0.2, 3.0]], np.float32), field_points=np.zeros((1, 3), np.float32),
              targets=[(plate, 0.001)], fields=[])
    load_scene(api, sc)
    api.project_source_points_to_objects(False)
    got = api.get_object_pressures(api.TARGET, 0)
    api.TearDownCuda()
    assert got.size * 16 > 4 * (8 << 20)
    o = oracle_scene(oracle_mod, sc)
    o.project_sources(False)
    ref = o.pressures(0, 0)
    o.close()
    assert got.shape == ref.shape
    assert np.count_nonzero(ref) > got.size // 3
    assert rel_l2(got, ref) < 1e-5
    # the last chunk's tail and a chunk seam, element by element
    for k in (got.size - 1, (8 << 20) // 16 - 1, (8 << 20) // 16):
        assert abs(got[k] - ref[k]) <= 1e-5 * abs(ref).max(), k
