"""The admissibility network on the GPU: its forward and backward kernels
against the FP64 oracle, Adam training, and the ablation that shows what the
trained network gains over compression without it.

Gradient check: GPU gradient of the mean squared error within 1e-4 relative
L2 of the oracle's FP64 gradient (FP32 kernels, 64-wide sums).
Ablation (trihedral, 30 kHz, network trained on its 20 and 25 kHz versions):
the network's proposals compress more of the bounce's pair work than the
separation rule at the same 1e-3 error bound, and need fewer approximation
attempts than trying every interacting block.
"""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import load_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def adm(api):
    import sonar_render_gb300.admissibility as a
    return a


def test_forward_and_gradient_match_oracle(adm, oracle_mod):
    adm.init(3)
    p = adm.get_params()
    assert len(p) == oracle_mod.mlp_param_count()
    rng = np.random.default_rng(11)
    X = rng.standard_normal((200, 8)).astype(np.float32)
    y = rng.standard_normal(200).astype(np.float32)
    pred = adm.predict(X)
    ref = oracle_mod.mlp_forward(p, X)
    e_fwd = rel_l2(pred, ref)
    loss, g = adm.grad(X, y)
    loss_ref, g_ref = oracle_mod.mlp_grad(p, X, y)
    e_grad = rel_l2(g, g_ref)
    print("network forward rel L2 %.2e, loss %.6f vs %.6f, gradient rel L2 %.2e" % (e_fwd, loss, loss_ref, e_grad))
    assert e_fwd < 1e-5
    assert abs(loss - loss_ref) < 1e-5 * max(1.0, loss_ref)
    assert e_grad < 1e-4
    # per layer (the last layers' gradients are the smallest)
    off = 0
    for fin, fout in ((8, 64), (64, 64), (64, 64), (64, 1)):
        n = fin * fout + fout
        assert rel_l2(g[off:off + n], g_ref[off:off + n]) < 1e-4
        off += n


def test_width128_tensor_core_inference_and_gradient(adm, oracle_mod):
    """Width 128: FP16 hidden layers on the tensor cores (tcgen05.mma, FP32
    accumulation) against the FP64 forward -- the FP16 rounding of
    activations and weights (2^-11 relative) bounds the error, 5e-3 relative
    L2 -- over more rows than one 128-row tile and a ragged last tile; the
    FP32 training kernels' gradient within 1e-4 of the FP64 one."""
    adm.set_width(128)
    oracle_mod.mlp_set_width(128)
    try:
        assert adm.width() == 128
        adm.init(7)
        p = adm.get_params()
        assert len(p) == oracle_mod.mlp_param_count() == 8 * 128 + 128 + 2 * (128 * 128 + 128) + 128 + 1
        rng = np.random.default_rng(12)
        X = rng.uniform(0.0, 4.0, (1000, 8)).astype(np.float32)
        y = rng.standard_normal(1000).astype(np.float32)
        pred = adm.predict(X)
        ref = oracle_mod.mlp_forward(p, X)
        e_fwd = rel_l2(pred, ref)
        loss, g = adm.grad(X[:300], y[:300])
        loss_ref, g_ref = oracle_mod.mlp_grad(p, X[:300], y[:300])
        e_grad = rel_l2(g, g_ref)
        print("width 128: tensor-core FP16 forward rel L2 %.2e (max abs %.2e), FP32 gradient rel L2 %.2e"
              % (e_fwd, np.abs(pred - ref).max(), e_grad))
        assert e_fwd < 5e-3
        assert e_grad < 1e-4
        # a second call gives the same bits (one tile per CTA, fixed order)
        assert np.array_equal(adm.predict(X), pred)
    finally:
        adm.set_width(64)
        oracle_mod.mlp_set_width(64)


def test_training_fits_a_smooth_function(adm):
    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, (4096, 8)).astype(np.float32)
    y = (np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2] + 0.5 * np.abs(X[:, 3])).astype(np.float32)
    adm.init(1)
    l0, _ = adm.grad(X, y)
    loss = adm.train(X, y, epochs=30, batch=128, lr=2e-3, seed=4)
    print("training loss %.4f -> %.5f" % (l0, loss))
    assert loss < 0.05 * l0
    # training is deterministic for a seed
    adm.init(1)
    loss2 = adm.train(X, y, epochs=30, batch=128, lr=2e-3, seed=4)
    assert loss2 == loss


def _tri(scenes, f):
    return scenes.trihedral_config(f, bounces=2, n_theta=4, n_phi=4)


def _run_bounces(api, scenes, f, compress, select=0):
    cfg = _tri(scenes, f)
    sc = dict(cp=cfg["cp"], f=cfg["frequency"], att=0.0, bounces=2, field_objects=False, sources=cfg["sources"],
              field_points=cfg["field_points"], targets=cfg["targets"], fields=[])
    api.set_option("compress", compress)
    api.set_option("compress_select", select)
    load_scene(api, sc)
    api.project_source_points_to_objects(False)
    P0 = api.get_object_pressures(api.TARGET, 0)
    api.set_option("reset_stats", 1)
    api.project_target_to_target_objects(2)
    P2 = api.get_object_pressures(api.TARGET, 0)
    hops = [h for h in api.stats()["hops"] if h["hop"] == 2]
    api.set_option("compress", 0)
    api.set_option("compress_select", 0)
    api.TearDownCuda()
    return P2 - P0, hops


def test_network_ablation(api, adm, scenes):
    X, y, loss = adm.train_on_scenes([_tri(scenes, 20e3), _tri(scenes, 25e3)], epochs=60, batch=128, lr=1e-3,
                                     seed=0)
    print("training samples %d, label mean %.2f, final loss %.4f" % (len(y), float(y.mean()), loss))
    assert len(y) > 1000
    plain, _ = _run_bounces(api, scenes, 30e3, 0)
    res = {}
    for name, sel in (("rule", 0), ("network", 2), ("exhaustive", 1)):
        out, hops = _run_bounces(api, scenes, 30e3, 1, sel)
        h = hops[0]
        res[name] = dict(err=rel_l2(out, plain), pairs=h["cmp_pairs"], total=h["pairs"], tried=h["cmp_blocks"],
                         accepted=h["cmp_accepted"], aca_ms=h["cmp_aca_ms"], build_ms=h["cmp_build_ms"],
                         bounce_ms=hops[1]["sum_ms"] + hops[1]["lr_ms"])
        print("%-10s err %.2e compressed pairs %.3f of all, tried %d accepted %d, aca %.2f ms build %.2f ms, "
              "second bounce %.3f ms" % (name, res[name]["err"], res[name]["pairs"] / (res[name]["total"] or 1),
                                         res[name]["tried"], res[name]["accepted"], res[name]["aca_ms"],
                                         res[name]["build_ms"], res[name]["bounce_ms"]))
    for r in res.values():
        assert r["err"] < 1e-3
    assert res["network"]["pairs"] > 1.2 * res["rule"]["pairs"]
    assert res["network"]["tried"] < res["exhaustive"]["tried"]
    assert res["network"]["pairs"] > 0.9 * res["exhaustive"]["pairs"]
