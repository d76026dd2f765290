"""Patch-aligned tiles (option tile_align, on by default).

The active fragments of a facet are reordered so that its full 16 x 16-cell
patches start on 256-fragment tile boundaries and its edge cells (readout
centroid on or outside the triangle) come last.  The order is internal:
every output goes through the fragment -> cell map, so the results must not
depend on it beyond the FP32 summation order.  On the 40 kHz trihedral the
aligned layout must also give the compressed path square interpolation
tiles (fewer nodes) and far fewer blocks that need per-pair bits.
"""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import load_scene

pytestmark = pytest.mark.gpu


def _trihedral(scenes, f):
    cfg = scenes.trihedral_config(f, bounces=2, n_theta=4, n_phi=4)
    return dict(cp=cfg["cp"], f=cfg["frequency"], att=0.0, bounces=2, field_objects=False, sources=cfg["sources"],
                field_points=cfg["field_points"], targets=cfg["targets"], fields=[])


def _run(api, sc, align, compress):
    api.set_option("tile_align", align)
    api.set_option("compress", compress)
    api.set_option("compress_select", 0)
    api.set_option("class_stats", 1)
    try:
        load_scene(api, sc)
        api.project_source_points_to_objects(False)
        P0 = api.get_object_pressures(api.TARGET, 0)
        api.set_option("reset_stats", 1)
        api.project_target_to_target_objects(2)
        P = api.get_object_pressures(api.TARGET, 0)
        api.project_target_to_field_points()
        F = api.get_field_point_pressures(len(sc["field_points"]))
        st = api.stats()
    finally:
        api.set_option("tile_align", 1)
        api.set_option("compress", 0)
        api.set_option("class_stats", 0)
        api.TearDownCuda()
    hop = [h for h in st["hops"] if h["hop"] == 2][0]
    cls = [c for c in (st.get("mask_classes") or []) if c["hop"] == 2]
    return P - P0, F, hop, cls[0] if cls else None


def test_alignment_keeps_plain_results(api, scenes):
    sc = _trihedral(scenes, 40e3)
    P1, F1, _, c1 = _run(api, sc, 1, 0)
    P0, F0, _, c0 = _run(api, sc, 0, 0)
    e_p, e_f = rel_l2(P1, P0), rel_l2(F1, F0)
    print("plain bounces, aligned vs patch order: %.2e, readout %.2e; blocks needing bits or gates %d -> %d"
          % (e_p, e_f, c0["bits"] + c0["clear"], c1["bits"] + c1["clear"]))
    assert e_p < 1e-6 and e_f < 1e-6
    assert c1["bits"] + c1["clear"] < 0.5 * (c0["bits"] + c0["clear"])


def test_alignment_interpolates_square_tiles(api, scenes):
    sc = _trihedral(scenes, 40e3)
    P1, _, h1, _ = _run(api, sc, 1, 1)
    P0, _, h0, _ = _run(api, sc, 0, 1)
    Pp, _, _, _ = _run(api, sc, 1, 0)
    print("compressed: interpolated blocks %d (mean nodes %.1f) aligned, %d (mean nodes %.1f) in patch order; "
          "vs plain %.2e, %.2e" % (h1["cmp_ip_blocks"], h1["cmp_ip_nodes"], h0["cmp_ip_blocks"], h0["cmp_ip_nodes"],
                                   rel_l2(P1, Pp), rel_l2(P0, Pp)))
    assert h1["cmp_ip_nodes"] < 0.8 * h0["cmp_ip_nodes"]
    assert rel_l2(P1, Pp) < 1e-3 and rel_l2(P0, Pp) < 1e-3
