"""Centroid-relative geometry of the source hop and the field-point readout
(option relative_geometry) at long range.

The reference forms every distance from absolute FP32 positions
(src/OptiX.cu:45-57, :150-153): at 30 m an FP32 coordinate is good to about
1e-6 m, i.e. 2e-4 rad of phase at 40 kHz.  The library's default path keeps
that rounding (parity with the reference, checked against the FP64 oracle,
which restates it).  With relative_geometry the phase distance is formed from
FP64 references -- the readout as r = R + (|o|^2 - 2 o.D) / (r + R) with o the
fragment's offset from its tile's centroid and R the FP64 distance of the
field point to that centroid, the source hop from its FP64 difference -- and
against the oracle's exact-geometry mode (FP64 distances from the same FP32
positions) its error must fall well below the default path's.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _scene(scenes):
    f = 40e3
    tris = scenes.plate_1x05()
    src = np.array([[3.0, 2.0, 29.7]], np.float32)  # ~30 m
    ang = np.linspace(-50.0, 50.0, 96)
    fp = scenes.arc_xz(30.0, ang)
    return f, tris, scenes.delta_for(f), src, fp


def _gpu(api, f, tris, delta, src, fp, rel):
    api.set_option("relative_geometry", rel)
    try:
        api.TearDownCuda()
        api.set_initial_conditions(1480.0, f, 0.0)
        api.load_stl_mesh_to_cuda(tris, api.TARGET, delta)
        api.load_points_to_cuda(src, isSource=True)
        api.load_points_to_cuda(fp, isSource=False)
        api.render_cuda()
        api.project_source_points_to_objects(False)
        P = api.get_object_pressures(api.TARGET, 0)
        api.project_target_to_field_points()
        F = api.get_field_point_pressures(len(fp))
        api.TearDownCuda()
    finally:
        api.set_option("relative_geometry", 0)
    return P, F


def _oracle(oracle_mod, f, tris, delta, src, fp, exact, P=None):
    o = oracle_mod.Oracle()
    o.set_initial_conditions(1480.0, f, 0.0)
    o.load_geometry(tris, 0, delta)
    o.load_source_points(src)
    o.load_field_points(fp)
    o.render()
    o.set_exact_geometry(exact)
    o.project_sources(False)
    Po = o.pressures(0, 0)
    if P is not None:
        o.set_pressures(0, 0, P)
    o.project_field_points()
    Fo = o.field_points()
    o.close()
    return Po, Fo


def test_relative_geometry_at_30m(api, oracle_mod, scenes):
    f, tris, delta, src, fp = _scene(scenes)
    P_abs, F_abs = _gpu(api, f, tris, delta, src, fp, 0)
    P_rel, F_rel = _gpu(api, f, tris, delta, src, fp, 1)
    # parity of the default path with the reference's rounding
    Pr, Fr = _oracle(oracle_mod, f, tris, delta, src, fp, False, P=P_abs)
    e_par_src, e_par_fp = rel_l2(P_abs, Pr), rel_l2(F_abs, Fr)
    # both paths against exact geometry, each readout given its own input
    Pe, Fe_abs = _oracle(oracle_mod, f, tris, delta, src, fp, True, P=P_abs)
    _, Fe_rel = _oracle(oracle_mod, f, tris, delta, src, fp, True, P=P_rel)
    e_abs_src, e_rel_src = rel_l2(P_abs, Pe), rel_l2(P_rel, Pe)
    e_abs_fp, e_rel_fp = rel_l2(F_abs, Fe_abs), rel_l2(F_rel, Fe_rel)
    print("30 m, 40 kHz: parity with the reference's rounding: source hop %.2e, readout %.2e" % (e_par_src, e_par_fp))
    print("against exact geometry: source hop %.2e (default) -> %.2e (relative), readout %.2e -> %.2e"
          % (e_abs_src, e_rel_src, e_abs_fp, e_rel_fp))
    assert e_par_src < 1e-5 and e_par_fp < 1e-5
    assert e_rel_src < 1e-5 and e_rel_fp < 1e-5
    assert e_rel_src < 0.3 * e_abs_src
    assert e_rel_fp < 0.5 * e_abs_fp
