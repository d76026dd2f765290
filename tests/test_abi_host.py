"""C-ABI library on the CPU: it loads, exports every symbol of
include/sonar_render.h, fragments bit-identically to the reference, and its
host-side error handling follows the documented rules.  No GPU work runs."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden


def header_symbols():
    src = open(os.path.join(ROOT, "include", "sonar_render.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M)
    return sorted(set(n for n in names if n not in ("defined",)))


def test_exports_every_declared_symbol(api):
    names = header_symbols()
    assert "render_cuda" in names and "ProjectTargetToTargetObjects" in names
    L = C.CDLL(api.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_reference_symbol_names_present(api):
    """The 13 entry points of the reference's python_interface.cpp:13-107."""
    ref = ["load_geometry", "load_field_points", "load_source_points", "set_initial_conditions", "render_cuda",
           "ProjectSrcPointsToObjects", "ProjectTargetToFieldObjects", "ProjectTargetToFieldPoints",
           "ProjectTargetToTargetObjects", "GetFieldPointPressures", "TearDownCuda", "RenderOpenGL",
           "SoundVisualisationInit"]
    assert set(ref) <= set(header_symbols())


def test_compat_library_name(api):
    compat = os.path.join(os.path.dirname(api.LIB_PATH), "libcuda_project.so")
    assert os.path.exists(compat)
    L = C.CDLL(compat)
    assert hasattr(L, "ProjectSrcPointsToObjects")


def test_fragmentation_matches_reference_bits(api):
    g = load_golden("fragmentation")
    for k, (t, d) in enumerate(zip(g["tris"], g["deltas"])):
        (nx, ny, neg), fr, a = api.fragment_triangle(t, float(d))
        assert (nx, ny, neg) == tuple(int(v) for v in g["ints"][k]), k
        assert np.array_equal(fr.view(np.uint32), g["frames"][k].view(np.uint32)), k
        ref = g["areas"][g["offsets"][k]:g["offsets"][k + 1]]
        assert np.array_equal(a.ravel().view(np.uint32), ref.view(np.uint32)), k


def test_fragmentation_random_vs_oracle(api, oracle_mod):
    rng = np.random.default_rng(7)
    for _ in range(200):
        t = (rng.normal(size=9) * rng.uniform(0.1, 3.0)).astype(np.float32)
        d = float(rng.uniform(0.005, 0.3))
        a = api.fragment_triangle(t, d)
        b = oracle_mod.fragment_triangle(t, d)
        assert a[0] == b[0]
        assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
        assert np.array_equal(a[2].view(np.uint32), b[2].view(np.uint32))


def test_fragment_area_sum_equals_triangle_area(api, scenes):
    """The check Facet.cpp:341-361 prints: clipped cell areas add up to the area."""
    for t in list(scenes.plate_1x05()) + list(scenes.trihedral(1.0)):
        (nx, ny, neg), fr, a = api.fragment_triangle(t, 0.0197)
        assert abs(a.sum(dtype=np.float64) - fr[16]) < 2e-3 * fr[16]


def test_degenerate_triangles(api, oracle_mod):
    """Collinear vertices: FP32 rounding leaves a sliver of cells (as in the
    reference), none of them above the 1e-6 area gate; coincident vertices
    give no cells at all."""
    t = np.array([0, 0, 0, 1, 1, 1, 2, 2, 2], np.float32)
    (nx, ny, neg), fr, a = api.fragment_triangle(t, 0.1)
    b = oracle_mod.fragment_triangle(t, 0.1)
    assert (nx, ny, neg) == b[0] and np.array_equal(a.view(np.uint32), b[2].view(np.uint32))
    assert (a > 1e-6).sum() == 0
    t = np.array([1, 1, 1, 1, 1, 1, 1, 1, 1], np.float32)
    (nx, ny, neg), fr, a = api.fragment_triangle(t, 0.1)
    assert a.size == 0


def test_invalid_object_type_sets_status_without_throwing(api):
    api.TearDownCuda()
    t = np.zeros((1, 9), np.float32)
    L = api.lib()
    L.load_geometry(t.ctypes.data_as(C.POINTER(C.c_float)), 1, 7, C.c_float(0.1))
    assert api.status() != 0
    assert "objectType" in api.last_error()
    # sticky: later loads are skipped until TearDownCuda
    L.load_geometry(t.ctypes.data_as(C.POINTER(C.c_float)), 1, 0, C.c_float(0.1))
    assert api.object_count(0) == 0
    api.TearDownCuda()
    assert api.status() == 0 and api.last_error() == ""


@pytest.mark.parametrize("bad", ["nan_vertex", "zero_delta", "neg_count"])
def test_invalid_geometry_is_rejected(api, bad):
    api.TearDownCuda()
    t = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    delta, n = 0.1, 1
    if bad == "nan_vertex":
        t[0, 4] = np.nan
    elif bad == "zero_delta":
        delta = 0.0
    else:
        n = -1
    api.lib().load_geometry(t.ctypes.data_as(C.POINTER(C.c_float)), n, 0, C.c_float(delta))
    assert api.status() != 0
    with pytest.raises(api.SonarError):
        api._check()
    api.TearDownCuda()


def test_projection_before_render_is_an_error(api):
    api.TearDownCuda()
    api.lib().ProjectTargetToFieldPoints()
    assert api.status() != 0 and "render_cuda" in api.last_error()
    api.TearDownCuda()


def test_cell_count_before_render(api, scenes):
    api.TearDownCuda()
    api.load_stl_mesh_to_cuda(scenes.plate_1x05(), api.TARGET, 0.05)
    n = api.object_cells(api.TARGET, 0)
    ints, areas = api.get_fragment_layout(api.TARGET, 0)
    assert n == int((ints[:, 0] * ints[:, 1]).sum()) == areas.size
    assert abs(areas.sum() - 0.5) < 1e-3
    api.TearDownCuda()


def test_render_opengl_needs_a_rendered_scene(api, tmp_path):
    """RenderOpenGL draws headless (CUDA rasteriser); without render_cuda it
    records an error instead of drawing, and TearDownCuda clears it."""
    api.TearDownCuda()
    out = str(tmp_path / "x.png")
    L = api.lib()
    vs = (C.c_float * 9)(10.0, 10.0, 10.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0)
    L.RenderOpenGL(64, 64, out.encode(), vs)
    assert L.sonar_status() != 0
    assert "render_cuda" in api.last_error()
    assert not os.path.exists(out)
    api.TearDownCuda()
    assert L.sonar_status() == 0


def test_options(api):
    api.set_option("split", 0)
    with pytest.raises(api.SonarError):
        api.set_option("no_such_option", 1)
    s = api.stats()
    assert "hops" in s


@pytest.mark.parametrize("bad", ["too_many_sources", "no_receivers", "zero_frequency", "nan_vertex", "empty_scene",
                                 "bad_offsets"])
def test_batch_plan_validates_before_touching_the_gpu(api, bad):
    """sonar_batch_plan checks every argument before any CUDA call and
    returns a negative code with a message (no GPU needed to see it)."""
    from sonar_render_gb300 import batch
    L = batch._lib()
    f_, i_ = C.POINTER(C.c_float), C.POINTER(C.c_int)
    tris = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    off = np.array([0, 1], np.int32)
    pts = np.zeros((65, 3), np.float32)
    pts[:, 2] = 10.0
    freqs = np.array([10e3], np.float32)
    nsrc, nrx = 4, 4
    if bad == "too_many_sources":
        nsrc = 65
    elif bad == "no_receivers":
        nrx = 0
    elif bad == "zero_frequency":
        freqs = np.array([0.0], np.float32)
    elif bad == "nan_vertex":
        tris = tris.copy()
        tris[0, 4] = np.nan
    elif bad == "empty_scene":
        off = np.array([0, 0], np.int32)
    elif bad == "bad_offsets":
        off = np.array([1, 1], np.int32)
    r = L.sonar_batch_plan(tris.ctypes.data_as(f_), off.ctypes.data_as(i_), 1, pts.ctypes.data_as(f_), nsrc,
                           pts.ctypes.data_as(f_), nrx, freqs.ctypes.data_as(f_), 1, C.c_float(1480.0),
                           C.c_float(0.0), C.c_float(7.5))
    assert r < 0
    assert L.sonar_last_error().decode().startswith("sonar_batch_plan")
    assert L.sonar_batch_run(12345, None) < 0  # unknown plan id
