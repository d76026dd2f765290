"""Python binding of the GB300 library, mirroring the reference's ctypes module
(run_scripts/modules/api.py:1-111): the same function names, argument meaning
and call order, over the same C symbols (include/sonar_render.h).

Differences from the reference wrapper:
  * ``set_initial_conditions`` passes all four arguments of the C function
    (the reference passes three to a four-argument function, api.py:11-14);
  * ``project_target_to_field_points`` calls ProjectTargetToFieldPoints (the
    reference calls the field-objects symbol, api.py:96-98);
  * ``load_stl_mesh_to_cuda`` takes an object with ``.vectors`` (numpy-stl) or
    any (n, 9) / (n, 3, 3) array;
  * every call checks the library status and raises ``SonarError`` when the
    library recorded an error (the C functions themselves never throw).

The library is loaded from ``build/libsonar_gb300.so`` next to this file
(built by ``build.py``).  There is no CPU fallback: without the library every
call raises.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libsonar_gb300.so")

TARGET, SOURCE, FIELD = 0, 1, 2
HOP_SOURCE, HOP_FIELD_POINTS, HOP_SELF, HOP_FIELD_OBJECT = 0, 1, 2, 3


class SonarError(RuntimeError):
    pass


_lib = None
_f = C.POINTER(C.c_float)
_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int)


def load_library(path: str | None = None, build: bool = False):
    """Load (optionally building first) the C-ABI library."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if build or not os.path.exists(path):
        if not build:
            raise SonarError("GB300 library not built: %s (run build.py)" % path)
        import importlib.util
        spec = importlib.util.spec_from_file_location("_sonar_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
    L = C.CDLL(path)
    L.set_initial_conditions.argtypes = [C.c_float] * 4
    L.load_geometry.argtypes = [_f, C.c_int, C.c_int, C.c_float]
    L.load_field_points.argtypes = [_f, C.c_int]
    L.load_source_points.argtypes = [_f, C.c_int]
    L.ProjectSrcPointsToObjects.argtypes = [C.c_bool]
    L.ProjectTargetToTargetObjects.argtypes = [C.c_int]
    L.GetFieldPointPressures.argtypes = [_d, C.c_int]
    L.RenderOpenGL.argtypes = [C.c_int, C.c_int, C.c_char_p, _f]
    L.SoundVisualisationInit.argtypes = [C.c_float, C.c_float, C.c_bool, C.c_bool]
    for n in ("render_cuda", "ProjectTargetToFieldObjects", "ProjectTargetToFieldPoints", "TearDownCuda",
              "set_initial_conditions", "load_geometry", "load_field_points", "load_source_points",
              "ProjectSrcPointsToObjects", "ProjectTargetToTargetObjects", "GetFieldPointPressures",
              "RenderOpenGL", "SoundVisualisationInit", "sonar_clear_error"):
        getattr(L, n).restype = None
    L.sonar_status.restype = C.c_int
    L.sonar_last_error.restype = C.c_char_p
    L.sonar_get_object_count.argtypes = [C.c_int]
    L.sonar_get_object_cells.argtypes = [C.c_int, C.c_int]
    L.sonar_get_object_cells.restype = C.c_longlong
    L.sonar_get_object_pressures.argtypes = [C.c_int, C.c_int, _d, C.c_longlong]
    L.sonar_get_fragment_layout.argtypes = [C.c_int, C.c_int, _i, C.c_int, _f, C.c_longlong]
    L.sonar_get_stats.argtypes = [C.c_char_p, C.c_int]
    L.sonar_set_option.argtypes = [C.c_char_p, C.c_double]
    L.sonar_get_mask.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_ubyte), C.c_longlong]
    L.sonar_get_mask.restype = C.c_longlong
    L.sonar_get_mask_rows.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_ubyte),
                                      C.c_longlong]
    L.sonar_get_mask_rows.restype = C.c_longlong
    L.sonar_audit_compression.argtypes = [C.c_int, C.c_uint, _f, _f, C.c_int]
    L.sonar_audit_compression.restype = C.c_int
    L.sonar_get_stream.restype = C.c_void_p
    L.sonar_get_surface_colours.argtypes = [C.c_int, C.c_int, _f, C.c_longlong]
    L.sonar_measure_peak.argtypes = [C.c_int]
    L.sonar_measure_peak.restype = C.c_double
    L.sonar_fragment_triangle.argtypes = [_f, C.c_float, _i, _f, _f, C.c_longlong]
    L.sonar_fragment_triangle.restype = C.c_longlong
    L.sonar_tile_order.argtypes = [_f, C.c_float, C.c_longlong, _i, C.c_longlong]
    L.sonar_tile_order.restype = C.c_longlong
    _lib = L
    return L


def lib():
    return load_library()


def _check():
    L = lib()
    st = L.sonar_status()
    if st != 0:
        raise SonarError("sonar error %d: %s" % (st, L.sonar_last_error().decode()))


def status():
    return int(lib().sonar_status())


def last_error():
    return lib().sonar_last_error().decode()


def clear_error():
    lib().sonar_clear_error()


# ---------------------------------------------------------------- reference API
def set_initial_conditions(cp, frequency, attenuation, density=1000.0):
    """Sets the wave number k = 2 pi f / cp (+ i attenuation)."""
    lib().set_initial_conditions(cp, frequency, attenuation, density)
    _check()


def load_points_to_cuda(points, isSource=False):
    """Loads source points (isSource) or field points."""
    p = np.ascontiguousarray(np.asarray(points, dtype=np.float32).reshape(-1, 3))
    ptr = p.ctypes.data_as(_f)
    if isSource:
        lib().load_source_points(ptr, int(p.shape[0]))
    else:
        lib().load_field_points(ptr, int(p.shape[0]))
    _check()


def _triangles(mesh):
    v = getattr(mesh, "vectors", mesh)
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(-1, 9))


def load_stl_mesh_to_cuda(stl_mesh, object_type, resolution=2e-3):
    """Loads a target (0), source (1) or field (2) surface."""
    t = _triangles(stl_mesh)
    lib().load_geometry(t.ctypes.data_as(_f), int(t.shape[0]), int(object_type), float(resolution))
    _check()


def render_cuda():
    """Fragment the loaded surfaces and upload the scene."""
    lib().render_cuda()
    _check()


def GetFieldPoints(NumFieldPnts):
    """Field point pressures as an (n, 2) array of (real, imag)."""
    out = np.zeros((NumFieldPnts, 2), dtype=np.double)
    lib().GetFieldPointPressures(out.ctypes.data_as(_d), int(NumFieldPnts))
    _check()
    return out


def render_openGL(width, height, viewSettings, filename="output"):
    """GL rendering is not available; records the reason (see last_error)."""
    vs = (C.c_float * len(viewSettings))(*viewSettings)
    lib().RenderOpenGL(int(width), int(height), (filename + ".png").encode(), vs)


def TearDownCuda():
    lib().TearDownCuda()


def project_source_points_to_objects(project_to_field_surface=False):
    lib().ProjectSrcPointsToObjects(bool(project_to_field_surface))
    _check()


def project_target_to_field_objects():
    lib().ProjectTargetToFieldObjects()
    _check()


def project_target_to_field_points():
    lib().ProjectTargetToFieldPoints()
    _check()


def project_target_to_target_objects(number_reflections):
    lib().ProjectTargetToTargetObjects(int(number_reflections))
    _check()


def sound_visualisation_init(max_db, min_db, render_phase_target, render_phase_field):
    lib().SoundVisualisationInit(max_db, min_db, bool(render_phase_target), bool(render_phase_field))


# ---------------------------------------------------------------- additive API
def object_count(object_type):
    return int(lib().sonar_get_object_count(int(object_type)))


def object_cells(object_type, idx=0):
    return int(lib().sonar_get_object_cells(int(object_type), int(idx)))


def get_object_pressures(object_type, idx=0):
    """Total pressure of every cell (facet-major, row-major y*nx + x) as complex128."""
    n = object_cells(object_type, idx)
    out = np.empty(max(n, 0), dtype=np.complex128)  # (re, im) double pairs, written in place
    r = lib().sonar_get_object_pressures(int(object_type), int(idx), out.ctypes.data_as(_d), n)
    _check()
    if r < 0:
        raise SonarError("sonar_get_object_pressures failed (%d)" % r)
    return out


def get_surface_colours(object_type, idx=0):
    """RGBA colours (float32, (ncells, 4)) of an object's surface cells."""
    n = object_cells(object_type, idx)
    out = np.zeros((max(n, 0), 4), dtype=np.float32)
    r = lib().sonar_get_surface_colours(int(object_type), int(idx), out.ctypes.data_as(_f), n)
    _check()
    if r < 0:
        raise SonarError("sonar_get_surface_colours failed (%d)" % r)
    return out


def get_field_point_pressures(n):
    v = GetFieldPoints(n)
    return v[:, 0] + 1j * v[:, 1]


def get_fragment_layout(object_type, idx=0):
    """((nfacets, 3) int32 nx/ny/neg, FP32 cell areas)."""
    L = lib()
    nf = L.sonar_get_fragment_layout(int(object_type), int(idx), None, 0, None, 0)
    if nf < 0:
        _check()
        raise SonarError("layout failed (%d)" % nf)
    ints = np.zeros((max(nf, 1), 3), np.int32)
    L.sonar_get_fragment_layout(int(object_type), int(idx), ints.ctypes.data_as(_i), nf, None, 0)
    n = int((ints[:nf, 0].astype(np.int64) * ints[:nf, 1]).sum())
    areas = np.zeros(max(n, 1), np.float32)
    L.sonar_get_fragment_layout(int(object_type), int(idx), None, 0, areas.ctypes.data_as(_f), n)
    _check()
    return ints[:nf], areas[:n]


def get_mask(hop, src_idx, dst_idx):
    """Interaction mask (ndst, nsrc) as uint8 (see sonar_get_mask)."""
    L = lib()
    n = L.sonar_get_mask(int(hop), int(src_idx), int(dst_idx), None, 0)
    _check()
    out = np.zeros(max(n, 1), np.uint8)
    r = L.sonar_get_mask(int(hop), int(src_idx), int(dst_idx), out.ctypes.data_as(C.POINTER(C.c_ubyte)), n)
    _check()
    if r < 0:
        raise SonarError("sonar_get_mask failed (%d)" % r)
    return out[:n]


def audit_compression(nsample=256, seed=0):
    """Full-tile errors of sampled accepted blocks of the last compressed
    bounce and the judge's sampled errors of the same blocks (see
    sonar_audit_compression): two float32 arrays."""
    full = np.zeros(max(nsample, 1), np.float32)
    judged = np.zeros(max(nsample, 1), np.float32)
    n = lib().sonar_audit_compression(int(nsample), int(seed), full.ctypes.data_as(_f), judged.ctypes.data_as(_f),
                                      int(nsample))
    _check()
    if n < 0:
        raise SonarError("sonar_audit_compression failed (%d)" % n)
    return full[:n], judged[:n]


def get_mask_rows(hop, src_idx, dst_idx, rows):
    """Rows of the interaction mask, (len(rows), nsrc) uint8 (see
    sonar_get_mask_rows)."""
    L = lib()
    rows = np.ascontiguousarray(np.asarray(rows, dtype=np.int32))
    rp = rows.ctypes.data_as(C.POINTER(C.c_int))
    n = L.sonar_get_mask_rows(int(hop), int(src_idx), int(dst_idx), rp, len(rows), None, 0)
    _check()
    out = np.zeros(max(n, 1), np.uint8)
    r = L.sonar_get_mask_rows(int(hop), int(src_idx), int(dst_idx), rp, len(rows),
                              out.ctypes.data_as(C.POINTER(C.c_ubyte)), n)
    _check()
    if r < 0:
        raise SonarError("sonar_get_mask_rows failed (%d)" % r)
    return out[:n].reshape(len(rows), -1)


def stats():
    L = lib()
    n = L.sonar_get_stats(None, 0)
    buf = C.create_string_buffer(n + 1)
    L.sonar_get_stats(buf, n + 1)
    return json.loads(buf.value.decode())


def set_option(key, value):
    r = lib().sonar_set_option(key.encode(), float(value))
    if r != 0:
        raise SonarError("unknown option %r" % key)


def measure_peak(which):
    """FP32 FLOP/s (0) or MUFU op/s (1) of the current GPU, measured now."""
    return float(lib().sonar_measure_peak(int(which)))


def stream_handle():
    """The library's cudaStream_t as an int (0 before render_cuda)."""
    return int(lib().sonar_get_stream() or 0)


def fragment_triangle(tri9, delta):
    """Host-only fragmentation of one triangle: ((nx, ny, neg), frame17, areas (ny, nx))."""
    L = lib()
    t = np.ascontiguousarray(np.asarray(tri9, dtype=np.float32).reshape(9))
    ints = np.zeros(3, np.int32)
    fr = np.zeros(17, np.float32)
    n = L.sonar_fragment_triangle(t.ctypes.data_as(_f), C.c_float(delta), ints.ctypes.data_as(_i),
                                  fr.ctypes.data_as(_f), None, 0)
    if n < 0:
        raise SonarError("sonar_fragment_triangle failed (%d)" % n)
    a = np.zeros(max(n, 1), np.float32)
    L.sonar_fragment_triangle(t.ctypes.data_as(_f), C.c_float(delta), ints.ctypes.data_as(_i),
                              fr.ctypes.data_as(_f), a.ctypes.data_as(_f), n)
    nx, ny, neg = (int(v) for v in ints)
    return (nx, ny, neg), fr, a[:n].reshape(ny, nx)


def tile_order(tri9, delta, start=0):
    """Host-only: the (x, y) grid cells of one triangle's active fragments in
    the order render_cuda stores them when the first one has index start
    (see sonar_tile_order); an (n, 2) int32 array."""
    L = lib()
    t = np.ascontiguousarray(np.asarray(tri9, dtype=np.float32).reshape(9))
    n = L.sonar_tile_order(t.ctypes.data_as(_f), C.c_float(delta), C.c_longlong(start), None, 0)
    if n < 0:
        raise SonarError("sonar_tile_order failed (%d)" % n)
    xy = np.zeros((max(n, 1), 2), np.int32)
    L.sonar_tile_order(t.ctypes.data_as(_f), C.c_float(delta), C.c_longlong(start), xy.ctypes.data_as(_i),
                       C.c_longlong(n))
    return xy[:n]


def run_scene(cfg, bounces=None, field_objects=True, field_points=True):
    """Load a scene dict (scenes.py), render and run the canonical order of the
    reference's run_rendering (run_scripts/modules/mh.py:43-70): sources ->
    objects, bounces, target -> field objects, target -> field points."""
    set_initial_conditions(cfg["cp"], cfg["frequency"], cfg.get("attenuation", 0.0))
    for tris, d in cfg["targets"]:
        load_stl_mesh_to_cuda(tris, TARGET, d)
    for tris, d in cfg.get("fields", []):
        load_stl_mesh_to_cuda(tris, FIELD, d)
    load_points_to_cuda(cfg["sources"], isSource=True)
    if cfg.get("field_points") is not None:
        load_points_to_cuda(cfg["field_points"], isSource=False)
    render_cuda()
    project_source_points_to_objects(False)
    nb = cfg.get("bounces", 0) if bounces is None else bounces
    if nb > 0:
        project_target_to_target_objects(nb)
    if field_objects and cfg.get("fields"):
        project_target_to_field_objects()
    if field_points and cfg.get("field_points") is not None:
        project_target_to_field_points()
