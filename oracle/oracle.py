"""ctypes face of the CPU oracle and of the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke`` and
by bench.py's CPU-baseline and reference legs.  The product package never
imports this module.

``Oracle`` wraps ``oracle/_build/libsonar_oracle.so`` (built from
``sonar_oracle.c`` by :func:`build`), a CPU restatement of the reference's
fragmentation (src/Facet.cpp:6-339), k (src/Model.cpp:44-54), the three sums
(src/OptiX.cu:35-406) and their sequencing (src/ModelCuda.cpp:242-356).

``RefHarness`` wraps ``oracle/_ref/libsonar_ref.so``: the reference's own
src/Facet.cpp and src/OptiX.cu compiled for the CPU by ``build_ref.sh``.  It
exists only where the reference sources were present at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsonar_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsonar_ref.so")

TARGET, SOURCE, FIELD = 0, 1, 2
HOP_SOURCE, HOP_FIELD_POINTS, HOP_SELF, HOP_FIELD_OBJECT = 0, 1, 2, 3

_f = C.POINTER(C.c_float)
_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int)
_l = C.POINTER(C.c_long)
_u8 = C.POINTER(C.c_uint8)
_vp = C.c_void_p


def build(force: bool = False) -> str:
    """Compile the oracle library with gcc (no fused multiply-add, OpenMP)."""
    srcs = [os.path.join(HERE, "sonar_oracle.c"), os.path.join(HERE, "mlp_oracle.c")]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(s) for s in srcs):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
                               "-fopenmp", "-o", tmp] + srcs + ["-lm"])
        os.replace(tmp, LIB)
    return LIB


# where the reference's sources lie in the build container (absent on the GPU
# machines, which use the harness built beforehand or none)
REFERENCE_ROOT = os.environ.get("SONAR_REFERENCE_ROOT", "/root/reference")


def build_ref(root: str | None = None) -> str | None:
    """Build the reference harness where the reference sources exist."""
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), root or REFERENCE_ROOT])
    return REF_LIB if os.path.exists(REF_LIB) else None


def _fp(a):
    return a.ctypes.data_as(_f)


def _dp(a):
    return a.ctypes.data_as(_d)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_new.restype = _vp
        L.orc_free.argtypes = [_vp]
        L.orc_add_object.argtypes = [_vp, _f, C.c_int, C.c_int, C.c_float]
        L.orc_add_sources.argtypes = [_vp, _f, C.c_int]
        L.orc_add_field_points.argtypes = [_vp, _f, C.c_int]
        L.orc_set_conditions.argtypes = [_vp, C.c_float, C.c_float, C.c_float, C.c_float]
        L.orc_set_exact_geometry.argtypes = [_vp, C.c_int]
        L.orc_get_k.argtypes = [_vp, C.c_int]
        L.orc_get_k.restype = C.c_double
        for n in ("orc_render", "orc_project_field_objects", "orc_project_field_points"):
            getattr(L, n).argtypes = [_vp]
        L.orc_project_sources.argtypes = [_vp, C.c_int]
        L.orc_project_bounces.argtypes = [_vp, C.c_int]
        L.orc_project_bounces_cross.argtypes = [_vp, C.c_int]
        L.orc_hop_subset.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _l, C.c_long, _d, _d, _u8]
        L.orc_hop_subset.restype = C.c_long
        L.orc_counter.argtypes = [_vp, C.c_int]
        L.orc_counter.restype = C.c_longlong
        L.orc_num_objects.argtypes = [_vp, C.c_int]
        for n in ("orc_object_ncells", "orc_object_nact"):
            getattr(L, n).argtypes = [_vp, C.c_int, C.c_int]
            getattr(L, n).restype = C.c_long
        L.orc_object_nfacets.argtypes = [_vp, C.c_int, C.c_int]
        L.orc_get_object_pressures.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _d]
        L.orc_set_object_pressures.argtypes = [_vp, C.c_int, C.c_int, C.c_int, _d]
        L.orc_get_areas.argtypes = [_vp, C.c_int, C.c_int, _f]
        L.orc_get_active.argtypes = [_vp, C.c_int, C.c_int, _l]
        L.orc_get_active.restype = C.c_long
        L.orc_get_facets.argtypes = [_vp, C.c_int, C.c_int, _i, _f]
        L.orc_get_field_points.argtypes = [_vp, _d]
        L.orc_fragment_triangle.argtypes = [_f, C.c_float, _i, _f, _f, C.c_long]
        L.orc_fragment_triangle.restype = C.c_long
        L.orc_segment.argtypes = [_vp, _d, _d, C.c_double, _i]
        L.orc_mlp_set_width.argtypes = [C.c_int]
        L.orc_mlp_forward.argtypes = [_f, _f, C.c_int, _d]
        L.orc_mlp_grad.argtypes = [_f, _f, _f, C.c_int, _d, _d]
        _lib = L
    return _lib


def colour_map(P, min_db, max_db, phase):
    """Reference surface colours (RGBA float32, (n, 4)) of complex pressures."""
    L = lib()
    P = np.asarray(P, dtype=np.complex128)
    buf = np.ascontiguousarray(np.stack([P.real, P.imag], axis=1))
    out = np.zeros((len(P), 4), np.float32)
    L.orc_colour_map.argtypes = [_d, C.c_long, C.c_float, C.c_float, C.c_int, _f]
    L.orc_colour_map(_dp(buf), len(P), C.c_float(min_db), C.c_float(max_db), int(phase), _fp(out))
    return out


def num_threads() -> int:
    return int(lib().orc_num_threads())


def fragment_triangle(tri9, delta):
    """(nx, ny, neg), 17 frame floats, area grid (ny, nx) of one triangle."""
    L = lib()
    t = np.ascontiguousarray(np.asarray(tri9, dtype=np.float32).reshape(9))
    ints = np.zeros(3, np.int32)
    fl = np.zeros(17, np.float32)
    n = L.orc_fragment_triangle(_fp(t), C.c_float(delta), ints.ctypes.data_as(_i), _fp(fl), None, 0)
    areas = np.zeros(max(n, 1), np.float32)
    L.orc_fragment_triangle(_fp(t), C.c_float(delta), ints.ctypes.data_as(_i), _fp(fl), _fp(areas), n)
    nx, ny, neg = (int(v) for v in ints)
    return (nx, ny, neg), fl, areas[:n].reshape(ny, nx)


def mlp_set_width(width):
    """Hidden width of the network restatement (64 or 128)."""
    lib().orc_mlp_set_width(int(width))


def mlp_param_count() -> int:
    return int(lib().orc_mlp_param_count())


def mlp_forward(params, X):
    """FP64 predictions of the admissibility network (n x 8 inputs)."""
    p = np.ascontiguousarray(params, np.float32)
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 8)
    out = np.zeros(len(X), np.float64)
    lib().orc_mlp_forward(_fp(p), _fp(X), C.c_int(len(X)), out.ctypes.data_as(_d))
    return out


def mlp_grad(params, X, y):
    """FP64 mean squared error and its gradient."""
    p = np.ascontiguousarray(params, np.float32)
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 8)
    y = np.ascontiguousarray(y, np.float32)
    g = np.zeros(mlp_param_count(), np.float64)
    loss = C.c_double(0.0)
    lib().orc_mlp_grad(_fp(p), _fp(X), _fp(y), C.c_int(len(X)), g.ctypes.data_as(_d), C.byref(loss))
    return loss.value, g


class Oracle:
    """One scene of the oracle, driven like the reference's C-ABI."""

    def __init__(self):
        self.L = lib()
        self.h = self.L.orc_new()
        self._nfp = 0

    def close(self):
        if self.h:
            self.L.orc_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- python_interface.cpp:21-59 equivalents
    def load_geometry(self, tris, object_type, resolution):
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.float32).reshape(-1, 9))
        return self.L.orc_add_object(self.h, _fp(t), int(t.shape[0]), int(object_type), C.c_float(resolution))

    def load_source_points(self, pts):
        p = np.ascontiguousarray(np.asarray(pts, dtype=np.float32).reshape(-1, 3))
        self.L.orc_add_sources(self.h, _fp(p), int(p.shape[0]))

    def load_field_points(self, pts):
        p = np.ascontiguousarray(np.asarray(pts, dtype=np.float32).reshape(-1, 3))
        self._nfp += p.shape[0]
        self.L.orc_add_field_points(self.h, _fp(p), int(p.shape[0]))

    def set_initial_conditions(self, cp, f, att, density=1000.0):
        self.L.orc_set_conditions(self.h, C.c_float(cp), C.c_float(f), C.c_float(att), C.c_float(density))

    def set_exact_geometry(self, on=True):
        """Source hop and field-point readout with FP64 distances and cosines
        from the FP32 positions (the reference rounds them in FP32)."""
        self.L.orc_set_exact_geometry(self.h, int(bool(on)))

    def k(self):
        return complex(self.L.orc_get_k(self.h, 0), self.L.orc_get_k(self.h, 1))

    def render(self):
        if self.L.orc_render(self.h) != 0:
            raise RuntimeError("oracle render failed")

    def project_sources(self, field_objects=False):
        self.L.orc_project_sources(self.h, int(bool(field_objects)))

    def project_bounces(self, n, cross_objects=False):
        """FACET_SELF bounces of every target (the reference's sequence); with
        cross_objects also FACET_RESP between every pair of targets."""
        if cross_objects:
            self.L.orc_project_bounces_cross(self.h, int(n))
        else:
            self.L.orc_project_bounces(self.h, int(n))

    def project_field_objects(self):
        self.L.orc_project_field_objects(self.h)

    def project_field_points(self):
        self.L.orc_project_field_points(self.h)

    # -- outputs
    def counters(self):
        return {k: int(self.L.orc_counter(self.h, i)) for i, k in enumerate(("pairs", "grazing", "selfplane"))}

    def ncells(self, t, i):
        return int(self.L.orc_object_ncells(self.h, t, i))

    def nact(self, t, i):
        return int(self.L.orc_object_nact(self.h, t, i))

    def pressures(self, t, i, which=0):
        out = np.zeros((self.ncells(t, i), 2))
        self.L.orc_get_object_pressures(self.h, t, i, which, _dp(out))
        return out[:, 0] + 1j * out[:, 1]

    def set_pressures(self, t, i, p, which=0):
        p = np.asarray(p, dtype=np.complex128)
        buf = np.ascontiguousarray(np.stack([p.real, p.imag], axis=1))
        self.L.orc_set_object_pressures(self.h, t, i, which, _dp(buf))

    def areas(self, t, i):
        out = np.zeros(self.ncells(t, i), np.float32)
        self.L.orc_get_areas(self.h, t, i, _fp(out))
        return out

    def active(self, t, i):
        n = self.L.orc_get_active(self.h, t, i, None)
        out = np.zeros(max(n, 1), np.int64)
        self.L.orc_get_active(self.h, t, i, out.ctypes.data_as(_l))
        return out[:n]

    def facets(self, t, i):
        nf = int(self.L.orc_object_nfacets(self.h, t, i))
        ints = np.zeros((max(nf, 1), 3), np.int32)
        fl = np.zeros((max(nf, 1), 17), np.float32)
        self.L.orc_get_facets(self.h, t, i, ints.ctypes.data_as(_i), _fp(fl))
        return ints[:nf], fl[:nf]

    def field_points(self):
        out = np.zeros((self._nfp, 2))
        self.L.orc_get_field_points(self.h, _dp(out))
        return out[:, 0] + 1j * out[:, 1]

    def hop_subset(self, hop, a_idx, b_idx, dst, pin=None, want_mask=False, nsrc=None):
        """Evaluate one hop at chosen destinations without changing state.

        Returns (values, mask) where mask[k, i] bit0 = pair interacts,
        bit1 = pair is grazing (only when want_mask)."""
        dst = np.ascontiguousarray(np.asarray(dst, dtype=np.int64))
        out = np.zeros((len(dst), 2))
        pin_p = None
        if pin is not None:
            pin = np.asarray(pin, dtype=np.complex128)
            pin_buf = np.ascontiguousarray(np.stack([pin.real, pin.imag], axis=1))
            pin_p = _dp(pin_buf)
        mask = None
        mp = None
        if want_mask:
            mask = np.zeros((len(dst), nsrc), np.uint8)
            mp = mask.ctypes.data_as(_u8)
        r = self.L.orc_hop_subset(self.h, hop, a_idx, b_idx, dst.ctypes.data_as(_l), len(dst), pin_p, _dp(out), mp)
        if r < 0:
            raise RuntimeError("orc_hop_subset failed (%d)" % r)
        return out[:, 0] + 1j * out[:, 1], mask


class RefHarness:
    """The reference's own Facet/OptiX sources run on the CPU (one global scene)."""

    def __init__(self, path=REF_LIB):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        L.ref_add_object.argtypes = [_f, C.c_int, C.c_int, C.c_float]
        L.ref_add_sources.argtypes = [_f, C.c_int]
        L.ref_add_field_points.argtypes = [_f, C.c_int]
        L.ref_set_conditions.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float]
        L.ref_project_sources.argtypes = [C.c_int]
        L.ref_project_bounces.argtypes = [C.c_int]
        L.ref_object_ncells.argtypes = [C.c_int, C.c_int]
        L.ref_object_ncells.restype = C.c_long
        L.ref_get_object_pressures.argtypes = [C.c_int, C.c_int, _d]
        L.ref_get_field_points.argtypes = [_d]
        L.ref_fragment_triangle.argtypes = [_f, C.c_float, _i, _f, _f, C.c_long]
        L.ref_fragment_triangle.restype = C.c_long
        self.L = L
        self._nfp = 0
        L.ref_reset()

    def reset(self):
        self.L.ref_reset()
        self._nfp = 0

    def load_geometry(self, tris, object_type, resolution):
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.float32).reshape(-1, 9))
        return self.L.ref_add_object(_fp(t), int(t.shape[0]), int(object_type), C.c_float(resolution))

    def load_source_points(self, pts):
        p = np.ascontiguousarray(np.asarray(pts, dtype=np.float32).reshape(-1, 3))
        self.L.ref_add_sources(_fp(p), int(p.shape[0]))

    def load_field_points(self, pts):
        p = np.ascontiguousarray(np.asarray(pts, dtype=np.float32).reshape(-1, 3))
        self._nfp += p.shape[0]
        self.L.ref_add_field_points(_fp(p), int(p.shape[0]))

    def set_initial_conditions(self, cp, f, att, density=1000.0):
        self.L.ref_set_conditions(C.c_float(cp), C.c_float(f), C.c_float(att), C.c_float(density))

    def render(self):
        if self.L.ref_render() != 0:
            raise RuntimeError("reference harness render failed")

    def project_sources(self, field_objects=False):
        self.L.ref_project_sources(int(bool(field_objects)))

    def project_bounces(self, n):
        self.L.ref_project_bounces(int(n))

    def project_field_objects(self):
        self.L.ref_project_field_objects()

    def project_field_points(self):
        self.L.ref_project_field_points()

    def pressures(self, t, i):
        n = int(self.L.ref_object_ncells(t, i))
        out = np.zeros((n, 2))
        self.L.ref_get_object_pressures(t, i, _dp(out))
        return out[:, 0] + 1j * out[:, 1]

    def field_points(self):
        out = np.zeros((self._nfp, 2))
        self.L.ref_get_field_points(_dp(out))
        return out[:, 0] + 1j * out[:, 1]

    def fragment_triangle(self, tri9, delta):
        t = np.ascontiguousarray(np.asarray(tri9, dtype=np.float32).reshape(9))
        ints = np.zeros(3, np.int32)
        fl = np.zeros(17, np.float32)
        n = self.L.ref_fragment_triangle(_fp(t), C.c_float(delta), ints.ctypes.data_as(_i), _fp(fl), None, 0)
        areas = np.zeros(max(n, 1), np.float32)
        self.L.ref_fragment_triangle(_fp(t), C.c_float(delta), ints.ctypes.data_as(_i), _fp(fl), _fp(areas), n)
        nx, ny, neg = (int(v) for v in ints)
        return (nx, ny, neg), fl, areas[:n].reshape(ny, nx)
