"""Many sources, receivers, frequencies and scenes in one run.

Python face of the library's ``sonar_batch_*`` entry points.  The reference
scripts answer "what does receiver p hear when source q radiates" with one
render per source and frequency (load_source_points, set_initial_conditions,
ProjectSrcPointsToObjects, ProjectTargetToFieldPoints, GetFieldPointPressures;
run_scripts/modules/mh.py:43-70).  A batch plan does all of them at once:
every (scene, frequency) item is fragmented and uploaded once, and a run is
one CUDA graph whose main kernel materialises the readout and incident
Green's-function tiles in shared memory and contracts them on the tensor
cores (split BF16, FP32 accumulation, FP64 per-item reduction).

``Plan.run()`` returns ``out[scene, freq, receiver, source]`` (complex128).
"""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from . import api

_f = C.POINTER(C.c_float)
_d = C.POINTER(C.c_double)
_i = C.POINTER(C.c_int)
_bound = False

MAX_POINTS = 64


def _lib():
    global _bound
    L = api.lib()
    if not _bound:
        L.sonar_batch_plan.argtypes = [_f, _i, C.c_int, _f, C.c_int, _f, C.c_int, _f, C.c_int, C.c_float,
                                       C.c_float, C.c_float]
        L.sonar_batch_plan.restype = C.c_longlong
        L.sonar_batch_run.argtypes = [C.c_longlong, _d]
        L.sonar_batch_stats.argtypes = [C.c_longlong, C.c_char_p, C.c_int]
        L.sonar_batch_stream.argtypes = [C.c_longlong, C.POINTER(C.c_void_p)]
        L.sonar_batch_set_points.argtypes = [C.c_longlong, _f, C.c_int, _f, C.c_int]
        L.sonar_batch_set_shape.argtypes = [C.c_longlong, C.c_int, C.c_int]
        L.sonar_batch_set_relative.argtypes = [C.c_longlong, C.c_int]
        L.sonar_batch_free.argtypes = [C.c_longlong]
        L.sonar_run_batch.argtypes = [_f, _i, C.c_int, _f, C.c_int, _f, C.c_int, _f, C.c_int, C.c_float,
                                      C.c_float, C.c_float, _d]
        L.sonar_last_error.restype = C.c_char_p
        _bound = True
    return L


def _err(what, code):
    return api.SonarError("%s failed (%d): %s" % (what, code, _lib().sonar_last_error().decode()))


def _inputs(scenes, sources, receivers, freqs):
    tris = [np.asarray(t, dtype=np.float32).reshape(-1, 9) for t in scenes]
    off = np.zeros(len(tris) + 1, np.int32)
    off[1:] = np.cumsum([t.shape[0] for t in tris])
    T = np.ascontiguousarray(np.concatenate(tris, axis=0)) if tris else np.zeros((0, 9), np.float32)
    S = np.ascontiguousarray(np.asarray(sources, dtype=np.float32).reshape(-1, 3))
    R = np.ascontiguousarray(np.asarray(receivers, dtype=np.float32).reshape(-1, 3))
    F = np.ascontiguousarray(np.asarray(freqs, dtype=np.float32).reshape(-1))
    return T, off, S, R, F


class Plan:
    """One batch: fragments, masks and the captured run graph on the GPU."""

    def __init__(self, scenes, sources, receivers, freqs, cp=1480.0, attenuation=0.0, per_wavelength=7.5):
        L = _lib()
        T, off, S, R, F = _inputs(scenes, sources, receivers, freqs)
        self._keep = (T, off, S, R, F)
        self.shape = (len(scenes), F.shape[0], R.shape[0], S.shape[0])
        pid = L.sonar_batch_plan(T.ctypes.data_as(_f), off.ctypes.data_as(_i), len(scenes), S.ctypes.data_as(_f),
                                 S.shape[0], R.ctypes.data_as(_f), R.shape[0], F.ctypes.data_as(_f), F.shape[0],
                                 C.c_float(cp), C.c_float(attenuation), C.c_float(per_wavelength))
        if pid <= 0:
            raise _err("sonar_batch_plan", pid)
        self.id = int(pid)
        self._out = np.zeros(self.shape + (2,), np.float64)

    def run(self, copy=True):
        """Replay the run graph; the result as complex128 [scene, freq, rx, src]
        (None when copy is False: the result stays on the device)."""
        r = _lib().sonar_batch_run(self.id, self._out.ctypes.data_as(_d) if copy else None)
        if r != 0:
            raise _err("sonar_batch_run", r)
        if not copy:
            return None
        return self._out[..., 0] + 1j * self._out[..., 1]

    def set_points(self, sources, receivers):
        """New source and receiver positions (same counts) for the next run."""
        S = np.ascontiguousarray(np.asarray(sources, np.float32).reshape(-1, 3))
        R = np.ascontiguousarray(np.asarray(receivers, np.float32).reshape(-1, 3))
        r = _lib().sonar_batch_set_points(self.id, S.ctypes.data_as(_f), S.shape[0], R.ctypes.data_as(_f), R.shape[0])
        if r != 0:
            raise _err("sonar_batch_set_points", r)

    def set_shape(self, fragments_per_stage, ctas_per_sm):
        """Run with this tile shape instead of the tuned one."""
        r = _lib().sonar_batch_set_shape(self.id, int(fragments_per_stage), int(ctas_per_sm))
        if r != 0:
            raise _err("sonar_batch_set_shape", r)

    def set_relative(self, on=True):
        """Centroid-relative phase (FP64 point offsets from each scene's box
        centre) instead of the reference's absolute FP32 distances."""
        r = _lib().sonar_batch_set_relative(self.id, int(bool(on)))
        if r != 0:
            raise _err("sonar_batch_set_relative", r)

    def stats(self):
        L = _lib()
        n = L.sonar_batch_stats(self.id, None, 0)
        if n < 0:
            raise _err("sonar_batch_stats", n)
        buf = C.create_string_buffer(n + 1)
        L.sonar_batch_stats(self.id, buf, n + 1)
        return json.loads(buf.value.decode())

    def stream_handle(self):
        s = C.c_void_p()
        r = _lib().sonar_batch_stream(self.id, C.byref(s))
        if r != 0:
            raise _err("sonar_batch_stream", r)
        return int(s.value or 0)

    def close(self):
        if getattr(self, "id", 0):
            _lib().sonar_batch_free(self.id)
            self.id = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_batch(scenes, sources, receivers, freqs, cp=1480.0, attenuation=0.0, per_wavelength=7.5):
    """Plan, run and free in one call (sonar_run_batch)."""
    L = _lib()
    T, off, S, R, F = _inputs(scenes, sources, receivers, freqs)
    out = np.zeros((len(scenes), F.shape[0], R.shape[0], S.shape[0], 2), np.float64)
    r = L.sonar_run_batch(T.ctypes.data_as(_f), off.ctypes.data_as(_i), len(scenes), S.ctypes.data_as(_f),
                          S.shape[0], R.ctypes.data_as(_f), R.shape[0], F.ctypes.data_as(_f), F.shape[0],
                          C.c_float(cp), C.c_float(attenuation), C.c_float(per_wavelength),
                          out.ctypes.data_as(_d))
    if r != 0:
        raise _err("sonar_run_batch", r)
    return out[..., 0] + 1j * out[..., 1]
