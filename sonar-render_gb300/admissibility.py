"""The admissibility network of the low-rank bounce blocks.

Python face of the library's ``sonar_mlp_*`` entry points and the procedure
that trains the network.  The reference evaluates every pair of every bounce;
the compressed bounce approximates blocks of 256 x 256 fragment pairs by
adaptive cross approximation, and this network decides which blocks to try
and with which rank cap.

Labels come from the exact method: a bounce with every interacting block
approximated (``compress_select`` 1) records, per block, its 8 descriptors and
log2(1 + rank) of the approximation the judge accepted (log2(1 + 2 cap) when
it rejected the block).  The library's own CUDA kernels train the network
(Adam on the mean squared error); with ``compress_select`` 2 it proposes the
blocks whose predicted rank is below ``compress_rcut`` and caps their rank at
1.5 x the prediction + 4.  The exact dense tile stays the fallback of every
block it does not propose and the judge of every block it does.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import api

_f = C.POINTER(C.c_float)
_bound = False


def _lib():
    global _bound
    L = api.lib()
    if not _bound:
        L.sonar_mlp_param_count.restype = C.c_int
        L.sonar_mlp_set_width.argtypes = [C.c_int]
        L.sonar_mlp_width.restype = C.c_int
        L.sonar_mlp_init.argtypes = [C.c_uint]
        L.sonar_mlp_set_params.argtypes = [_f, C.c_longlong]
        L.sonar_mlp_get_params.argtypes = [_f, C.c_longlong]
        L.sonar_mlp_grad.argtypes = [_f, _f, C.c_int, _f, _f]
        L.sonar_mlp_train.argtypes = [_f, _f, C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint, _f]
        L.sonar_mlp_predict.argtypes = [_f, C.c_int, _f]
        L.sonar_get_block_samples.argtypes = [_f, _f, C.c_longlong]
        L.sonar_get_block_samples.restype = C.c_longlong
        _bound = True
    return L


def _call(r, what):
    if r != 0:
        L = api.lib()
        msg = L.sonar_last_error().decode()
        L.sonar_clear_error()
        raise api.SonarError("%s failed (%d): %s" % (what, r, msg))


def _fa(a):
    return a.ctypes.data_as(_f)


def set_width(width: int):
    """Hidden width 64 (FP32 inference) or 128 (FP16 hidden layers on the
    tensor cores); drops the parameters."""
    _call(_lib().sonar_mlp_set_width(int(width)), "sonar_mlp_set_width")


def width() -> int:
    return int(_lib().sonar_mlp_width())


def param_count() -> int:
    return int(_lib().sonar_mlp_param_count())


def init(seed: int = 0):
    _call(_lib().sonar_mlp_init(int(seed)), "sonar_mlp_init")


def set_params(p):
    p = np.ascontiguousarray(p, np.float32)
    _call(_lib().sonar_mlp_set_params(_fa(p), len(p)), "sonar_mlp_set_params")


def get_params():
    p = np.zeros(param_count(), np.float32)
    _call(_lib().sonar_mlp_get_params(_fa(p), len(p)), "sonar_mlp_get_params")
    return p


def grad(X, y):
    """Mean squared error and its gradient from the GPU's backward kernels."""
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 8)
    y = np.ascontiguousarray(y, np.float32)
    g = np.zeros(param_count(), np.float32)
    loss = C.c_float(0.0)
    _call(_lib().sonar_mlp_grad(_fa(X), _fa(y), len(X), _fa(g), C.byref(loss)), "sonar_mlp_grad")
    return float(loss.value), g


def train(X, y, epochs=40, batch=256, lr=1e-3, seed=0):
    """Adam on the GPU; returns the mean squared error of the last epoch."""
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 8)
    y = np.ascontiguousarray(y, np.float32)
    loss = C.c_float(0.0)
    _call(_lib().sonar_mlp_train(_fa(X), _fa(y), len(X), int(epochs), int(batch), float(lr), int(seed),
                                 C.byref(loss)), "sonar_mlp_train")
    return float(loss.value)


def predict(X):
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 8)
    out = np.zeros(len(X), np.float32)
    _call(_lib().sonar_mlp_predict(_fa(X), len(X), _fa(out)), "sonar_mlp_predict")
    return out


def block_samples():
    """(descriptors n x 8, labels n) of the blocks the last compressed bounce
    approximated."""
    L = _lib()
    n = int(L.sonar_get_block_samples(None, None, 0))
    X = np.zeros((max(n, 1), 8), np.float32)
    y = np.zeros(max(n, 1), np.float32)
    if n > 0:
        L.sonar_get_block_samples(_fa(X), _fa(y), n)
    return X[:n], y[:n]


def label_scene(cfg, rmax=32):
    """Run the source hop and one bounce of a scene with every interacting
    block approximated; return its block samples (descriptors, labels)."""
    api.set_option("compress", 1)
    api.set_option("compress_select", 1)
    api.set_option("compress_rmax", rmax)
    try:
        api.TearDownCuda()
        api.run_scene(cfg, bounces=1, field_objects=False, field_points=False)
        return block_samples()
    finally:
        api.set_option("compress_select", 0)
        api.set_option("compress", 0)
        api.TearDownCuda()


def train_on_scenes(cfgs, epochs=40, batch=256, lr=1e-3, seed=0, rmax=32):
    """Label every scene with the exact method, initialise and train the
    network; returns (X, y, final loss)."""
    Xs, ys = [], []
    for cfg in cfgs:
        X, y = label_scene(cfg, rmax=rmax)
        Xs.append(X)
        ys.append(y)
    X = np.concatenate(Xs)
    y = np.concatenate(ys)
    init(seed)
    loss = train(X, y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return X, y, loss
