"""sonar_readout_noalloc: the readout for callers that cannot allocate device
memory (their framework owns every device byte, or they allocate only at
start-up).  They pass their own device buffers; the library's only scratch is
a fixed array inside the library.

The test runs the library's usual readout (ProjectTargetToFieldPoints) on a
plate, which nothing occludes, then feeds the same fragments -- centroids,
areas, normals and the pressures the source hop left -- to the no-allocation
entry point through the C ABI twice in a row, and compares both results with
the usual readout at the tolerance of the other parity tests (1e-5 relative
L2).  This file is collected last so that a failure here never hides the
other tests' results.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _fragments(api, tris, delta, P):
    """Active fragments in the library's order: centroid (no x shift), area,
    normal and pressure, with the library's FP32 rounding."""
    pos, nrm, pres = [], [], []
    cell0 = 0
    d = np.float32(delta)
    for t in tris:
        (nx, ny, neg), fr, a = api.fragment_triangle(t, delta)
        ys, xs = np.nonzero(a > 1e-6)
        xo = d * (xs - neg).astype(np.float32)
        yo = d * ys.astype(np.float32) + d / np.float32(2)
        base, xa, ya = fr[3:6], fr[6:9], fr[9:12]
        p = (base[None, :] + xa[None, :] * xo[:, None]) + ya[None, :] * yo[:, None]
        pos.append(np.concatenate([p, a[ys, xs][:, None]], axis=1))
        nrm.append(np.tile(np.append(fr[0:3], 0.0).astype(np.float32), (len(xs), 1)))
        pres.append(P[cell0 + ys * nx + xs])
        cell0 += nx * ny
    pres = np.concatenate(pres)
    return (np.ascontiguousarray(np.concatenate(pos), np.float32), np.ascontiguousarray(np.concatenate(nrm)),
            np.ascontiguousarray(np.stack([pres.real, pres.imag], axis=1)))


def _k(cp, f):
    omega = np.float32(2 * np.pi * np.float64(np.float32(f)))
    return float(np.float32(omega / np.float32(cp)))


def test_noalloc_readout_matches_library_readout(api, scenes):
    import torch
    cfg = scenes.plate_config()
    tris, delta = cfg["targets"][0]
    pts = scenes.grid_xy(32, 1.0, 3.0)
    api.TearDownCuda()
    api.set_initial_conditions(cfg["cp"], cfg["frequency"], 0.0)
    api.load_stl_mesh_to_cuda(tris, api.TARGET, delta)
    api.load_points_to_cuda(cfg["sources"], isSource=True)
    api.load_points_to_cuda(pts, isSource=False)
    api.render_cuda()
    api.project_source_points_to_objects(False)
    P = api.get_object_pressures(api.TARGET, 0)
    api.project_target_to_field_points()
    ref = api.get_field_point_pressures(len(pts))
    api.TearDownCuda()

    pos, nrm, pres = _fragments(api, tris, delta, P)
    assert len(pos) > 1200
    dev = torch.device("cuda", torch.cuda.current_device())
    t_pos = torch.from_numpy(pos).to(dev)
    t_nrm = torch.from_numpy(nrm).to(dev)
    t_pres = torch.from_numpy(pres).to(dev)
    t_pts = torch.from_numpy(np.ascontiguousarray(np.concatenate([pts, np.zeros((len(pts), 1), np.float32)], 1))).to(dev)
    out = torch.zeros((len(pts), 2), dtype=torch.float64, device=dev)
    L = api.lib()
    L.sonar_readout_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                        C.c_float, C.c_float, C.c_void_p, C.c_void_p]
    L.sonar_readout_noalloc.restype = C.c_int
    k = _k(cfg["cp"], cfg["frequency"])
    stream = torch.cuda.current_stream(dev).cuda_stream
    results = []
    for _ in range(2):  # two calls in a row share the library's scratch array
        out.zero_()
        rc = L.sonar_readout_noalloc(t_pos.data_ptr(), t_nrm.data_ptr(), t_pres.data_ptr(), len(pos),
                                     t_pts.data_ptr(), len(pts), k, 0.0, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize(dev)
        o = out.cpu().numpy()
        results.append(o[:, 0] + 1j * o[:, 1])
    for r in results:
        err = rel_l2(r, ref)
        print("no-alloc readout vs ProjectTargetToFieldPoints: rel L2 %.3e" % err)
        assert err < 1e-5
    assert rel_l2(results[0], results[1]) < 1e-12


def test_noalloc_rejects_too_many_points(api):
    L = api.lib()
    L.sonar_readout_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                        C.c_float, C.c_float, C.c_void_p, C.c_void_p]
    L.sonar_readout_noalloc.restype = C.c_int
    rc = L.sonar_readout_noalloc(None, None, None, 0, None, 524288 + 1, 1.0, 0.0, None, None)
    assert rc == -2
    assert L.sonar_readout_noalloc(None, None, None, -1, None, 4, 1.0, 0.0, None, None) == -1
