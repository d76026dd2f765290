"""sonar_readout_noalloc: the readout for callers that cannot allocate device
memory (their framework owns every device byte, or they allocate only at
start-up).  They pass their own device buffers; the library's only scratch is
a fixed array inside the library.

Each case runs the library's usual readout (ProjectTargetToFieldPoints) on a
plate, which nothing occludes, then feeds the same fragments -- centroids,
areas, normals and the pressures the source hop left -- to the
no-allocation entry point through the C ABI twice in a row, and compares both
results with the usual readout and with the FP64 oracle at the tolerance of
the other parity tests (1e-5 relative L2).  The cases cover an attenuating
medium (k_im != 0), several tiles per source split and a field-point count
large enough that the scratch size caps the number of splits, and the
device's free memory is checked to stay the same across calls.  This file is
collected last so that a failure here never hides the other tests' results.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

MAX_PARTIALS = 1 << 19  # double2 entries of the library's scratch array


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


def _entry(api):
    L = api.lib()
    L.sonar_readout_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                        C.c_float, C.c_float, C.c_void_p, C.c_void_p]
    L.sonar_readout_noalloc.restype = C.c_int
    return L.sonar_readout_noalloc


def _library_readout(api, cfg, pts, att):
    """Source hop and the library's own readout; returns the target's cell
    pressures and the field-point pressures."""
    tris, delta = cfg["targets"][0]
    api.TearDownCuda()
    api.set_initial_conditions(cfg["cp"], cfg["frequency"], att)
    api.load_stl_mesh_to_cuda(tris, api.TARGET, delta)
    api.load_points_to_cuda(cfg["sources"], isSource=True)
    api.load_points_to_cuda(pts, isSource=False)
    api.render_cuda()
    api.project_source_points_to_objects(False)
    P = api.get_object_pressures(api.TARGET, 0)
    api.project_target_to_field_points()
    ref = api.get_field_point_pressures(len(pts))
    api.TearDownCuda()
    return P, ref


def _oracle_readout(oracle_mod, cfg, pts, att, P, dst):
    """The FP64 oracle's readout at the field points dst, given the GPU's
    cell pressures (the readout's input)."""
    tris, delta = cfg["targets"][0]
    o = oracle_mod.Oracle()
    o.set_initial_conditions(cfg["cp"], cfg["frequency"], att)
    o.load_geometry(tris, 0, delta)
    o.load_source_points(cfg["sources"])
    o.load_field_points(pts)
    o.render()
    o.set_pressures(0, 0, P)
    v, _ = o.hop_subset(1, 0, 0, dst)
    o.close()
    return v


def _run_noalloc(api, pos, nrm, pres, pts, k_re, k_im, calls=2):
    """Copies the inputs into device buffers of its own (as a caller that
    owns its memory would) and calls the entry point `calls` times in a row;
    returns the results and the device's free memory before and after the
    calls (after a warm-up call)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    t_pos = torch.from_numpy(pos).to(dev)
    t_nrm = torch.from_numpy(nrm).to(dev)
    t_pres = torch.from_numpy(pres).to(dev)
    p4 = np.ascontiguousarray(np.concatenate([pts, np.zeros((len(pts), 1), np.float32)], 1))
    t_pts = torch.from_numpy(p4).to(dev)
    out = torch.zeros((len(pts), 2), dtype=torch.float64, device=dev)
    fn = _entry(api)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def call():
        out.zero_()
        rc = fn(t_pos.data_ptr(), t_nrm.data_ptr(), t_pres.data_ptr(), len(pos), t_pts.data_ptr(), len(pts),
                k_re, k_im, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize(dev)
        o = out.cpu().numpy()
        return o[:, 0] + 1j * o[:, 1]

    call()  # the first call in this context looks up the scratch array's address
    free0 = torch.cuda.mem_get_info(dev)[0]
    results = [call() for _ in range(calls)]
    free1 = torch.cuda.mem_get_info(dev)[0]
    return results, (free0, free1)


def _check(results, ref, oracle_vals, dst, what):
    for r in results:
        e_lib = rel_l2(r, ref)
        e_orc = rel_l2(r[dst], oracle_vals)
        print("%s: no-alloc readout vs ProjectTargetToFieldPoints %.3e, vs FP64 oracle %.3e" % (what, e_lib, e_orc))
        assert e_lib < 1e-5 and e_orc < 1e-5
    assert rel_l2(results[0], results[1]) < 1e-12


def test_noalloc_readout_matches_library_readout(api, oracle_mod, scenes):
    cfg = scenes.plate_config()
    tris, delta = cfg["targets"][0]
    pts = scenes.grid_xy(32, 1.0, 3.0)
    P, ref = _library_readout(api, cfg, pts, 0.0)
    pos, nrm, pres = _fragments(api, tris, delta, P)
    assert len(pos) > 1200
    results, (free0, free1) = _run_noalloc(api, pos, nrm, pres, pts, _k(cfg["cp"], cfg["frequency"]), 0.0)
    dst = np.arange(len(pts))
    _check(results, ref, _oracle_readout(oracle_mod, cfg, pts, 0.0, P, dst), dst, "plate 10 kHz")
    assert free0 == free1, "device memory changed across calls: %d -> %d free bytes" % (free0, free1)


def test_noalloc_readout_attenuating_medium(api, oracle_mod, scenes):
    """k_im != 0: every term carries exp(-k_im r)."""
    cfg = scenes.plate_config()
    tris, delta = cfg["targets"][0]
    pts = scenes.grid_xy(24, 1.5, 2.0)
    att = 0.35
    P, ref = _library_readout(api, cfg, pts, att)
    pos, nrm, pres = _fragments(api, tris, delta, P)
    results, _ = _run_noalloc(api, pos, nrm, pres, pts, _k(cfg["cp"], cfg["frequency"]), att)
    dst = np.arange(len(pts))
    _check(results, ref, _oracle_readout(oracle_mod, cfg, pts, att, P, dst), dst, "plate 10 kHz, attenuation")


def test_noalloc_readout_many_tiles_scratch_capped_splits(api, oracle_mod, scenes):
    """More than 64 tiles of fragments (each split sums several tiles) and so
    many field points that the scratch array holds only one partial per
    point (a single split over every tile)."""
    cfg = scenes.plate_config(frequency=40e3)
    tris, delta = cfg["targets"][0]
    n_side = 600  # 360,000 field points: 524,288 // 360,000 = 1 split
    pts = scenes.grid_xy(n_side, 2.0, 3.0)
    assert MAX_PARTIALS // len(pts) == 1
    P, ref = _library_readout(api, cfg, pts, 0.0)
    pos, nrm, pres = _fragments(api, tris, delta, P)
    assert len(pos) > 64 * 256
    results, (free0, free1) = _run_noalloc(api, pos, nrm, pres, pts, _k(cfg["cp"], cfg["frequency"]), 0.0)
    dst = np.sort(np.random.default_rng(17).choice(len(pts), 256, replace=False))
    _check(results, ref, _oracle_readout(oracle_mod, cfg, pts, 0.0, P, dst), dst, "plate 40 kHz, 360k points")
    assert free0 == free1


def test_noalloc_rejects_bad_arguments(api):
    """Checked on the host before anything is queued: too many points, a
    negative size, and a buffer that does not start on a 16-byte boundary."""
    import torch
    fn = _entry(api)
    assert fn(None, None, None, 0, None, 524288 + 1, 1.0, 0.0, None, None) == -2
    assert fn(None, None, None, -1, None, 4, 1.0, 0.0, None, None) == -1
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    base = buf.data_ptr()
    # field points at base + 8: misaligned; nothing is launched
    assert fn(base, base, base, 4, base + 8, 4, 1.0, 0.0, base, None) == -1
    assert fn(base + 4, base, base, 4, base, 4, 1.0, 0.0, base, None) == -1
