"""The headless RenderOpenGL: the library's CUDA rasteriser against the CPU
restatement of the reference's GL pipeline (oracle/raster_oracle.py).

Tolerance: pixel centres lying on a triangle edge can be decided differently
in FP32 and FP64, and bilinear weights round differently, so at most 1 % of
the pixels may differ by more than 2 levels and the rest by at most 2."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def scene(api, scenes):
    api.TearDownCuda()
    f = 8e3
    api.set_initial_conditions(1480.0, f, 0.0)
    plate = scenes.rotate(scenes.rectangle(1.0, 0.6), "x", 10.0)
    box = scenes.translate(scenes.box(0.25, 0.2, 0.3), (0.2, 0.1, 0.35))
    field = np.array([[-1.5, -1.0, -0.6, 1.5, -1.0, -0.6, 1.5, 1.2, -0.6],
                      [-1.5, -1.0, -0.6, 1.5, 1.2, -0.6, -1.5, 1.2, -0.6]], np.float32)
    api.load_stl_mesh_to_cuda(np.concatenate([plate, box]), api.TARGET, scenes.delta_for(f))
    api.load_stl_mesh_to_cuda(field, api.FIELD, 0.03)
    api.load_points_to_cuda(np.array([[0.5, 0.8, 4.0]], np.float32), isSource=True)
    api.render_cuda()
    api.sound_visualisation_init(0.0, -60.0, False, False)
    api.project_source_points_to_objects(True)
    tris = np.concatenate([plate, box, field]).reshape(-1, 9)
    return tris


def textures(api, tris, n_target):
    """Per triangle the (ny, nx, 4) colour grid of its facet."""
    out = []
    for t_type, idx, rng in ((api.TARGET, 0, range(n_target)), (api.FIELD, 0, range(n_target, len(tris)))):
        col = api.get_surface_colours(t_type, idx)
        ints, areas = api.get_fragment_layout(t_type, idx)[:2]
        off = 0
        for k, (nx, ny, neg) in enumerate(ints):
            out.append(col[off:off + nx * ny].reshape(ny, nx, 4))
            off += nx * ny
    return out


def test_render_matches_cpu_restatement(api, scenes, tmp_path):
    import raster_oracle as R
    tris = scene(api, scenes)
    tex = textures(api, tris, 14)
    L = api.lib()
    L.sonar_render_image.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_ubyte)]
    for (w, h, vs) in ((320, 240, (3.0, 2.5, 4.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0)),
                       (200, 300, (-2.0, -1.5, 3.0, 0.2, 0.1, 0.0, 0.0, 0.0, 1.0))):
        img = np.zeros((h, w, 3), np.uint8)
        vsa = (C.c_float * 9)(*vs)
        r = L.sonar_render_image(w, h, vsa, img.ctypes.data_as(C.POINTER(C.c_ubyte)))
        assert r == 0, api.last_error()
        ref = R.render(tris, tex, w, h, vs)
        diff = np.abs(img.astype(int) - ref.astype(int)).max(axis=2)
        bad = float((diff > 2).mean())
        covered = float((ref != np.array([245, 245, 219], np.uint8)).any(axis=2).mean())
        print("render %dx%d: %.1f %% of pixels covered, %.3f %% differ by > 2 levels, max diff %d"
              % (w, h, 100 * covered, 100 * bad, diff.max()))
        assert covered > 0.05
        assert bad < 0.01
    # RenderOpenGL writes the same picture as a PNG
    out = str(tmp_path / "frame.png")
    vs = (C.c_float * 9)(3.0, 2.5, 4.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0)
    L.RenderOpenGL(320, 240, out.encode(), vs)
    assert L.sonar_status() == 0, api.last_error()
    import zlib
    data = open(out, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    # IDAT payload decompresses to 240 rows of 1 + 320 * 3 bytes
    pos, idat = 8, b""
    while pos < len(data):
        n = int.from_bytes(data[pos:pos + 4], "big")
        tag = data[pos + 4:pos + 8]
        if tag == b"IDAT":
            idat += data[pos + 8:pos + 8 + n]
        pos += 12 + n
    raw = zlib.decompress(idat)
    assert len(raw) == 240 * (1 + 320 * 3)
    rows = np.frombuffer(raw, np.uint8).reshape(240, 1 + 320 * 3)[:, 1:].reshape(240, 320, 3)
    img = np.zeros((240, 320, 3), np.uint8)
    L.sonar_render_image(320, 240, vs, img.ctypes.data_as(C.POINTER(C.c_ubyte)))
    assert np.array_equal(rows, img)
    api.TearDownCuda()
