"""Scene I/O and the reference's scene builders (run_scripts/modules/geo.py),
restated without numpy-stl / trimesh, on the CPU.

The builders use the reference's vertex and face tables, so a reference
script's scene gives the same triangles (and so the same facet frames and
fragment grids); the winding is the reference's even where it points a face
inward (the front face of geo.py's make_cube).
"""
import numpy as np


def tri_normals(t):
    t = np.asarray(t, np.float64).reshape(-1, 3, 3)
    return np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])


def area(t):
    return 0.5 * np.linalg.norm(tri_normals(t), axis=1).sum()


def test_stl_round_trip(tmp_path, scenes):
    for k, m in enumerate([scenes.make_cube(), scenes.icosphere(1, 0.3), scenes.create_reflector(0.5, 0.01)]):
        p = tmp_path / ("m%d.stl" % k)
        scenes.write_stl(str(p), m)
        back = scenes.read_stl(str(p))
        assert back.dtype == np.float32 and back.shape == m.shape
        assert np.array_equal(back, m)
        raw = p.read_bytes()
        assert len(raw) == 84 + 50 * len(m)
        # the record normals are the unit (v2 - v1) x (v3 - v1)
        n = np.frombuffer(raw, np.uint8, offset=84).reshape(-1, 50)[:, :12].copy().view("<f4").reshape(-1, 3)
        ref = tri_normals(m)
        ref /= np.linalg.norm(ref, axis=1, keepdims=True)
        assert np.allclose(n, ref, atol=1e-6)


def test_halve_facets_order_area_normals(scenes):
    t = scenes.icosphere(0, 1.0)
    h = scenes.halve_facets(t)
    assert len(h) == 4 * len(t)
    assert abs(area(h) - area(t)) < 1e-5 * area(t)
    n0 = tri_normals(t)
    n1 = tri_normals(h).reshape(-1, 4, 3)
    for k in range(4):
        cosang = np.einsum("ij,ij->i", n0, n1[:, k]) / (np.linalg.norm(n0, axis=1) * np.linalg.norm(n1[:, k], axis=1))
        assert np.all(cosang > 1 - 1e-6)
    # the reference's vertex order: (v1, m12, m31), (m12, v2, m23), (m23, v3, m31), (m12, m23, m31)
    v = t.reshape(-1, 3, 3)[0].astype(np.float64)
    m12, m23, m31 = (v[0] + v[1]) / 2, (v[1] + v[2]) / 2, (v[2] + v[0]) / 2
    want = np.array([[v[0], m12, m31], [m12, v[1], m23], [m23, v[2], m31], [m12, m23, m31]], np.float32)
    assert np.array_equal(h[:4].reshape(4, 3, 3), want)


def test_builders(scenes):
    c = scenes.make_cube()
    assert c.shape == (12, 9) and abs(area(c) - 6.0) < 1e-6
    assert c.min() == 0.0 and c.max() == 1.0
    r = scenes.make_rectangle(1.0, 0.5)
    assert np.array_equal(r, scenes.rectangle(1.0, 0.5))
    assert np.allclose(tri_normals(scenes.make_rectangle(1.0, 0.5, xy_plane=False))[:, [0, 2]], 0.0)
    assert abs(area(scenes.make_right_angle_triangle(0.3, 0.4)) - 0.06) < 1e-7
    p = scenes.create_plate(1.0, 0.5, 0.02)
    assert p.shape == (12, 9) and abs(area(p) - (2 * 0.5 + 2 * 0.02 * 1.5)) < 1e-5
    pt = scenes.create_plate_triangle(1.0, 0.5, 0.02)
    assert pt.shape == (8, 9)
    refl = scenes.create_reflector(1.0, 0.02)
    assert refl.shape == (32, 9) and np.all(np.isfinite(refl))
    tri = scenes.create_trihedral_reflector(1.0, 0.02)
    assert tri.shape == (36, 9) and abs(area(tri) - 3 * (2.0 + 4 * 0.02)) < 1e-4
    j = scenes.join(c, r)
    assert np.array_equal(j[:12], c) and np.array_equal(j[12:], r)
    # translation: FP64 sum stored as FP32
    tr = scenes.translate(c, (0.1, 0.2, 0.3))
    assert np.array_equal(tr, (c.reshape(-1, 3, 3).astype(np.float64) + [0.1, 0.2, 0.3]).astype(np.float32).reshape(-1, 9))


def test_builder_scene_fragments_to_its_area(api, scenes):
    """Every triangle of a generated reflector through the library's host-side
    fragmentation (Facet.cpp:111-339): the cell areas add up to the triangle's
    (the reference prints the same check, Facet.cpp:341-361)."""
    tri = scenes.create_trihedral_reflector(0.5, 0.02)
    d = scenes.delta_for(20e3)
    for t in tri:
        (nx, ny, neg), fr, a = api.fragment_triangle(t, d)
        ta = 0.5 * np.linalg.norm(tri_normals(t))
        assert a.shape == (ny, nx)
        assert abs(a.astype(np.float64).sum() - ta) <= 2e-3 * ta + 1e-7
