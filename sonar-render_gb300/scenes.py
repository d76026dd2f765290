"""Synthetic scenes for the discrete Kirchhoff path (numpy only).

Triangle arrays are float32 of shape (n, 9): v1, v2, v3 per triangle, the
layout ``load_geometry`` takes (python_interface.cpp:26-41).  The winding sets
the scattering side: the reference's normal is unit((v2-v1) x (v3-v1))
(Facet.cpp:95-109).

The workloads below are the benchmark configurations of this path, restated
as seeded synthetic inputs of the same shapes and sizes:

* ``plate_config``      1.0 x 0.5 m plate, 10 kHz, one source, 64 x 64 field grid
* ``sphere_config``     r = 1 m icosphere (subdivision 4), 20 kHz, source at 10 m,
                        field plane through the centre
* ``trihedral_config``  orthogonal trihedral, 1 m legs, 3 bounces at 40 kHz
                        (60 kHz, 2 bounces for the compression workload)
* ``batch_config``      16 seeded plates, boxes and spheres (2k-200k fragments),
                        64 arc positions as sources and receivers, 8 frequencies

Mesh helpers mirror the reference's run_scripts/modules/geo.py builders
(make_rectangle, make_right_angle_triangle, make_cube, create_plate,
create_plate_triangle, create_reflector, create_trihedral_reflector,
halve_facets, rotate, translate, join, generate_field_points) without
numpy-stl / trimesh; ``read_stl`` and ``write_stl`` read and write binary STL.
"""
from __future__ import annotations

import math
import struct

import numpy as np

CP_WATER = 1480.0


def delta_for(frequency, cp=CP_WATER, per_wavelength=7.5):
    """Fragment side of lambda / 7.5, the convention of the reference scripts."""
    return (cp / frequency) / per_wavelength


# ---------------------------------------------------------------- meshes
def plate_1x05():
    """The 1.0 x 0.5 m plate in z = 0, normal +z (two triangles)."""
    return np.array([[-0.5, -0.25, 0.0, 0.5, -0.25, 0.0, 0.5, 0.25, 0.0],
                     [-0.5, -0.25, 0.0, 0.5, 0.25, 0.0, -0.5, 0.25, 0.0]], np.float32)


def rectangle(width, height, z=0.0, normal_up=True):
    """Axis-aligned rectangle centred at the origin in the plane z (two triangles)."""
    w, h = width / 2.0, height / 2.0
    a, b, c, d = (-w, -h, z), (w, -h, z), (w, h, z), (-w, h, z)
    if normal_up:
        t = [a + b + c, a + c + d]
    else:
        t = [a + c + b, a + d + c]
    return np.array(t, np.float32)


def halve_facets(tris):
    """Split every triangle into four through its edge midpoints, in the
    reference's vertex order (geo.py:158-196): (v1, m12, m31), (m12, v2, m23),
    (m23, v3, m31), (m12, m23, m31).  The order fixes each facet's frame, so
    the fragment grids equal the reference's."""
    t = np.asarray(tris, np.float64).reshape(-1, 3, 3)
    a, b, c = t[:, 0], t[:, 1], t[:, 2]
    ab, bc, ca = (a + b) / 2, (b + c) / 2, (c + a) / 2
    out = np.stack([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1),
                    np.stack([bc, c, ca], 1), np.stack([ab, bc, ca], 1)], 1)
    return out.reshape(-1, 9).astype(np.float32)


def box(sx, sy, sz, center=(0.0, 0.0, 0.0)):
    """Closed box with outward normals (12 triangles)."""
    x0, y0, z0 = (np.asarray(center) - np.array([sx, sy, sz]) / 2).tolist()
    x1, y1, z1 = x0 + sx, y0 + sy, z0 + sz
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]])
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (3, 0, 4, 7)]
    tris = []
    for q in quads:
        tris.append(np.concatenate([v[q[0]], v[q[1]], v[q[2]]]))
        tris.append(np.concatenate([v[q[0]], v[q[2]], v[q[3]]]))
    return np.array(tris, np.float32)


def icosphere(subdivisions=4, radius=1.0, center=(0.0, 0.0, 0.0)):
    """Icosphere with outward normals: 20 * 4**subdivisions triangles."""
    p = (1.0 + 5 ** 0.5) / 2
    verts = [(-1, p, 0), (1, p, 0), (-1, -p, 0), (1, -p, 0), (0, -1, p), (0, 1, p),
             (0, -1, -p), (0, 1, -p), (p, 0, -1), (p, 0, 1), (-p, 0, -1), (-p, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}

        def mid(i, j):
            key = (min(i, j), max(i, j))
            if key not in cache:
                m = verts[i] + verts[j]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.array(verts) * radius + np.asarray(center, np.float64)
    F = np.array(faces)
    tris = np.concatenate([V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]], axis=1)
    # orient outward: (v2-v1) x (v3-v1) along the centroid direction
    t = tris.reshape(-1, 3, 3)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    outward = np.einsum("ij,ij->i", n, t.mean(1) - np.asarray(center)) > 0
    t[~outward] = t[~outward][:, [0, 2, 1]]
    return t.reshape(-1, 9).astype(np.float32)


def trihedral(leg=1.0):
    """Orthogonal trihedral corner reflector: three right triangles with legs
    ``leg`` along +x, +y, +z from the origin corner; normals point into the
    octant (the reflecting side)."""
    L = float(leg)
    return np.array([[0, 0, 0, L, 0, 0, 0, L, 0],     # z = 0, normal +z
                     [0, 0, 0, 0, L, 0, 0, 0, L],     # x = 0, normal +x
                     [0, 0, 0, 0, 0, L, L, 0, 0]],    # y = 0, normal +y
                    np.float32)


def read_stl(path):
    """Binary STL -> (n, 9) float32 triangles (normals in the file are ignored)."""
    with open(path, "rb") as fh:
        data = fh.read()
    n = struct.unpack_from("<I", data, 80)[0]
    rec = np.frombuffer(data, dtype=np.uint8, count=n * 50, offset=84).reshape(n, 50)
    return np.ascontiguousarray(rec[:, 12:48]).view("<f4").reshape(n, 9).astype(np.float32)


def translate(tris, offset):
    """Shift by offset (geo.py:456-472: the sum in FP64, stored as FP32)."""
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3).astype(np.float64) + np.asarray(offset, np.float64)
    return t.reshape(-1, 9).astype(np.float32)


def write_stl(path, tris, header=b"sonar-render_gb300"):
    """(n, 9) triangles -> binary STL; each record's normal is
    unit((v2 - v1) x (v3 - v1)), the normal the library derives itself."""
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    n = np.cross((t[:, 1] - t[:, 0]).astype(np.float64), (t[:, 2] - t[:, 0]).astype(np.float64))
    L = np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(L > 0, n / np.where(L > 0, L, 1.0), 0.0).astype("<f4")
    rec = np.zeros(len(t), dtype=[("n", "<f4", 3), ("v", "<f4", 9), ("attr", "<u2")])
    rec["n"] = n
    rec["v"] = t.reshape(-1, 9)
    with open(path, "wb") as fh:
        fh.write(header[:80].ljust(80, b"\0"))
        fh.write(struct.pack("<I", len(t)))
        fh.write(rec.tobytes())


def join(*meshes):
    """Concatenate triangle arrays (geo.py:244-264 join_meshes)."""
    return np.concatenate([np.asarray(m, np.float32).reshape(-1, 9) for m in meshes])


# Solids built from vertex and face tables: the tables (coordinates, face
# order and winding) are the reference's (geo.py), so that a scene script
# produces the same triangles -- and so the same facet frames -- here.
def _from_table(vertices, faces):
    v = np.asarray(vertices, np.float64)
    f = np.asarray(faces, np.int64)
    return np.concatenate([v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]], axis=1).astype(np.float32)


def make_rectangle(length, width, xy_plane=True):
    """Two-triangle rectangle centred at the origin in the xy-plane (normal
    +z) or the xz-plane (geo.py:75-113)."""
    l, w = length / 2.0, width / 2.0
    if xy_plane:
        v = [(-l, -w, 0.0), (l, -w, 0.0), (l, w, 0.0), (-l, w, 0.0)]
    else:
        v = [(-l, 0.0, -w), (l, 0.0, -w), (l, 0.0, w), (-l, 0.0, w)]
    return _from_table(v, [(0, 1, 2), (0, 2, 3)])


def make_right_angle_triangle(x_length, y_length):
    """One right triangle in the xy-plane, right angle at the origin (geo.py:115-145)."""
    return _from_table([(0, 0, 0), (x_length, 0, 0), (0, y_length, 0)], [(0, 1, 2)])


def make_cube():
    """Unit cube [0, 1]^3, 12 triangles (geo.py:198-242)."""
    v = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    f = [(2, 1, 0), (3, 2, 0), (5, 6, 4), (6, 7, 4), (0, 4, 5), (0, 5, 1),
         (6, 2, 3), (7, 6, 3), (7, 3, 0), (4, 7, 0), (6, 5, 1), (2, 6, 1)]
    return _from_table(v, f)


def create_plate(length, width, thickness=0.01):
    """Plate of the given thickness above z = 0, 12 triangles (geo.py:282-310)."""
    l, w, t = length / 2.0, width / 2.0, thickness
    v = [(-l, -w, 0), (l, -w, 0), (l, w, 0), (-l, w, 0), (-l, -w, t), (l, -w, t), (l, w, t), (-l, w, t)]
    f = [(2, 1, 0), (3, 2, 0), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
         (1, 2, 6), (1, 6, 5), (2, 3, 7), (2, 7, 6), (3, 0, 4), (3, 4, 7)]
    return _from_table(v, f)


def create_plate_triangle(length, width, thickness=0.01):
    """Triangular prism (base length along x, apex at the origin side), 8
    triangles (geo.py:313-356)."""
    l, w, t = length / 2.0, width / 2.0, thickness
    v = [(-l, -w, 0), (l, -w, 0), (0, 0, 0), (-l, -w, t), (l, -w, t), (0, 0, t)]
    f = [(2, 1, 0), (4, 5, 3), (0, 1, 4), (0, 4, 3), (1, 2, 5), (1, 5, 4), (2, 0, 3), (2, 3, 5)]
    return _from_table(v, f)


def create_reflector(width, thickness):
    """Four triangular prisms forming a corner reflector (geo.py:359-384)."""
    side = (2 * ((width / 2) ** 2)) ** 0.5
    p1 = rotate(create_plate_triangle(side, width, thickness), "x", 45)
    p2 = rotate(create_plate_triangle(side, width, thickness), "x", -45)
    p3 = rotate(rotate(create_plate_triangle(side, width, thickness), "y", 90), "z", 45)
    p4 = rotate(rotate(create_plate_triangle(side, width, thickness), "y", 90), "z", -45)
    return rotate(join(p1, p2, p3, p4), "x", -90)


def create_trihedral_reflector(side_length, thickness):
    """Three thick square plates meeting at a corner (geo.py:387-411)."""
    xy = rotate(create_plate(side_length, side_length, thickness), "z", 45)
    xz = rotate(rotate(create_plate(side_length, side_length, thickness), "z", 45), "y", 90)
    yz = rotate(rotate(create_plate(side_length, side_length, thickness), "z", 45), "x", 90)
    return rotate(rotate(join(xy, xz, yz), "z", 45), "x", 45)


def rotate(tris, axis, degrees):
    """Rotate about a coordinate axis through the origin (geo.py:414-446)."""
    a = math.radians(degrees)
    c, s = math.cos(a), math.sin(a)
    R = {"x": [[1, 0, 0], [0, c, -s], [0, s, c]],
         "y": [[c, 0, s], [0, 1, 0], [-s, 0, c]],
         "z": [[c, -s, 0], [s, c, 0], [0, 0, 1]]}[axis]
    t = np.asarray(tris, np.float64).reshape(-1, 3, 3) @ np.array(R).T
    return t.reshape(-1, 9).astype(np.float32)


# ---------------------------------------------------------------- points
def grid_xy(n, half, z):
    """n x n points on [-half, half]^2 in the plane z (row-major in y then x)."""
    g = np.linspace(-half, half, n)
    X, Y = np.meshgrid(g, g)
    return np.stack([X.ravel(), Y.ravel(), np.full(X.size, z)], 1).astype(np.float32)


def arc_xz(radius, angles_deg):
    """Points on an arc in the xz-plane (geo.py:64-73 generate_field_points)."""
    a = np.radians(np.asarray(angles_deg, np.float64))
    return np.stack([radius * np.sin(a), np.zeros_like(a), radius * np.cos(a)], 1).astype(np.float32)


def hemisphere(n_theta, n_phi, radius, axis=(1.0, 1.0, 1.0), center=(0.0, 0.0, 0.0)):
    """n_theta x n_phi points on the hemisphere of given radius around ``axis``."""
    ax = np.asarray(axis, np.float64)
    ax = ax / np.linalg.norm(ax)
    tmp = np.array([1.0, 0.0, 0.0]) if abs(ax[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    u = np.cross(ax, tmp)
    u /= np.linalg.norm(u)
    w = np.cross(ax, u)
    th = (np.arange(n_theta) + 0.5) / n_theta * (math.pi / 2)
    ph = np.arange(n_phi) / n_phi * 2 * math.pi
    T, P = np.meshgrid(th, ph, indexing="ij")
    d = (np.cos(T)[..., None] * ax + np.sin(T)[..., None] * (np.cos(P)[..., None] * u + np.sin(P)[..., None] * w))
    return (np.asarray(center) + radius * d.reshape(-1, 3)).astype(np.float32)


# ---------------------------------------------------------------- workloads
def plate_config(frequency=10e3):
    """Plate, 10 kHz, source at (0, 0, 5), 64 x 64 field points at z = 3."""
    f = float(frequency)
    return dict(name="plate_1x0.5m_%dkHz" % int(f / 1e3), frequency=f, cp=CP_WATER, attenuation=0.0,
                targets=[(plate_1x05(), delta_for(f))], fields=[],
                sources=np.array([[0.0, 0.0, 5.0]], np.float32),
                field_points=grid_xy(64, 1.0, 3.0), bounces=0)


def sphere_config(field_points_side=512, field_surface=True, frequency=20e3):
    """Icosphere (r = 1 m, 5,120 triangles), 20 kHz, source at 10 m on +z;
    readout onto the 4 x 4 m field plane x = 0 through the centre."""
    f = float(frequency)
    plane = np.array([[0, -2, -2, 0, 2, -2, 0, 2, 2], [0, -2, -2, 0, 2, 2, 0, -2, 2]], np.float32)
    fields = [(plane, 4.0 / field_points_side)] if field_surface else []
    g = np.linspace(-2, 2, field_points_side)
    Y, Z = np.meshgrid(g, g)
    fp = np.stack([np.zeros(Y.size), Y.ravel(), Z.ravel()], 1).astype(np.float32)
    return dict(name="icosphere_r1m_%dkHz" % int(f / 1e3), frequency=f, cp=CP_WATER, attenuation=0.0,
                targets=[(icosphere(4, 1.0), delta_for(f))], fields=fields,
                sources=np.array([[0.0, 0.0, 10.0]], np.float32),
                field_points=None if field_surface else fp, bounces=0)


def trihedral_config(frequency=40e3, bounces=3, n_theta=256, n_phi=256):
    """Trihedral (1 m legs), source at 20 m on the (1,1,1) diagonal, bounces,
    readout to an n_theta x n_phi hemisphere of radius 2 m (none when either
    count is 0)."""
    src = (20.0 / math.sqrt(3.0)) * np.ones((1, 3), np.float32)
    fp = hemisphere(n_theta, n_phi, 2.0) if n_theta and n_phi else None
    return dict(name="trihedral_1m_%dkHz_%db" % (int(frequency / 1e3), bounces), frequency=frequency,
                cp=CP_WATER, attenuation=0.0, targets=[(trihedral(1.0), delta_for(frequency))], fields=[],
                sources=src, field_points=fp, bounces=bounces)


def batch_config(seed=0, nscenes=16, npos=64, nfreq=8, n_lo=2000, n_hi=200000, f_lo=5e3, f_hi=40e3):
    """Seeded batch of scenes for the many-source, many-frequency path.

    ``nscenes`` scenes (plates, boxes and spheres, drawn uniformly) sized so
    that each has about U[n_lo, n_hi] active fragments at the top frequency
    (fragment side lambda / 7.5); ``npos`` positions on a 30 m arc in the
    xz-plane from -60 to +60 degrees, used both as sources and as receivers
    (monostatic and bistatic pairs); ``nfreq`` frequencies log-spaced from
    f_lo to f_hi.  The fragment count of a scene scales with f^2 below the top
    frequency, and every (scene, frequency) is fragmented separately."""
    rng = np.random.default_rng(seed)
    d_hi = delta_for(f_hi)
    scenes, kinds, targets = [], [], []
    for _ in range(nscenes):
        kind = ("plate", "box", "sphere")[int(rng.integers(0, 3))]
        n = float(rng.uniform(n_lo, n_hi))
        area = n * d_hi * d_hi
        if kind == "plate":
            ar = float(rng.uniform(0.5, 2.0))
            w = math.sqrt(area * ar)
            t = rectangle(w, area / w)
            t = rotate(t, "x", float(rng.uniform(-20.0, 20.0)))
            t = rotate(t, "z", float(rng.uniform(0.0, 180.0)))
        elif kind == "box":
            a, b, c = 1.0, float(rng.uniform(0.5, 1.5)), float(rng.uniform(0.5, 1.5))
            s = math.sqrt(area / (2.0 * (a * b + b * c + c * a)))
            t = box(a * s, b * s, c * s)
            t = rotate(t, "y", float(rng.uniform(0.0, 90.0)))
        else:
            t = icosphere(3, math.sqrt(area / (4.0 * math.pi)))
        scenes.append(np.asarray(t, np.float32))
        kinds.append(kind)
        targets.append(int(n))
    pos = arc_xz(30.0, np.linspace(-60.0, 60.0, npos))
    freqs = np.geomspace(f_lo, f_hi, nfreq).astype(np.float32)
    return dict(name="batch_%dscenes_%dpos_%dfreq" % (nscenes, npos, nfreq), scenes=scenes, kinds=kinds,
                target_fragments=targets, sources=pos, receivers=pos, freqs=freqs, cp=CP_WATER, attenuation=0.0,
                per_wavelength=7.5)
