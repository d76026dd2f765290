"""CPU restatement of the reference's GL picture (RenderOpenGL).

TEST INFRASTRUCTURE ONLY: imported by tests/ to check the library's CUDA
rasteriser.  The reference draws every facet of the target and field objects
with its colour-mapped pressure grid as a texture (src/ModelGl.cpp:222-341,
src/ObjectGl.cpp:64-110, texture coordinates src/Facet.cpp:18-60, shader
src/ModelGl.cpp:128-160) through OpenGL: camera glm::perspective(45 deg,
w/h, 0.1, 10000) * glm::lookAt(eye, centre, up) (src/ModelGl.cpp:98-106),
depth test GL_LESS, texture sampling GL_LINEAR with the default GL_REPEAT
wrap, clear colour (0.96, 0.96, 0.86), the frame flipped so that the top row
comes first (src/ModelGl.cpp:321-330).  The GL pipeline itself cannot run
here (no graphics stack), so this is the pipeline's arithmetic in numpy
(FP64): pixel centres, barycentric coverage, linear window depth,
perspective-correct texture coordinates, bilinear filtering, rounding to 8
bits.  Parity with the reference's actual GL output is unpinned.
"""
from __future__ import annotations

import math

import numpy as np


def camera(width, height, vs):
    fovy = math.radians(45.0)
    aspect = width / height
    zn, zf = 0.1, 10000.0
    th = math.tan(fovy / 2.0)
    P = np.array([[1.0 / (aspect * th), 0, 0, 0], [0, 1.0 / th, 0, 0],
                  [0, 0, -(zf + zn) / (zf - zn), -(2.0 * zf * zn) / (zf - zn)], [0, 0, -1.0, 0]])
    eye, ctr, up = np.asarray(vs[0:3], float), np.asarray(vs[3:6], float), np.asarray(vs[6:9], float)
    f = ctr - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    V = np.array([[s[0], s[1], s[2], -s @ eye], [u[0], u[1], u[2], -u @ eye], [-f[0], -f[1], -f[2], f @ eye],
                  [0, 0, 0, 1.0]])
    return P @ V


def facet_uv(tri):
    """Texture coordinates of the three vertices: base origin (0, 0), base end
    (1, 0), apex (BaseLengthNeg / BaseLength, 1); the base is the longest edge
    (first maximum of |v1v2|, |v1v3|, |v2v3|)."""
    v = np.asarray(tri, float).reshape(3, 3)
    e = [np.linalg.norm(v[0] - v[1]), np.linalg.norm(v[0] - v[2]), np.linalg.norm(v[1] - v[2])]
    m = 0
    if e[1] > e[m]:
        m = 1
    if e[2] > e[m]:
        m = 2
    origin, end = (1 if m == 2 else 0), (1 if m == 0 else 2)
    apex = 2 if m == 0 else (1 if m == 1 else 0)
    ax = v[end] - v[origin]
    L = np.linalg.norm(ax)
    neg = float(np.dot(v[apex] - v[origin], ax / L))  # distance origin -> foot of the altitude
    uv = np.zeros((3, 2))
    uv[origin] = (0.0, 0.0)
    uv[end] = (1.0, 0.0)
    uv[apex] = (neg / L, 1.0)
    return uv


def render(tris, textures, width, height, vs):
    """tris: (T, 9) vertices in drawing order; textures: per triangle an
    (ny, nx, 4) RGBA array.  Returns (height, width, 3) uint8, top row first."""
    M = camera(width, height, vs)
    depth = np.full((height, width), np.inf)
    owner = np.full((height, width), -1, np.int64)
    scr = []
    for t, tri in enumerate(np.asarray(tris, float).reshape(-1, 3, 3)):
        c = (M @ np.concatenate([tri, np.ones((3, 1))], axis=1).T).T
        if not (c[:, 3] > 0.1).all():
            scr.append(None)
            continue
        x = (c[:, 0] / c[:, 3] + 1.0) * 0.5 * width
        y = (c[:, 1] / c[:, 3] + 1.0) * 0.5 * height
        z = c[:, 2] / c[:, 3]
        scr.append((x, y, z, 1.0 / c[:, 3]))
        area = (x[1] - x[0]) * (y[2] - y[0]) - (x[2] - x[0]) * (y[1] - y[0])
        if area == 0.0:
            continue
        x0, x1 = max(0, int(math.floor(x.min()))), min(width - 1, int(math.ceil(x.max())))
        y0, y1 = max(0, int(math.floor(y.min()))), min(height - 1, int(math.ceil(y.max())))
        if x0 > x1 or y0 > y1:
            continue
        PX, PY = np.meshgrid(np.arange(x0, x1 + 1) + 0.5, np.arange(y0, y1 + 1) + 0.5)
        e0 = (x[2] - x[1]) * (PY - y[1]) - (y[2] - y[1]) * (PX - x[1])
        e1 = (x[0] - x[2]) * (PY - y[2]) - (y[0] - y[2]) * (PX - x[2])
        e2 = (x[1] - x[0]) * (PY - y[0]) - (y[1] - y[0]) * (PX - x[0])
        inside = ((e0 >= 0) & (e1 >= 0) & (e2 >= 0)) if area > 0 else ((e0 <= 0) & (e1 <= 0) & (e2 <= 0))
        zz = (e0 * z[0] + e1 * z[1] + e2 * z[2]) / area
        inside &= (zz >= -1.0) & (zz <= 1.0)
        d = (zz + 1.0) * 0.5
        sub_d = depth[y0:y1 + 1, x0:x1 + 1]
        win = inside & (d < sub_d)
        sub_d[win] = d[win]
        owner[y0:y1 + 1, x0:x1 + 1][win] = t
    img = np.empty((height, width, 3))
    img[:] = (0.96, 0.96, 0.86)
    uvs = [facet_uv(tri) for tri in np.asarray(tris, float).reshape(-1, 9)]
    for t in np.unique(owner[owner >= 0]):
        x, y, z, iw = scr[t]
        area = (x[1] - x[0]) * (y[2] - y[0]) - (x[2] - x[0]) * (y[1] - y[0])
        py, px = np.nonzero(owner == t)
        PX, PY = px + 0.5, py + 0.5
        b0 = ((x[2] - x[1]) * (PY - y[1]) - (y[2] - y[1]) * (PX - x[1])) / area
        b1 = ((x[0] - x[2]) * (PY - y[2]) - (y[0] - y[2]) * (PX - x[2])) / area
        b2 = ((x[1] - x[0]) * (PY - y[0]) - (y[1] - y[0]) * (PX - x[0])) / area
        q = np.stack([b0 * iw[0], b1 * iw[1], b2 * iw[2]], 1)
        uv = (q @ uvs[t]) / q.sum(1, keepdims=True)
        tex = np.asarray(textures[t], float)
        ny, nx = tex.shape[:2]
        fx, fy = uv[:, 0] * nx - 0.5, uv[:, 1] * ny - 0.5
        ix, iy = np.floor(fx).astype(np.int64), np.floor(fy).astype(np.int64)
        ax, ay = (fx - ix)[:, None], (fy - iy)[:, None]
        c00 = tex[iy % ny, ix % nx]
        c10 = tex[iy % ny, (ix + 1) % nx]
        c01 = tex[(iy + 1) % ny, ix % nx]
        c11 = tex[(iy + 1) % ny, (ix + 1) % nx]
        col = (1 - ay) * ((1 - ax) * c00 + ax * c10) + ay * ((1 - ax) * c01 + ax * c11)
        img[py, px] = col[:, :3]
    out = np.rint(np.clip(img, 0.0, 1.0) * 255.0).astype(np.uint8)
    return out[::-1].copy()
