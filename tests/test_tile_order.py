"""Host-only check of the patch-aligned fragment order (sonar_tile_order,
the order render_cuda stores a facet's active fragments in; no GPU).

On a trihedral face at 60 kHz (grid rows along the hypotenuse, both legs
cut at 45 degrees) the order must be a permutation of the active cells; every
full 16 x 16 patch must be exactly one 256-fragment tile, whatever the
facet's start offset; the cells whose readout centroid (the cell's left
edge, no x shift) lies on or outside the triangle must come last; and the
tiles of partial patches, taken along the boundary, must stay compact."""
import numpy as np
import pytest


def _face(scenes):
    return scenes.trihedral(1.0)[0], scenes.delta_for(60e3)


def _readout(fr, neg, d, xy):
    base, xa, ya = fr[3:6].astype(np.float64), fr[6:9].astype(np.float64), fr[9:12].astype(np.float64)
    xo = d * (xy[:, 0] - neg).astype(np.float64)
    yo = d * xy[:, 1].astype(np.float64) + d / 2
    return base + xo[:, None] * xa + yo[:, None] * ya


def _inside(tri, P):
    v = np.asarray(tri, np.float64).reshape(3, 3)
    n = np.cross(v[1] - v[0], v[2] - v[0])
    ok = np.ones(len(P), bool)
    for a, b in ((v[0], v[1]), (v[1], v[2]), (v[2], v[0])):
        e = np.cross(n, b - a)
        e /= np.linalg.norm(e)
        ok &= (P - a) @ e > 1e-6 * max(1.0, np.linalg.norm(b - a))
    return ok


@pytest.mark.parametrize("start", [0, 100, 46437])
def test_tile_order_aligns_full_patches(api, scenes, start):
    tri, d = _face(scenes)
    (nx, ny, neg), fr, area = api.fragment_triangle(tri, d)
    xy = api.tile_order(tri, d, start)
    act = np.argwhere(area > 1e-6)[:, ::-1]  # (x, y)
    assert len(xy) == len(act)
    assert set(map(tuple, xy)) == set(map(tuple, act))
    # full patches of the grid, and the tiles that are one of them
    pid = (xy[:, 1] // 16) * ((nx + 15) // 16) + xy[:, 0] // 16
    counts = np.bincount(pid)
    nfull = int((counts == 256).sum())
    need = (256 - start % 256) % 256
    whole = 0
    for t0 in range(need, len(xy) - 255, 256):
        if len(set(pid[t0:t0 + 256])) == 1:
            whole += 1
    print("start %d: %d active cells, %d full patches, %d tiles that are one patch" % (start, len(xy), nfull, whole))
    assert nfull > 100 and whole == nfull


def test_tile_order_edge_cells_last_and_partial_tiles_compact(api, scenes):
    tri, d = _face(scenes)
    (nx, ny, neg), fr, area = api.fragment_triangle(tri, d)
    xy = api.tile_order(tri, d, 0)
    inside = _inside(tri, _readout(fr, neg, d, xy))
    nedge = int((~inside).sum())
    assert 0 < nedge < len(xy) // 50
    assert not inside[len(xy) - nedge:].any() and inside[:len(xy) - nedge].all()
    # tiles of partial patches (after the full ones, before the edge cells) follow one leg at a time: boxes
    # of at most 48 x 48 cells (in patch order a tile would take partial cells of both legs, ~400 cells apart)
    pid = (xy[:, 1] // 16) * ((nx + 15) // 16) + xy[:, 0] // 16
    full = np.bincount(pid)[pid] == 256
    first_partial = int(np.argmax(~full[256:])) + 256  # start 0: no cells in front of the full patches
    boxes = []
    for t0 in range(first_partial - first_partial % 256 + 256, len(xy) - nedge - 256, 256):
        c = xy[t0:t0 + 256]
        boxes.append((c[:, 0].max() - c[:, 0].min() + 1, c[:, 1].max() - c[:, 1].min() + 1))
    print("partial tiles: %d, boxes %s" % (len(boxes), sorted(set(boxes))))
    assert len(boxes) > 5
    assert all(bx <= 48 and by <= 48 for bx, by in boxes)


def _patch_order(nx, area):
    """The active cells in patch order (patch row, patch column, rows inside)."""
    ny = area.shape[0]
    out = []
    for py in range(0, ny, 16):
        for px in range(0, nx, 16):
            for y in range(py, min(ny, py + 16)):
                for x in range(px, min(nx, px + 16)):
                    if area[y, x] > 1e-6:
                        out.append((x, y))
    return np.array(out, np.int32).reshape(-1, 2)


_SHAPES = {
    "acute": ([0, 0, 0, 1, 0, 0, 0.3, 0.8, 0], 40e3),
    "tilted": ([0, 0, 0, 0.6, 0.2, 0.5, 0.1, 0.9, 0.3], 40e3),
    "obtuse": ([0, 0, 0, 1.2, 0, 0, 1.5, 0.4, 0.1], 30e3),
    "sliver": ([0, 0, 0, 1, 0, 0, 0.5, 0.02, 0], 40e3),
    "long sliver": ([0, 0, 0, 2.5, 0, 0, 1.2, 0.02, 0], 40e3),
    "small": ([0, 0, 0, 0.05, 0, 0, 0, 0.05, 0], 40e3),
}


@pytest.mark.parametrize("shape", sorted(_SHAPES))
@pytest.mark.parametrize("start", [0, 77, 300])
def test_tile_order_any_triangle(api, scenes, shape, start):
    """Any triangle: a permutation of the active cells; with a full patch, at
    least 512 cells and enough partial cells inside the triangle to fill the
    first tile, every full patch is one tile and the partial cells whose
    readout centroid is on or outside the triangle come last; otherwise the
    patch order stays."""
    tri, f = _SHAPES[shape]
    d = float(np.float32(scenes.delta_for(f)))
    (nx, ny, neg), fr, area = api.fragment_triangle(tri, d)
    xy = api.tile_order(tri, d, start)
    po = _patch_order(nx, area)
    assert len(xy) == len(po)
    assert set(map(tuple, xy)) == set(map(tuple, po))
    pid = (po[:, 1] // 16) * ((nx + 15) // 16) + po[:, 0] // 16
    counts = np.bincount(pid) if len(pid) else np.zeros(0, int)
    full_cell = counts[pid] == 256 if len(pid) else np.zeros(0, bool)
    inside = _inside(tri, _readout(fr, neg, d, po))
    need = (256 - start % 256) % 256
    ngood = int((~full_cell & inside).sum())
    aligned = full_cell.any() and (~full_cell).any() and len(po) >= 512 and ngood >= need
    print("%s start %d: %d cells, %d full patches, %d good partial cells, aligned %s"
          % (shape, start, len(po), int(full_cell.sum()) // 256, ngood, aligned))
    if not aligned:
        assert np.array_equal(xy, po)
        return
    # every full patch is exactly one tile of the global index space
    pid_xy = (xy[:, 1] // 16) * ((nx + 15) // 16) + xy[:, 0] // 16
    for p in np.flatnonzero(counts == 256):
        at = np.flatnonzero(pid_xy == p)
        assert len(at) == 256 and at[-1] - at[0] == 255 and (start + at[0]) % 256 == 0
    # the partial cells on or outside the triangle come last
    edge = set(map(tuple, po[~full_cell & ~inside]))
    ne = len(edge)
    if ne:
        assert set(map(tuple, xy[len(xy) - ne:])) == edge
