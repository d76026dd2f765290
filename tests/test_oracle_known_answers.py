"""Known-answer tests of the FP64 oracle's sums, on the CPU.

Each sum is recomputed here from the reference's formulas, independently of
the oracle's code, with the reference's rounding: fragment positions, r,
1/r, the unit vector and the cosines in FP32 (no contraction), k = float(2 pi
f) / c in FP32, the Green's functions in FP64 (src/OptiX.cu:35-406,
src/Model.cpp:44-54).  Pinned quirks: the half-cell x shift of the source
hop, no 4 pi and no area on the source hop, the FP32 1/r^2 term outside the
exponential, the r < delta regularisation, the 0.9 damping, the zero-input
skip that also drops the reciprocal write, attenuation as the imaginary part
of k.  Visibility is not re-derived here: pairs are taken where the oracle's
mask says the ray is clear (the masks have their own tests).
"""
import math

import numpy as np
import pytest

f32 = np.float32


def k_of(f, cp=1480.0, att=0.0):
    omega = f32(2.0 * math.pi * f)
    k = f32(omega / f32(cp))
    return complex(float(k), float(f32(att)))  # the attenuation is a float too (Model.cpp:44-54)


def frames(o, t, i, delta):
    ints, fl = o.facets(t, i)
    out, cell0 = [], 0
    for (nx, ny, neg), F in zip(ints, fl):
        out.append(dict(nx=int(nx), ny=int(ny), neg=int(neg), n=F[0:3].astype(f32), base=F[3:6].astype(f32),
                        xa=F[6:9].astype(f32), ya=F[9:12].astype(f32), cell0=cell0, d=f32(delta)))
        cell0 += int(nx) * int(ny)
    return out


def cell_facet(frs, c):
    for fi, F in enumerate(frs):
        if F["cell0"] <= c < F["cell0"] + F["nx"] * F["ny"]:
            k = c - F["cell0"]
            return fi, k % F["nx"], k // F["nx"]
    raise ValueError(c)


def frag_pos(F, x, y, src_hop):
    d = F["d"]
    xoff = f32(d * f32(x - F["neg"]))
    if src_hop:
        xoff = f32(xoff + f32(d / f32(2)))
    yoff = f32(f32(d * f32(y)) + f32(d / f32(2)))
    xa, ya = (F["xa"] * xoff).astype(f32), (F["ya"] * yoff).astype(f32)
    return ((F["base"] + xa).astype(f32) + ya).astype(f32)


def dot(a, b):
    return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))


def ray(pa, pb):
    v = (pb - pa).astype(f32)
    r = f32(np.sqrt(dot(v, v)))
    inv = f32(f32(1) / r)
    return r, (v * inv).astype(f32)


def green(k, r):
    rd = float(r)
    g = -np.exp(1j * k * rd) / (4 * math.pi) * (1j * k / rd)
    return g + float(f32(f32(1) / f32(r * r)))


def load(oracle_mod, tris, delta, f, att=0.0, src=None):
    o = oracle_mod.Oracle()
    o.set_initial_conditions(1480.0, f, att)
    for t in tris:
        o.load_geometry(t, 0, delta)
    o.load_source_points(np.asarray(src if src is not None else [[0.0, 0.0, 5.0]], np.float32))
    o.load_field_points(np.zeros((1, 3), np.float32))
    o.render()
    return o


@pytest.mark.parametrize("att", [0.0, 0.4])
def test_source_hop(oracle_mod, scenes, att):
    """P_j = cos_inc e^{ikr} / r at the half-cell-shifted centroid; unit source."""
    f, delta = 3e3, 0.06
    tris = [scenes.rotate(scenes.rectangle(0.3, 0.2), "x", 25.0)]
    src = np.array([[0.2, -0.4, 1.5]], np.float32)
    o = load(oracle_mod, tris, delta, f, att, src)
    frs = frames(o, 0, 0, delta)
    k = k_of(f, att=att)
    o.project_sources(False)
    got = o.pressures(0, 0)
    want = np.zeros_like(got)
    for c in range(len(got)):
        fi, x, y = cell_facet(frs, c)
        r, uv = ray(src[0], frag_pos(frs[fi], x, y, True))
        ci = dot((-uv).astype(f32), frs[fi]["n"])
        if ci < f32(1e-6):
            continue
        want[c] = float(ci) * np.exp(1j * k * float(r)) / float(r)
    assert np.abs(want).max() > 0
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)


def test_bounce_regularisation_damping_reciprocity(oracle_mod, scenes):
    """Two small facets 6 mm apart face each other (delta = 1 cm, so every
    pair is regularised: G = 0.9 i k / 4 pi), plus a third facet further away
    (plain G); the destination-owned bounce at each active cell equals the
    forward terms from lower facets plus the reciprocal terms from higher
    ones, all with A_src cos_scat cos_inc P_in G and the 0.9 damping."""
    f, delta = 6e3, 0.01
    a = np.array([[0, 0, 0, 0.012, 0, 0, 0, 0.012, 0]], np.float32)              # z = 0, normal +z
    b = np.array([[0, 0, 0.006, 0, 0.012, 0.006, 0.012, 0, 0.006]], np.float32)  # z = 6 mm, normal -z
    c = np.array([[0, 0, 0.05, 0, 0.03, 0.05, 0.03, 0, 0.05]], np.float32)       # z = 5 cm, normal -z
    o = load(oracle_mod, [np.concatenate([a, b, c])], delta, f)
    frs = frames(o, 0, 0, delta)
    act = o.active(0, 0)
    area = o.areas(0, 0)
    rng = np.random.default_rng(3)
    pin = np.zeros(o.ncells(0, 0), np.complex128)
    pin[act] = rng.standard_normal(len(act)) + 1j * rng.standard_normal(len(act))
    got, mask = o.hop_subset(2, 0, 0, np.arange(len(act)), pin=pin, want_mask=True, nsrc=len(act))
    k = k_of(f)
    n_reg = 0
    for q, cj in enumerate(act):
        fb, xj, yj = cell_facet(frs, cj)
        pj = frag_pos(frs[fb], xj, yj, False)
        acc = 0j
        for s_, ci in enumerate(act):
            fa, xi, yi = cell_facet(frs, ci)
            if fa == fb or not (mask[q, s_] & 1):
                continue
            pi_ = frag_pos(frs[fa], xi, yi, False)
            fwd = fa < fb
            pA, pB = (pi_, pj) if fwd else (pj, pi_)
            FA, FB = (frs[fa], frs[fb]) if fwd else (frs[fb], frs[fa])
            r, uv = ray(pA, pB)
            cs = dot(uv, FA["n"])
            cin = dot((-uv).astype(f32), FB["n"])
            if cs < f32(1e-6) or cin < f32(1e-6):
                continue
            if not fwd and pin[cj] == 0:
                continue  # the zero-input skip of the A side drops the reciprocal write
            if fwd and pin[ci] == 0:
                continue
            if r < f32(delta):
                g, n_reg = 1j * k / (4 * math.pi), n_reg + 1
            else:
                g = green(k, r)
            w = float(f32(f32(area[ci] * cs) * cin))
            acc += w * pin[ci] * 0.9 * g
        assert abs(got[q] - acc) <= 1e-12 * max(abs(acc), 1e-300) + 1e-15, (q, got[q], acc)
    assert n_reg > 0


def test_zero_input_skip_drops_reciprocal_terms(oracle_mod, scenes):
    """Trihedral corner: a destination cell of facet 1 whose own input is 0
    receives only the forward terms of facet 0; with a non-zero input it also
    receives the reciprocal terms of facet 2 (src/OptiX.cu:241-245, :367-390)."""
    f, delta = 6e3, 0.01
    o = load(oracle_mod, [scenes.trihedral(0.04)], delta, f)
    act = o.active(0, 0)
    frs = frames(o, 0, 0, delta)
    fac = np.array([cell_facet(frs, c)[0] for c in act])
    rng = np.random.default_rng(5)
    pin = np.zeros(o.ncells(0, 0), np.complex128)
    pin[act] = rng.standard_normal(len(act)) + 1j * rng.standard_normal(len(act))
    dst = np.nonzero(fac == 1)[0]
    full, _ = o.hop_subset(2, 0, 0, dst, pin=pin)
    only0 = pin.copy()
    only0[act[fac == 2]] = 0.0          # facet 2 silent: forward terms from facet 0 only
    fwd0, _ = o.hop_subset(2, 0, 0, dst, pin=only0)
    zero_dst = pin.copy()
    zero_dst[act[dst]] = 0.0            # the destinations' own inputs 0: reciprocal terms dropped
    got, _ = o.hop_subset(2, 0, 0, dst, pin=zero_dst)
    assert np.abs(full - fwd0).max() > 0  # facet 2 does reach facet 1 when the input is non-zero
    np.testing.assert_array_equal(got, fwd0)
