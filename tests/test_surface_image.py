"""Headless surface colouring: the GPU colour map against the oracle's
restatement of the reference's MakeSurface / hsv2rgb arithmetic, and the PNG
writer."""
import os

import numpy as np
import pytest

from conftest import golden_scene, load_golden


def test_png_roundtrip(tmp_path):
    from sonar_render_gb300 import image
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, size=(7, 11, 4), dtype=np.uint8)
    p = image.write_png(os.path.join(tmp_path, "x.png"), img)
    assert np.array_equal(image.read_png_rgba(p), img)


def test_oracle_colour_map_known_values(oracle_mod):
    # |p| = 1 -> 0 dB -> top of a [-60, 0] window; grey mode 0.8
    c = oracle_mod.colour_map(np.array([1.0 + 0j, 1e-3 + 0j, 0j]), -60.0, 0.0, 0)
    assert np.allclose(c[0], [0.8, 0.8, 0.8, 1.0])
    assert np.allclose(c[1], [0.0, 0.0, 0.0, 1.0], atol=1e-5)  # -60 dB -> bottom
    # phase mode: +1 has phase 0 -> hue 0.5 -> cyan-ish (r = m, g = c + m, b = x + m)
    c = oracle_mod.colour_map(np.array([-1.0 + 1e-12j]), -60.0, 0.0, 1)
    assert c[0, 3] == 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("phase", [0, 1])
def test_gpu_colour_map_matches_oracle(api, oracle_mod, phase):
    g = load_golden("trihedral_bounces")
    sc = golden_scene(g)
    from test_gpu_parity import run_gpu
    run_gpu(api, sc)
    api.sound_visualisation_init(-20.0, -90.0, bool(phase), bool(phase))
    for t in (api.TARGET, api.FIELD):
        P = api.get_object_pressures(t, 0)
        got = api.get_surface_colours(t, 0)
        ref = oracle_mod.colour_map(P, -90.0, -20.0, phase)
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) < 2e-5
        assert np.unique(np.round(got[:, 0], 3)).size > 10  # a real gradient, not a constant
    api.TearDownCuda()


@pytest.mark.gpu
def test_surface_png(api, tmp_path):
    from sonar_render_gb300 import image
    g = load_golden("trihedral_bounces")
    sc = golden_scene(g)
    from test_gpu_parity import run_gpu
    run_gpu(api, sc)
    api.sound_visualisation_init(-20.0, -90.0, True, True)
    p = image.save_object_png(api, api.FIELD, 0, os.path.join(tmp_path, "field.png"))
    img = image.read_png_rgba(p)
    api.TearDownCuda()
    assert img.shape[2] == 4 and img[..., 3].max() == 255
