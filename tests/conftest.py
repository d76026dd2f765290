"""Shared test setup: the gpu marker, the package loader and the oracle.

CPU tests (``-m "not gpu"``) check the oracle against the golden fixtures made
from the reference's own code, the host logic and the C ABI's exports; GPU
tests (``-m gpu``) run the CUDA path through the C ABI and compare it with the
oracle.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__ as ge  # noqa: E402

ge.load_package()
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_scene(g):
    """Rebuild a scene definition from a golden file's inputs."""
    sc = dict(cp=float(g["cp"]), f=float(g["f"]), att=float(g["att"]), bounces=int(g["bounces"]),
              field_objects=bool(int(g["field_objects"])), sources=g["sources"], field_points=g["field_points"],
              targets=[(g["target%d" % i], float(g["target%d_delta" % i])) for i in range(int(g["n_targets"]))],
              fields=[(g["field%d" % i], float(g["field%d_delta" % i])) for i in range(int(g["n_fields"]))])
    return sc


GOLDEN_SCENES = ["plate_10khz", "trihedral_bounces", "occluded_plates", "attenuated_box"]


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def api():
    from sonar_render_gb300 import api as a
    from sonar_render_gb300 import build as b
    b.build()
    a.load_library()
    return a


@pytest.fixture(scope="session")
def scenes():
    from sonar_render_gb300 import scenes as s
    return s
