"""Writes the golden fixtures of tests/golden/ from the reference's own code.

Run where the reference's sources are present:

    python tests/golden/make_golden.py [reference-root]

It builds oracle/_ref/libsonar_ref.so (oracle/build_ref.sh: the reference's
unmodified src/Facet.cpp and src/OptiX.cu compiled for the CPU) and records:

  fragmentation.npz  frames and area grids of seeded random triangles and of
                     the benchmark meshes (src/Facet.cpp:6-339)
  <scene>.npz        surface and field-point pressures of small scenes after
                     the reference's projections (src/OptiX.cu:35-445 with the
                     sequencing of src/ModelCuda.cpp:242-356)

The scene inputs are stored in the same files, so the tests replay them
without the reference.
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "sonar-render_gb300"))

import oracle as O  # noqa: E402
import scenes as S  # noqa: E402


def scene_defs():
    """Small scenes whose shadow verdicts are far from every tolerance."""
    out = {}
    plate = S.plate_config()
    out["plate_10khz"] = dict(targets=[(plate["targets"][0][0], 0.02)], fields=[],
                              sources=plate["sources"], field_points=S.grid_xy(16, 1.0, 3.0),
                              cp=1480.0, f=10e3, att=0.0, bounces=0, field_objects=False)
    tri = S.trihedral(0.3)
    out["trihedral_bounces"] = dict(targets=[(tri, 0.02)], fields=[(S.rectangle(1.0, 1.0, z=0.6), 0.05)],
                                    sources=np.array([[2.0, 2.0, 2.0]], np.float32),
                                    field_points=S.hemisphere(8, 8, 1.0, axis=(1.0, 1.2, 0.9),
                                                              center=(0.05, 0.08, 0.03)),
                                    cp=1480.0, f=10e3, att=0.0,
                                    bounces=2, field_objects=True)
    # an occluder: a small plate at z = 0.5 shadows part of a larger plate at
    # z = 0 from a source above both; readout above the small plate's edge
    big = S.rectangle(1.2, 1.2, z=0.0)
    small = S.rectangle(0.3, 0.3, z=0.5)
    out["occluded_plates"] = dict(targets=[(big, 0.03), (small, 0.03)], fields=[],
                                  sources=np.array([[0.05, 0.02, 2.0]], np.float32),
                                  field_points=S.grid_xy(12, 0.8, 1.5), cp=1480.0, f=5e3, att=0.0,
                                  bounces=1, field_objects=False)
    out["attenuated_box"] = dict(targets=[(S.box(0.3, 0.2, 0.25), 0.025)], fields=[],
                                 sources=np.array([[0.7, 0.4, 0.9], [-0.5, 0.6, -0.8]], np.float32),
                                 field_points=S.grid_xy(8, 1.0, 1.2), cp=1500.0, f=8e3, att=0.05,
                                 bounces=1, field_objects=False)
    return out


def run_scene(eng, sc):
    eng.set_initial_conditions(sc["cp"], sc["f"], sc["att"])
    for tris, d in sc["targets"]:
        eng.load_geometry(tris, 0, d)
    for tris, d in sc["fields"]:
        eng.load_geometry(tris, 2, d)
    eng.load_source_points(sc["sources"])
    eng.load_field_points(sc["field_points"])
    eng.render()
    eng.project_sources(False)
    if sc["bounces"]:
        eng.project_bounces(sc["bounces"])
    if sc["field_objects"]:
        eng.project_field_objects()
    eng.project_field_points()
    res = {}
    for i in range(len(sc["targets"])):
        res["P_target%d" % i] = eng.pressures(0, i)
    for i in range(len(sc["fields"])):
        res["P_field%d" % i] = eng.pressures(2, i)
    res["P_points"] = eng.field_points()
    return res


def pack_inputs(sc):
    d = dict(cp=sc["cp"], f=sc["f"], att=sc["att"], bounces=sc["bounces"], field_objects=int(sc["field_objects"]),
             sources=sc["sources"], field_points=sc["field_points"],
             n_targets=len(sc["targets"]), n_fields=len(sc["fields"]))
    for i, (t, dl) in enumerate(sc["targets"]):
        d["target%d" % i] = t
        d["target%d_delta" % i] = np.float32(dl)
    for i, (t, dl) in enumerate(sc["fields"]):
        d["field%d" % i] = t
        d["field%d_delta" % i] = np.float32(dl)
    return d


def main(ref_root=None):
    args = ["sh", os.path.join(ROOT, "oracle", "build_ref.sh")] + ([ref_root] if ref_root else [])
    subprocess.check_call(args)
    ref = O.RefHarness()

    # fragmentation
    rng = np.random.default_rng(20240601)
    tris = [rng.normal(size=9).astype(np.float32) * np.float32(rng.uniform(0.2, 2.0)) for _ in range(64)]
    deltas = [np.float32(rng.uniform(0.01, 0.15)) for _ in range(64)]
    for t in S.plate_1x05():
        tris.append(t); deltas.append(np.float32(S.delta_for(10e3)))
    for t in S.trihedral(1.0):
        tris.append(t); deltas.append(np.float32(S.delta_for(40e3)))
    for t in S.icosphere(1, 1.0)[:8]:
        tris.append(t); deltas.append(np.float32(0.02))
    frag = {"tris": np.array(tris, np.float32), "deltas": np.array(deltas, np.float32)}
    ints, frames, areas, offs = [], [], [], [0]
    for t, d in zip(tris, deltas):
        (nx, ny, neg), fr, a = ref.fragment_triangle(t, float(d))
        ints.append((nx, ny, neg)); frames.append(fr); areas.append(a.ravel())
        offs.append(offs[-1] + a.size)
    frag["ints"] = np.array(ints, np.int32)
    frag["frames"] = np.array(frames, np.float32)
    frag["areas"] = np.concatenate(areas).astype(np.float32)
    frag["offsets"] = np.array(offs, np.int64)
    np.savez_compressed(os.path.join(HERE, "fragmentation.npz"), **frag)

    for name, sc in scene_defs().items():
        ref.reset()
        res = run_scene(ref, sc)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **pack_inputs(sc), **res)
        print("golden", name, {k: v.shape for k, v in res.items()})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
