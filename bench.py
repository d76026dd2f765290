"""Benchmark of the discrete Kirchhoff hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload trihedral60|trihedral40|sphere|plate]

Metric: fragment-pair interactions per second (the reference loops' candidate
pairs after the area gates, before the cosine and visibility gates): source
hop S * N_cells, bounces sum_{a != b} n_a n_b, readout N_active * M.

Workload (default): the learned-compression configuration's scene, run with
the plain FP32 path -- orthogonal trihedral with 1 m legs at 60 kHz
(delta = lambda / 7.5 = 3.29 mm, ~138.7k fragments), one source at 20 m on the
(1,1,1) diagonal, 2 fragment -> fragment bounces, readout to a 256 x 256
hemisphere of radius 2 m.  Synthetic, seeded inputs; nothing is read from disk.

A step is one full pass of the path on the resident scene: interaction masks
rebuilt (visibility included), source hop, 2 bounces, readout.  Each step is
bracketed by CUDA events on the library's own stream; the L2 is flushed
between steps (a 256 MB write) outside the events.  ``e2e`` runs the same
work through the public C ABI from host buffers each step: load the
triangles and points, set_initial_conditions, render_cuda (fragmentation,
upload), the projections and GetFieldPointPressures (device -> host).

N > 1 runs N independent replicas (the path runs on one GPU; there is no
data-path collective): value = pairs of all ranks / max-over-ranks time.

``--impl reference`` times the CPU oracle (a restatement of the reference's
sums, all host threads) on a bounded sample of the same workload; rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fragment-pair interactions/s on 1 GB300: plain vs compressed, at 1e-3 rel err"
UNIT = "pairs/s"
FLOP_PER_PAIR = 40.0   # algorithmic FP32 flop per interaction of the sum kernel
SFU_PER_PAIR = 3.0     # rsqrt, sin, cos


def workload(name):
    import __graft_entry__ as ge
    ge.load_package()
    from sonar_render_gb300 import scenes
    if name == "trihedral60":
        cfg = scenes.trihedral_config(60e3, bounces=2, n_theta=256, n_phi=256)
    elif name == "trihedral40":
        cfg = scenes.trihedral_config(40e3, bounces=3, n_theta=256, n_phi=256)
    elif name == "sphere":
        cfg = scenes.sphere_config(512, field_surface=True)
    elif name == "plate":
        cfg = scenes.plate_config()
    else:
        raise SystemExit("unknown workload %s" % name)
    return cfg


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_rank%d.csv" % gpu_index)

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def load_scene(api, cfg):
    api.TearDownCuda()
    api.set_initial_conditions(cfg["cp"], cfg["frequency"], cfg.get("attenuation", 0.0))
    for tris, d in cfg["targets"]:
        api.load_stl_mesh_to_cuda(tris, api.TARGET, d)
    for tris, d in cfg.get("fields", []):
        api.load_stl_mesh_to_cuda(tris, api.FIELD, d)
    api.load_points_to_cuda(cfg["sources"], isSource=True)
    if cfg.get("field_points") is not None:
        api.load_points_to_cuda(cfg["field_points"], isSource=False)
    api.render_cuda()


def projections(api, cfg):
    api.project_source_points_to_objects(False)
    if cfg.get("bounces", 0):
        api.project_target_to_target_objects(cfg["bounces"])
    if cfg.get("fields"):
        api.project_target_to_field_objects()
    if cfg.get("field_points") is not None:
        api.project_target_to_field_points()


def step_pairs(stats):
    return sum(h["pairs"] for h in stats["hops"])


def run_gb300(args):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as ge
    ge.load_package()
    from sonar_render_gb300 import api, build
    build.build()
    api.load_library()
    cfg = workload(args.workload)

    train_info = None
    if args.compress and args.select == 2:
        # the admissibility network learns from the exact method's blocks of
        # the same trihedral at other frequencies (untimed set-up)
        from sonar_render_gb300 import admissibility, scenes
        t0 = time.time()
        train_cfgs = [scenes.trihedral_config(f, bounces=1, n_theta=4, n_phi=4) for f in (40e3, 50e3)]
        X, y, loss = admissibility.train_on_scenes(train_cfgs, epochs=args.train_epochs, batch=256, lr=1e-3, seed=0)
        train_info = {"samples": int(len(y)), "scenes": ["trihedral_1m_40kHz", "trihedral_1m_50kHz"],
                      "epochs": args.train_epochs, "final_mse": loss, "seconds": round(time.time() - t0, 2)}
        print("network trained: %s" % json.dumps(train_info), file=sys.stderr)

    # ---- device-timed steps on the resident scene
    api.set_option("compress", args.compress)
    api.set_option("compress_select", args.select)
    load_scene(api, cfg)
    ext = torch.cuda.ExternalStream(api.stream_handle())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def one_step():
        api.set_option("drop_masks", 1)
        api.set_option("reset_pressures", 1)
        projections(api, cfg)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    if args.profile_only:
        # device work only, for profiler captures: no e2e, no CPU legs, no JSON line
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            one_step()
        torch.cuda.synchronize()
        print("profile-only: %d steps of %s done" % (args.steps, cfg["name"]))
        print(json.dumps(api.stats()["hops"][-4:]))
        api.TearDownCuda()
        return
    if world > 1:
        dist.barrier()
    api.set_option("reset_stats", 1)
    clocks = Clocks(local)
    clocks.start()
    times = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        one_step()
        e1.record(ext)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    clk = clocks.stop()
    if world > 1:
        dist.barrier()
    stats = api.stats()
    total_ms = float(sum(times))
    pairs_rank = step_pairs(stats)  # all timed steps
    t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_ms = float(t.item())
    value = pairs_rank * world / (max_ms * 1e-3)
    per_step = stats["hops"][: len(stats["hops"]) // max(args.steps, 1)]

    # ---- kernel breakdown and roofline of the dominant kernel
    kern = {}
    for h in stats["hops"]:
        name = {0: "source", 1: "field_points", 2: "bounce", 3: "field_object"}[h["hop"]]
        kern.setdefault("mask_" + name, 0.0)
        kern.setdefault("sum_" + name, 0.0)
        kern["mask_" + name] += h["mask_ms"]
        kern["sum_" + name] += h["sum_ms"]
    share = {k: round(v / total_ms, 4) for k, v in kern.items() if v > 0}
    f2f = [h for h in stats["hops"] if h["hop"] == 2]
    fp32_peak = api.measure_peak(0)
    mufu_peak = api.measure_peak(1)
    roofline = None
    if f2f and fp32_peak > 0 and mufu_peak > 0:
        # the bounce sum evaluates one Green's function per unordered pair and
        # applies it in both directions: per ordered pair 20 flop (half of the
        # 40-flop evaluation incl. one complex MAC) + 4 (the second MAC) and 1.5
        # MUFU ops; roofline pairs/s = min(FP32 / 24, MUFU / 1.5)
        flop_pp, sfu_pp = 24.0, 1.5
        roof = min(fp32_peak / flop_pp, mufu_peak / sfu_pp)
        launch_ms = sum(h["sum_ms"] for h in f2f) / len(f2f)
        pairs_launch = f2f[0]["pairs"]
        achieved = pairs_launch * flop_pp / (launch_ms * 1e-3) / 1e12
        peak = roof * flop_pp / 1e12
        roofline = {"kernel": "k_sum_f2f_sym (bounce sum, reciprocity)", "bound": "fp32+sfu",
                    "achieved": round(achieved, 3), "peak": round(peak, 3), "unit": "TFLOP/s",
                    "frac": round(achieved / peak, 4), "traffic": None, "pairs_per_launch": pairs_launch,
                    "pairs_per_s": round(pairs_launch / (launch_ms * 1e-3), 1), "launch_ms": round(launch_ms, 4),
                    "peak_source": "measured now by sonar_measure_peak: FP32 %.1f TFLOP/s, MUFU %.2f Top/s; "
                                   "roofline = min(FP32/24, MUFU/1.5) ordered pairs/s x 24 flop"
                                   % (fp32_peak / 1e12, mufu_peak / 1e12)}
    mask_f2f = [h for h in stats["hops"] if h["hop"] == 2 and h["mask_ms"] > 0]
    mask_info = None
    if mask_f2f:
        ms = sum(h["mask_ms"] for h in mask_f2f) / len(mask_f2f)
        nact = int(round(math.sqrt(max(f2f[0]["pairs"], 1))))
        mask_info = {"kernel": "k_mask<F2F>", "launch_ms": round(ms, 4),
                     "mask_bytes_written": None, "note": "1 bit per ordered pair"}

    # block classes of the interaction masks (an untimed extra step)
    api.set_option("class_stats", 1)
    api.set_option("drop_masks", 1)
    api.set_option("reset_pressures", 1)
    api.set_option("reset_stats", 1)
    projections(api, cfg)
    mask_classes = api.stats().get("mask_classes")
    api.set_option("class_stats", 0)

    # ---- end to end through the C ABI from host buffers
    api.TearDownCuda()
    e2e_times = []
    h2d = d2h = 0
    npts = 0 if cfg.get("field_points") is None else len(cfg["field_points"])
    for k in range(max(1, min(args.steps, 3)) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        load_scene(api, cfg)
        projections(api, cfg)
        res = api.GetFieldPoints(npts) if npts else api.get_object_pressures(api.TARGET, 0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        st = api.stats()
        if k > 0:  # the first one warms the host allocator and the driver
            e2e_times.append(t1 - t0)
            h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
        api.TearDownCuda()
    e2e_s = statistics.median(e2e_times)
    e2e_pairs = pairs_rank / max(args.steps, 1)
    e2e = {"value": e2e_pairs * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "s_per_step": round(e2e_s, 4)}

    # ---- error vs FP64 on a seeded subset (bounce 1) and CPU baseline, rank 0
    extra = {}
    cpu = None
    if rank == 0:
        extra = check_error(api, cfg)
        cpu = cpu_baseline(cfg, args.cpu_seconds)
    launches = stats["launches"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded trihedral mesh and points, generated in-process)",
        "config": {"workload": cfg["name"] + "_plain_fp32", "fragments": extra.get("fragments"),
                   "bounces": cfg.get("bounces", 0), "sources": int(len(cfg["sources"])),
                   "field_points": npts, "pairs_per_step": e2e_pairs, "l2": "flushed between steps (256 MB write)",
                   "path": "plain FP32 sums + interaction masks (rebuilt every step)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": roofline, "mask_kernel": mask_info, "kernel_share": share, "mask_block_classes": mask_classes,
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": launches,
        "rel_err_vs_fp64": extra.get("errors"), "grazing": extra.get("grazing"),
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def check_error(api, cfg):
    """Bounce-1 and readout relative L2 error vs the FP64 oracle on seeded
    destinations, given the GPU's own inputs."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    out = {}
    try:
        load_scene(api, cfg)
        api.project_source_points_to_objects(False)
        P0 = api.get_object_pressures(api.TARGET, 0)
        api.project_target_to_target_objects(1)
        P1 = api.get_object_pressures(api.TARGET, 0)
        npts = len(cfg["field_points"]) if cfg.get("field_points") is not None else 0
        if npts:
            api.project_target_to_field_points()
            fp = api.GetFieldPoints(npts)
            fp = fp[:, 0] + 1j * fp[:, 1]
        api.TearDownCuda()
        o = O.Oracle()
        o.set_initial_conditions(cfg["cp"], cfg["frequency"], cfg.get("attenuation", 0.0))
        for tris, d in cfg["targets"]:
            o.load_geometry(tris, 0, d)
        o.load_source_points(cfg["sources"])
        if npts:
            o.load_field_points(cfg["field_points"])
        o.render()
        act = o.active(0, 0)
        out["fragments"] = int(len(act))
        rng = np.random.default_rng(2024)
        q = np.sort(rng.choice(len(act), min(32, len(act)), replace=False))
        nact = len(act)
        v1, m1 = o.hop_subset(2, 0, 0, q, pin=P0, want_mask=True, nsrc=nact)
        c1 = o.counters()
        g1 = (m1 & 2).any(axis=1)
        d1 = (P1 - P0)[act[q]]
        e = {"bounce1": float(np.linalg.norm(d1 - v1) / np.linalg.norm(v1))}
        if (~g1).any():
            e["bounce1_nongrazing_dst"] = float(np.linalg.norm((d1 - v1)[~g1]) / np.linalg.norm(v1[~g1]))
        graze = {"bounce_pairs_checked": c1["pairs"], "bounce_grazing": c1["grazing"]}
        if npts:
            o.set_pressures(0, 0, P1)
            jj = np.sort(rng.choice(npts, min(32, npts), replace=False))
            vf, mf = o.hop_subset(1, 0, 0, jj, want_mask=True, nsrc=nact)
            c2 = o.counters()
            gf = (mf & 2).any(axis=1)
            e["readout"] = float(np.linalg.norm(fp[jj] - vf) / np.linalg.norm(vf))
            if (~gf).any():
                e["readout_nongrazing_dst"] = float(np.linalg.norm((fp[jj] - vf)[~gf]) / np.linalg.norm(vf[~gf]))
            graze.update({"readout_pairs_checked": c2["pairs"], "readout_grazing": c2["grazing"],
                          "readout_dst_with_grazing": int(gf.sum())})
        out["errors"] = e
        out["grazing"] = graze
    except Exception as ex:  # the error check must not hide the timing
        out["errors"] = {"failed": str(ex)}
    return out


def cpu_sample(cfg, seconds, threads=None):
    """Time the FP64 oracle on bounce destinations until ~seconds of work."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    o = O.Oracle()
    o.set_initial_conditions(cfg["cp"], cfg["frequency"], cfg.get("attenuation", 0.0))
    for tris, d in cfg["targets"]:
        o.load_geometry(tris, 0, d)
    o.load_source_points(cfg["sources"])
    o.render()
    o.project_sources(False)
    P = o.pressures(0, 0)
    nact = o.nact(0, 0)
    rng = np.random.default_rng(99)
    n = 8
    t0 = time.perf_counter()
    o.hop_subset(2, 0, 0, np.sort(rng.choice(nact, n, replace=False)), pin=P)
    dt = max(time.perf_counter() - t0, 1e-3)
    n = int(min(nact, max(8, n * seconds / dt)))
    q = np.sort(rng.choice(nact, n, replace=False))
    t0 = time.perf_counter()
    o.hop_subset(2, 0, 0, q, pin=P)
    dt = time.perf_counter() - t0
    pairs = o.counters()["pairs"]
    return pairs, dt, n, O.num_threads()


def cpu_baseline(cfg, seconds):
    try:
        pairs, dt, n, th = cpu_sample(cfg, seconds)
        return {"value": pairs / dt, "unit": UNIT, "cores": th, "kind": "port",
                "sample": "FP64 oracle, bounce sums of %d seeded destinations (%d pairs, %.1f s), %d threads"
                          % (n, pairs, dt, th)}
    except Exception as ex:
        return {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": "failed: %s" % ex}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    cfg = workload(args.workload)
    vals = []
    info = None
    for k in range(args.warmup + args.steps):
        pairs, dt, n, th = cpu_sample(cfg, args.cpu_seconds / max(args.steps, 1))
        if k >= args.warmup:
            vals.append(pairs / dt)
            info = (pairs, dt, n, th)
    v = statistics.median(vals)
    pairs, dt, n, th = info
    cpu = {"value": v, "unit": UNIT, "cores": th, "kind": "port",
           "sample": "FP64 oracle restating the reference's sums (src/OptiX.cu:192-406), bounce destinations: "
                     "%d per step, %d pairs, %.1f s, %d threads" % (n, pairs, dt, th)}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": cfg["name"] + "_plain_fp32", "sample": "bounce destinations on host cores"},
            "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference's own hot path is OptiX GPU code; its CPU restatement (the oracle) runs here"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="trihedral60")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--profile-only", action="store_true",
                    help="run warm-up and steps of device work only (for ncu captures)")
    ap.add_argument("--compress", type=int, default=0, help="compress admissible bounce blocks (low rank)")
    ap.add_argument("--select", type=int, default=0,
                    help="compressed blocks: 0 separation rule, 1 every interacting block, 2 the trained network")
    ap.add_argument("--train-epochs", type=int, default=40)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
