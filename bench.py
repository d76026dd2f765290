"""Benchmark of the discrete Kirchhoff hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload trihedral60|trihedral40|sphere|plate|batch] [--mode both|plain|compressed]
                    [--batch 0|1]

Metric: fragment-pair interactions per second (the reference loops' candidate
pairs after the area gates, before the cosine and visibility gates): source
hop S * N_cells, bounces sum_{a != b} n_a n_b, readout N_active * M.  A
compressed bounce performs the same interactions through low-rank factors, so
its rate is those pairs over its time.

Workload (default, trihedral60): the learned-compression configuration --
orthogonal trihedral with 1 m legs at 60 kHz (delta = lambda / 7.5 =
3.29 mm, ~139k fragments), one source at 20 m on the (1,1,1) diagonal, source
hop then 2 fragment -> fragment bounces.  Synthetic, seeded inputs; nothing is
read from disk.  Two paths run on it:
  plain       every pair on the fly in FP32 (hand-written sums), masks rebuilt
              every step;
  compressed  the admissibility network proposes blocks and rank caps, cross
              approximation builds them and the exact entries judge them, the
              rest stays on the plain kernel -- masks, descriptors, network
              inference and approximation rebuilt every step.
``value`` is the compressed path's rate, ``plain`` the plain one's; both are
checked against each other over every fragment and against the FP64 oracle
on seeded destinations of each bounce.  The network is trained before the
timed region on the same trihedral at 40 and 50 kHz (never on the 60 kHz
blocks it is evaluated on).

Each step is bracketed by CUDA events on the library's own stream; the L2 is
flushed between steps (a 256 MB write) outside the events.  ``e2e`` runs the
same work through the public C ABI from host buffers each step: load the
triangles and points, set_initial_conditions, render_cuda (fragmentation,
upload), the projections and the read-back of the surface pressures.

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
        cfg = scenes.trihedral_config(60e3, bounces=2, n_theta=0, n_phi=0)
    elif name == "trihedral40":
        cfg = scenes.trihedral_config(40e3, bounces=3, n_theta=256, n_phi=256)
    elif name == "trihedral40_2b":
        cfg = scenes.trihedral_config(40e3, bounces=2, n_theta=0, n_phi=0)
    elif name == "sphere":
        cfg = scenes.sphere_config(512, field_surface=True)
    elif name == "sphere10":
        # the same scene at 10 kHz (a quarter of the fragments): profiler captures
        cfg = scenes.sphere_config(512, field_surface=True, frequency=10e3)
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
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix="sonar_clocks_rank%d_" % self.idx, suffix=".csv")
            self.fh = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.fh,
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
        try:
            os.remove(self.path)
        except OSError:
            pass
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


RCUT = [32.0]  # the admissibility network proposes blocks with predicted rank below this
TOL = [7e-4]   # cross-approximation tolerance (the judge accepts 3 x this RMS error)
ACA_VARIANT = [8]  # cross-approximation kernel shape (k_aca / k_aca2, factor ranks in shared memory, CTAs per SM)
OVERLAP = [1]      # compressed bounce: low-rank apply on a second stream beside the dense remainder
LR_CTAS = [4]      # low-rank apply: resident CTAs per SM (register cap)
FUSED = [1]        # k_aca2: the first bounce's low-rank apply fused into the cross approximation
INTERP = [1]       # far class-ALL blocks between planar tiles by directional interpolation
BUILD_OVERLAP = [1]  # interpolation build on a second stream beside the cross approximation
TILE_ALIGN = [1]     # full patches of the fragment grid on 256-fragment tile boundaries
IP_TRANSPOSE = [0]   # 1: interpolation tiles taller than wide take the grid's y axis first


def set_path(api, compressed, select):
    api.set_option("compress", 1 if compressed else 0)
    api.set_option("compress_select", select if compressed else 0)
    api.set_option("compress_rcut", RCUT[0])
    api.set_option("compress_tol", TOL[0])
    api.set_option("compress_judge", 3.0 * TOL[0])
    api.set_option("aca_variant", ACA_VARIANT[0])
    api.set_option("aca_fused_apply", FUSED[0])
    api.set_option("lr_block_ctas", LR_CTAS[0])
    api.set_option("overlap_streams", OVERLAP[0])
    api.set_option("compress_interp", INTERP[0])
    api.set_option("compress_build_overlap", BUILD_OVERLAP[0])
    api.set_option("tile_align", TILE_ALIGN[0])
    api.set_option("ip_transpose", IP_TRANSPOSE[0])


def time_path(api, cfg, args, flush, local, world, reuse=False):
    """Warm-up and K timed steps of the current path on the loaded scene;
    returns (times ms, stats, clocks).  Events are recorded on the library's
    stream of this scene (load_scene recreates it).  Every step rebuilds the
    interaction masks (and with them the compressed blocks) unless reuse is
    set: then the first warm-up step builds them and the others reuse them
    (a static target, as for a sequence of pings)."""
    import torch
    import torch.distributed as dist
    ext = torch.cuda.ExternalStream(api.stream_handle())

    def one_step():
        if not reuse:
            api.set_option("drop_masks", 1)
        api.set_option("reset_pressures", 1)
        projections(api, cfg)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
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
    return times, api.stats(), clk


def max_over_ranks(ms, world, device="cuda"):
    """The slowest rank's time (replicas: the job ends with its last rank)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(pairs_step, steps, world, total_ms):
    """Whole-job pairs/s: every rank runs the same workload (weak scaling),
    over the slowest rank's time."""
    return pairs_step * steps * world / (total_ms * 1e-3)


def kernel_times(stats, steps):
    """Per-step device time of each kernel group from the library's records."""
    k = {}
    for h in stats["hops"]:
        name = {0: "source", 1: "field_points", 2: "bounce", 3: "field_object", 4: "cross_object",
                5: "piston_target", 6: "piston_field_object"}.get(h["hop"], "hop%d" % h["hop"])
        k["mask_" + name] = k.get("mask_" + name, 0.0) + h["mask_ms"]
        k["sum_" + name] = k.get("sum_" + name, 0.0) + h["sum_ms"]
        if h.get("lr_ms"):
            k["lowrank_apply"] = k.get("lowrank_apply", 0.0) + h["lr_ms"]
        if h.get("cmp_build_ms"):
            k["select_blocks"] = k.get("select_blocks", 0.0) + h["cmp_select_ms"]
            # the cross approximation and the interpolation run on two streams
            # side by side: each one's own time, and both together
            k["cross_approx"] = k.get("cross_approx", 0.0) + h["cmp_aca_ms"]
            k["interpolation"] = k.get("interpolation", 0.0) + h.get("cmp_ip_ms", 0.0)
            appr = h.get("cmp_approx_ms") or h["cmp_aca_ms"]
            k["approximation_both"] = k.get("approximation_both", 0.0) + appr
            k["build_other"] = k.get("build_other", 0.0) + h["cmp_build_ms"] - h["cmp_select_ms"] - appr
    return {n: v / max(steps, 1) for n, v in k.items() if v > 0}


def sym_roofline(api, f2f):
    fp32_peak = api.measure_peak(0)
    mufu_peak = api.measure_peak(1)
    if not f2f or not (fp32_peak > 0 and mufu_peak > 0):
        return None, fp32_peak
    # the bounce sum evaluates one Green's function per unordered pair and
    # applies it in both directions: per ordered pair 20 flop (half of the
    # 40-flop evaluation incl. one complex MAC) + 4 (the second MAC) and 1.5
    # MUFU ops; roofline pairs/s = min(FP32 / 24, MUFU / 1.5)
    flop_pp, sfu_pp = 24.0, 1.5
    roof = min(fp32_peak / flop_pp, mufu_peak / sfu_pp)
    launch_ms = sum(h["sum_ms"] for h in f2f) / len(f2f)
    # on the compressed path the kernel evaluates only the pairs outside the accepted blocks
    pairs_launch = f2f[0]["pairs"] - f2f[0].get("cmp_pairs", 0)
    achieved = pairs_launch * flop_pp / (launch_ms * 1e-3) / 1e12
    peak = roof * flop_pp / 1e12
    name = "k_sum_f2f_sym (bounce sum, reciprocity)" if not f2f[0].get("cmp_pairs") else \
        "k_sum_f2f_sym (dense remainder of the compressed bounce)"
    return {"kernel": name, "bound": "fp32+sfu",
            "achieved": round(achieved, 3), "peak": round(peak, 3), "unit": "TFLOP/s",
            "frac": round(achieved / peak, 4), "traffic": None, "pairs_per_launch": pairs_launch,
            "pairs_per_s": round(pairs_launch / (launch_ms * 1e-3), 1), "launch_ms": round(launch_ms, 4),
            "peak_source": "measured now by sonar_measure_peak: FP32 %.1f TFLOP/s, MUFU %.2f Top/s; "
                           "roofline = min(FP32/24, MUFU/1.5) ordered pairs/s x 24 flop"
                           % (fp32_peak / 1e12, mufu_peak / 1e12)}, fp32_peak


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        for k in ("hbm_gbs", "hbm_GBs", "hbm"):
            if k in d:
                v = d[k]
                return float(v if not isinstance(v, dict) else v.get("value")), "MEASURED_PEAKS.json hbm_gbs"
    except Exception:
        pass
    return 6800.0, "fallback 6.8 TB/s"


def lowrank_roofline(stats):
    """The second bounce's apply of the accepted blocks: the factor blocks
    (k_lr_block) are HBM-bound -- per block U, V (rank x 256 complex FP32
    each) read once -- the interpolated blocks' (k_ip apply) read their node
    entries ((P (P | 1) + 156) complex FP32) and are bound by FP32 issue;
    every block writes 2 x 256 complex FP32 outputs that the gather reads
    back.  The figure is the HBM rate of these bytes over the whole apply."""
    hops = [h for h in stats["hops"] if h["hop"] == 2 and h.get("lr_ms")]
    if not hops:
        return None
    h = hops[0]
    nacc = h["cmp_accepted"]
    nip = h.get("cmp_ip_blocks", 0)
    P = h.get("cmp_ip_nodes", 0.0)
    factor_bytes = (nacc - nip) * h["cmp_mean_rank"] * 256 * 8 * 2
    node_bytes = nip * (P * (int(P) | 1) + 156) * 8
    bytes_launch = factor_bytes + node_bytes + nacc * 256 * 8 * 2 * 2
    ms = sum(x["lr_ms"] for x in hops) / len(hops)
    peak, src = hbm_peak()
    ach = bytes_launch / (ms * 1e-3) / 1e9
    # k_lr_block's DRAM bytes were 0.985 x these algorithmic bytes in the ncu
    # capture on the 40 kHz trihedral at tolerance 5e-4 (1.141 GB for 19,502
    # blocks at rank 13.5)
    return {"kernel": "k_lr_block + k_ip apply + k_lr_gather (second bounce's apply of the accepted blocks)",
            "bound": "hbm for the factor blocks; fp32 issue for the interpolated ones", "achieved": round(ach, 1),
            "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4), "traffic": round(0.985 * bytes_launch),
            "traffic_source": "ncu dram bytes of k_lr_block on the 40 kHz capture, scaled by algorithmic bytes",
            "bytes_per_launch": int(bytes_launch), "launch_ms": round(ms, 4), "peak_source": src,
            "blocks": nacc, "interpolated_blocks": nip, "mean_rank": h["cmp_mean_rank"]}


def aca_roofline(stats, fp32_peak):
    """Cross approximation (k_aca2: with the first bounce's low-rank apply of
    every accepted block fused), FP32 work per launch: per approximated block
    of rank k, 2 k residual rows/columns of 256 entries plus 512 judged
    entries at 48 flop per Green's function evaluation, the residual updates
    (2 x 256 x k (k - 1) / 2 complex MACs, 8 flop each), the judged entries'
    approximations (512 k complex MACs) and the fused apply (4 x 256 x k
    complex MACs); k = the mean accepted rank."""
    hops = [h for h in stats["hops"] if h["hop"] == 2 and h.get("cmp_aca_ms")]
    if not hops or not fp32_peak:
        return None
    h = hops[0]
    k = h["cmp_mean_rank"]
    nb = h["cmp_blocks"] - h.get("cmp_ip_blocks", 0)  # the interpolated blocks have their own kernel
    flop_block = 48.0 * (2 * 256 * k + 512) + 8.0 * 256 * k * (k - 1) + 8.0 * 512 * k + 8.0 * 4 * 256 * k
    ms = sum(x["cmp_aca_ms"] for x in hops) / len(hops)
    ach = nb * flop_block / (ms * 1e-3) / 1e12
    peak = fp32_peak / 1e12
    # DRAM bytes per (block x rank) from the ncu capture of this kernel on the
    # 40 kHz trihedral with every interacting block approximated at tolerance
    # 5e-4 (0.116 GB read + 1.138 GB written for 20,170 blocks at mean rank
    # 13.5: the factors written once), scaled to this launch by blocks x rank
    traffic = 4605.0 * nb * k
    return {"kernel": "k_aca2 (cross approximation + exact-entry judge + first bounce's low-rank apply)",
            "bound": "fp32 issue / load latency (serial pivots)",
            "achieved": round(ach, 3), "peak": round(peak, 3), "unit": "TFLOP/s", "frac": round(ach / peak, 4),
            "traffic": round(traffic), "traffic_source": "ncu dram bytes of the 40 kHz capture, scaled by blocks x rank",
            "blocks_per_launch": nb, "mean_rank": k, "flop_per_block": round(flop_block),
            "launch_ms": round(ms, 4), "peak_source": "FP32 FMA rate measured now by sonar_measure_peak"}


def ip_roofline(stats, fp32_peak):
    """Directional interpolation build (k_ip<BUILD>: node entries, judge and
    the first bounce's apply), FP32 work per launch.  Per interpolated block
    of P nodes (px x py, px = sqrt(1.4 P) for the mean level) and the 4 x 3
    smooth nodes: (P^2 + 144) node entries at 45 flop; the judge, 8 P^2 +
    96 x 12 complex MACs (8 flop) and 64 exact entries at 48 flop; the apply,
    per side a projection and an expansion over the 16 x 16 occupied cells
    (16 x 16 x px + P x 16 complex MACs each) and the smooth part's
    (16 x 16 x 4 + 12 x 16 real x complex, 4 flop), and the couplings 2 P^2
    complex and 2 x 144 real x complex MACs."""
    hops = [h for h in stats["hops"] if h["hop"] == 2 and h.get("cmp_ip_ms")]
    if not hops or not fp32_peak or not hops[0].get("cmp_ip_blocks"):
        return None
    h = hops[0]
    P = h["cmp_ip_nodes"]
    nb = h["cmp_ip_blocks"]
    px = (1.4 * P) ** 0.5
    apply = 8.0 * 4 * (256 * px + 16 * P) + 4.0 * 4 * (256 * 4 + 12 * 16) + 8.0 * 2 * P * P + 4.0 * 2 * 144
    flop_block = 45.0 * (P * P + 144) + 8.0 * (8 * P * P + 96 * 12) + 48.0 * 64 + apply
    ms = sum(x["cmp_ip_ms"] for x in hops) / len(hops)
    ach = nb * flop_block / (ms * 1e-3) / 1e12
    peak = fp32_peak / 1e12
    # DRAM: the node entries written once; the ncu capture at 40 kHz wrote
    # 77.7 MB for 11,535 blocks of mean 28.2 nodes (6.7 KB per block), here
    # scaled by the stored entries per block
    traffic = nb * (P * P + 156) * 8.0 * (77.7e6 / (11535 * (28.2 * 28.2 + 156) * 8.0))
    return {"kernel": "k_ip build (directional interpolation: node entries + 8 x 8 exact-entry judge + first bounce's "
                      "apply)", "bound": "fp32 issue / barrier latency (seven dependent phases per block)",
            "achieved": round(ach, 3), "peak": round(peak, 3), "unit": "TFLOP/s", "frac": round(ach / peak, 4),
            "traffic": round(traffic), "traffic_source": "ncu dram bytes of the 40 kHz capture per stored entry",
            "blocks_per_launch": nb, "mean_nodes": P, "flop_per_block": round(flop_block),
            "launch_ms": round(ms, 4), "timed": "its own stream's span",
            "peak_source": "FP32 FMA rate measured now by sonar_measure_peak"}


def e2e_path(api, cfg, args, world, pairs_step):
    import torch
    api.TearDownCuda()
    e2e_times, render_ms = [], []
    h2d = d2h = 0
    npts = 0 if cfg.get("field_points") is None else len(cfg["field_points"])
    for k in range(max(1, min(args.steps, 3)) + 1):
        api.set_option("reset_stats", 1)  # the transfer counters of this step only
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        load_scene(api, cfg)
        projections(api, cfg)
        api.GetFieldPoints(npts) if npts else api.get_object_pressures(api.TARGET, 0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        st = api.stats()
        if k > 0:  # the first one warms the host allocator and the driver
            e2e_times.append(t1 - t0)
            h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
            render_ms.append(st.get("render_host_ms") or {})
        api.TearDownCuda()
    e2e_s = statistics.median(e2e_times)
    # host time of render_cuda inside the step (facet frames, fragment grids and
    # areas, tile order, uploads), median over the steps per part
    parts = sorted({p for r in render_ms for p in r})
    host = {p: round(statistics.median([float(r.get(p, 0.0)) for r in render_ms]), 4) for p in parts}
    return {"value": pairs_step * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "s_per_step": round(e2e_s, 4), "render_host_ms": host}


def batch_leg(args, flush, rank):
    """The many-source, many-frequency batch (16 seeded scenes, 64 arc
    positions as sources and receivers, 8 frequencies): device time of the
    captured run graph (CUDA events inside the graph, on the plan's stream),
    L2 flushed between runs; e2e = plan + run + result read-back + free
    through the C ABI from host buffers; error vs the FP64 oracle on sampled
    items and sources (rank 0)."""
    import torch
    from sonar_render_gb300 import api as api_mod, batch, scenes
    cfg = scenes.batch_config(0)
    args_b = (cfg["scenes"], cfg["sources"], cfg["receivers"], cfg["freqs"], cfg["cp"], cfg["attenuation"],
              cfg["per_wavelength"])
    t0 = time.perf_counter()
    plan = batch.Plan(*args_b)
    plan_s = time.perf_counter() - t0
    for _ in range(max(args.warmup, 1)):
        plan.run(copy=False)
    dev = []
    parts = {"vis_ms": [], "gemm_ms": [], "reduce_ms": []}
    for _ in range(max(args.steps, 1)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        plan.run(copy=False)
        st = plan.stats()
        for k in parts:
            parts[k].append(st[k])
        dev.append(st["vis_ms"] + st["gemm_ms"] + st["reduce_ms"])
    out = plan.run()
    st = plan.stats()
    ms = statistics.median(dev)
    pairs = st["pairs"]
    # the same runs with the centroid-relative phase (FP64 point offsets from
    # each scene's box centre): its device time and its result
    plan.set_relative(True)
    for _ in range(max(args.warmup, 1)):
        plan.run(copy=False)
    dev_rel, gemm_rel = [], []
    for _ in range(max(args.steps, 1)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        plan.run(copy=False)
        sr = plan.stats()
        dev_rel.append(sr["vis_ms"] + sr["gemm_ms"] + sr["reduce_ms"])
        gemm_rel.append(sr["gemm_ms"])
    out_rel = plan.run()
    plan.set_relative(False)
    ms_rel = statistics.median(dev_rel)
    # e2e through the reused plan, as a sequence of pings at the same scenes:
    # each run uploads its source and receiver positions from host memory,
    # runs the graph and reads the result back
    e2e_reuse = []
    for _ in range(max(args.steps, 3)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plan.set_points(cfg["sources"], cfg["receivers"])
        plan.run(copy=True)
        e2e_reuse.append(time.perf_counter() - t0)
    e2e_reuse_s = statistics.median(e2e_reuse)
    # and the one-shot entry point from host buffers (fragmentation on the
    # host, uploads, tuning from the process cache, graph, run, read-back)
    e2e = []
    for _ in range(2):
        t0 = time.perf_counter()
        batch.run_batch(*args_b)
        e2e.append(time.perf_counter() - t0)
    e2e_s = min(e2e)
    nfrag = st["fragments"]
    # operand generation against its MUFU bound: every evaluation takes 3 MUFU
    # ops (rsqrt, sin, cos); evaluations per run = fragments x (receivers + sources)
    mufu = api_mod.measure_peak(1)
    evals = nfrag * (st["receivers"] + st["sources"])
    gem = statistics.median(parts["gemm_ms"])
    gen = {"green_evaluations_per_s": evals / (gem * 1e-3), "mufu_ops_per_evaluation": 3,
           "mufu_peak_ops_per_s": mufu,
           "frac_of_mufu_bound": round(evals * 3 / (gem * 1e-3) / mufu, 4) if mufu > 0 else None}
    h2d = int(nfrag * (3 * 16 + 4) + sum(t.nbytes for t in cfg["scenes"]))
    d2h = int(out.size * 16)
    err = None
    if rank == 0:
        err = batch_error(cfg, out, out_rel, st)
    # tensor-core work of the run: 3 split products x 2 (real embedding)
    # x 2 flop per MAC over the 128 x 64 x (2 K) products
    flops = 3 * 2 * 128 * 64 * 2 * nfrag
    res = {"workload": cfg["name"], "items": st["items"], "fragments": nfrag, "pairs_per_run": pairs,
           "value": pairs / (ms * 1e-3), "unit": UNIT, "ms_per_run": round(ms, 4),
           "kernel_ms": {k: round(statistics.median(v), 4) for k, v in parts.items()},
           "tensor_tflops_achieved": round(flops / (statistics.median(parts["gemm_ms"]) * 1e-3) / 1e12, 2),
           "green_evaluations_per_run": int(nfrag * (st["receivers"] + st["sources"])),
           "tuning": st["tuning"], "plan_s": round(plan_s, 3), "convex_scenes": st["convex_scenes"],
           "shadow_tests_per_run": st.get("shadow_tests"),
           "e2e": {"value": pairs / e2e_reuse_s, "unit": UNIT,
                   "h2d_bytes_per_step": int(len(cfg["sources"]) * 12 + len(cfg["receivers"]) * 12),
                   "d2h_bytes_per_step": d2h, "s_per_step": round(e2e_reuse_s, 5),
                   "path": "reused plan: set_points + run + read-back per run (sonar_batch_set_points, sonar_batch_run)"},
           "e2e_one_shot": {"value": pairs / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                            "s_per_step": round(e2e_s, 4), "path": "sonar_run_batch: plan, tune (cached), run, free"},
           "generation": gen,
           "relative_phase": {"ms_per_run": round(ms_rel, 4), "slowdown": round(ms_rel / ms - 1.0, 4),
                              "gemm_ms": round(statistics.median(gemm_rel), 4),
                              "path": "sonar_batch_set_relative(plan, 1): points as FP64 offsets from the scene's "
                                      "box centre, k R reduced on the host"},
           "rel_err_vs_fp64": err, "dtype": "split bf16 x3, fp32 accumulate, compensated reduce combined in fp64",
           "l2": "flushed between runs (256 MB write)"}
    plan.close()
    return res


def sum_roofline(stats, hop, fp32_peak, mufu_peak, name):
    """FP32 + MUFU roofline of one hop's sum kernel (k_sum: 40 flop + 3 MUFU
    per ordered pair): algorithmic flop per launch over its event time."""
    hs = [h for h in stats["hops"] if h["hop"] == hop and h["sum_ms"] > 0]
    if not hs or not (fp32_peak > 0 and mufu_peak > 0):
        return None
    pairs = sum(h["pairs"] for h in hs) / len(hs)
    ms = sum(h["sum_ms"] for h in hs) / len(hs)
    roof = min(fp32_peak / FLOP_PER_PAIR, mufu_peak / SFU_PER_PAIR)
    ach = pairs * FLOP_PER_PAIR / (ms * 1e-3) / 1e12
    peak = roof * FLOP_PER_PAIR / 1e12
    return {"kernel": name, "bound": "fp32+sfu", "achieved": round(ach, 3), "peak": round(peak, 3),
            "unit": "TFLOP/s", "frac": round(ach / peak, 4), "traffic": None, "pairs_per_launch": int(pairs),
            "launch_ms": round(ms, 4),
            "peak_source": "measured now by sonar_measure_peak: FP32 %.1f TFLOP/s, MUFU %.2f Top/s; roofline = "
                           "min(FP32/40, MUFU/3) pairs/s x 40 flop" % (fp32_peak / 1e12, mufu_peak / 1e12)}


def mask_roofline(stats, hop, name):
    """The mask kernel against HBM at its algorithmic 0.125 B (one bit) per
    candidate pair: how far the shadow tests keep it from the bandwidth
    bound."""
    hs = [h for h in stats["hops"] if h["hop"] == hop and h["mask_ms"] > 0]
    if not hs:
        return None
    pairs = sum(h["pairs"] for h in hs) / len(hs)
    ms = sum(h["mask_ms"] for h in hs) / len(hs)
    peak, src = hbm_peak()
    ach = pairs * 0.125 / (ms * 1e-3) / 1e9
    return {"kernel": name, "bound": "hbm (algorithmic bit per pair); shadow tests make it ALU/issue-bound",
            "achieved": round(ach, 1), "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4), "traffic": None,
            "launch_ms": round(ms, 4), "pairs_per_launch": int(pairs), "peak_source": src}


def config5_as_written(api, cfg, args, flush, local, world, rank, select):
    """The learned-compression configuration as written: cross-approximation
    tolerance 1e-4 (judge limit 3e-4), the 4-layer width-128 network with
    FP16 hidden layers on the tensor cores (FP32 input and output layers,
    FP32 training), trained on labels at that tolerance (40 and 50 kHz
    trihedral, as the headline)."""
    from sonar_render_gb300 import admissibility, scenes
    saved_tol, saved_params = TOL[0], admissibility.get_params()
    saved_width = admissibility.width()
    try:
        TOL[0] = 1e-4
        admissibility.set_width(128)
        admissibility.init(0)
        api.set_option("compress_tol", TOL[0])
        api.set_option("compress_judge", 3.0 * TOL[0])
        t0 = time.time()
        train_cfgs = [scenes.trihedral_config(f, bounces=1, n_theta=0, n_phi=0) for f in (40e3, 50e3)]
        _, y, loss = admissibility.train_on_scenes(train_cfgs, epochs=args.train_epochs, batch=256, lr=1e-3, seed=0)
        train_s = time.time() - t0
        set_path(api, True, select)
        load_scene(api, cfg)
        import types
        A = types.SimpleNamespace(steps=max(3, min(args.steps, 10)), warmup=3)
        times, stats, clk = time_path(api, cfg, A, flush, local, world)
        total_ms = max_over_ranks(float(sum(times)), world)
        pairs_step = step_pairs(stats) / A.steps
        h = [x for x in stats["hops"] if x["hop"] == 2 and x.get("cmp_build_ms")][0]
        res = {"tolerance": TOL[0], "judge_limit": 3.0 * TOL[0],
               "network": "8-128-128-128-1: FP16 hidden layers on the tensor cores (tcgen05), FP32 input/output "
                          "layers and training",
               "training_samples": int(len(y)), "training_mse_log2rank": round(loss, 5), "training_s": round(train_s, 2),
               "value": job_value(pairs_step, A.steps, world, total_ms), "unit": UNIT,
               "ms_per_step": round(total_ms / A.steps, 4), "steps": A.steps,
               "kernel_ms_per_step": {k: round(v, 4) for k, v in kernel_times(stats, A.steps).items()},
               "accepted": h["cmp_accepted"], "approximated": h["cmp_blocks"], "mean_rank": h["cmp_mean_rank"],
               "clocks": clk}
        if rank == 0:
            res["rel_err_vs_fp64"] = check_error(api, cfg).get("errors")
        return res
    finally:
        TOL[0] = saved_tol
        admissibility.set_width(saved_width)
        admissibility.set_params(saved_params)
        set_path(api, True, select)


def config_leg(api, name, args, flush, local, world, rank):
    """One of the other benchmark configurations on the plain FP32 path:
    device-timed steps (masks rebuilt every step, L2 flushed between steps),
    pairs/s, kernel times, the dominant kernels' rooflines, error vs the
    FP64 oracle on seeded destinations and the grazing counts (rank 0).
      sphere20   r = 1 m icosphere (5,120 triangles) at 20 kHz, source at
                 10 m, shadowed source hop + FACET_NO_RESP onto the 512 x 512
                 cell field plane through the centre;
      trihedral40  trihedral at 40 kHz, source hop, 3 bounces, readout to a
                 256 x 256 hemisphere of field points."""
    from sonar_render_gb300 import scenes
    if name == "sphere20":
        cfg = scenes.sphere_config(512, field_surface=True)
    else:
        cfg = scenes.trihedral_config(40e3, bounces=3, n_theta=256, n_phi=256)
    set_path(api, False, 0)
    load_scene(api, cfg)

    import types
    A = types.SimpleNamespace(steps=max(3, min(args.steps, 10)), warmup=3)
    times, stats, clk = time_path(api, cfg, A, flush, local, world)
    total_ms = max_over_ranks(float(sum(times)), world)
    pairs_step = step_pairs(stats) / A.steps
    kms = {k: round(v, 4) for k, v in kernel_times(stats, A.steps).items()}
    fp32_peak, mufu_peak = api.measure_peak(0), api.measure_peak(1)
    res = {"workload": cfg["name"], "value": job_value(pairs_step, A.steps, world, total_ms), "unit": UNIT,
           "ms_per_step": round(total_ms / A.steps, 4), "steps": A.steps, "warmup": A.warmup,
           "pairs_per_step": pairs_step, "kernel_ms_per_step": kms, "clocks": clk,
           "l2": "flushed between steps (256 MB write)", "dtype": "fp32"}
    if name == "sphere20":
        # the sum evaluates only the blocks its mask does not classify NONE
        # (most of the field plane lies behind the sphere for most fragments):
        # its roofline counts the pairs of those blocks (an upper bound at
        # the tiles' ragged edges), from one untimed step's block classes
        api.set_option("class_stats", 1)
        api.set_option("drop_masks", 1)
        api.set_option("reset_pressures", 1)
        api.set_option("reset_stats", 1)
        projections(api, cfg)
        api.set_option("class_stats", 0)
        cls3 = [c for c in api.stats().get("mask_classes", []) if c["hop"] == 3]
        evaluated = None
        if cls3:
            c = cls3[0]
            evaluated = (c["bits"] + c["clear"] + c["all"]) * 256 * 256
        roof = sum_roofline(stats, 3, fp32_peak, mufu_peak, "k_sum<NORESP> (sphere -> field plane)")
        if roof and evaluated:
            scale = evaluated / roof["pairs_per_launch"]
            roof.update({"achieved": round(roof["achieved"] * scale, 3), "frac": round(roof["frac"] * scale, 4),
                         "pairs_evaluated_per_launch": int(evaluated), "block_classes": cls3[0],
                         "note": "work = pairs of the blocks not classified NONE (at most), not the candidate pairs"})
        res["roofline_sum"] = roof
        res["roofline_mask"] = mask_roofline(stats, 3, "k_mask<NORESP> (sphere -> field plane, shadowed)")
    else:
        roof, _ = sym_roofline(api, [h for h in stats["hops"] if h["hop"] == 2])
        res["roofline_bounce_sum"] = roof
        res["roofline_readout"] = sum_roofline(stats, 1, fp32_peak, mufu_peak, "k_sum<FP> (readout)")
    res["dominant_kernel"] = max(kms, key=kms.get) if kms else None
    if rank == 0:
        res.update(config_error(api, cfg, name))
    api.TearDownCuda()
    return res


def config_error(api, cfg, name):
    """Errors vs the FP64 oracle of the configuration legs on seeded
    destinations, each hop given the GPU's own input, and grazing counts."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    try:
        load_scene(api, cfg)
        api.project_source_points_to_objects(False)
        P0 = api.get_object_pressures(api.TARGET, 0)
        o = O.Oracle()
        o.set_initial_conditions(cfg["cp"], cfg["frequency"], cfg.get("attenuation", 0.0))
        for tris, d in cfg["targets"]:
            o.load_geometry(tris, 0, d)
        for tris, d in cfg.get("fields", []):
            o.load_geometry(tris, 2, d)
        o.load_source_points(cfg["sources"])
        if cfg.get("field_points") is not None:
            o.load_field_points(cfg["field_points"])
        o.render()
        rng = np.random.default_rng(7)
        act = o.active(0, 0)
        e, g = {}, {}
        cs = np.sort(rng.choice(o.ncells(0, 0), 1024, replace=False))
        v0, m0 = o.hop_subset(0, 0, 0, cs, want_mask=True, nsrc=1)
        e["source_hop"] = float(np.linalg.norm(P0[cs] - v0) / np.linalg.norm(v0))
        g["source_hop_grazing"] = int(((m0 & 2) != 0).sum())
        if name == "sphere20":
            api.project_target_to_field_objects()
            F = api.get_object_pressures(api.FIELD, 0)
            actf = o.active(2, 0)
            q = np.sort(rng.choice(len(actf), 256, replace=False))
            o.set_pressures(0, 0, P0)
            v, m = o.hop_subset(3, 0, 0, q, want_mask=True, nsrc=len(act))
            c = o.counters()
            e["field_surface"] = float(np.linalg.norm(F[actf[q]] - v) / np.linalg.norm(v))
            g.update({"field_surface_pairs_checked": c["pairs"], "field_surface_grazing": c["grazing"],
                      "destinations_checked": len(q)})
        else:
            outs = [P0]
            tot = [P0]
            for nb in (1, 2, 3):
                load_scene(api, cfg)
                api.project_source_points_to_objects(False)
                api.project_target_to_target_objects(nb)
                tot.append(api.get_object_pressures(api.TARGET, 0))
                outs.append(tot[-1] - tot[-2])
            api.project_target_to_field_points()
            fp = api.get_field_point_pressures(len(cfg["field_points"]))
            q = np.sort(rng.choice(len(act), 256, replace=False))
            for k in (1, 2, 3):
                v, m = o.hop_subset(2, 0, 0, q, pin=outs[k - 1], want_mask=(k == 1), nsrc=len(act))
                e["bounce%d" % k] = float(np.linalg.norm(outs[k][act[q]] - v) / np.linalg.norm(v))
                if k == 1:
                    c = o.counters()
                    g.update({"bounce_pairs_checked": c["pairs"], "bounce_grazing": c["grazing"]})
            o.set_pressures(0, 0, tot[3])
            jj = np.sort(rng.choice(len(cfg["field_points"]), 1024, replace=False))
            vf, mf = o.hop_subset(1, 0, 0, jj, want_mask=True, nsrc=len(act))
            c = o.counters()
            e["readout"] = float(np.linalg.norm(fp[jj] - vf) / np.linalg.norm(vf))
            # a grazing pair's visibility may go either way (the reference's own
            # answer depends on OptiX's rounding): the field points without one
            clean = ~((mf & 2) != 0).any(axis=1)
            if clean.any():
                e["readout_nongrazing_dst"] = float(np.linalg.norm(fp[jj][clean] - vf[clean]) / np.linalg.norm(vf[clean]))
            g.update({"readout_pairs_checked": c["pairs"], "readout_grazing": c["grazing"],
                      "readout_dst": len(jj), "readout_dst_without_grazing": int(clean.sum())})
        o.close()
        api.TearDownCuda()
        return {"rel_err_vs_fp64": e, "grazing": g}
    except Exception as ex:
        return {"rel_err_vs_fp64": {"failed": str(ex)}}


def batch_error(cfg, out, out_rel, st):
    """Relative L2 error of sampled (scene, frequency) items, 4 sources each,
    against the FP64 oracle's per-source runs: the default run against the
    oracle's restatement of the reference's FP32 distances (parity), and
    both runs (default and centroid-relative phase) against its exact
    geometry (FP64 distances from the same FP32 positions)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    try:
        nf = len(cfg["freqs"])
        nfr = st["item_fragments"]
        rng = np.random.default_rng(11)
        # the items with the fewest fragments above 1,000 (the oracle is serial per source),
        # and at the top frequency, where the phase rounding of FP32 distances is largest,
        # the smallest item and the smallest plate
        order = [int(i) for i in np.argsort(nfr) if nfr[i] >= 1000][:3]
        top = [i for i in np.argsort(nfr) if int(i) % nf == nf - 1]
        plates = [i for i in top if cfg["kinds"][int(i) // nf] == "plate"]
        for i in top[:1] + plates[:1]:
            if int(i) not in order:
                order.append(int(i))
        errs, exact_abs, exact_rel = {}, {}, {}
        for it in order:
            s, k = int(it) // nf, int(it) % nf
            f = float(cfg["freqs"][k])
            delta = float(np.float32(cfg["cp"]) / np.float32(f) / np.float32(cfg["per_wavelength"]))
            qs = np.sort(rng.choice(len(cfg["sources"]), 4, replace=False))
            ref = {False: np.zeros((len(cfg["receivers"]), len(qs)), np.complex128)}
            ref[True] = ref[False].copy()
            for exact in (False, True):
                for c, q in enumerate(qs):
                    o = O.Oracle()
                    o.set_initial_conditions(cfg["cp"], f, cfg["attenuation"])
                    o.load_geometry(cfg["scenes"][s], 0, delta)
                    o.load_source_points(cfg["sources"][q:q + 1])
                    o.load_field_points(cfg["receivers"])
                    o.render()
                    o.set_exact_geometry(exact)
                    o.project_sources(False)
                    o.project_field_points()
                    ref[exact][:, c] = o.field_points()
                    o.close()
            key = "scene%d_%s_%.0fHz_%dfrag" % (s, cfg["kinds"][s], f, nfr[it])
            rl2 = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
            errs[key] = rl2(out[s, k][:, qs], ref[False])
            exact_abs[key] = rl2(out[s, k][:, qs], ref[True])
            exact_rel[key] = rl2(out_rel[s, k][:, qs], ref[True])
        errs["vs_exact_geometry"] = {"absolute": exact_abs, "relative_phase": exact_rel,
                                     "worst_absolute": max(exact_abs.values()),
                                     "worst_relative_phase": max(exact_rel.values())}
        return errs
    except Exception as ex:
        return {"failed": str(ex)}


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
    if args.workload == "batch":
        # the many-source, many-frequency batch alone
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        if args.profile_only:
            from sonar_render_gb300 import batch, scenes
            bc = scenes.batch_config(0)
            plan = batch.Plan(bc["scenes"], bc["sources"], bc["receivers"], bc["freqs"], bc["cp"], bc["attenuation"],
                              bc["per_wavelength"])
            for _ in range(args.warmup + args.steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                plan.run(copy=False)
            st = plan.stats()
            st.pop("item_fragments")
            st.pop("item_cells")
            print("profile-only: %d runs of %s done" % (args.warmup + args.steps, bc["name"]))
            print(json.dumps(st))
            plan.close()
        else:
            print(json.dumps(batch_leg(args, flush, rank)))
        return
    cfg = workload(args.workload)
    modes = ["plain", "compressed"] if args.mode == "both" else [args.mode]
    select = args.select

    train_info = None
    if "compressed" in modes and select == 2:
        # the admissibility network learns from the exact method's blocks of
        # the same trihedral at other frequencies (untimed set-up); with
        # --mlp-cache the trained parameters are kept in a file and reused
        # (profiler runs then launch no training kernels)
        from sonar_render_gb300 import admissibility, scenes
        t0 = time.time()
        # the configuration's network: width 128, FP16 hidden layers on the tensor cores
        admissibility.set_width(args.mlp_width)
        if args.mlp_cache and os.path.exists(args.mlp_cache):
            admissibility.set_params(np.load(args.mlp_cache))
            train_info = {"loaded": os.path.basename(args.mlp_cache)}
        else:
            # labels: the exact method's ranks at the tolerance the timed path uses
            api.set_option("compress_tol", TOL[0])
            api.set_option("compress_judge", 3.0 * TOL[0])
            train_cfgs = [scenes.trihedral_config(f, bounces=1, n_theta=0, n_phi=0) for f in (40e3, 50e3)]
            X, y, loss = admissibility.train_on_scenes(train_cfgs, epochs=args.train_epochs, batch=256, lr=1e-3,
                                                       seed=0)
            train_info = {"samples": int(len(y)), "scenes": ["trihedral_1m_40kHz", "trihedral_1m_50kHz"],
                          "width": args.mlp_width, "epochs": args.train_epochs, "final_mse_log2rank": round(loss, 5),
                          "seconds": round(time.time() - t0, 2)}
            if args.mlp_cache:
                np.save(args.mlp_cache, admissibility.get_params())

    load_scene(api, cfg)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    if args.profile_only:
        # device work only, for profiler captures: no e2e, no CPU legs, no JSON line
        for m in modes:
            set_path(api, m == "compressed", select)
            for _ in range(args.warmup + args.steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                api.set_option("drop_masks", 1)
                api.set_option("reset_pressures", 1)
                projections(api, cfg)
            torch.cuda.synchronize()
            print("profile-only: %d steps of %s (%s) done" % (args.warmup + args.steps, cfg["name"], m))
            print(json.dumps(api.stats()["hops"][-3:]))
        api.TearDownCuda()
        return

    res = {}
    for m in modes:
        set_path(api, m == "compressed", select)
        load_scene(api, cfg)
        times, stats, clk = time_path(api, cfg, args, flush, local, world)
        total_ms = max_over_ranks(float(sum(times)), world)
        pairs_step = step_pairs(stats) / max(args.steps, 1)
        res[m] = {"times": times, "stats": stats, "clocks": clk, "ms_per_step": total_ms / args.steps,
                  "value": job_value(pairs_step, args.steps, world, total_ms), "pairs_step": pairs_step,
                  "kernels_ms_per_step": {k: round(v, 4) for k, v in kernel_times(stats, args.steps).items()},
                  "launches_per_step": stats["launches"] / max(args.steps, 1)}
    # the same steps with the masks and compressed blocks of the static target
    # built once and reused (kept apart from the headline, which rebuilds them)
    reuse = {}
    for m in modes:
        set_path(api, m == "compressed", select)
        load_scene(api, cfg)
        times, stats, _ = time_path(api, cfg, args, flush, local, world, reuse=True)
        total_ms = max_over_ranks(float(sum(times)), world)
        pairs_step = step_pairs(stats) / max(args.steps, 1)
        reuse[m] = {"value": job_value(pairs_step, args.steps, world, total_ms), "ms_per_step": total_ms / args.steps,
                    "kernel_ms_per_step": {k: round(v, 4) for k, v in kernel_times(stats, args.steps).items()}}
    # the low-rank apply timed alone (one stream, reused operator): its
    # roofline; in the steps above it shares the SMs with the dense remainder
    lr_alone = None
    # and the two approximation kernels of the build (interpolation, cross
    # approximation) each alone: in the headline steps they share the SMs on
    # two streams, so neither stream's span is a kernel duration
    build_alone = None
    if "compressed" in modes:
        set_path(api, True, select)
        api.set_option("overlap_streams", 0)
        load_scene(api, cfg)
        _, lr_alone, _ = time_path(api, cfg, args, flush, local, world, reuse=True)
        load_scene(api, cfg)
        _, build_alone, _ = time_path(api, cfg, args, flush, local, world)
        api.set_option("overlap_streams", OVERLAP[0])
    batch_res = batch_leg(args, flush, rank) if args.batch else None
    legs = {}
    for leg in [x for x in args.configs.split(",") if x]:
        if leg == "trihedral60_tol1e-4":
            if "compressed" in modes and select == 2:
                legs[leg] = config5_as_written(api, cfg, args, flush, local, world, rank, select)
        else:
            legs[leg] = config_leg(api, leg, args, flush, local, world, rank)
    load_scene(api, cfg)
    f2f_plain = [h for h in res.get("plain", res[modes[0]])["stats"]["hops"] if h["hop"] == 2]
    roof_sym, fp32_peak = sym_roofline(api, f2f_plain)

    # audit of the judge: full-tile errors of sampled accepted blocks after
    # one untimed compressed step
    audit = None
    if "compressed" in modes:
        try:
            set_path(api, True, select)
            api.set_option("drop_masks", 1)
            api.set_option("reset_pressures", 1)
            projections(api, cfg)
            full, judged = api.audit_compression(512, seed=11)
            lim = 3.0 * TOL[0]
            audit = {"blocks_audited": int(len(full)), "judge_limit": lim,
                     "fraction_full_tile_error_above_limit": round(float(np.mean(full > lim)), 4),
                     "full_tile_error_median": float(np.median(full)), "full_tile_error_max": float(full.max()),
                     "judged_error_median": float(np.median(judged)),
                     "median_full_over_judged": round(float(np.median(full / np.maximum(judged, 1e-12))), 3)}
        except Exception as ex:
            audit = {"failed": str(ex)}

    # block classes of the interaction masks (an untimed extra step)
    set_path(api, False, 0)
    api.set_option("class_stats", 1)
    api.set_option("drop_masks", 1)
    api.set_option("reset_pressures", 1)
    api.set_option("reset_stats", 1)
    projections(api, cfg)
    mask_classes = api.stats().get("mask_classes")
    api.set_option("class_stats", 0)

    # ---- end to end through the C ABI from host buffers
    for m in modes:
        set_path(api, m == "compressed", select)
        res[m]["e2e"] = e2e_path(api, cfg, args, world, res[m]["pairs_step"])

    # ---- errors (vs FP64 on seeded destinations, compressed vs plain) and CPU baseline, rank 0
    errs, cpu, frag = {}, None, None
    if rank == 0:
        outs = {}
        for m in modes:
            set_path(api, m == "compressed", select)
            e = check_error(api, cfg)
            errs[m] = e.get("errors")
            frag = e.get("fragments", frag)
            outs[m] = e.get("out")
            if m == "plain":
                errs["grazing"] = e.get("grazing")
        if "plain" in outs and "compressed" in outs and outs["plain"] is not None and outs["compressed"] is not None:
            a, b = outs["compressed"], outs["plain"]
            errs["compressed_vs_plain_all_fragments"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        cpu = cpu_baseline(cfg, args.cpu_seconds)
    set_path(api, False, 0)

    head = "compressed" if "compressed" in modes else modes[0]
    H = res[head]
    st = H["stats"]
    cmp_hops = [h for h in st["hops"] if h["hop"] == 2 and h.get("cmp_build_ms")]
    compression = None
    if cmp_hops:
        h = cmp_hops[0]
        compression = {"select": {0: "separation rule", 1: "every interacting block", 2: "admissibility network"}
                       [h["cmp_select"]], "candidate_blocks": h["cmp_cand"], "approximated": h["cmp_blocks"],
                       "accepted": h["cmp_accepted"], "pair_fraction_compressed": round(h["cmp_pairs"] / h["pairs"], 4),
                       "mean_rank": h["cmp_mean_rank"], "max_judged_block_err": h["cmp_max_err"],
                       "interpolated_blocks": h.get("cmp_ip_blocks", 0), "interpolation_mean_nodes": h.get("cmp_ip_nodes", 0.0),
                       "interpolation_kept": h.get("cmp_ip_kept", 0),
                       "tolerance": TOL[0], "judge_limit": 3.0 * TOL[0], "network_training": train_info,
                       "judge_audit": audit}
    kms = H["kernels_ms_per_step"]
    kshare = {k: round(v / H["ms_per_step"], 4) for k, v in kms.items()}
    roof_lr = lowrank_roofline(lr_alone) if head == "compressed" and lr_alone else None
    if roof_lr:
        roof_lr["timed"] = "alone (one stream), operator reused; the headline step overlaps it with the dense remainder"
    roof_aca = aca_roofline(build_alone or st, fp32_peak) if head == "compressed" else None
    roof_ip = ip_roofline(build_alone or st, fp32_peak) if head == "compressed" else None
    for r in (roof_aca, roof_ip):
        if r and build_alone:
            r["timed"] = ("alone: the same rebuilt steps with the build on one stream; the headline step runs the "
                          "interpolation beside the cross approximation on a second stream")
    # the roofline object describes the dominant kernel of the headline step
    # (not the two approximation kernels' joint span)
    single = {k: v for k, v in kms.items() if k != "approximation_both"}
    alone_ms = None
    if build_alone:
        ka = kernel_times(build_alone, args.steps)
        alone_ms = {k: round(ka[k], 4) for k in ("interpolation", "cross_approx") if k in ka}
        single.update(alone_ms)
    dominant = max(single, key=single.get) if single else None
    if dominant == "cross_approx" and roof_aca:
        roof_main = roof_aca
    elif dominant == "interpolation" and roof_ip:
        roof_main = roof_ip
    elif dominant == "lowrank_apply" and roof_lr:
        roof_main = roof_lr
    else:
        roof_main = roof_sym
    line = {
        "metric": METRIC, "value": H["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": H["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded trihedral mesh and source, generated in-process)",
        "config": {"workload": cfg["name"] + ("_compressed" if head == "compressed" else "_plain"),
                   "fragments": frag, "bounces": cfg.get("bounces", 0), "sources": int(len(cfg["sources"])),
                   "field_points": 0 if cfg.get("field_points") is None else len(cfg["field_points"]),
                   "pairs_per_step": H["pairs_step"], "l2": "flushed between steps (256 MB write)",
                   "path": ("network-proposed low-rank blocks + plain FP32 sums for the rest; masks, network "
                            "inference and approximation rebuilt every step") if head == "compressed" else
                           "plain FP32 sums + interaction masks (rebuilt every step)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": roof_main, "roofline_bounce_sum": roof_sym, "roofline_lowrank": roof_lr,
        "roofline_cross_approx": roof_aca, "roofline_interpolation": roof_ip, "dominant_kernel": dominant,
        "kernel_ms_per_step": kms, "kernel_share": kshare, "build_kernels_alone_ms_per_step": alone_ms,
        "compression": compression,
        "mask_block_classes": mask_classes,
        "cpu_baseline": cpu, "e2e": H["e2e"], "clocks": H["clocks"], "gpu_launches": int(H["launches_per_step"] * args.steps),
        "rel_err_vs_fp64": errs.get(head), "grazing": errs.get("grazing"),
        "batch_config": batch_res,
        "config_sphere20": legs.get("sphere20"), "config_trihedral40_3b": legs.get("trihedral40"),
        "config_trihedral60_as_written": legs.get("trihedral60_tol1e-4"),
        "operator_reuse": dict(reuse, note="masks and compressed blocks built once per target and reused by every "
                                           "step (not the headline: the headline rebuilds them every step)"),
    }
    if "plain" in reuse and "compressed" in reuse:
        line["operator_reuse"]["compressed_over_plain"] = round(reuse["compressed"]["value"] / reuse["plain"]["value"], 3)
    if head == "compressed":
        line["rel_err_compressed_vs_plain"] = errs.get("compressed_vs_plain_all_fragments")
    if "plain" in res and head != "plain":
        P = res["plain"]
        line["plain"] = {"value": P["value"], "ms_per_step": P["ms_per_step"], "e2e": P["e2e"],
                         "kernel_ms_per_step": P["kernels_ms_per_step"], "clocks": P["clocks"],
                         "rel_err_vs_fp64": errs.get("plain"), "gpu_launches": int(P["launches_per_step"] * args.steps)}
        line["compressed_over_plain"] = round(H["value"] / P["value"], 3)
        line["compressed_over_plain_e2e"] = round(H["e2e"]["value"] / P["e2e"]["value"], 3)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def check_error(api, cfg):
    """Per-bounce relative L2 error vs the FP64 oracle on seeded destinations,
    each bounce given the GPU's own input, and the readout's when the
    workload has field points.  Also returns the GPU's bounce output."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    out = {}
    try:
        nb = int(cfg.get("bounces", 0))
        load_scene(api, cfg)
        api.project_source_points_to_objects(False)
        Ps = [api.get_object_pressures(api.TARGET, 0)]
        for _ in range(nb):
            api.project_target_to_target_objects(1)
            Ps.append(api.get_object_pressures(api.TARGET, 0))
        npts = len(cfg["field_points"]) if cfg.get("field_points") is not None else 0
        if npts:
            api.project_target_to_field_points()
            fp = api.GetFieldPoints(npts)
            fp = fp[:, 0] + 1j * fp[:, 1]
        api.TearDownCuda()
        out["out"] = Ps[-1] - Ps[0]
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
        nact = len(act)
        e = {}
        graze = {}
        for k in range(nb):
            q = np.sort(rng.choice(nact, min(256, nact), replace=False))
            # bounce k+1 input: the pressure after bounce k (P_out <- P)
            v, m = o.hop_subset(2, 0, 0, q, pin=Ps[k], want_mask=(k == 0), nsrc=nact)
            c = o.counters()
            d = (Ps[k + 1] - Ps[k])[act[q]]
            e["bounce%d" % (k + 1)] = float(np.linalg.norm(d - v) / np.linalg.norm(v))
            if k == 0:
                g1 = (m & 2).any(axis=1)
                if (~g1).any():
                    e["bounce1_nongrazing_dst"] = float(np.linalg.norm((d - v)[~g1]) / np.linalg.norm(v[~g1]))
                graze = {"bounce_pairs_checked": c["pairs"], "bounce_grazing": c["grazing"]}
        if npts:
            o.set_pressures(0, 0, Ps[-1])
            jj = np.sort(rng.choice(npts, min(1024, npts), replace=False))
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
    # grow the destination sample until a probe takes a tenth of the budget,
    # then size the timed sample to the budget
    n, dt = 64, 0.0
    while n < nact:
        t0 = time.perf_counter()
        o.hop_subset(2, 0, 0, np.sort(rng.choice(nact, n, replace=False)), pin=P)
        dt = time.perf_counter() - t0
        if dt >= 0.1 * seconds:
            break
        n = min(nact, n * 4)
    n = int(min(nact, max(8, n * seconds / max(dt, 1e-3))))
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
            "config": {"workload": cfg["name"] + "_compressed", "sample": "bounce destinations on host cores"},
            "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference's own hot path is OptiX GPU code; its CPU restatement (the oracle) runs here"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="trihedral60")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--profile-only", action="store_true",
                    help="run warm-up and steps of device work only (for ncu captures)")
    ap.add_argument("--mode", default="both", choices=["both", "plain", "compressed"])
    ap.add_argument("--aca-variant", type=int, default=8, choices=tuple(range(11)),
                    help="cross-approximation kernel: k_aca (one row and column per thread): 0 = 8 factor ranks in "
                         "shared memory, 4 CTAs per SM; 1 = 12 ranks, 4 CTAs; 2 = 16 ranks, 3 CTAs; k_aca2 (two rows "
                         "and columns per thread, first bounce's apply fused): 3 = 8 ranks, 4 CTAs; 4 = 6 ranks, "
                         "5 CTAs; 5 = 4 ranks, 6 CTAs; 6 = 2 ranks, 8 CTAs; 7 = 3 ranks, 7 CTAs; without the fragment "
                         "staging: 8 = 8 ranks, 6 CTAs; 9 = 6 ranks, 7 CTAs; 10 = 4 ranks, 8 CTAs")
    ap.add_argument("--lr-ctas", type=int, default=4, choices=(4, 6, 8),
                    help="low-rank apply kernel: resident CTAs per SM (its register cap)")
    ap.add_argument("--fused-apply", type=int, default=1, choices=(0, 1),
                    help="k_aca2: apply the accepted blocks to the first bounce's inputs in the same kernel")
    ap.add_argument("--mlp-width", type=int, default=128, choices=(64, 128),
                    help="admissibility network width: 128 = FP16 hidden layers on the tensor cores (the "
                         "configuration's), 64 = FP32 on the CUDA cores")
    ap.add_argument("--interp", type=int, default=1, choices=(0, 1),
                    help="compressed bounce: far class-ALL blocks between planar tiles by directional interpolation "
                         "(the rest by cross approximation)")
    ap.add_argument("--overlap", type=int, default=1, choices=(0, 1),
                    help="compressed bounce: low-rank apply on a second stream beside the dense remainder")
    ap.add_argument("--tile-align", type=int, default=1, choices=(0, 1),
                    help="active fragments: full patches on 256-fragment tile boundaries")
    ap.add_argument("--ip-transpose", type=int, default=0, choices=(0, 1),
                    help="interpolation tiles taller than wide take the fragment grid's y axis as the first axis")
    ap.add_argument("--build-overlap", type=int, default=1, choices=(0, 1),
                    help="compressed build: interpolation on a second stream beside the cross approximation")
    ap.add_argument("--tol", type=float, default=7e-4,
                    help="cross-approximation tolerance of the compressed path (judge limit 3 x tol); the "
                         "default keeps the step's error about 3x below the 1e-3 target (5e-4: about 4x)")
    ap.add_argument("--rcut", type=float, default=32.0,
                    help="network: propose blocks whose predicted rank is below this")
    ap.add_argument("--select", type=int, default=2,
                    help="compressed blocks: 0 separation rule, 1 every interacting block, 2 the trained network")
    ap.add_argument("--train-epochs", type=int, default=40)
    ap.add_argument("--mlp-cache", default="",
                    help="file (.npy) for the trained network's parameters: loaded when present, else written")
    ap.add_argument("--batch", type=int, default=1,
                    help="also run the many-source, many-frequency batch configuration (0: skip)")
    ap.add_argument("--configs", default="sphere20,trihedral40,trihedral60_tol1e-4",
                    help="other configurations timed beside the headline (comma list of sphere20, trihedral40, "
                         "trihedral60_tol1e-4 = the headline workload at the stated tolerance 1e-4; empty: none)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    RCUT[0] = args.rcut
    ACA_VARIANT[0] = args.aca_variant
    OVERLAP[0] = args.overlap
    BUILD_OVERLAP[0] = args.build_overlap
    TILE_ALIGN[0] = args.tile_align
    IP_TRANSPOSE[0] = args.ip_transpose
    FUSED[0] = args.fused_apply
    INTERP[0] = args.interp
    LR_CTAS[0] = args.lr_ctas
    TOL[0] = args.tol
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
