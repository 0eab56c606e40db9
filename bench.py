#!/usr/bin/env python
"""Benchmark of the grouped gravity solver on one GB300.

Workload (the reference's headline metric at N = 2,000,000): one full force
evaluation -- octree build with FP64 moments, grouped walk, FP32 list
evaluation, scatter -- of a Hernquist galaxy (disk 40 %, bulge 13 %, halo
47 %, seed 1), theta = 0.75, group_size = 32, leaf_size = 8, softening 0.025,
quadrupoles on, sibling packing on. A "step" is one force evaluation.

  value   ms per force evaluation, inputs resident in HBM, CUDA events on the
          solver's stream around each call, L2 flushed (256 MiB write) before
          every timed call, mean over the timed steps;
  e2e     the same through the public host-array call (gtc_group_force):
          pinned host positions/masses in, accelerations/potentials out;
  roofline  the list-evaluation kernel: algorithmic FP32 flops (20 per body
          interaction, 64 per quadrupole cell interaction) / its event time,
          against this GPU's FP32 FMA peak measured in the same run;
  accuracy  p99 and median of |a - a_FP64| / |a_FP64| on the reference
          bench's 4096-particle sample, FP64 direct sums on the device;
  cpu_baseline  the oracle's restatement of the reference's OpenMP group and
          tree solvers on this machine's host cores, one evaluation each;
  learned   the same workload with the learned opening criterion (the
          committed model, alpha calibrated on another galaxy by the training
          script), timed the same way after warm-up solves that supply the
          previous accelerations it needs: ms, breakdown, interactions, p99 on
          the same sample, and its ratio to the plain theta = 0.75 value.

--impl reference times the reference's own CPU solver on the host cores
(its build when present, else the oracle restatement) on the same workload.
"""

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SOLVER = dict(G=1.0, theta=0.75, eps=0.025, quadrupole=True, group_size=32, leaf_size=8)
METRIC = "ms/force-eval at N=2M, p99 err vs FP64 direct; learned vs plain \u03b8=0.75 on GB300"
MODEL = ROOT / "galactic-tides_gb300" / "criterion_model.f32"
MODEL_INFO = ROOT / "galactic-tides_gb300" / "criterion_model.json"
WORKLOAD = "hernquist-galaxy N=2M, group solver theta=0.75 gs=32 leaf=8 eps=0.025 quadrupole"
FLOPS_BODY, FLOPS_CELL_QUAD, FLOPS_CELL_MONO = 20, 64, 21


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=2_000_000)
    ap.add_argument("--sample", type=int, default=4096)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-criterion measurement")
    ap.add_argument("--no-200k", action="store_true",
                    help="skip the N = 200k group and direct lines")
    ap.add_argument("--only-direct", action="store_true",
                    help="the tiled FP32 direct kernel on --n bodies only (for profiler runs)")
    ap.add_argument("--walk-warps", type=int, default=-1, choices=[-1, 0, 1],
                    help="the plain walk: -1 the solver's choice, 0 threads, 1 warps")
    ap.add_argument("--direct-targets", type=int, default=0, choices=[0, 2, 4],
                    help="the direct kernel's targets per thread (0: the default)")
    ap.add_argument("--only-steps", action="store_true",
                    help="warm-up and timed steps only (for profiler launch lists)")
    ap.add_argument("--learned-steps", action="store_true",
                    help="with --only-steps: the learned criterion's warm-up and timed steps")
    return ap.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def read_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text()), "measured"
        except Exception:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed loop runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        time.sleep(0.15)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def galaxy(n, seed=1):
    """The benchmark galaxy, from the pure-numpy generator loaded by its path
    (the package itself, and with it libgtc.so, stays unloaded: the reference
    arm uses this too)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "gtc_bench_galaxy", ROOT / "galactic-tides_gb300" / "galaxy.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    pos, vel, mass, _ = mod.make_galaxy(n, seed=seed)
    return pos, vel, mass


def warmup_steps(args):
    return max(3, args.warmup)


def bench_config(n):
    """The workload, identical in both arms."""
    return {"workload": WORKLOAD, "n": n,
            "l2": ("inputs and working set larger than L2 (2M bodies: 64 MB in, about 3.5 GB "
                   "on the device); the GPU arm also writes 256 MiB before every timed step")}


def cpu_group_ms(pos, mass, use_ref):
    """One evaluation (after one warm-up) of the reference's CPU group solver."""
    sys.path.insert(0, str(ROOT / "tests"))
    import native
    if use_ref:
        impl = native.Ref()
        impl.group_force(pos, mass, pack=False, **SOLVER)
        t0 = time.perf_counter()
        _, _, tm = impl.group_force(pos, mass, pack=False, **SOLVER)
        return (time.perf_counter() - t0) * 1e3, tm
    impl = native.Oracle()
    impl.group_force(pos, mass, pack=False, **SOLVER)
    t0 = time.perf_counter()
    _, _, tm = impl.group_force(pos, mass, pack=False, **SOLVER)
    return (time.perf_counter() - t0) * 1e3, tm


def cpu_tree_ms(pos, mass):
    sys.path.insert(0, str(ROOT / "tests"))
    import native
    kw = {k: v for k, v in SOLVER.items() if k != "group_size"}
    t0 = time.perf_counter()
    _, _, st = native.Oracle().tree_force(pos, mass, **kw)
    return (time.perf_counter() - t0) * 1e3, st


def run_reference(args):
    """The reference's CPU group solver on the host cores: its own sources
    built by oracle/Makefile.ref where they are present, else the oracle's
    restatement of it (pinned to that build bit for bit)."""
    rank, _, world = dist_info()
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "tests"))
    import native
    use_ref = native.have_ref()
    impl = native.Ref() if use_ref else native.Oracle()
    pos, _, mass = galaxy(args.n)
    warm = warmup_steps(args)
    for _ in range(warm):
        impl.group_force(pos, mass, pack=False, **SOLVER)
    times, budget, t_start = [], 150.0, time.perf_counter()
    for k in range(args.steps):
        t0 = time.perf_counter()
        _, _, tm = impl.group_force(pos, mass, pack=False, **SOLVER)
        times.append((time.perf_counter() - t0) * 1e3)
        if time.perf_counter() - t_start > budget:
            break
    ms = statistics.mean(times)
    cores = os.cpu_count()
    kind = "reference" if use_ref else "port"
    sample = (f"{len(times)} full force evaluations at N={args.n} after {warm} warm-up, group "
              f"solver unpacked (the reference's CPU default), OpenMP over {cores} threads")
    line = {"impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": "ms",
            "n_gpus": world, "steps": len(times), "warmup": warm,
            "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 tree+walk, f32 evaluation",
            "data": "synthetic (Hernquist galaxy, seed 1)",
            "config": bench_config(args.n), "parallelism": "openmp host",
            "breakdown_ms": {"tree": tm["tree"] * 1e3, "lists": tm["lists"] * 1e3,
                             "evaluate": tm["evaluate"] * 1e3},
            "cpu_baseline": {"value": round(ms, 3), "unit": "ms", "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(ms, 3), "unit": "ms", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# Algorithmic bytes of the build's stages: what each must read and write once
# (B per body, B per node); the sort's come from its pass count.
KEYS_B_BODY = 24 + 24 + 13          # box: pos; keys: pos in, key + index + tiny flag out
SORT_B_BODY_PASS = 24               # key and index in and out per 8-bit pass
TOPO_B_BODY, TOPO_B_NODE = 118, 88  # levels, node count + scan, nodes, leaf and tree order
# FP64 moments in two passes: bodies in for each; per node the centres of mass
# pass reads geometry, children and ranges and writes the centre of mass,
# delta and both walk records; the quadrupole pass reads centres of mass,
# children and ranges and writes the quadrupole and the FP32 cell
MOM_B_BODY, MOM_COM_B_NODE, MOM_QUAD_B_NODE = 32, 230, 169
PACK_B_BODY = 48                    # FP32 bodies from the tree-order copies


def timed_events(step, flush, stream, reps):
    """Mean CUDA-event time of step() over reps calls on `stream`, L2
    flushed before each."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps)]
    with torch.cuda.stream(stream):
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / reps


def measure_stages(ctx, step, flush, stream, n, hbm_gbs, reps=5):
    """Per-stage device times of the plain solver (CUDA events at the stage
    boundaries, context option stage_events) and their HBM rates: algorithmic
    bytes / time, against the measured copy bandwidth."""
    import torch
    ctx.set_option("stage_events", 1)
    acc = []
    with torch.cuda.stream(stream):
        for _ in range(reps):
            flush.zero_()
            step()
            acc.append((ctx.stage_times(), ctx.stats()))
    ctx.set_option("stage_events", 0)
    tm = {k: statistics.mean(a[k] for a, _ in acc) for k in acc[0][0] if k != "sort_passes"}
    passes = acc[-1][0]["sort_passes"]
    st = acc[-1][1]
    m, g = st["n_nodes"], st["n_groups"]
    entries = st["n_cell_list"] + st["n_body_list"]
    b_keys = KEYS_B_BODY * n
    b_sort = SORT_B_BODY_PASS * passes * n
    b_topo = TOPO_B_BODY * n + TOPO_B_NODE * m
    b_mom = MOM_B_BODY * n + MOM_COM_B_NODE * m
    b_quad = MOM_B_BODY * n + MOM_QUAD_B_NODE * m
    b_build = b_keys + b_sort + b_topo + b_mom + PACK_B_BODY * n
    # the walk: node records read once, group boxes and ranges read, lists and
    # group records written; `requested` counts every record test's 48 B
    b_walk = 48 * m + 40 * g + 4 * entries + 64 * g

    def rate(b, ms):
        if ms is None or ms <= 0:
            return None
        gbs = b / (ms * 1e-3) / 1e9
        return {"bytes": int(b), "ms": round(ms, 4), "gbs": round(gbs, 1),
                "frac": round(gbs / hbm_gbs, 4)}

    return {"note": ("algorithmic bytes (each stage's inputs read and outputs written once) / "
                     "CUDA-event stage time, against the measured copy bandwidth; mean of "
                     f"{reps} solves after the timed steps, L2 flushed before each"),
            "hbm_peak_gbs": hbm_gbs, "sort_passes": passes,
            "keys": rate(b_keys, tm["keys_ms"]), "radix_sort": rate(b_sort, tm["sort_ms"]),
            "topology": rate(b_topo, tm["topology_ms"]),
            "moments_com": rate(b_mom, tm["moments_ms"]),
            "moments_quad_beside_walk": rate(b_quad, tm["quad_ms"]),
            "tree_build": rate(b_build, tm["build_ms"]), "walk": rate(b_walk, tm["walk_ms"]),
            "walk_record_bytes_requested": 48 * st["walk_nodes"],
            "walk_requested_gbs": (round(48 * st["walk_nodes"] / (tm["walk_ms"] * 1e-3) / 1e9, 1)
                                   if tm["walk_ms"] > 0 else None)}


def sm_count(device):
    import torch
    return torch.cuda.get_device_properties(device).multi_processor_count


def measure_200k(gtc, device, flush, sample, peak_fp32, sm_mhz, steps=10):
    """The same galaxy model at N = 200k (the size of the reference's only
    published GPU figures): the plain group solver (ms, breakdown, p99
    against FP64 direct on the bench sample) and the tiled FP32 direct
    kernel (ms, FP32 rate against this GPU's measured FMA peak and against
    the spec bound SMs x 128 FMA/clk x the sampled SM clock)."""
    import torch
    n = 200_000
    pos, _, mass = galaxy(n)
    dev = torch.device("cuda", device)
    dpos = torch.from_numpy(pos).to(dev)
    dmass = torch.from_numpy(mass).to(dev)
    dacc = torch.empty((n, 3), dtype=torch.float64, device=dev)
    dpot = torch.empty(n, dtype=torch.float64, device=dev)
    c = gtc.Context(device)
    stream = torch.cuda.ExternalStream(c.stream, device=dev)
    torch.cuda.synchronize()

    def group():
        c.group_force_device(dpos.data_ptr(), dmass.data_ptr(), n, dacc.data_ptr(),
                             dpot.data_ptr(), pack=True, **SOLVER)

    for _ in range(3):
        group()
    torch.cuda.synchronize()
    stats = []

    def group_stats():
        group()
        stats.append(c.stats())

    g_ms = timed_events(group_stats, flush, stream, steps)
    mean = lambda key: statistics.mean(s[key] for s in stats)
    st = stats[-1]
    idx = gtc.sample_indices(n, sample, 1)
    didx = torch.from_numpy(idx.astype(np.int64)).to(dev)
    racc = torch.empty((len(idx), 3), dtype=torch.float64, device=dev)
    rpot = torch.empty(len(idx), dtype=torch.float64, device=dev)
    c.direct_fp64_device(dpos.data_ptr(), dmass.data_ptr(), n, didx.data_ptr(), len(idx),
                         racc.data_ptr(), rpot.data_ptr(), G=SOLVER["G"], eps=SOLVER["eps"])
    torch.cuda.synchronize()
    ref = racc.cpu().numpy()
    got = dacc.cpu().numpy()[idx.astype(np.int64)]
    err = np.sort(np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1))
    group_line = {"ms": round(g_ms, 4),
                  "breakdown_ms": {"tree": round(mean("tree_ms"), 4),
                                   "lists": round(mean("lists_ms"), 4),
                                   "evaluate": round(mean("evaluate_ms"), 4)},
                  "interactions_per_particle": (st["cell_interactions"]
                                                + st["body_interactions"]) / n,
                  "p99": float(err[len(err) * 99 // 100]), "sample": len(idx),
                  "reference_published": {"group_ms": 16.0, "split_ms": [3.7, 5.6, 6.6],
                                          "hardware": "Apple M4 Max (Metal), README.md:65-70",
                                          "note": "unavailable on this box; context only"}}

    def direct():
        c.direct_force_device(dpos.data_ptr(), dmass.data_ptr(), n, dacc.data_ptr(),
                              dpot.data_ptr(), **SOLVER)

    direct()
    torch.cuda.synchronize()
    dstats = []

    def direct_stats():
        direct()
        dstats.append(c.stats())

    d_ms = timed_events(direct_stats, flush, stream, 5)
    k_ms = statistics.mean(s["eval_kernel_ms"] for s in dstats)
    flops = FLOPS_BODY * n * (n - 1)
    tflops = flops / (k_ms * 1e-3) / 1e12
    spec = (sm_count(device) * 256 * sm_mhz * 1e6 / 1e12) if sm_mhz else None
    c.close()
    direct_line = {"ms": round(d_ms, 4), "kernel_ms": round(k_ms, 4),
                   "flops_per_launch": flops, "achieved_tflops": round(tflops, 2),
                   "frac_of_measured_fp32": round(tflops / peak_fp32, 4),
                   "spec_fp32_tflops": round(spec, 2) if spec else None,
                   "frac_of_spec": round(tflops / spec, 4) if spec else None,
                   "reference_published": {"direct_ms": 122.0,
                                           "hardware": "Apple M4 Max (Metal), README.md:66",
                                           "note": "unavailable on this box; context only"}}
    return group_line, direct_line


def measure_learned(gtc, n, dpos, dmass, dacc, dpot, flush, stream, args, idx, ref, plain_ms,
                    device):
    """The learned criterion on the same bodies, timed like the plain solver."""
    import torch
    info = json.loads(MODEL_INFO.read_text())
    alpha = float(info["alpha"])
    lctx = gtc.Context(device)
    lctx.learned_set_model(np.fromfile(MODEL, dtype="<f4"))

    def step():
        lctx.group_force_device(dpos.data_ptr(), dmass.data_ptr(), n, dacc.data_ptr(),
                                dpot.data_ptr(), pack=True, criterion=gtc.CRITERION_LEARNED,
                                alpha=alpha, **SOLVER)

    for _ in range(max(3, args.warmup) + 1):  # the first is the theta fallback
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    stats = []
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
            stats.append(lctx.stats())
    torch.cuda.synchronize()
    lms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    got = dacc.cpu().numpy()[idx.astype(np.int64)]
    err = np.sort(np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1))
    st = stats[-1]
    mean = lambda key: statistics.mean(s[key] for s in stats)
    model = np.fromfile(MODEL, dtype="<f4")
    lctx.close()
    return {"ms": round(lms, 4), "ratio_vs_plain": round(lms / plain_ms, 4),
            "criterion_used": "learned" if st["criterion_used"] == gtc.CRITERION_LEARNED else "theta",
            "breakdown_ms": {"tree": round(mean("tree_ms"), 4), "lists": round(mean("lists_ms"), 4),
                             "evaluate": round(mean("evaluate_ms"), 4),
                             "evaluate_kernel": round(mean("eval_kernel_ms"), 4)},
            "interactions": {"cell": st["cell_interactions"], "body": st["body_interactions"],
                             "per_particle": (st["cell_interactions"] + st["body_interactions"]) / n},
            "accuracy": {"p99": float(err[len(err) * 99 // 100]),
                         "median": float(err[len(err) // 2]), "sample": len(idx),
                         "judge": "fp64 direct"},
            "network_rows": st["mlp_rows"], "network_batches": st["mlp_batches"],
            "alpha": alpha, "band": float(model[-1]),
            "model": "galactic-tides_gb300/criterion_model.f32 (6-64-64-1, BF16 inference)",
            "alpha_source": ("band and alpha calibrated on a 2M galaxy of seed 7: per band the "
                             "largest alpha with p99 <= plain theta=0.75, then the fastest pair"),
            "gpu_launches": sum(s["kernel_launches"] for s in stats)}


def run_direct_only(args):
    """The direct kernel alone on the galaxy of --n bodies: warm-up and timed
    launches through gtc_direct_force_device, one JSON line."""
    import torch
    import __graft_entry__
    gtc = __graft_entry__.load_package().gtc
    n = args.n
    pos, _, mass = galaxy(n)
    dev = torch.device("cuda", 0)
    dpos, dmass = torch.from_numpy(pos).to(dev), torch.from_numpy(mass).to(dev)
    dacc = torch.empty((n, 3), dtype=torch.float64, device=dev)
    dpot = torch.empty(n, dtype=torch.float64, device=dev)
    with gtc.Context(0) as c:
        if args.direct_targets:
            c.set_option("direct_targets", args.direct_targets)
        for _ in range(warmup_steps(args)):
            c.direct_force_device(dpos.data_ptr(), dmass.data_ptr(), n, dacc.data_ptr(),
                                  dpot.data_ptr(), **SOLVER)
        ms = []
        for _ in range(args.steps):
            c.direct_force_device(dpos.data_ptr(), dmass.data_ptr(), n, dacc.data_ptr(),
                                  dpot.data_ptr(), **SOLVER)
            ms.append(c.stats()["eval_kernel_ms"])
    k = statistics.mean(ms)
    print(json.dumps({"direct_n": n, "kernel_ms": round(k, 4), "steps": args.steps,
                      "tflops": round(FLOPS_BODY * n * (n - 1) / (k * 1e-3) / 1e12, 2)}),
          flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.only_direct:
        return run_direct_only(args)
    import torch
    rank, local_rank, world = dist_info()
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__
    gtc = __graft_entry__.load_package().gtc
    ctx = gtc.Context(local_rank)
    ctx.set_option("walk_warps", args.walk_warps)
    n = args.n
    pos, _, mass = galaxy(n)

    dev = torch.device("cuda", local_rank)
    dpos = torch.from_numpy(pos).to(dev)
    dmass = torch.from_numpy(mass).to(dev)
    dacc = torch.empty((n, 3), dtype=torch.float64, device=dev)
    dpot = torch.empty(n, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)

    def step():
        ctx.group_force_device(dpos.data_ptr(), dmass.data_ptr(), n, dacc.data_ptr(),
                               dpot.data_ptr(), pack=True, **SOLVER)

    if args.only_steps and args.learned_steps:
        info = json.loads(MODEL_INFO.read_text())
        ctx.learned_set_model(np.fromfile(MODEL, dtype="<f4"))

        def step():  # noqa: F811  (the learned solver on the same bodies)
            ctx.group_force_device(dpos.data_ptr(), dmass.data_ptr(), n, dacc.data_ptr(),
                                   dpot.data_ptr(), pack=True, criterion=gtc.CRITERION_LEARNED,
                                   alpha=float(info["alpha"]), **SOLVER)

    for _ in range(warmup_steps(args)):
        step()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank)
    sampler.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    stats = []
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
            stats.append(ctx.stats())
    torch.cuda.synchronize()
    clocks = sampler.stop()
    times = [a.elapsed_time(b) for a, b in ev]
    total = sum(times)
    if world > 1:
        t = torch.tensor([total], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())
    ms = total / args.steps
    value = ms / world  # replicas: force evaluations of the whole job per ms

    if args.only_steps:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 4), "unit": "ms",
                              "n": n, "steps": args.steps, "only_steps": True,
                              "eval_kernel_ms": round(statistics.mean(
                                  s["eval_kernel_ms"] for s in stats), 4),
                              "lists_ms": round(statistics.mean(
                                  s["lists_ms"] for s in stats), 4)}), flush=True)
        ctx.close()
        return
    st = stats[-1]
    mean = lambda key: statistics.mean(s[key] for s in stats)
    cell_int, body_int = st["cell_interactions"], st["body_interactions"]
    fl_cell = FLOPS_CELL_QUAD if SOLVER["quadrupole"] else FLOPS_CELL_MONO
    flops = FLOPS_BODY * body_int + fl_cell * cell_int
    kernel_ms = mean("eval_kernel_ms")
    launches = sum(s["kernel_launches"] for s in stats)

    # accuracy against FP64 direct sums on the reference bench's sample
    idx = gtc.sample_indices(n, args.sample, 1)
    didx = torch.from_numpy(idx.astype(np.int64)).to(dev)
    racc = torch.empty((len(idx), 3), dtype=torch.float64, device=dev)
    rpot = torch.empty(len(idx), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    ctx.direct_fp64_device(dpos.data_ptr(), dmass.data_ptr(), n, didx.data_ptr(), len(idx),
                           racc.data_ptr(), rpot.data_ptr(), G=SOLVER["G"], eps=SOLVER["eps"])
    ref = racc.cpu().numpy()
    got = dacc.cpu().numpy()[idx.astype(np.int64)]
    err = np.sort(np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1))
    p99, med = float(err[len(err) * 99 // 100]), float(err[len(err) // 2])

    # end to end through the host-array call, pinned buffers
    hpos = torch.from_numpy(pos).pin_memory().numpy()
    hmass = torch.from_numpy(mass).pin_memory().numpy()
    hacc = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
    hpot = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    import ctypes
    gp = gtc.gravity_params(pack=True, **SOLVER)

    def e2e_step():
        rc = gtc.lib.gtc_group_force(ctx.h, hpos.ctypes.data, hmass.ctypes.data, n,
                                     ctypes.byref(gp), hacc.ctypes.data, hpot.ctypes.data)
        ctx._check(rc)

    e2e_step()
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps

    learned = None
    if not args.no_learned and MODEL.exists():
        learned = measure_learned(gtc, n, dpos, dmass, dacc, dpot, flush, stream, args, idx, ref,
                                  ms, local_rank)
    peak_fp32 = ctx.fp32_peak_tflops()
    peaks, peak_src = read_peaks()
    stages = measure_stages(ctx, step, flush, stream, n, peaks.get("hbm_gbs", 6800.0))
    n200k = direct200k = None
    if not args.no_200k:
        n200k, direct200k = measure_200k(gtc, local_rank, flush, args.sample, peak_fp32,
                                         clocks.get("sm_mhz"))
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    traffic = None
    tf = ROOT / "profiles" / "evaluate_traffic.json"
    if tf.exists():
        try:
            t = json.loads(tf.read_text())
            traffic = float(t["dram_bytes_per_launch"]) * n / float(t["n"])
        except Exception:
            traffic = None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, str(ROOT / "tests"))
        import native
        use_ref = native.have_ref()
        g_ms, g_tm = cpu_group_ms(pos, mass, use_ref)
        t_ms, t_st = cpu_tree_ms(pos, mass)
        cores = os.cpu_count()
        cpu = {"value": round(g_ms, 2), "unit": "ms", "cores": cores,
               "kind": "reference" if use_ref else "port",
               "sample": (f"1 full force evaluation at N={n} after 1 warm-up: the reference's "
                          f"OpenMP group solver (unpacked, its CPU default) over {cores} threads"),
               "group_breakdown_ms": {"tree": g_tm["tree"] * 1e3, "lists": g_tm["lists"] * 1e3,
                                      "evaluate": g_tm["evaluate"] * 1e3},
               "tree_cpu_ms": round(t_ms, 2),
               "tree_cpu_interactions_per_particle": (t_st[0] + t_st[1]) / n}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": "ms", "n_gpus": world,
            "steps": args.steps, "warmup": warmup_steps(args), "ms_per_step": round(ms, 4),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 tree+walk, f32 evaluation", "data": "synthetic (Hernquist galaxy, seed 1)",
            "config": bench_config(n), "parallelism": "replicas" if world > 1 else "1 gpu",
            "breakdown_ms": {"tree": round(mean("tree_ms"), 4), "lists": round(mean("lists_ms"), 4),
                             "evaluate": round(mean("evaluate_ms"), 4),
                             "evaluate_kernel": round(kernel_ms, 4)},
            "interactions": {"cell": cell_int, "body": body_int,
                             "per_particle": (cell_int + body_int) / n,
                             "per_s": (cell_int + body_int) / (ms * 1e-3)},
            "accuracy": {"p99": p99, "median": med, "sample": len(idx), "judge": "fp64 direct"},
            "tree": {"nodes": st["n_nodes"], "groups": st["n_groups"], "depth": st["depth"],
                     "max_list": st["max_list"], "mean_fill": n / max(1, st["n_groups"]),
                     "walk_tests_fp64": st["walk_tests_fp64"]},
            "e2e": {"value": round(e2e_ms, 4), "unit": "ms", "h2d_bytes_per_step": n * 32,
                    "d2h_bytes_per_step": n * 32, "steps": e2e_steps},
            "roofline": {"kernel": "k_eval (warp-per-group list evaluation)", "bound": "fp32",
                         "achieved": round(achieved, 3), "peak": round(peak_fp32, 3),
                         "unit": "TFLOP/s", "frac": round(achieved / peak_fp32, 4),
                         "traffic": traffic,
                         "peak_source": "FP32 FMA throughput measured in this run by a dense FMA "
                                        "kernel on every SM (no FP32 figure in MEASURED_PEAKS.json)",
                         "flops_per_launch": flops},
            "peaks": {"hbm_gbs": peaks.get("hbm_gbs"), "bf16_tflops": peaks.get("bf16_tflops"),
                      "source": peak_src, "fp32_measured_tflops": round(peak_fp32, 3),
                      "fp32_spec_tflops": (round(sm_count(local_rank) * 256 * clocks["sm_mhz"]
                                                 * 1e6 / 1e12, 2) if clocks.get("sm_mhz") else None),
                      "fp32_spec_note": "SMs x 128 FMA/clk x 2 flops x the median SM clock sampled "
                                        "during the timed steps"},
            "stages": stages,
            "n200k_group": n200k,
            "n200k_direct": direct200k,
            "gpu_launches": launches,
            "clocks": clocks,
            "cpu_baseline": cpu,
            "learned": learned,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    ctx.close()


if __name__ == "__main__":
    main()
