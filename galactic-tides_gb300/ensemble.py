#!/usr/bin/env python
"""A batched ensemble of independent galaxies, on one GPU or sharded over
several (one process per GPU).

  python galactic-tides_gb300/ensemble.py [--galaxies 64] [--steps 10]
  torchrun --nproc-per-node N galactic-tides_gb300/ensemble.py ...

Galaxies: N log-uniform in [10k, 500k], disk mass 0.5-2, bulge-to-disk
mass 0-0.5, halo mass 3-10 (the benchmark model's other fields), one seed
each; every rank draws the same list. Galaxies are independent, so the
ensemble shards by galaxy: `partition_by_cost` gives each rank a set of
galaxies of about equal N log N cost (largest first, each to the least
loaded rank), each rank advances its own set on its own GPU, and the
per-galaxy results (interactions, p99 error, time) are gathered to rank 0 on
the host. There is no exchange in the data path.

On each GPU: each galaxy's group_size and packing threshold come from the
autotuner (gtc_autotune_group); the rank's galaxies then advance together as
one forest (gtc_ensemble_leapfrog: every stage one launch for all galaxies,
every step one CUDA graph launch; --forest 0: one kernel chain per galaxy
in the graph instead, each with its tuned walk). Reported: the aggregate
interactions/s of the whole job (all ranks' interactions over the slowest
rank's time, steady state), what one leapfrog call adds once, the same
galaxies solved one after another with the default parameters, and each
galaxy's p99 force error against FP64 direct sums on a sample. Rank 0
prints one JSON object.
"""

import argparse
import importlib.util
import json
import math
import os
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

SOLVER = dict(G=1.0, theta=0.75, eps=0.025, quadrupole=True, group_size=32, leaf_size=8,
              pack=True)


def _galaxy_module():
    spec = importlib.util.spec_from_file_location("gtc_ensemble_galaxy", HERE / "galaxy.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def draw_models(k, seed):
    """The ensemble's k galaxy models (the same on every rank)."""
    galaxy = _galaxy_module()
    rng = np.random.default_rng(seed)
    models = []
    for i in range(k):
        n = int(round(np.exp(rng.uniform(np.log(10_000), np.log(500_000)))))
        disk = rng.uniform(0.5, 2.0)
        bulge = max(rng.uniform(0.0, 0.5), 0.005) * disk
        halo = rng.uniform(3.0, 10.0)
        models.append(galaxy.galaxy_model(n, 1000 + i, disk_mass=disk, bulge_mass=bulge,
                                          halo_mass=halo))
    return models


def galaxy_cost(n):
    """Estimated cost of one step of a galaxy of n bodies: N log N."""
    return n * math.log2(max(n, 2))


def partition_by_cost(sizes, ranks):
    """Galaxy indices per rank, about equal total cost: largest galaxy first,
    each to the rank with the least cost so far (ties: the lowest rank).
    Each rank's list is in galaxy order."""
    if ranks < 1:
        raise ValueError("need at least one rank")
    load = [0.0] * ranks
    parts = [[] for _ in range(ranks)]
    for i in sorted(range(len(sizes)), key=lambda i: (-galaxy_cost(sizes[i]), i)):
        r = min(range(ranks), key=lambda r: (load[r], r))
        parts[r].append(i)
        load[r] += galaxy_cost(sizes[i])
    return [sorted(p) for p in parts]


def gather_shards(shard, rank, world):
    """Every rank's shard result on rank 0 (a list in rank order), None on
    the others; the host-side gather of per-galaxy statistics."""
    if world == 1:
        return [shard]
    import torch.distributed as dist
    out = [None] * world if rank == 0 else None
    dist.gather_object(shard, out, dst=0)
    return out


def combine(shards, steps):
    """The job's figures from the ranks' shard results: per-galaxy rows in
    galaxy order, interactions/s of all ranks over the slowest rank's time."""
    rows = sorted((g for s in shards for g in s["galaxies"]), key=lambda g: g["galaxy"])
    t_job = max(s["ensemble_seconds"] for s in shards)
    inter = sum(g["interactions"] for g in rows)
    p99 = [g["p99"] for g in rows]
    return {
        "ranks": len(shards), "galaxies": len(rows), "particles": sum(g["n"] for g in rows),
        "steps": steps,
        "ensemble_ms_per_step": round(1e3 * t_job / steps, 4),
        "call_overhead_ms": round(1e3 * max(s.get("call_overhead_seconds", 0.0) for s in shards), 3),
        "ensemble_interactions_per_s": inter / (t_job / steps) if t_job > 0 else None,
        "per_rank": [{"rank": s["rank"], "galaxies": len(s["galaxies"]),
                      "particles": sum(g["n"] for g in s["galaxies"]),
                      "cost": sum(galaxy_cost(g["n"]) for g in s["galaxies"]),
                      "ms_per_step": round(1e3 * s["ensemble_seconds"] / steps, 4)}
                     for s in shards],
        "p99": {"max": max(p99), "median": float(np.median(p99)), "per_galaxy": p99},
        "tuned": [{k: g[k] for k in ("galaxy", "n", "group_size", "pack", "walk_warps",
                                     "tuned_ms") if k in g} for g in rows],
    }


def run_shard(models, mine, args, device):
    """Advances galaxies `mine` on GPU `device`: autotune, one eager pass as
    the unbatched baseline, then the ensemble; the p99 error of each
    galaxy's last forces. Returns the shard's result."""
    import torch
    import __graft_entry__
    gtc = __graft_entry__.load_package().gtc
    galaxy = _galaxy_module()
    dev = torch.device("cuda", device)
    gal = []
    for i in mine:
        pos, vel, mass, _ = galaxy.make_galaxy(model=models[i])
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        n = len(mass)
        gal.append(dict(galaxy=i, n=n, pos=t(pos), vel=t(vel), mass=t(mass),
                        acc=torch.zeros((n, 3), dtype=torch.float64, device=dev),
                        pot=torch.zeros(n, dtype=torch.float64, device=dev)))
    shard = {"rank": args.rank, "galaxies": [], "ensemble_seconds": 0.0}
    if not gal:
        return shard

    tuner = gtc.Context(device)
    t0 = time.perf_counter()
    for g in gal:
        if args.tune:
            gs, pack, ms, walk = tuner.autotune_group(g["pos"].data_ptr(), g["mass"].data_ptr(),
                                                      g["n"], **SOLVER)
        else:  # the benchmark's defaults
            gs, pack, ms, walk = SOLVER["group_size"], 1, 0.0, -1
        g.update(group_size=gs, pack=pack, tuned_ms=ms, walk_warps=walk)
    shard["autotune_seconds"] = time.perf_counter() - t0

    # one after another, default parameters, eager: the unbatched baseline
    for g in (gal if args.sequential else []):
        tuner.group_force_device(g["pos"].data_ptr(), g["mass"].data_ptr(), g["n"],
                                 g["acc"].data_ptr(), g["pot"].data_ptr(), **SOLVER)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    seq_inter = 0
    for g in (gal if args.sequential else []):
        tuner.group_force_device(g["pos"].data_ptr(), g["mass"].data_ptr(), g["n"],
                                 g["acc"].data_ptr(), g["pot"].data_ptr(), **SOLVER)
        st = tuner.stats()
        seq_inter += st["cell_interactions"] + st["body_interactions"]
    torch.cuda.synchronize(dev)
    shard["sequential_seconds"] = time.perf_counter() - t0
    shard["sequential_interactions"] = seq_inter
    tuner.close()

    # the ensemble: tuned parameters, one graph launch per step
    ens = gtc.Ensemble(len(gal), device)
    for k, g in enumerate(gal):
        kw = dict(SOLVER, group_size=g["group_size"], pack=g["pack"])
        ens.set_system(k, g["pos"].data_ptr(), g["vel"].data_ptr(), g["mass"].data_ptr(),
                       g["acc"].data_ptr(), g["pot"].data_ptr(), g["n"], **kw)
        ens.context(k).set_option("walk_warps", g["walk_warps"])
    ens.set_option("forest", args.forest)
    torch.cuda.synchronize(dev)
    ens.leapfrog(args.dt, 2, prime=True, graph=True)  # capture and warm up
    # A call pays once for its set-up (gathering the systems, a sizing
    # solve, the graph capture); a call of 1 step and one of 1 + steps steps
    # give the steady per-step time (their difference) and that overhead.
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    ens.leapfrog(args.dt, 1, prime=False, graph=True)
    torch.cuda.synchronize(dev)
    t_one = time.perf_counter() - t0
    t0 = time.perf_counter()
    ens.leapfrog(args.dt, 1 + args.steps, prime=False, graph=True)
    torch.cuda.synchronize(dev)
    t_many = time.perf_counter() - t0
    shard["ensemble_seconds"] = t_many - t_one
    shard["call_overhead_seconds"] = t_one - shard["ensemble_seconds"] / args.steps
    for k, g in enumerate(gal):
        st = ens.context(k).stats()
        g["interactions"] = st["cell_interactions"] + st["body_interactions"]
        g["graph_steps"] = st["graph_steps"]

    # accuracy of each galaxy's last forces against FP64 direct sums
    chk = gtc.Context(device)
    for g in gal:
        n = g["n"]
        idx = gtc.sample_indices(n, args.sample, 1).astype(np.int64)
        didx = torch.from_numpy(idx).to(dev)
        racc = torch.empty((len(idx), 3), dtype=torch.float64, device=dev)
        rpot = torch.empty(len(idx), dtype=torch.float64, device=dev)
        chk.direct_fp64_device(g["pos"].data_ptr(), g["mass"].data_ptr(), n, didx.data_ptr(),
                               len(idx), racc.data_ptr(), rpot.data_ptr(), G=1.0, eps=0.025)
        ref = racc.cpu().numpy()
        got = g["acc"].cpu().numpy()[idx]
        e = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        g["p99"] = float(np.percentile(e, 99))
    chk.close()
    ens.close()
    shard["galaxies"] = [{k: g[k] for k in ("galaxy", "n", "group_size", "pack", "walk_warps",
                                             "tuned_ms", "interactions", "graph_steps", "p99")}
                         for g in gal]
    return shard


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--galaxies", type=int, default=64)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--dt", type=float, default=0.01)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--sample", type=int, default=1024)
    ap.add_argument("--forest", type=int, default=-1, choices=(-1, 0, 1),
                    help="the ensemble as one forest: -1 when eligible, 0 never, 1 always")
    ap.add_argument("--tune", type=int, default=1, choices=(0, 1),
                    help="0: the benchmark's group size and packing for every galaxy")
    ap.add_argument("--sequential", type=int, default=1, choices=(0, 1),
                    help="0: no one-after-another baseline")
    args = ap.parse_args()
    args.rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    device = int(os.environ.get("LOCAL_RANK", 0))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")  # host-side gather of statistics only
    models = draw_models(args.galaxies, args.seed)
    parts = partition_by_cost([m.n for m in models], world)
    shard = run_shard(models, parts[args.rank], args, device)
    shards = gather_shards(shard, args.rank, world)
    if args.rank == 0:
        out = combine(shards, args.steps)
        seq_t = sum(s.get("sequential_seconds", 0.0) for s in shards)
        out["sequential_interactions_per_s"] = (
            sum(s.get("sequential_interactions", 0) for s in shards) / seq_t
            if seq_t and args.sequential else None)
        out["autotune_seconds"] = round(max(s.get("autotune_seconds", 0.0) for s in shards), 2)
        out["note"] = ("ensemble steps include kicks and drifts, timed in steady state (a call of "
                       "1 + steps steps less a call of 1 step); call_overhead_ms is what a "
                       "leapfrog call adds once (set-up, sizing solve, graph capture); the "
                       "sequential baseline is one force evaluation per galaxy with default "
                       "group_size 32, packing on")
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
