#!/usr/bin/env python
"""A batched ensemble of independent galaxies on one GPU.

  python galactic-tides_gb300/ensemble.py [--galaxies 64] [--steps 10]

Galaxies: N log-uniform in [10k, 500k], disk mass 0.5-2, bulge-to-disk
mass 0-0.5, halo mass 3-10 (the benchmark model's other fields), one seed
each. Each galaxy's group_size and sibling packing come from the autotuner
(gtc_autotune_group); all galaxies then advance together, every step one
CUDA graph launch (gtc_ensemble_leapfrog). Reported: the aggregate
interactions/s of the ensemble, the same galaxies stepped one after another
with the default parameters, and each galaxy's p99 force error against FP64
direct sums on a sample. Prints one JSON object.
"""

import argparse
import json
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

SOLVER = dict(G=1.0, theta=0.75, eps=0.025, quadrupole=True, group_size=32, leaf_size=8,
              pack=True)


def draw_models(gtc, k, seed):
    rng = np.random.default_rng(seed)
    models = []
    for i in range(k):
        n = int(round(np.exp(rng.uniform(np.log(10_000), np.log(500_000)))))
        disk = rng.uniform(0.5, 2.0)
        bulge = max(rng.uniform(0.0, 0.5), 0.005) * disk
        halo = rng.uniform(3.0, 10.0)
        m = gtc.galaxy_model(n, 1000 + i, disk_mass=disk, bulge_mass=bulge, halo_mass=halo)
        models.append(m)
    return models


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--galaxies", type=int, default=64)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--dt", type=float, default=0.01)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--sample", type=int, default=1024)
    args = ap.parse_args()
    import torch
    import __graft_entry__
    gtc = __graft_entry__.load_package().gtc
    dev = torch.device("cuda", 0)
    models = draw_models(gtc, args.galaxies, args.seed)
    gal = []
    for m in models:
        pos, vel, mass, _ = gtc.make_galaxy(model=m)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        n = len(mass)
        gal.append(dict(n=n, pos0=pos, vel0=vel, pos=t(pos), vel=t(vel), mass=t(mass),
                        acc=torch.zeros((n, 3), dtype=torch.float64, device=dev),
                        pot=torch.zeros(n, dtype=torch.float64, device=dev)))
    total_n = sum(g["n"] for g in gal)

    # the autotuner, per galaxy
    tuner = gtc.Context(0)
    t0 = time.perf_counter()
    for g in gal:
        gs, pack, ms = tuner.autotune_group(g["pos"].data_ptr(), g["mass"].data_ptr(), g["n"],
                                            **SOLVER)
        g.update(group_size=gs, pack=pack, tuned_ms=ms)
    t_tune = time.perf_counter() - t0

    # one after another, default parameters, eager: the unbatched baseline
    for g in gal:
        tuner.group_force_device(g["pos"].data_ptr(), g["mass"].data_ptr(), g["n"],
                                 g["acc"].data_ptr(), g["pot"].data_ptr(), **SOLVER)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq_inter = 0
    for g in gal:
        tuner.group_force_device(g["pos"].data_ptr(), g["mass"].data_ptr(), g["n"],
                                 g["acc"].data_ptr(), g["pot"].data_ptr(), **SOLVER)
        st = tuner.stats()
        seq_inter += st["cell_interactions"] + st["body_interactions"]
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    tuner.close()

    # the ensemble: tuned parameters, one graph launch per step
    ens = gtc.Ensemble(len(gal))
    for i, g in enumerate(gal):
        kw = dict(SOLVER, group_size=g["group_size"], pack=g["pack"])
        ens.set_system(i, g["pos"].data_ptr(), g["vel"].data_ptr(), g["mass"].data_ptr(),
                       g["acc"].data_ptr(), g["pot"].data_ptr(), g["n"], **kw)
    ens.leapfrog(args.dt, 2, prime=True, graph=True)  # capture and warm up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ens.leapfrog(args.dt, args.steps, prime=False, graph=True)
    torch.cuda.synchronize()
    t_ens = time.perf_counter() - t0
    inter = 0
    replays = []
    for i in range(len(gal)):
        st = ens.context(i).stats()
        inter += st["cell_interactions"] + st["body_interactions"]
        replays.append(st["graph_steps"])

    # accuracy of each galaxy's last forces against FP64 direct sums
    chk = gtc.Context(0)
    p99 = []
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
        p99.append(float(np.percentile(e, 99)))
    chk.close()
    ens.close()
    out = {
        "galaxies": len(gal), "particles": total_n, "steps": args.steps, "dt": args.dt,
        "ensemble_ms_per_step": round(1e3 * t_ens / args.steps, 4),
        "ensemble_interactions_per_s": inter / (t_ens / args.steps),
        "graph_replays_per_galaxy": [min(replays), max(replays)],
        "sequential_force_eval_ms": round(1e3 * t_seq, 4),
        "sequential_interactions_per_s": seq_inter / t_seq,
        "note": ("ensemble steps include kicks and drifts; the sequential baseline is one force "
                 "evaluation per galaxy with default group_size 32, packing on"),
        "autotune_seconds": round(t_tune, 2),
        "tuned": [dict(n=g["n"], group_size=g["group_size"], pack=g["pack"],
                       ms=round(g["tuned_ms"], 4)) for g in gal],
        "p99": {"max": max(p99), "median": float(np.median(p99)), "per_galaxy": p99},
    }
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
