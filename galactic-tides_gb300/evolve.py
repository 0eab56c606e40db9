#!/usr/bin/env python
"""Evolves a galaxy or a parabolic encounter with the device leapfrog.

  python galactic-tides_gb300/evolve.py galaxy     [--n 50000]   [--steps 10]
  python galactic-tides_gb300/evolve.py encounter  [--n 1000000] [--steps 2000]

galaxy: the benchmark galaxy model (seed 1); one force evaluation, then
`steps` leapfrog steps of dt = 0.01, eagerly and replayed from the CUDA
graph (the two must agree bitwise).
encounter: two copies of the model (n each, seeds 1 and 2) inclined 30 and
60 degrees on a parabolic orbit with pericentre 2 from 15 apart, centre of
mass at rest (apps/galactic_tides_ics.cpp:78-97); `steps` steps of 0.01,
each replayed from the CUDA graph. Every `--every` steps: the energy drift
and the p99 force error against FP64 direct sums on a 4096-particle sample.
Prints one JSON object.
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["galaxy", "encounter"])
    ap.add_argument("--n", type=int, default=None, help="particles (per galaxy)")
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--dt", type=float, default=0.01)
    ap.add_argument("--sample", type=int, default=4096)
    args = ap.parse_args()
    import torch
    import __graft_entry__
    gtc = __graft_entry__.load_package().gtc
    dev = torch.device("cuda", 0)
    if args.mode == "galaxy":
        n_each, steps = args.n or 50_000, args.steps if args.steps is not None else 10
        pos, vel, mass, _ = gtc.make_galaxy(n_each, seed=1)
    else:
        n_each, steps = args.n or 1_000_000, args.steps if args.steps is not None else 2000
        pos, vel, mass, _ = gtc.make_encounter(n_each, seed=1, incl1=30.0, incl2=60.0, rp=2.0,
                                               r0=15.0)
    n = len(mass)
    ctx = gtc.Context(0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dpos, dvel, dmass = t(pos), t(vel), t(mass)
    dacc = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    dpot = torch.zeros(n, dtype=torch.float64, device=dev)
    idx = gtc.sample_indices(n, args.sample, 1).astype(np.int64)
    didx = torch.from_numpy(idx).to(dev)
    racc = torch.empty((len(idx), 3), dtype=torch.float64, device=dev)
    rpot = torch.empty(len(idx), dtype=torch.float64, device=dev)

    def p99():
        ctx.direct_fp64_device(dpos.data_ptr(), dmass.data_ptr(), n, didx.data_ptr(), len(idx),
                               racc.data_ptr(), rpot.data_ptr(), G=SOLVER["G"], eps=SOLVER["eps"])
        ref = racc.cpu().numpy()
        got = dacc.cpu().numpy()[idx]
        e = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        return float(np.percentile(e, 99))

    def diag(time_now):
        return ctx.diagnostics_device(dpos.data_ptr(), dvel.data_ptr(), dmass.data_ptr(),
                                      dpot.data_ptr(), n, time_now)

    def leapfrog(k, prime=False, graph=True):
        ctx.leapfrog_device(dpos.data_ptr(), dvel.data_ptr(), dmass.data_ptr(), dacc.data_ptr(),
                            dpot.data_ptr(), n, args.dt, k, prime=prime, graph=graph, **SOLVER)

    out = {"mode": args.mode, "n": n, "dt": args.dt, "steps": steps, "solver": SOLVER}
    leapfrog(0, prime=True)
    torch.cuda.synchronize()
    d0 = diag(0.0)
    log = [{"step": 0, "time": 0.0, "energy": d0["total"], "dE/E0": 0.0,
            "virial": d0["virial_ratio"], "p99": p99()}]
    graph_steps = 0
    t_run = 0.0
    done = 0
    while done < steps:
        k = min(args.every, steps - done)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        leapfrog(k)
        torch.cuda.synchronize()
        t_run += time.perf_counter() - t0
        graph_steps += ctx.stats()["graph_steps"]
        done += k
        d = diag(done * args.dt)
        log.append({"step": done, "time": done * args.dt, "energy": d["total"],
                    "dE/E0": d["total"] / d0["total"] - 1, "virial": d["virial_ratio"],
                    "p99": p99(), "momentum": d["momentum"]})
    out.update(ms_per_step=round(1e3 * t_run / max(1, steps), 4), graph_steps=graph_steps,
               log=log, max_abs_dE=max(abs(r["dE/E0"]) for r in log),
               max_p99=max(r["p99"] for r in log))
    if args.mode == "galaxy":
        # the same steps eagerly from the same start: bitwise the same
        e_pos = t(pos)
        e_vel = t(vel)
        e_acc = torch.zeros_like(dacc)
        e_pot = torch.zeros_like(dpot)
        ctx.leapfrog_device(e_pos.data_ptr(), e_vel.data_ptr(), dmass.data_ptr(), e_acc.data_ptr(),
                            e_pot.data_ptr(), n, args.dt, steps, prime=True, graph=False, **SOLVER)
        torch.cuda.synchronize()
        out["graph_equals_eager"] = bool(torch.equal(e_pos, dpos) and torch.equal(e_vel, dvel))
    print(json.dumps(out), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
