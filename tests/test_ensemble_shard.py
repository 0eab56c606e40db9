"""The batched ensemble sharded over ranks (galactic-tides_gb300/ensemble.py):
the cost partition and the host-side gather, run as two `gloo` ranks on the
CPU with a stand-in for each rank's GPU work. Galaxies are independent, so
the only multi-rank step is gathering per-galaxy statistics to rank 0."""

import importlib.util
import math
import os
import pathlib
import socket

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def load_ensemble():
    spec = importlib.util.spec_from_file_location(
        "gtc_ensemble", ROOT / "galactic-tides_gb300" / "ensemble.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_partition_covers_every_galaxy_once_and_balances_cost():
    ens = load_ensemble()
    models = ens.draw_models(64, seed=4)
    sizes = [m.n for m in models]
    assert all(10_000 <= n <= 500_000 for n in sizes)
    for ranks in (1, 2, 3, 4, 8):
        parts = ens.partition_by_cost(sizes, ranks)
        assert len(parts) == ranks
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        assert all(p == sorted(p) for p in parts)
        cost = [sum(ens.galaxy_cost(sizes[i]) for i in p) for p in parts]
        # greedy largest-first: the spread is at most one galaxy's cost
        assert max(cost) - min(cost) <= max(ens.galaxy_cost(n) for n in sizes)
    assert ens.partition_by_cost([5, 7], 4)[2:] == [[], []]  # more ranks than galaxies
    with pytest.raises(ValueError):
        ens.partition_by_cost([5], 0)
    assert ens.draw_models(8, seed=4)[3].n == models[3].n  # the same on every rank


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ens = load_ensemble()
        models = ens.draw_models(12, seed=7)
        parts = ens.partition_by_cost([m.n for m in models], world)
        # stand-in for run_shard: per-galaxy figures that depend on the galaxy
        shard = {"rank": rank, "ensemble_seconds": 0.5 + rank,
                 "galaxies": [{"galaxy": i, "n": models[i].n, "group_size": 16, "pack": True,
                               "tuned_ms": 1.0, "interactions": 100 * models[i].n,
                               "graph_steps": 10, "p99": 1e-3 * (i + 1)} for i in parts[rank]]}
        shards = ens.gather_shards(shard, rank, world)
        if rank == 0:
            out.put(("ok", ens.combine(shards, steps=10), [len(p) for p in parts]))
        else:
            assert shards is None
        dist.barrier()
    except Exception as e:  # surfaced to the parent
        out.put(("error", repr(e), None))
        raise
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_every_galaxy_on_rank_zero():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    status, res, counts = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert status == "ok", res
    ens = load_ensemble()
    models = ens.draw_models(12, seed=7)
    assert res["ranks"] == 2 and res["galaxies"] == 12 and sum(counts) == 12
    assert res["particles"] == sum(m.n for m in models)
    assert res["p99"]["per_galaxy"] == [1e-3 * (i + 1) for i in range(12)]  # galaxy order
    assert [r["galaxies"] for r in res["per_rank"]] == counts
    # the job's time is the slowest rank's: 1.5 s over 10 steps
    assert res["ensemble_ms_per_step"] == 150.0
    total = sum(100 * m.n for m in models)
    assert math.isclose(res["ensemble_interactions_per_s"], total / 0.15)
