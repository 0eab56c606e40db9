"""The device solver on the benchmark galaxy and the reference's accuracy and
invariant tests, on the GPU."""

import numpy as np
import pytest

from checks import (check_lists, check_packing, compare_lists, compare_trees, dev_children,
                    rel_errors, scatter, sorted_per_group)
from native import lopsided_sphere

pytestmark = pytest.mark.gpu


def galaxy_parity(ctx, oracle, gtc, n, sample=4096):
    """The benchmark galaxy of n bodies (seed 1, theta 0.75, group_size 32,
    leaf 8, packing, eps 0.025, quadrupoles): tree order, every node, the
    groups, both lists and the list counters identical to the oracle's; the
    forces against the oracle's evaluation of the same lists; and the p99
    error against FP64 direct sums on the reference bench's sample
    (apps/galactic_tides_bench.cpp:74-95, 142-149) within 0.1 % of the CPU
    path's. Returns the force errors against the oracle for the caller to
    bound."""
    pos, _, mass, _ = gtc.make_galaxy(n, seed=1)
    kw = dict(theta=0.75, group_size=32, leaf_size=8, pack=True)
    acc, pot = ctx.group_force(pos, mass, G=1.0, eps=0.025, quadrupole=True, **kw)
    st = ctx.stats()
    dev = ctx.export()
    nodes, order, lists = oracle.lists(pos, mass, **kw)
    assert np.array_equal(dev["order"], order)
    assert compare_trees(dev["nodes"], nodes) == []
    assert compare_lists(dev, dev["nodes"], lists, nodes) == []
    for k in ("cell_interactions", "body_interactions", "max_list", "max_group"):
        assert st[k] == getattr(lists.stats, k), k
    want = oracle.eval_lists(lists, G=1.0, eps=0.025, quadrupole=True)
    ref_acc = scatter(want[:, :3].astype(np.float64), order)
    ref_pot = scatter(want[:, 3].astype(np.float64), order)
    err = rel_errors(acc, ref_acc)
    perr = np.abs(pot / ref_pot - 1)
    # tree-order output scattered to the caller's order exactly
    assert np.array_equal(acc[order.astype(np.int64)], dev["out"][:, :3].astype(np.float64))
    idx = gtc.sample_indices(len(mass), sample, 1).astype(np.int64)
    racc, _ = oracle.direct_fp64(pos, mass, eps=0.025, idx=idx)
    e_dev = np.sort(rel_errors(acc[idx], racc))
    e_cpu = np.sort(rel_errors(ref_acc[idx], racc))
    p = len(e_dev) * 99 // 100
    assert abs(e_dev[p] / e_cpu[p] - 1) < 1e-3
    print(f"\n[galaxy {n}] vs oracle lists evaluation: accel median {np.median(err):.3e} "
          f"p99 {np.percentile(err, 99):.3e} max {err.max():.3e}; potential median "
          f"{np.median(perr):.3e} max {perr.max():.3e}; p99 vs FP64 direct device "
          f"{e_dev[p]:.5e} cpu {e_cpu[p]:.5e}; depth {st['depth']} nodes {st['n_nodes']} "
          f"fp64 walk tests {st['walk_tests_fp64']}")
    return err, perr


def test_galaxy_200k_matches_oracle(ctx, oracle, gtc):
    """The benchmark model at 200k bodies."""
    err, perr = galaxy_parity(ctx, oracle, gtc, 200_000)
    assert np.median(err) < 1e-5 and np.percentile(err, 99) < 1e-4 and err.max() < 1e-3
    assert np.median(perr) < 1e-5 and perr.max() < 1e-4


def test_galaxy_2M_matches_oracle(ctx, oracle, gtc):
    """The benchmark configuration itself, 2M bodies: the deepest trees, the
    most FP64 fallbacks of the banded walk test, and the partial-level radix
    sort all at their largest."""
    err, perr = galaxy_parity(ctx, oracle, gtc, 2_000_000)
    assert np.median(err) < 1e-5 and np.percentile(err, 99) < 1e-4 and err.max() < 1e-3
    assert np.median(perr) < 1e-5 and perr.max() < 1e-4


def test_direct_200k_matches_oracle(ctx, oracle, gtc):
    """The tiled FP32 direct kernel at 200k bodies (the reference's `direct`
    benchmark size): on a 4096-body sample of targets, against the oracle's
    FP32 restatement of gt_direct_accel on the same packed bodies, and
    against FP64 direct sums with the error the FP32 CPU kernel itself has
    (tests/test_gpu_kernels.cpp:211-234)."""
    pos, _, mass, _ = gtc.make_galaxy(200_000, seed=1)
    centre = 0.5 * (pos.min(0) + pos.max(0))
    bodies = oracle.pack_bodies(pos, mass, centre)
    got = ctx.direct(bodies, G=1.0, eps2=np.float32(0.025 * 0.025))
    idx = gtc.sample_indices(len(mass), 4096, 1).astype(np.int64)
    want = oracle.direct_fp32(bodies, G=1.0, eps=0.025, idx=idx.astype(np.uint64))
    e32 = rel_errors(got[idx, :3].astype(np.float64), want[:, :3].astype(np.float64))
    p32 = np.abs(got[idx, 3].astype(np.float64) / want[:, 3] - 1)
    racc, rpot = oracle.direct_fp64(pos, mass, G=1.0, eps=0.025, idx=idx)
    e_dev = np.sort(rel_errors(got[idx, :3].astype(np.float64), racc))
    e_cpu = np.sort(rel_errors(want[:, :3].astype(np.float64), racc))
    p64 = np.abs(got[idx, 3].astype(np.float64) / rpot - 1)
    print(f"\n[direct 200k] vs FP32 oracle: median {np.median(e32):.3e} max {e32.max():.3e} "
          f"pot max {p32.max():.3e}; vs FP64: device median {e_dev[len(e_dev) // 2]:.3e} "
          f"max {e_dev[-1]:.3e} pot max {p64.max():.3e}, cpu FP32 median "
          f"{e_cpu[len(e_cpu) // 2]:.3e} max {e_cpu[-1]:.3e}")
    # the reference's bounds against FP64 (tests/test_gpu_kernels.cpp:232-234)
    assert e_dev[len(e_dev) // 2] < 1e-5 and e_dev[-1] < 1e-3 and p64.max() < 1e-5
    # no further from FP64 than the FP32 CPU kernel (the device sums each
    # source slice and the even and odd sources apart: shorter sums)
    assert e_dev[len(e_dev) // 2] <= 1.05 * e_cpu[len(e_cpu) // 2] + 1e-7
    # and the FP32 kernels agree to their own summation error
    assert np.median(e32) < 1e-5 and e32.max() < 1e-3 and p32.max() < 1e-3


@pytest.mark.parametrize("pack", [False, True])
@pytest.mark.parametrize("gs", [1, 7, 32])
def test_device_list_invariants(ctx, pack, gs):
    for n, seed in ((3000, 11), (6000, 21)):
        pos, mass = lopsided_sphere(n, seed)
        ctx.group_force(pos, mass, theta=0.7, eps=0.01, group_size=gs, pack=pack)
        d = ctx.export()
        nd = d["nodes"]
        assert check_lists(nd["begin"], nd["end"], d["groups"], d["cell_list"], d["body_list"],
                           n, gs) == 0
        assert check_packing(nd["begin"], nd["end"], dev_children(nd), d["groups"]) == 0
        st = ctx.stats()
        assert st["max_group"] <= gs
        if n == 3000:  # the reference's heuristic, on the shape of its own test system
            mean = (st["cell_interactions"] + st["body_interactions"]) / n
            assert st["max_list"] < 3 * mean + 64


@pytest.mark.parametrize("theta", [0.5, 0.7, 1.0])
def test_group_accuracy_vs_cpu_tree(ctx, oracle, theta):
    """The grouped walk is never looser than the per-particle walk
    (tests/test_gpu_kernels.cpp:315-333)."""
    pos, mass = lopsided_sphere(3000, 11)
    ref_acc, ref_pot = oracle.direct_fp64(pos, mass, eps=0.01)
    t_acc, _, _ = oracle.tree_force(pos, mass, theta=theta, eps=0.01)
    q_acc, q_pot = ctx.group_force(pos, mass, theta=theta, eps=0.01, pack=theta == 0.7)
    et, eq = np.sort(rel_errors(t_acc, ref_acc)), np.sort(rel_errors(q_acc, ref_acc))
    n = len(mass)
    assert eq[n // 2] <= 1.05 * et[n // 2] + 2e-6
    assert eq[n * 99 // 100] <= 1.05 * et[n * 99 // 100] + 2e-5
    assert np.abs(q_pot / ref_pot - 1).max() < 2e-3


def test_momentum_conservation(ctx):
    """Sum of m a is small against sum of m |a| (tests/test_octree.cpp:92-104)."""
    pos, mass = lopsided_sphere(4000, 42)
    acc, _ = ctx.group_force(pos, mass, theta=0.6, eps=0.01)
    f = (mass[:, None] * acc).sum(0)
    assert np.linalg.norm(f) / (mass * np.linalg.norm(acc, axis=1)).sum() < 1e-3


def test_repeat_calls_reuse_buffers(ctx, gtc):
    """Repeated solves on one context give identical results (buffers reused)."""
    pos, _, mass, _ = gtc.make_galaxy(50_000, seed=1)
    a1, p1 = ctx.group_force(pos, mass)
    small, smass = lopsided_sphere(1000, 1)
    ctx.group_force(small, smass)
    a2, p2 = ctx.group_force(pos, mass)
    assert np.array_equal(a1, a2) and np.array_equal(p1, p2)


def test_one_pass_walk_matches_two_passes(gtc):
    """A repeated solve walks once, into per-group slots sized by the first
    walk's longest lists; its lists (exported back to back) and forces are
    the two-pass walk's, bit for bit."""
    pos, _, mass, _ = gtc.make_galaxy(100_000, seed=3)
    kw = dict(G=1.0, eps=0.025, quadrupole=True, theta=0.75, group_size=32, leaf_size=8,
              pack=True)
    c = gtc.Context(0)
    try:
        a1, p1 = c.group_force(pos, mass, **kw)
        d1, s1 = c.export(), c.stats()
        a2, p2 = c.group_force(pos, mass, **kw)
        d2, s2 = c.export(), c.stats()
    finally:
        c.close()
    assert (s1["list_passes"], s2["list_passes"], s2["spilled_groups"]) == (2, 1, 0)
    assert s2["kernel_launches"] < s1["kernel_launches"]  # no count pass, no list scans
    assert np.array_equal(a1, a2) and np.array_equal(p1, p2)
    for k in ("groups", "cell_list", "body_list"):
        assert np.array_equal(d1[k], d2[k]), k
    for k in ("cell_interactions", "body_interactions", "max_list", "max_group",
              "n_cell_list", "n_body_list", "walk_tests_fp64"):
        assert s1[k] == s2[k], k


def test_one_pass_walk_overflow_falls_back(ctx, gtc, oracle):
    """Slots sized by a loose walk (theta 1.0) are outgrown by a tighter one
    (theta 0.4): that solve falls back to counting first and still gives the
    oracle's lists."""
    pos, _, mass, _ = gtc.make_galaxy(60_000, seed=5)
    c = gtc.Context(0)
    try:
        kw = dict(G=1.0, eps=0.025, quadrupole=True, group_size=32, leaf_size=8, pack=True)
        c.group_force(pos, mass, theta=1.0, **kw)
        c.group_force(pos, mass, theta=1.0, **kw)
        n_short = c.stats()["max_list"]
        acc, pot = c.group_force(pos, mass, theta=0.4, **kw)
        d = c.export()
        assert c.stats()["max_list"] > n_short
        ref_acc, ref_pot = ctx.group_force(pos, mass, theta=0.4, **kw)
    finally:
        c.close()
    nodes, order, lists = oracle.lists(pos, mass, theta=0.4, group_size=32, leaf_size=8, pack=True)
    assert compare_lists(d, d["nodes"], lists, nodes) == []
    assert np.array_equal(acc, ref_acc) and np.array_equal(pot, ref_pot)


def test_one_pass_walk_spills_outgrown_groups(gtc, oracle):
    """Slots sized on a uniform cube are outgrown by a few groups once a
    dense clump is added: those groups' lists are written again, whole,
    into the overflow pools, the others stay in their slots, and lists and
    forces are the two-pass walk's."""
    rng = np.random.default_rng(2)
    n = 20_000
    pos = rng.uniform(-1, 1, (n, 3))
    mass = np.full(n, 1.0 / n)
    pos2 = np.vstack([pos, rng.normal(0, 0.01, (4000, 3)) + 0.3])
    mass2 = np.full(len(pos2), 1.0 / len(pos2))
    kw = dict(G=1.0, eps=0.01, quadrupole=True, theta=0.75, group_size=32, leaf_size=8, pack=True)
    c, fresh = gtc.Context(0), gtc.Context(0)
    try:
        c.group_force(pos, mass, **kw)
        acc, pot = c.group_force(pos2, mass2, **kw)
        st, d = c.stats(), c.export()
        ref_acc, ref_pot = fresh.group_force(pos2, mass2, **kw)
        assert fresh.stats()["list_passes"] == 2
    finally:
        c.close()
        fresh.close()
    assert st["list_passes"] == 1 and 0 < st["spilled_groups"] < st["n_groups"] // 10
    nodes, order, lists = oracle.lists(pos2, mass2, theta=0.75, group_size=32, leaf_size=8,
                                       pack=True)
    assert compare_lists(d, d["nodes"], lists, nodes) == []
    assert np.array_equal(acc, ref_acc) and np.array_equal(pot, ref_pot)


def test_warp_walk_matches_thread_walk(gtc, oracle):
    """The walk by warps (the default) and by threads (option walk_warps 0)
    test the same nodes: the exported cell lists are identical and in the
    reference's order, each group's bodies are the same multiset (the thread
    walk's in the reference's order too), the counters are equal, and the
    forces differ by summation order only. Two solves each: count + fill,
    then one pass."""
    pos, _, mass, _ = gtc.make_galaxy(100_000, seed=4)
    kw = dict(G=1.0, eps=0.025, quadrupole=True, theta=0.75, group_size=32, leaf_size=8,
              pack=True)
    res = {}
    for warps in (1, 0):
        c = gtc.Context(0)
        try:
            c.set_option("walk_warps", warps)
            for _ in range(2):
                acc, pot = c.group_force(pos, mass, **kw)
                res[(warps, c.stats()["list_passes"])] = (acc, pot, c.export(), c.stats())
        finally:
            c.close()
    nodes, order, lists = oracle.lists(pos, mass, theta=0.75, group_size=32, leaf_size=8, pack=True)
    for passes in (2, 1):
        (aw, pw, dw, sw), (at, pt, dt, st) = res[(1, passes)], res[(0, passes)]
        for k in ("groups", "cell_list"):
            assert np.array_equal(dw[k], dt[k]), (passes, k)
        g = dw["groups"]
        assert np.array_equal(sorted_per_group(dw["body_list"], g[:, 4], g[:, 5]),
                              sorted_per_group(dt["body_list"], g[:, 4], g[:, 5]))
        # the walk by threads keeps the reference's order of every list
        assert compare_lists(dt, dt["nodes"], lists, nodes, body_order=True) == []
        assert compare_lists(dw, dw["nodes"], lists, nodes) == []
        for k in ("cell_interactions", "body_interactions", "max_list", "walk_tests_fp64"):
            assert sw[k] == st[k], (passes, k)
        # the thread walk tests the root too; the warp walk opens it untested
        assert st["walk_nodes"] - sw["walk_nodes"] == len(dw["groups"])
        err = rel_errors(aw, at)
        assert np.median(err) < 1e-6 and err.max() < 1e-4
        assert np.abs(pw / pt - 1).max() < 1e-5
