"""The oracle against fixtures generated by the reference itself
(tests/golden/make_golden.py): bit-identical trees, lists, list evaluations,
group-solver forces and direct sums."""

import pathlib

import numpy as np
import pytest

from native import NO_PARALLEL

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
CASES = ["lopsided_3000", "lopsided_613", "coincident_150"]
VARIANTS = [(0.7, 7, False), (0.7, 32, False), (0.7, 32, True), (1.0, 32, True)]
EPS = 0.01


@pytest.fixture(scope="module", params=CASES)
def case(request):
    return request.param, np.load(GOLDEN / f"{request.param}.npz")


@pytest.mark.parametrize("leaf", [1, 8])
def test_tree(oracle, case, leaf):
    _, z = case
    nodes, order, depth = oracle.tree(z["pos"], z["mass"], leaf, NO_PARALLEL)
    assert nodes.tobytes() == z[f"tree_leaf{leaf}_nodes"].tobytes()
    assert np.array_equal(order, z[f"tree_leaf{leaf}_order"])
    assert depth == int(z[f"tree_leaf{leaf}_depth"])


@pytest.mark.parametrize("theta,gs,pack", VARIANTS)
def test_lists_and_evaluation(oracle, case, theta, gs, pack):
    _, z = case
    key = f"lists_t{theta}_gs{gs}_p{int(pack)}"
    _, _, L = oracle.lists(z["pos"], z["mass"], theta=theta, group_size=gs, leaf_size=8, pack=pack)
    for f in ("groups", "cell_list", "body_list", "cells", "bodies"):
        assert np.array_equal(getattr(L, f), z[f"{key}_{f}"]), f
    st = z[f"{key}_stats"]
    assert [L.stats.cell_interactions, L.stats.body_interactions, L.stats.max_list,
            L.stats.max_group] == [int(x) for x in st]
    out = oracle.eval_lists(L, G=1.0, eps=EPS, quadrupole=True)
    assert np.array_equal(out, z[f"{key}_eval"])


def test_group_and_tree_solvers(oracle, case):
    _, z = case
    acc, pot, _ = oracle.group_force(z["pos"], z["mass"], theta=0.6, eps=EPS, pack=False)
    assert np.array_equal(acc, z["group_acc"]) and np.array_equal(pot, z["group_pot"])
    acc, pot, st = oracle.tree_force(z["pos"], z["mass"], theta=0.6, eps=EPS)
    assert np.array_equal(acc, z["tree_acc"]) and np.array_equal(pot, z["tree_pot"])
    assert list(st) == [int(x) for x in z["tree_stats"]]


def test_direct_sums(oracle, case):
    _, z = case
    acc, pot = oracle.direct_fp64(z["pos"], z["mass"], eps=EPS)
    assert np.array_equal(acc, z["direct64_acc"]) and np.array_equal(pot, z["direct64_pot"])
    bodies = oracle.pack_bodies(z["pos"], z["mass"], [1.0, 1.0, 1.0])
    assert np.array_equal(bodies, z["direct32_bodies"])
    assert np.array_equal(oracle.direct_fp32(bodies, eps=EPS), z["direct32_out"])


def test_parallel_layout_is_the_same_tree(oracle, case):
    """Serial and parallel builds: same nodes up to numbering, same order
    (tests/test_octree.cpp:134-176)."""
    from checks import compare_trees
    _, z = case
    ser, so, _ = oracle.tree(z["pos"], z["mass"], 8, NO_PARALLEL)
    par, po, _ = oracle.tree(z["pos"], z["mass"], 8, 1)
    assert np.array_equal(so, po)
    dev_like = np.zeros(len(par), dtype=[("begin", "<u4"), ("end", "<u4"), ("depth", "<i4"),
                                         ("half", "<f8"), ("center", "<f8", 3),
                                         ("com", "<f8", 3), ("mass", "<f8"), ("quad", "<f8", 6),
                                         ("delta", "<f8"), ("n_children", "<i4")])
    from checks import ref_depths
    for f in ("begin", "end", "half", "center", "com", "mass", "quad", "delta", "n_children"):
        dev_like[f] = par[f]
    dev_like["depth"] = ref_depths(par)
    assert compare_trees(dev_like, ser) == []
