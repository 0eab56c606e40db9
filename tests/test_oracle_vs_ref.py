"""The oracle against the reference built from its own sources, on more
inputs than the fixtures hold (runs only where the reference is present)."""

import numpy as np
import pytest

from native import NO_PARALLEL, coincident_system, lopsided_sphere

SYSTEMS = {"lopsided_4000": lambda: lopsided_sphere(4000, 42),
           "lopsided_1001": lambda: lopsided_sphere(1001, 9),
           "coincident": coincident_system}


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("threshold", [NO_PARALLEL, 1])
def test_tree_layouts(oracle, ref, name, threshold):
    pos, mass = SYSTEMS[name]()
    a = oracle.tree(pos, mass, 8, threshold)
    b = ref.tree(pos, mass, 8, threshold)
    assert a[0].tobytes() == b[0].tobytes() and np.array_equal(a[1], b[1]) and a[2] == b[2]


@pytest.mark.parametrize("name", list(SYSTEMS))
@pytest.mark.parametrize("gs,pack", [(1, True), (7, False), (32, True), (64, False), (64, True)])
def test_lists(oracle, ref, name, gs, pack):
    pos, mass = SYSTEMS[name]()
    _, _, lo = oracle.lists(pos, mass, theta=0.75, group_size=gs, pack=pack)
    _, _, lr, er = ref.lists(pos, mass, theta=0.75, group_size=gs, pack=pack, eps=0.025,
                             evaluate=True)
    for f in ("groups", "cell_list", "body_list", "cells", "bodies"):
        assert np.array_equal(getattr(lo, f), getattr(lr, f)), f
    assert np.array_equal(oracle.eval_lists(lo, eps=0.025), er)


def test_galaxy_group_solver(oracle, ref):
    pos, _, mass, _ = ref.galaxy(n=30000, seed=3)
    a, p, ta = oracle.group_force(pos, mass, pack=True)
    b, q, tb = ref.group_force(pos, mass, pack=True)
    assert np.array_equal(a, b) and np.array_equal(p, q)
    assert ta["cell_interactions"] == tb["cell_interactions"]


def test_leapfrog(oracle, ref):
    pos, vel, mass, _ = ref.galaxy(n=3000, seed=2)
    a = oracle.leapfrog_group(pos, vel, mass, dt=0.01, steps=3)
    b = ref.leapfrog_group(pos, vel, mass, dt=0.01, steps=3)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
