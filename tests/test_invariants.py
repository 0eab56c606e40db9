"""The reference's list invariants on the oracle's output
(tests/test_gpu_kernels.cpp:254-288): coverage, no self-acceptance, packing
of siblings only, no list dwarfing the mean."""

import numpy as np
import pytest

from checks import check_lists, check_packing, ref_children
from native import coincident_system, lopsided_sphere


@pytest.mark.parametrize("pack", [False, True])
@pytest.mark.parametrize("gs", [1, 7, 32, 64])
def test_list_invariants(oracle, pack, gs):
    pos, mass = lopsided_sphere(3000, 11)
    nodes, _, L = oracle.lists(pos, mass, theta=0.7, group_size=gs, pack=pack)
    n = len(mass)
    assert check_lists(nodes["begin"], nodes["end"], L.groups, L.cell_list, L.body_list, n,
                       gs) == 0
    assert check_packing(nodes["begin"], nodes["end"], ref_children(nodes), L.groups) == 0
    mean = (L.stats.cell_interactions + L.stats.body_interactions) / n
    assert L.stats.max_list < 3 * mean + 64
    assert L.stats.max_group <= gs


def test_oversized_leaf_is_cut(oracle):
    pos, mass = coincident_system()
    for pack in (False, True):
        nodes, _, L = oracle.lists(pos, mass, theta=0.75, group_size=32, pack=pack)
        assert check_lists(nodes["begin"], nodes["end"], L.groups, L.cell_list, L.body_list,
                           len(mass), 32) == 0
        assert L.stats.max_group <= 32
