"""Parity of the CUDA backend with the oracle (the reference's CPU algorithm).

* tree: node set, ranges, FP64 centres/moments and tree order bit-identical;
* lists: groups, cell lists and body lists identical, in order;
* forces: the FP32 list evaluation within 1e-5 relative (median) of the CPU
  evaluation of the same lists -- the reference's own GPU-vs-CPU bound
  (tests/test_metal.cpp:315-316: median < 1e-5, max < 1e-3);
* direct: FP32 kernel against the FP64 sum with the bounds of
  tests/test_gpu_kernels.cpp:232-234.
"""

import numpy as np
import pytest

from checks import compare_lists, compare_trees, rel_errors, scatter
from native import coincident_system, lopsided_sphere

pytestmark = pytest.mark.gpu

KW = dict(G=1.0, eps=0.025, quadrupole=True, leaf_size=8)


def solve_and_compare(ctx, oracle, pos, mass, theta, gs, pack, leaf_size=8, eps=0.025,
                      quadrupole=True):
    acc, pot = ctx.group_force(pos, mass, G=1.0, theta=theta, eps=eps, quadrupole=quadrupole,
                               group_size=gs, leaf_size=leaf_size, pack=pack)
    dev = ctx.export()
    nodes, order, lists = oracle.lists(pos, mass, theta=theta, group_size=gs,
                                       leaf_size=leaf_size, pack=pack)
    assert np.array_equal(dev["order"], order), "tree order"
    assert compare_trees(dev["nodes"], nodes) == []
    assert compare_lists(dev, dev["nodes"], lists, nodes) == []
    assert np.array_equal(dev["bodies"], lists.bodies)
    # the FP32 cells the evaluator reads, in the device's node numbering
    rk = {(int(b), int(d)): i for i, (b, d) in
          enumerate(zip(nodes["begin"], __import__("checks").ref_depths(nodes)))}
    perm = np.array([rk[(int(b), int(d))] for b, d in
                     zip(dev["nodes"]["begin"], dev["nodes"]["depth"])], dtype=np.int64)
    assert np.array_equal(dev["cells"], lists.cells[perm])
    want = oracle.eval_lists(lists, G=1.0, eps=eps, quadrupole=quadrupole)
    ref_acc = scatter(want[:, :3].astype(np.float64), order)
    ref_pot = scatter(want[:, 3].astype(np.float64), order)
    err = rel_errors(acc, ref_acc)
    perr = np.abs(pot / ref_pot - 1)
    st = ctx.stats()
    assert st["cell_interactions"] == lists.stats.cell_interactions
    assert st["body_interactions"] == lists.stats.body_interactions
    assert st["max_list"] == lists.stats.max_list
    assert st["max_group"] == lists.stats.max_group
    return err, perr


@pytest.mark.parametrize("pack", [False, True])
@pytest.mark.parametrize("gs", [1, 7, 32])
def test_group_lists_and_forces(ctx, oracle, pack, gs):
    pos, mass = lopsided_sphere(3000, 11)
    err, perr = solve_and_compare(ctx, oracle, pos, mass, theta=0.7, gs=gs, pack=pack, eps=0.01)
    assert np.median(err) < 1e-5 and err.max() < 1e-3
    assert np.median(perr) < 1e-5 and perr.max() < 1e-4


@pytest.mark.parametrize("theta", [0.5, 0.75, 1.0])
def test_theta_range(ctx, oracle, theta):
    pos, mass = lopsided_sphere(20011, 3)
    err, _ = solve_and_compare(ctx, oracle, pos, mass, theta=theta, gs=32, pack=True)
    assert np.median(err) < 1e-5 and err.max() < 1e-3


@pytest.mark.parametrize("leaf", [1, 4, 8, 16])
def test_leaf_sizes(ctx, oracle, leaf):
    pos, mass = lopsided_sphere(4001, 7)
    err, _ = solve_and_compare(ctx, oracle, pos, mass, theta=0.75, gs=32, pack=True,
                               leaf_size=leaf)
    assert np.median(err) < 1e-5


def test_monopole_only(ctx, oracle):
    pos, mass = lopsided_sphere(3001, 2)
    err, _ = solve_and_compare(ctx, oracle, pos, mass, theta=0.75, gs=32, pack=True,
                               quadrupole=False)
    assert np.median(err) < 1e-5


def test_coincident_bodies(ctx, oracle):
    """100 coincident bodies: a chain of single-child nodes down to the tiny-node
    rule at depth 42, then a leaf far larger than a group, cut into chunks
    (tests/test_gpu_kernels.cpp:276-288)."""
    pos, mass = coincident_system()
    for pack in (False, True):
        err, _ = solve_and_compare(ctx, oracle, pos, mass, theta=0.6, gs=32, pack=pack)
        assert np.all(np.isfinite(err))
    assert ctx.stats()["depth"] == 42


def test_deep_clump(ctx, oracle):
    """A dense clump inside a wide system: leaves below the 21 levels of the
    first key word, resolved by a second word."""
    rng = np.random.default_rng(4)
    pos = np.concatenate([rng.normal(size=(2000, 3)) * 10.0,
                          1.0 + rng.normal(size=(300, 3)) * 1e-7])
    mass = rng.random(len(pos)) + 0.5
    solve_and_compare(ctx, oracle, pos, mass, theta=0.75, gs=32, pack=True)
    assert ctx.stats()["depth"] > 21


def test_trees_deeper_and_shallower_than_the_last(gtc, oracle):
    """The sort orders only the key levels the context's last tree needed,
    plus one: a deeper tree is sorted again on all 21 levels (and with a
    second key word where needed), then shallower ones follow; each is the
    oracle's tree."""
    rng = np.random.default_rng(12)
    wide = rng.normal(size=(3000, 3)) * 10.0

    def clump(scale):
        return np.concatenate([wide, 1.0 + rng.normal(size=(300, 3)) * scale])

    cases = [wide, clump(1e-3), clump(1e-7), wide, clump(1e-3)]
    depths = []
    with gtc.Context(0) as c:
        for pos in cases:
            mass = np.full(len(pos), 1.0 / len(pos))
            solve_and_compare(c, oracle, pos, mass, theta=0.75, gs=32, pack=True)
            depths.append(c.stats()["depth"])
    assert depths[0] < depths[1] <= 21 < depths[2], depths
    assert depths[3] == depths[0] and depths[4] == depths[1], depths


def test_tiny_inputs(ctx, oracle):
    for n in (1, 2, 3, 8, 9, 33):
        pos, mass = lopsided_sphere(n, n)
        acc, pot = ctx.group_force(pos, mass, theta=0.75, group_size=32, pack=True, **KW)
        want, wpot, _ = oracle.group_force(pos, mass, theta=0.75, group_size=32, pack=True,
                                           parallel_threshold=1 << 40, **KW)
        assert np.allclose(acc, want, rtol=1e-5, atol=1e-7 * np.abs(want).max())
    acc, pot = ctx.group_force(np.zeros((0, 3)), np.zeros(0), theta=0.75, group_size=32, **KW)
    assert acc.shape == (0, 3)


def test_eval_on_reference_lists(ctx, oracle):
    """The list evaluator alone, on lists built by the oracle (metal::Context::tree)."""
    pos, mass = lopsided_sphere(5003, 5)
    for gs in (8, 32):
        _, order, lists = oracle.lists(pos, mass, theta=0.5, group_size=gs, pack=True)
        want = oracle.eval_lists(lists, G=1.0, eps=0.01, quadrupole=True)
        got = ctx.tree(lists.bodies, lists.cells, lists.cell_list, lists.body_list, lists.groups,
                       G=1.0, eps2=np.float32(0.01 * 0.01), quadrupole=True)
        err = rel_errors(got[:, :3].astype(np.float64), want[:, :3].astype(np.float64))
        assert np.median(err) < 1e-5 and err.max() < 1e-3


def test_eval_rejects_wide_groups(ctx, gtc, oracle):
    pos, mass = lopsided_sphere(3000, 1)
    _, _, lists = oracle.lists(pos, mass, theta=0.7, group_size=64, pack=True)
    with pytest.raises(gtc.GtcInvalidArgument):
        ctx.tree(lists.bodies, lists.cells, lists.cell_list, lists.body_list, lists.groups)
    with pytest.raises(gtc.GtcInvalidArgument):
        ctx.group_force(pos, mass, group_size=33)


def test_direct_against_fp64(ctx, oracle):
    """tests/test_gpu_kernels.cpp:211-234 and tests/test_metal.cpp:289-291."""
    pos, mass = lopsided_sphere(5003, 5)
    acc, pot = ctx.direct_force(pos, mass, G=1.0, eps=0.01)
    racc, rpot = oracle.direct_fp64(pos, mass, G=1.0, eps=0.01)
    err = rel_errors(acc, racc)
    assert np.median(err) < 1e-5 and err.max() < 1e-3
    assert np.abs(pot / rpot - 1).max() < 1e-5


def test_direct_kernel_against_fp32_cpu(ctx, oracle):
    pos, mass = lopsided_sphere(2049, 9)
    bodies = oracle.pack_bodies(pos, mass, [1.0, 1.0, 1.0])
    want = oracle.direct_fp32(bodies, G=1.0, eps=0.02)
    got = ctx.direct(bodies, G=1.0, eps2=np.float32(0.02 * 0.02))
    err = rel_errors(got[:, :3].astype(np.float64), want[:, :3].astype(np.float64))
    assert err.max() < 1e-4
    one = ctx.direct(np.array([[0.5, 0, 0, 1]], np.float32), G=1.0, eps2=0.0)
    assert np.all(one == 0)


def test_fp64_sample_kernel(ctx, oracle):
    import torch
    pos, mass = lopsided_sphere(4000, 12)
    idx = np.random.default_rng(1).permutation(len(mass))[:300].astype(np.uint64)
    racc, rpot = oracle.direct_fp64(pos, mass, G=1.0, eps=0.025, idx=idx)
    dp = torch.tensor(pos, device="cuda")
    dm = torch.tensor(mass, device="cuda")
    di = torch.tensor(idx.astype(np.int64), device="cuda")
    da = torch.zeros((len(idx), 3), dtype=torch.float64, device="cuda")
    dpot = torch.zeros(len(idx), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.direct_fp64_device(dp.data_ptr(), dm.data_ptr(), len(mass), di.data_ptr(), len(idx),
                           da.data_ptr(), dpot.data_ptr(), G=1.0, eps=0.025)
    err = rel_errors(da.cpu().numpy(), racc)
    assert err.max() < 1e-12
    assert np.abs(dpot.cpu().numpy() / rpot - 1).max() < 1e-12


def test_rejects_non_finite_positions(ctx, gtc):
    pos, mass = lopsided_sphere(1000, 3)
    pos[17, 1] = np.nan
    with pytest.raises(gtc.GtcInvalidArgument):
        ctx.group_force(pos, mass)
    pos[17, 1] = np.inf
    with pytest.raises(gtc.GtcInvalidArgument):
        ctx.group_force(pos, mass)
    pos, mass = lopsided_sphere(1000, 3)   # the context stays usable
    acc, _ = ctx.group_force(pos, mass)
    assert np.all(np.isfinite(acc))


def test_unsoftened_self_exclusion(ctx, oracle):
    """eps = 0: the evaluator tests every body entry against the target."""
    pos, mass = lopsided_sphere(2000, 8)
    err, _ = solve_and_compare(ctx, oracle, pos, mass, theta=0.7, gs=32, pack=True, eps=0.0)
    assert np.all(np.isfinite(err)) and np.median(err) < 1e-5


@pytest.mark.parametrize("theta,quad,eps", [(0.5, True, 0.01), (0.7, True, 0.0), (1.0, False, 0.02)])
def test_tree_solver_matches_oracle_bitwise(ctx, oracle, theta, quad, eps):
    """The per-particle walk (gtc_tree_force: compute_gravity_tree and
    Octree::accel_pot, src/gravity.cpp:7-26, src/octree.cpp:275-344) in FP64
    on the device tree: forces, potentials and interaction counts identical
    to the oracle's restatement of the reference, which the golden fixtures
    pin to the reference itself."""
    pos, mass = lopsided_sphere(3000, 11)
    acc, pot = ctx.tree_force(pos, mass, G=1.0, theta=theta, eps=eps, quadrupole=quad)
    st = ctx.stats()
    want, wpot, (nc, npart) = oracle.tree_force(pos, mass, G=1.0, theta=theta, eps=eps,
                                                quadrupole=quad)
    assert np.array_equal(acc, want) and np.array_equal(pot, wpot)
    assert (st["cell_interactions"], st["body_interactions"]) == (nc, npart)


def test_tree_solver_galaxy_and_coincident(ctx, oracle, gtc):
    pos, _, mass, _ = gtc.make_galaxy(50_000, seed=2)
    acc, pot = ctx.tree_force(pos, mass, theta=0.75, eps=0.025)
    want, wpot, _ = oracle.tree_force(pos, mass, theta=0.75, eps=0.025)
    assert np.array_equal(acc, want) and np.array_equal(pot, wpot)
    pos, mass = coincident_system()
    acc, pot = ctx.tree_force(pos, mass, theta=0.75, eps=0.01)
    want, wpot, _ = oracle.tree_force(pos, mass, theta=0.75, eps=0.01)
    assert np.array_equal(acc, want) and np.array_equal(pot, wpot)
