"""The batched ensemble as one forest (csrc/forest.cu): every system's
bodies in one arena, one tree per system, each stage one launch for all
systems. Each system must move to the same doubles as on its own: the
forest against the same ensemble stepped system by system (option
"forest" 0), bitwise, over systems that exercise every branch of the
build -- galaxies of uneven N with their own group size and packing, a
clump deeper than one key word, coincident bodies (the tiny-node rule),
and systems smaller than a group or a leaf."""

import numpy as np
import pytest

from native import coincident_system, lopsided_sphere

gpu = pytest.mark.gpu

SOLVER = dict(G=1.0, theta=0.75, eps=0.025, quadrupole=True, leaf_size=8)


def systems(gtc):
    """(pos, vel, mass, group_size, pack) of each system."""
    rng = np.random.default_rng(31)
    out = []
    for n, seed, gs, pack in [(12_000, 1, 32, 1), (30_000, 2, 16, 0), (8_000, 3, 24, 12)]:
        pos, vel, mass, _ = gtc.make_galaxy(n, seed=seed)
        out.append((pos, vel, mass, gs, pack))
    wide = rng.normal(size=(3000, 3)) * 10.0
    clump = np.concatenate([wide, 1.0 + rng.normal(size=(300, 3)) * 1e-7])
    out.append((clump, rng.normal(size=clump.shape) * 0.1, rng.random(len(clump)) + 0.5, 8, 6))
    pos, mass = coincident_system()
    out.append((pos, np.zeros_like(pos), mass, 32, 1))
    pos, mass = lopsided_sphere(5000, 7)
    out.append((pos, rng.normal(size=pos.shape) * 0.05, mass, 16, 1))
    for n in (1, 9):
        pos, mass = lopsided_sphere(n, n + 40)
        out.append((pos, np.zeros_like(pos), mass, 8, 1))
    return out


def run(gtc, specs, forest, walk, steps, prime=True, graph=False, headroom=None):
    import torch
    d = torch.device("cuda", 0)
    bufs = []
    stats = []
    with gtc.Ensemble(len(specs)) as ens:
        for i, (pos, vel, mass, gs, pack) in enumerate(specs):
            t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(d)
            n = len(mass)
            b = dict(pos=t(pos), vel=t(vel), mass=t(mass),
                     acc=torch.zeros((n, 3), dtype=torch.float64, device=d),
                     pot=torch.zeros(n, dtype=torch.float64, device=d))
            bufs.append(b)
            ens.set_system(i, b["pos"].data_ptr(), b["vel"].data_ptr(), b["mass"].data_ptr(),
                           b["acc"].data_ptr(), b["pot"].data_ptr(), n,
                           **dict(SOLVER, group_size=gs, pack=pack))
            ens.context(i).set_option("walk_warps", walk)
        ens.set_option("forest", forest)
        ens.set_option("walk_warps", walk)
        if headroom is not None:
            ens.set_option("graph_headroom", headroom)
        torch.cuda.synchronize()  # the arrays are written on torch's stream
        ens.leapfrog(0.01, steps, prime=prime, graph=graph)
        torch.cuda.synchronize()
        for i in range(len(specs)):
            st = ens.context(i).stats()
            stats.append((st["cell_interactions"], st["body_interactions"], st["n_groups"],
                          st["graph_steps"]))
    return [{k: v.cpu().numpy() for k, v in b.items()} for b in bufs], stats


@gpu
@pytest.mark.parametrize("walk", [0, 1])
def test_forest_steps_equal_each_system_stepped_alone(gtc, walk):
    specs = systems(gtc)
    got, got_stats = run(gtc, specs, forest=1, walk=walk, steps=3)
    want, want_stats = run(gtc, specs, forest=0, walk=walk, steps=3)
    for i, (g, w) in enumerate(zip(got, want)):
        for k in ("pos", "vel", "acc", "pot"):
            assert np.array_equal(g[k], w[k]), (i, k)
        assert np.all(np.isfinite(g["acc"]))
    assert got_stats == want_stats


@gpu
@pytest.mark.parametrize("deep, headroom", [(False, 0.25), (False, 0.0), (True, 0.25)])
def test_forest_graph_steps_equal_eager_steps(gtc, deep, headroom):
    """Every step replayed from one captured graph of the whole forest step
    gives bitwise the eager steps. With no headroom most replays outgrow the
    captured sizes, and a tree that needs a second key word aborts every
    replay: those steps are redone eagerly, to the same doubles."""
    specs = [s for i, s in enumerate(systems(gtc)) if deep or i not in (3, 4)]  # (deeper than 21)
    got, got_stats = run(gtc, specs, forest=1, walk=0, steps=4, graph=True, headroom=headroom)
    want, want_stats = run(gtc, specs, forest=1, walk=0, steps=4)
    for i, (g, w) in enumerate(zip(got, want)):
        for k in ("pos", "vel", "acc", "pot"):
            assert np.array_equal(g[k], w[k]), (i, k)
    assert [s[:3] for s in got_stats] == [s[:3] for s in want_stats]
    replays = got_stats[0][3]
    if deep:
        assert replays == 0
    elif headroom > 0:
        assert replays == 4
    assert all(s[3] == replays for s in got_stats)


@gpu
def test_forest_force_evaluation_alone_equals_group_force(gtc):
    """A prime with no steps is one forest force evaluation: each system's
    forces are its own group_force's (walk by threads, the reference's list
    order), bitwise."""
    specs = systems(gtc)[:6]
    got, _ = run(gtc, specs, forest=1, walk=0, steps=0)
    with gtc.Context(0) as c:
        c.set_option("walk_warps", 0)
        for i, (pos, _, mass, gs, pack) in enumerate(specs):
            acc, pot = c.group_force(pos, mass, group_size=gs, pack=pack, **SOLVER)
            assert np.array_equal(got[i]["acc"], acc), i
            assert np.array_equal(got[i]["pot"], pot), i


@gpu
def test_forest_refuses_mixed_parameters(gtc):
    import torch
    d = torch.device("cuda", 0)
    pos, vel, mass, _ = gtc.make_galaxy(2000, seed=3)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(d)
    arrays = [[t(pos), t(vel), t(mass), t(np.zeros((2000, 3))), t(np.zeros(2000))]
              for _ in range(2)]
    with gtc.Ensemble(2) as ens:
        for i, (dp, dv, dm, da, dpt) in enumerate(arrays):
            kw = dict(SOLVER, group_size=16, pack=1, theta=0.75 if i == 0 else 0.6)
            ens.set_system(i, dp.data_ptr(), dv.data_ptr(), dm.data_ptr(), da.data_ptr(),
                           dpt.data_ptr(), 2000, **kw)
        ens.set_option("forest", 1)
        with pytest.raises(gtc.GtcInvalidArgument, match="forest"):
            ens.leapfrog(0.01, 1, prime=True, graph=False)
        ens.set_option("forest", -1)  # not eligible: system by system
        ens.leapfrog(0.01, 1, prime=True, graph=False)
    with pytest.raises(gtc.GtcInvalidArgument):
        with gtc.Ensemble(1) as ens:
            ens.set_option("forest", 2)


@gpu
def test_forest_graph_kept_across_calls(gtc):
    """A second call on the same systems and dt (no priming) replays the
    graph the first call captured: two calls of two steps give bitwise the
    four eager steps."""
    import torch
    d = torch.device("cuda", 0)
    specs = [s for i, s in enumerate(systems(gtc)) if i not in (3, 4)]
    want, _ = run(gtc, specs, forest=1, walk=0, steps=4)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(d)
    bufs = []
    with gtc.Ensemble(len(specs)) as ens:
        for i, (pos, vel, mass, gs, pack) in enumerate(specs):
            n = len(mass)
            b = dict(pos=t(pos), vel=t(vel), mass=t(mass), acc=t(np.zeros((n, 3))),
                     pot=t(np.zeros(n)))
            bufs.append(b)
            ens.set_system(i, b["pos"].data_ptr(), b["vel"].data_ptr(), b["mass"].data_ptr(),
                           b["acc"].data_ptr(), b["pot"].data_ptr(), n,
                           **dict(SOLVER, group_size=gs, pack=pack))
        ens.set_option("forest", 1)
        ens.set_option("walk_warps", 0)
        torch.cuda.synchronize()
        ens.leapfrog(0.01, 2, prime=True, graph=True)
        ens.leapfrog(0.01, 2, prime=False, graph=True)
        torch.cuda.synchronize()
        assert ens.context(0).stats()["graph_steps"] == 2
    for i, (b, w) in enumerate(zip(bufs, want)):
        for k in ("pos", "vel", "acc", "pot"):
            assert np.array_equal(b[k].cpu().numpy(), w[k]), (i, k)


@gpu
def test_forest_of_many_small_systems(gtc):
    """300 systems of 20..2000 bodies: the sort's pass by system takes two
    8-bit digits and each system's split table fewer levels (15 within the
    budget); each system still moves to the doubles of its own step."""
    rng = np.random.default_rng(77)
    specs = []
    for k in range(300):
        n = int(rng.integers(20, 2000))
        pos, mass = lopsided_sphere(n, 1000 + k)
        pos = pos * rng.uniform(0.1, 10.0) + rng.normal(size=3) * 50.0
        specs.append((pos, rng.normal(size=pos.shape) * 0.05, mass, int(rng.choice([8, 16, 32])),
                      int(rng.choice([0, 1]))))
    got, got_stats = run(gtc, specs, forest=1, walk=0, steps=2)
    want, want_stats = run(gtc, specs, forest=0, walk=0, steps=2)
    for i, (g, w) in enumerate(zip(got, want)):
        for k in ("pos", "vel", "acc", "pot"):
            assert np.array_equal(g[k], w[k]), (i, k)
    assert [s[:3] for s in got_stats] == [s[:3] for s in want_stats]
