"""The device leapfrog and diagnostics: the reference's integrator tests
(tests/test_integrator.cpp: a circular binary, a Plummer sphere in
equilibrium), the oracle's leapfrog, the CUDA-graph step against the eager
step (bitwise), and the encounter set-up (apps/galactic_tides_ics.cpp)."""

import numpy as np
import pytest

SOLVER = dict(G=1.0, theta=0.75, eps=0.025, quadrupole=True, group_size=32, leaf_size=8,
              pack=True)


def plummer(n, seed=1):
    """Plummer sphere in Henon units sampled from its distribution function
    (Aarseth, Henon & Wielen 1974), as tests/test_integrator.cpp:44-58 draws it."""
    rng = np.random.default_rng(seed)
    a = 3 * np.pi / 16

    def direction(k):
        cz = 2 * rng.random(k) - 1
        ph = 2 * np.pi * rng.random(k)
        s = np.sqrt(1 - cz * cz)
        return np.stack([s * np.cos(ph), s * np.sin(ph), cz], axis=1)

    r = np.empty(0)
    while r.size < n:
        u = rng.random(2 * n)
        rr = a / np.sqrt(u ** (-2.0 / 3.0) - 1)
        r = np.concatenate([r, rr[rr <= 10 * a]])
    r = r[:n]
    q = np.empty(0)
    while q.size < n:
        qq, g = rng.random(4 * n), 0.1 * rng.random(4 * n)
        q = np.concatenate([q, qq[g <= qq * qq * (1 - qq * qq) ** 3.5]])
    q = q[:n]
    vesc = np.sqrt(2.0) * (r * r + a * a) ** -0.25
    pos = r[:, None] * direction(n)
    vel = (q * vesc)[:, None] * direction(n)
    pos -= pos.mean(0)
    vel -= vel.mean(0)
    return pos, vel, np.full(n, 1.0 / n)


# ---------------------------------------------------------------- CPU only

def test_parabolic_orbit_has_zero_energy(gtc):
    dx, dv = gtc.parabolic_orbit(1.0, 7.13, 7.13, 2.0, 15.0)
    assert abs(np.linalg.norm(dx) - 15.0) < 1e-12
    assert abs(0.5 * dv @ dv - 14.26 / np.linalg.norm(dx)) < 1e-12
    assert dx @ dv < 0  # approaching
    h = np.cross(dx, dv)
    assert abs(h @ h - 2 * 14.26 * 2.0) < 1e-9  # pericentre rp: h^2 = 2 G M rp
    with pytest.raises(ValueError):
        gtc.parabolic_orbit(1.0, 1.0, 1.0, 5.0, 2.0)


def test_encounter_is_in_its_centre_of_mass_frame(gtc):
    pos, vel, mass, typ = gtc.make_encounter(20_000, seed=5, incl1=30, incl2=60)
    assert pos.shape == (40_000, 3)
    m = mass[:, None]
    assert np.abs((m * pos).sum(0)).max() < 1e-9 and np.abs((m * vel).sum(0)).max() < 1e-9
    # the two galaxies' centres are r0 apart
    c1 = (m[:20_000] * pos[:20_000]).sum(0) / mass[:20_000].sum()
    c2 = (m[20_000:] * pos[20_000:]).sum(0) / mass[20_000:].sum()
    assert abs(np.linalg.norm(c2 - c1) - 15.0) < 1e-9
    # galaxy 1's disk is inclined 30 degrees: its angular momentum about its
    # centre makes that angle with z
    disk = np.where(typ[:20_000] == 2)[0]
    v1 = (m[:20_000] * vel[:20_000]).sum(0) / mass[:20_000].sum()
    L = np.cross(pos[disk] - c1, vel[disk] - v1).sum(0)
    assert abs(np.degrees(np.arccos(L[2] / np.linalg.norm(L))) - 30.0) < 0.5


def test_orient_rotates_rigidly(gtc):
    rng = np.random.default_rng(2)
    pos, vel = rng.normal(size=(100, 3)), rng.normal(size=(100, 3))
    p0, v0 = pos.copy(), vel.copy()
    gtc.orient(pos, vel, 37.0, 11.0)
    assert np.allclose(np.linalg.norm(pos, axis=1), np.linalg.norm(p0, axis=1), atol=1e-12)
    assert np.allclose(pos @ pos.T, p0 @ p0.T, atol=1e-10)
    assert np.allclose(np.einsum("ij,ij->i", pos, vel), np.einsum("ij,ij->i", p0, v0), atol=1e-12)


# ---------------------------------------------------------------- GPU

gpu = pytest.mark.gpu


def _dev(*arrays):
    import torch
    d = torch.device("cuda", 0)
    return [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(d) for a in arrays]


def _run(ctx, pos, vel, mass, dt, steps, prime=True, graph=False, **kw):
    import torch
    n = len(mass)
    dpos, dvel, dmass = _dev(pos, vel, mass)
    dacc = torch.zeros((n, 3), dtype=torch.float64, device=dpos.device)
    dpot = torch.zeros(n, dtype=torch.float64, device=dpos.device)
    args = dict(SOLVER)
    args.update(kw)
    ctx.leapfrog_device(dpos.data_ptr(), dvel.data_ptr(), dmass.data_ptr(), dacc.data_ptr(),
                        dpot.data_ptr(), n, dt, steps, prime=prime, graph=graph, **args)
    d = ctx.diagnostics_device(dpos.data_ptr(), dvel.data_ptr(), dmass.data_ptr(),
                               dpot.data_ptr(), n)
    return dpos.cpu().numpy(), dvel.cpu().numpy(), dacc.cpu().numpy(), dpot.cpu().numpy(), d


def _diag(ctx, pos, vel, mass, pot):
    dpos, dvel, dmass, dpot = _dev(pos, vel, mass, pot)
    return ctx.diagnostics_device(dpos.data_ptr(), dvel.data_ptr(), dmass.data_ptr(),
                                  dpot.data_ptr(), len(mass))


@gpu
def test_diagnostics_match_fp64_sums(ctx):
    rng = np.random.default_rng(3)
    n = 100_003
    pos, vel = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    mass, pot = rng.random(n), -rng.random(n)
    d = _diag(ctx, pos, vel, mass, pot)
    m = mass[:, None]
    assert abs(d["kinetic"] - 0.5 * (mass * (vel * vel).sum(1)).sum()) < 1e-10 * d["kinetic"]
    assert abs(d["potential"] - 0.5 * (mass * pot).sum()) < 1e-10 * abs(d["potential"])
    assert np.allclose(d["momentum"], (m * vel).sum(0), rtol=1e-9, atol=1e-9)
    assert np.allclose(d["angular_momentum"], (m * np.cross(pos, vel)).sum(0), rtol=1e-9, atol=1e-9)
    assert np.allclose(d["centre_of_mass"], (m * pos).sum(0) / mass.sum(), rtol=1e-9, atol=1e-12)
    assert abs(d["total"] - d["kinetic"] - d["potential"]) < 1e-12 * abs(d["total"])


@gpu
@pytest.mark.parametrize("graph", [False, True])
def test_circular_binary(ctx, graph):
    """tests/test_integrator.cpp:13-35 with the device leapfrog."""
    pos = np.array([[0.5, 0, 0], [-0.5, 0, 0]], float)
    vel = np.array([[0, 0.5, 0], [0, -0.5, 0]], float)
    mass = np.array([0.5, 0.5])
    period, steps = 2 * np.pi, 2000
    dt = 10 * period / steps
    kw = dict(eps=0.0, theta=0.5)
    p0, v0, a0, phi0, d0 = _run(ctx, pos, vel, mass, dt, 0, **kw)
    p1, v1, _, _, d1 = _run(ctx, pos, vel, mass, dt, steps, graph=graph, **kw)
    assert abs(d1["total"] - d0["total"]) < 1e-5 * abs(d0["total"])
    assert np.linalg.norm(p1[0] - [0.5, 0, 0]) < 0.02
    # the reference checks 1e-12 with FP64 forces; FP32 forces carry a
    # relative rounding of about 1e-7 that does not cancel exactly
    assert abs(d1["angular_momentum"][2] - d0["angular_momentum"][2]) < 1e-7 * 0.25


@gpu
def test_plummer_sphere_conserves_energy(ctx):
    """tests/test_integrator.cpp:37-79: 2000 bodies, eps 0.02, theta 0.6,
    500 steps of 0.01: |dE/E| < 5e-3, virial ratio within 0.1 of 1."""
    pos, vel, mass = plummer(2000)
    _, _, _, _, d0 = _run(ctx, pos, vel, mass, 0.01, 0, eps=0.02, theta=0.6)
    assert abs(d0["virial_ratio"] - 1.0) < 0.1
    _, _, _, _, d1 = _run(ctx, pos, vel, mass, 0.01, 500, eps=0.02, theta=0.6, graph=True)
    assert abs(d1["total"] / d0["total"] - 1) < 5e-3
    assert abs(d1["virial_ratio"] - 1.0) < 0.1


@gpu
def test_leapfrog_matches_oracle(ctx, oracle, gtc):
    """The device integrator against the oracle's restatement of
    LeapfrogKDK with the group solver (FP64 kicks and drifts, FP32 forces)."""
    pos, vel, mass, _ = gtc.make_galaxy(6000, seed=4)
    dt, steps = 0.01, 5
    p_dev, v_dev, _, _, _ = _run(ctx, pos, vel, mass, dt, steps, pack=False)
    p_orc, v_orc, _ = oracle.leapfrog_group(pos, vel, mass, dt, steps, theta=0.75, eps=0.025,
                                            group_size=32, leaf_size=8, pack=False)
    assert np.abs(p_dev - p_orc).max() < 1e-9 * np.abs(p_orc).max()
    assert np.abs(v_dev - v_orc).max() < 1e-6 * np.abs(v_orc).max()


@gpu
def test_graph_step_is_the_eager_step(ctx, gtc):
    """configs[0]: one force evaluation and 10 leapfrog steps of 0.01 at
    N = 50,000, eagerly and replayed from a CUDA graph: bitwise equal."""
    pos, vel, mass, _ = gtc.make_galaxy(50_000, seed=1)
    eager = _run(ctx, pos, vel, mass, 0.01, 10)
    graph = _run(ctx, pos, vel, mass, 0.01, 10, graph=True)
    assert ctx.stats()["graph_steps"] == 10
    for a, b in zip(eager[:4], graph[:4]):
        assert np.array_equal(a, b)
    assert abs(graph[4]["total"] / eager[4]["total"] - 1) < 1e-15


@gpu
def test_graph_replays_that_outgrow_their_buffers_are_redone(gtc):
    """With no headroom most replays outgrow the captured sizes; each is
    redone eagerly and the trajectory is still the eager one, bitwise."""
    pos, vel, mass, _ = gtc.make_galaxy(20_000, seed=2)
    with gtc.Context(0) as c:
        eager = _run(c, pos, vel, mass, 0.02, 12)
    with gtc.Context(0) as c:
        c.set_option("graph_headroom", 0.0)
        graph = _run(c, pos, vel, mass, 0.02, 12, graph=True)
        replayed = c.stats()["graph_steps"]
    assert replayed < 12
    for a, b in zip(eager[:4], graph[:4]):
        assert np.array_equal(a, b)


@gpu
def test_encounter_energy_drift(gtc):
    """A scaled-down parabolic encounter (2 x 20,000 bodies, 100 steps of
    0.01 from 15 apart): energy conserved to 2e-3, momentum stays ~0."""
    pos, vel, mass, _ = gtc.make_encounter(20_000, seed=1, incl1=30, incl2=60, rp=2.0, r0=15.0)
    with gtc.Context(0) as c:
        _, _, _, _, d0 = _run(c, pos, vel, mass, 0.01, 0)
        _, _, _, _, d1 = _run(c, pos, vel, mass, 0.01, 100, graph=True)
        assert c.stats()["graph_steps"] >= 90
    assert abs(d1["total"] / d0["total"] - 1) < 2e-3
    assert np.abs(d1["momentum"]).max() < 1e-3 * np.abs(mass).sum()


@gpu
@pytest.mark.parametrize("forest", [0, 1])
def test_ensemble_step_graph_equals_each_system_alone(gtc, forest):
    """Three galaxies advanced together, with tuned-like parameters per
    system -- one graph launch per step of every system's kernel chains, or
    as one forest -- give bitwise the trajectories each gives alone."""
    import torch
    specs = [(12_000, 1, 32, True), (30_000, 2, 16, False), (8_000, 3, 24, True)]
    alone = []
    with gtc.Context(0) as c:
        for n, seed, gs, pack in specs:
            pos, vel, mass, _ = gtc.make_galaxy(n, seed=seed)
            alone.append(_run(c, pos, vel, mass, 0.01, 5, group_size=gs, pack=pack))
    d = torch.device("cuda", 0)
    bufs = []
    with gtc.Ensemble(len(specs)) as ens:
        for i, (n, seed, gs, pack) in enumerate(specs):
            pos, vel, mass, _ = gtc.make_galaxy(n, seed=seed)
            dpos, dvel, dmass = _dev(pos, vel, mass)
            dacc = torch.zeros((n, 3), dtype=torch.float64, device=d)
            dpot = torch.zeros(n, dtype=torch.float64, device=d)
            bufs.append((dpos, dvel, dacc, dpot, dmass))
            kw = dict(SOLVER, group_size=gs, pack=pack)
            ens.set_system(i, dpos.data_ptr(), dvel.data_ptr(), dmass.data_ptr(), dacc.data_ptr(),
                           dpot.data_ptr(), n, **kw)
        ens.set_option("forest", forest)
        ens.leapfrog(0.01, 5, prime=True, graph=True)
        torch.cuda.synchronize()
        for i in range(len(specs)):
            assert ens.context(i).stats()["graph_steps"] == 5
    for (dpos, dvel, dacc, dpot, _), want in zip(bufs, alone):
        assert np.array_equal(dpos.cpu().numpy(), want[0])
        assert np.array_equal(dvel.cpu().numpy(), want[1])
        assert np.array_equal(dacc.cpu().numpy(), want[2])


@gpu
def test_autotuner_returns_a_timed_configuration(ctx, gtc):
    """group_size, packing (off, a threshold, a group's worth) and the walk;
    the context's own options stay as they were; the direct kernel's tile
    shape is kept in the context."""
    pos, _, mass, _ = gtc.make_galaxy(60_000, seed=9)
    dpos, dmass = _dev(pos, mass)
    gs, pack, ms, walk = ctx.autotune_group(dpos.data_ptr(), dmass.data_ptr(), len(mass),
                                            **SOLVER)
    assert gs in (8, 16, 24, 32) and pack in (0, 1, gs // 2, 3 * gs // 4) and ms > 0
    assert walk in (0, 1)
    k, kms = ctx.autotune_direct(dpos.data_ptr(), dmass.data_ptr(), len(mass), **SOLVER)
    assert k in (2, 4) and kms > 0
    # the tuned parameters solve, with the chosen walk, to the same lists
    c = gtc.Context(0)
    try:
        kw = dict(SOLVER, group_size=gs, pack=pack)
        c.set_option("walk_warps", walk)
        acc, _ = c.group_force(pos, mass, **kw)
        d = c.export()
        c.set_option("walk_warps", 1 - walk)
        acc2, _ = c.group_force(pos, mass, **kw)
        d2 = c.export()
    finally:
        c.close()
    assert np.array_equal(d["cell_list"], d2["cell_list"])
    assert np.abs(acc - acc2).max() <= 1e-4 * np.abs(acc).max()


@gpu
def test_autotuner_picks_the_evaluation_tile_shape(gtc):
    """gtc_autotune_eval times the list evaluation's tile shapes and keeps
    the fastest in the context. Staged pairs per iteration do not change the
    forces (bitwise); the pass cost changes the slicing, so the summation
    order only."""
    pos, _, mass, _ = gtc.make_galaxy(60_000, seed=9)
    dpos, dmass = _dev(pos, mass)
    res = {}
    c = gtc.Context(0)
    try:
        k, cost, ms = c.autotune_eval(dpos.data_ptr(), dmass.data_ptr(), len(mass), **SOLVER)
        assert k in (1, 2) and cost in (8, 16, 24, 32, 48) and ms > 0
        for pairs, pass_cost in ((2, 24), (1, 24), (2, 8), (1, 48)):
            c.set_option("eval_pairs", pairs)
            c.set_option("eval_pass_cost", pass_cost)
            res[(pairs, pass_cost)] = c.group_force(pos, mass, **SOLVER)
        with pytest.raises(gtc.GtcInvalidArgument):
            c.set_option("eval_pairs", 3)
        with pytest.raises(gtc.GtcInvalidArgument):
            c.autotune_eval(dpos.data_ptr(), dmass.data_ptr(), len(mass),
                            **dict(SOLVER, quadrupole=False))
    finally:
        c.close()
    for a, b in zip(res[(2, 24)], res[(1, 24)]):
        assert np.array_equal(a, b)
    ref = res[(2, 24)][0]
    for key in ((2, 8), (1, 48)):
        assert np.abs(res[key][0] - ref).max() <= 1e-5 * np.abs(ref).max()


@gpu
def test_packing_threshold_keeps_sibling_runs(ctx):
    """pack = k >= 2 merges small siblings while the run holds at most k
    bodies: groups are still whole nodes, leaf chunks or sibling runs, the
    lists cover every body once, and merged runs stay within k."""
    from checks import check_lists, check_packing, dev_children
    from native import lopsided_sphere
    pos, mass = lopsided_sphere(6000, 21)
    counts = {}
    for pack in (0, 12, 24, 1):
        ctx.group_force(pos, mass, theta=0.7, eps=0.01, group_size=32, pack=pack)
        d = ctx.export()
        nd = d["nodes"]
        assert check_lists(nd["begin"], nd["end"], d["groups"], d["cell_list"], d["body_list"],
                           len(mass), 32) == 0
        assert check_packing(nd["begin"], nd["end"], dev_children(nd), d["groups"]) == 0
        counts[pack] = len(d["groups"])
    assert counts[0] >= counts[12] >= counts[24] >= counts[1]
    assert counts[0] > counts[1]
