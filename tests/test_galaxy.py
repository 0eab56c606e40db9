"""The synthetic galaxy generator (galactic-tides_gb300/galaxy.py): counts,
masses, the centre-of-mass frame, each component's profile against its
closed form, and the distributions against a galaxy the reference's own
make_hernquist_galaxy drew (tests/golden/galaxy_6000.npz, same model)."""

import importlib.util
import pathlib

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"


@pytest.fixture(scope="module")
def galaxy():
    # loaded by path: the generator is pure numpy and needs no compiled library
    spec = importlib.util.spec_from_file_location(
        "gtc_galaxy", ROOT / "galactic-tides_gb300" / "galaxy.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def big(galaxy):
    return galaxy.make_galaxy(200_000, seed=3)


def test_counts_masses_frame(galaxy, big):
    pos, vel, mass, typ = big
    assert pos.shape == (200_000, 3) and vel.shape == (200_000, 3)
    assert [(typ == t).sum() for t in (1, 2, 3)] == [94_000, 80_000, 26_000]
    for t, m in ((1, 5.8), (2, 1.0), (3, 0.33)):
        sel = typ == t
        assert np.isclose(mass[sel].sum(), m) and np.all(mass[sel] == mass[sel][0])
    assert np.abs((mass[:, None] * pos).sum(0)).max() < 1e-12
    assert np.abs((mass[:, None] * vel).sum(0)).max() < 1e-12
    assert np.isfinite(pos).all() and np.isfinite(vel).all()


def test_same_seed_same_galaxy(galaxy):
    a = galaxy.make_galaxy(5000, seed=9)
    b = galaxy.make_galaxy(5000, seed=9)
    c = galaxy.make_galaxy(5000, seed=10)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert not np.array_equal(a[0], c[0])


def test_profiles_against_closed_forms(galaxy):
    m = galaxy.galaxy_model(400_000, seed=5)
    pos, vel, mass, typ = galaxy.make_galaxy(model=m)
    p = pos  # moved to the centre-of-mass frame: shifts of order 1e-3
    # bulge: M(<r) / M = (r / (r + a))^2 / (rmax / (rmax + a))^2
    r = np.sort(np.linalg.norm(p[typ == 3], axis=1))
    q = np.array([0.1, 0.25, 0.5, 0.75, 0.9])
    s = np.sqrt(q * (m.bulge_rmax / (m.bulge_rmax + m.bulge_a)) ** 2)
    want = m.bulge_a * s / (1 - s)
    got = r[(q * len(r)).astype(int)]
    assert np.allclose(got, want, rtol=0.02)
    # disk: 1 - (1 + x) e^-x in R / h, sech^2 heights
    d = p[typ == 2]
    R = np.hypot(d[:, 0], d[:, 1]) / m.disk_h
    cdf = lambda x: 1 - (1 + x) * np.exp(-x)
    for x in (0.5, 1.0, 2.0, 4.0):
        assert abs(np.mean(R < x) - cdf(x) / cdf(m.disk_rmax / m.disk_h)) < 4e-3
    z = d[:, 2] / m.disk_z0
    for zz in (0.25, 0.5, 1.0, 2.0):  # P(|z| < zz) = tanh(zz)
        assert abs(np.mean(np.abs(z) < zz) - np.tanh(zz)) < 4e-3
    assert R.max() <= m.disk_rmax / m.disk_h + 0.02
    # halo: within its cut-off radius
    assert np.linalg.norm(p[typ == 1], axis=1).max() <= m.halo_rmax + 0.02


def ks_statistic(a, b):
    """Largest distance between the empirical distribution functions."""
    a, b = np.sort(a), np.sort(b)
    x = np.concatenate([a, b])
    return np.abs(np.searchsorted(a, x, "right") / len(a)
                  - np.searchsorted(b, x, "right") / len(b)).max()


def test_distributions_match_the_references_generator(galaxy, big):
    """Per component, the distributions of radius and height against the
    6000-body galaxy the reference drew for the same model: two-sample
    Kolmogorov-Smirnov statistics below the 0.1 % critical value (1.95
    sqrt((n1 + n2) / (n1 n2))). Velocities come from the same moment
    equations, but the reference takes the field from its own tree on the
    realised bodies and this generator from the analytic model, so they are
    compared by their rms speed per component (within 5 %)."""
    z = np.load(GOLDEN / "galaxy_6000.npz")
    pos, vel, mass, typ = big
    for t in (1, 2, 3):
        a, b = typ == t, z["type"] == t
        crit = 1.95 * np.sqrt((a.sum() + b.sum()) / (a.sum() * b.sum()))
        for name, f in (("radius", lambda p: np.linalg.norm(p, axis=1)),
                        ("height", lambda p: np.abs(p[:, 2]))):
            d = ks_statistic(f(pos[a]), f(z["pos"][b]))
            assert d < crit, (t, name, d, crit)
        va = np.sqrt((vel[a] ** 2).sum(1).mean())
        vb = np.sqrt((z["vel"][b] ** 2).sum(1).mean())
        assert abs(va / vb - 1) < 0.05, (t, va, vb)


def test_disk_rotates_and_spheroids_do_not(galaxy, big):
    pos, vel, mass, typ = big
    R = np.hypot(pos[:, 0], pos[:, 1])
    vphi = (pos[:, 0] * vel[:, 1] - pos[:, 1] * vel[:, 0]) / np.maximum(R, 1e-12)
    assert vphi[typ == 2].mean() > 0.6
    assert abs(vphi[typ == 1].mean()) < 0.02 and abs(vphi[typ == 3].mean()) < 0.03


def test_parabolic_orbit_and_encounter(galaxy):
    dx, dv = galaxy.parabolic_orbit(1.0, 7.13, 7.13, 2.0, 15.0)
    mu = 14.26
    assert np.isclose(np.linalg.norm(dx), 15.0)
    assert abs(0.5 * dv @ dv - mu / np.linalg.norm(dx)) < 1e-12 * mu   # zero energy
    ell = np.cross(dx, dv)[2]
    assert np.isclose(ell ** 2 / (2 * mu), 2.0)                         # pericentre
    assert dx @ dv < 0                                                  # approaching
    with pytest.raises(ValueError):
        galaxy.parabolic_orbit(1.0, 1.0, 1.0, 5.0, 2.0)
    pos, vel, mass, typ = galaxy.make_encounter(5000, seed=5, incl1=30, incl2=60)
    assert len(mass) == 10_000
    assert np.abs((mass[:, None] * pos).sum(0)).max() < 1e-10
    assert np.abs((mass[:, None] * vel).sum(0)).max() < 1e-10
    m1, m2 = mass[:5000].sum(), mass[5000:].sum()
    c1 = (mass[:5000, None] * pos[:5000]).sum(0) / m1
    c2 = (mass[5000:, None] * pos[5000:]).sum(0) / m2
    assert np.isclose(np.linalg.norm(c2 - c1), 15.0)


def test_orient_rotates_rigidly(galaxy):
    pos, vel, mass, _ = galaxy.make_galaxy(3000, seed=2)
    p0, v0 = pos.copy(), vel.copy()
    galaxy.orient(pos, vel, 37.0, 11.0)
    assert np.allclose(np.linalg.norm(pos, axis=1), np.linalg.norm(p0, axis=1))
    assert np.allclose((pos * vel).sum(1), (p0 * v0).sum(1))
    L0 = np.cross(p0, v0).sum(0)
    L = np.cross(pos, vel).sum(0)
    i = np.radians(37.0)
    # a spin along +z tilts by the inclination
    assert np.isclose(np.linalg.norm(L), np.linalg.norm(L0))
    assert np.isclose(L[2], L0[2] * np.cos(i) + L0[1] * np.sin(i))
