"""Synthetic disk + bulge + halo galaxies: the inputs of the benchmarks, the
encounter and ensemble runs, and the large tests.

The mass model is the one galactic-tides' benchmark galaxy uses
(include/galactic_tides/hernquist_ics.h:55-77, after Hernquist 1993):

* an exponential disk, surface density ~ exp(-R/h) cut at R = disk_rmax, with
  a sech^2(z/z0) vertical profile;
* a Hernquist bulge, rho ~ a / (r (r + a)^3), cut at bulge_rmax;
* a truncated isothermal halo, rho ~ exp(-r^2/rc^2) / (r^2 + gamma^2), cut at
  halo_rmax;

each component of equal-mass particles. This module draws its own particles
from that model with numpy's PCG64 generator: the same distributions as the
reference's generator, not the same particles.

Positions: the bulge by its closed-form cumulative mass r^2 / (r + a)^2; the
halo by interpolating its tabulated cumulative mass; disk radii by Newton
iterations on 1 - (1 + x) e^-x; heights by inverting the sech^2 profile
(z = z0 atanh(2u - 1)); directions isotropic.

Velocities (so that integration runs start near equilibrium): the spheroids
from the isotropic Jeans equation in the enclosed mass of all three components
(the disk counted as spherical), Gaussian components truncated at
vesc_fraction of the local escape speed; the disk from the epicyclic
approximation in the spheroids' field plus the thin disk's own (Freeman
1970) -- Toomre-Q normalised radial dispersion ~ exp(-R / 2h),
sigma_phi from kappa^2 / 4 Omega^2, isothermal-sheet sigma_z, and the
asymmetric-drift mean rotation. The system is moved to its centre-of-mass
frame.

numpy and scipy only; it loads no compiled library of this project.
"""

from dataclasses import dataclass, replace

import numpy as np
from scipy import special

# particle types, as GADGET numbers them (include/galactic_tides/particles.h:15-22)
HALO, DISK, BULGE = 1, 2, 3


@dataclass
class GalaxyModel:
    G: float = 1.0
    disk_n: int = 0
    bulge_n: int = 0
    halo_n: int = 0
    disk_mass: float = 1.0
    disk_h: float = 1.0
    disk_z0: float = 0.1
    disk_rmax: float = 10.0
    disk_Q: float = 1.5
    disk_Q_radius: float = 2.43
    bulge_mass: float = 0.33
    bulge_a: float = 0.2
    bulge_rmax: float = 4.0
    halo_mass: float = 5.8
    halo_core: float = 1.0
    halo_cutoff: float = 10.0
    halo_rmax: float = 30.0
    vesc_fraction: float = 0.95
    seed: int = 1

    @property
    def n(self):
        return self.disk_n + self.bulge_n + self.halo_n


def galaxy_model(n, seed=1, **fields):
    """The benchmark galaxy of n particles: disk 40 % (M = 1, h = 1,
    z0 = 0.1), bulge 13 % (M = 0.33, a = 0.2), halo the rest (M = 5.8,
    core 1, cutoff 10); keyword fields override."""
    disk_n = n * 40 // 100
    bulge_n = n * 13 // 100
    m = GalaxyModel(disk_n=disk_n, bulge_n=bulge_n, halo_n=n - disk_n - bulge_n, seed=seed)
    return replace(m, **fields) if fields else m


# ---------------------------------------------------------------- profiles

class _Halo:
    """Truncated isothermal sphere, its cumulative mass tabulated."""

    def __init__(self, m):
        self.mass, self.rmax = m.halo_mass, m.halo_rmax
        g, rc = m.halo_core, m.halo_cutoff
        self.shape = lambda r: np.exp(-(r / rc) ** 2) / (r * r + g * g)
        rmin = 1e-5 * (min(g, rc) if g > 0 else rc)
        r = np.concatenate([[0.0], np.geomspace(rmin, self.rmax, 8192)])
        shell = 4 * np.pi * r * r * self.shape(np.maximum(r, rmin))
        shell[0] = 0.0
        cum = np.concatenate([[0.0], np.cumsum(0.5 * (shell[1:] + shell[:-1]) * np.diff(r))])
        self.norm = self.mass / cum[-1]
        self.r, self.cum = r, cum * self.norm

    def density(self, r):
        return np.where((r > 0) & (r <= self.rmax), self.norm * self.shape(np.maximum(r, 1e-300)),
                        0.0)

    def enclosed(self, r):
        return np.interp(r, self.r, self.cum)

    def radius(self, u):
        return np.interp(u * self.mass, self.cum, self.r)


class _Bulge:
    """Hernquist sphere cut at rmax, normalised to its mass inside rmax."""

    def __init__(self, m):
        self.mass, self.a, self.rmax = m.bulge_mass, m.bulge_a, m.bulge_rmax
        self.frac = (self.rmax / (self.rmax + self.a)) ** 2

    def density(self, r):
        a = self.a
        rs = np.maximum(r, 1e-300)
        rho = self.mass / self.frac * a / (2 * np.pi * rs * (rs + a) ** 3)
        return np.where((r > 0) & (r <= self.rmax), rho, 0.0)

    def enclosed(self, r):
        rr = np.minimum(r, self.rmax)
        return self.mass / self.frac * (rr / (rr + self.a)) ** 2

    def radius(self, u):
        s = np.sqrt(u * self.frac)
        return self.a * s / (1 - s)


class _Disk:
    """Exponential disk cut at rmax; sech^2 layers of scale height z0."""

    def __init__(self, m):
        self.mass, self.h, self.rmax, self.z0 = m.disk_mass, m.disk_h, m.disk_rmax, m.disk_z0
        self.xmax = self.rmax / self.h
        self.fmax = self.cdf(self.xmax)
        self.sigma0 = self.mass / (2 * np.pi * self.h ** 2 * self.fmax)

    @staticmethod
    def cdf(x):
        return 1.0 - (1.0 + x) * np.exp(-x)

    def surface(self, R):
        return np.where(R > self.rmax, 0.0, self.sigma0 * np.exp(-R / self.h))

    def enclosed(self, r):
        return self.mass * self.cdf(np.minimum(r, self.rmax) / self.h) / self.fmax

    def radius(self, u):
        t = u * self.fmax
        # start from a table, polish with Newton on cdf(x) = t (cdf' = x e^-x)
        xs = np.linspace(0.0, self.xmax, 4097)
        x = np.interp(t, self.cdf(xs), xs)
        for _ in range(4):
            d = x * np.exp(-x)
            x = np.clip(x - (self.cdf(x) - t) / np.maximum(d, 1e-300), 0.0, self.xmax)
        return x * self.h


def _open_uniform(rng, size):
    u = rng.random(size)
    bad = u <= 0.0
    while bad.any():
        u[bad] = rng.random(int(bad.sum()))
        bad = u <= 0.0
    return u


def _directions(rng, n):
    cz = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2 * np.pi, n)
    s = np.sqrt(np.maximum(0.0, 1 - cz * cz))
    return np.stack([s * np.cos(ph), s * np.sin(ph), cz], axis=1)


# ---------------------------------------------------------------- galaxies

def make_galaxy(n=None, seed=1, model=None, **fields):
    """-> pos (n,3), vel (n,3), mass (n,), type (n,): halo bodies first, then
    disk, then bulge, centre of mass at rest at the origin."""
    m = model if model is not None else galaxy_model(n, seed, **fields)
    for comp, cnt, mass in (("disk", m.disk_n, m.disk_mass), ("bulge", m.bulge_n, m.bulge_mass),
                            ("halo", m.halo_n, m.halo_mass)):
        if cnt < 0 or (cnt > 0 and not mass > 0):
            raise ValueError(f"invalid {comp}: {cnt} bodies of total mass {mass}")
    if m.n == 0:
        raise ValueError("a galaxy needs at least one body")
    rng = np.random.Generator(np.random.PCG64(m.seed))
    halo, bulge, disk = _Halo(m), _Bulge(m), _Disk(m)
    parts = []
    if m.halo_n:
        r = halo.radius(_open_uniform(rng, m.halo_n))
        parts.append((r[:, None] * _directions(rng, m.halo_n), m.halo_mass / m.halo_n, HALO))
    if m.disk_n:
        R = disk.radius(_open_uniform(rng, m.disk_n))
        ph = rng.uniform(0.0, 2 * np.pi, m.disk_n)
        z = m.disk_z0 * np.arctanh(2 * _open_uniform(rng, m.disk_n) - 1)
        parts.append((np.stack([R * np.cos(ph), R * np.sin(ph), z], axis=1),
                      m.disk_mass / m.disk_n, DISK))
    if m.bulge_n:
        r = bulge.radius(_open_uniform(rng, m.bulge_n))
        parts.append((r[:, None] * _directions(rng, m.bulge_n), m.bulge_mass / m.bulge_n, BULGE))
    pos = np.concatenate([p for p, _, _ in parts])
    mass = np.concatenate([np.full(len(p), mk) for p, mk, _ in parts])
    typ = np.concatenate([np.full(len(p), t, np.int32) for p, _, t in parts])
    vel = _velocities(m, rng, pos, typ, halo if m.halo_n else None,
                      bulge if m.bulge_n else None, disk if m.disk_n else None)
    mt = mass.sum()
    pos -= (mass[:, None] * pos).sum(0) / mt
    vel -= (mass[:, None] * vel).sum(0) / mt
    return np.ascontiguousarray(pos), np.ascontiguousarray(vel), mass, typ


def _velocities(m, rng, pos, typ, halo, bulge, disk):
    G = m.G
    comps = [c for c in (halo, bulge, disk) if c is not None]
    scales = [x for x in (m.halo_core if m.halo_core > 0 else m.halo_cutoff, m.bulge_a, m.disk_h)]
    rlo = 1e-4 * min(scales)
    rhi = max(m.halo_rmax, m.bulge_rmax, m.disk_rmax)
    rg = np.geomspace(rlo, rhi, 2000)
    menc = sum(c.enclosed(rg) for c in comps)
    grav = G * menc / rg ** 2
    dr = np.diff(rg)
    # potential: -G M / r outside, inward integral of the field inside
    seg = 0.5 * (grav[1:] + grav[:-1]) * dr
    phi = -G * menc[-1] / rhi - np.concatenate([np.cumsum(seg[::-1])[::-1], [0.0]])
    vel = np.zeros_like(pos)
    r = np.linalg.norm(pos, axis=1)

    for comp, t in ((halo, HALO), (bulge, BULGE)):
        if comp is None:
            continue
        sel = np.nonzero(typ == t)[0]
        rho = comp.density(rg)
        flux = 0.5 * (rho[1:] * grav[1:] + rho[:-1] * grav[:-1]) * dr
        outer = np.concatenate([np.cumsum(flux[::-1])[::-1], [0.0]])
        s2 = np.where(rho > 0, outer / np.maximum(rho, 1e-300), 0.0)
        ri = np.maximum(r[sel], rlo)
        sigma = np.sqrt(np.maximum(0.0, np.interp(ri, rg, s2)))
        pot = np.where(r[sel] >= rhi, -G * menc[-1] / np.maximum(r[sel], 1e-300),
                       np.interp(ri, rg, phi))
        vmax = m.vesc_fraction * np.sqrt(np.maximum(0.0, -2.0 * pot))
        v = sigma[:, None] * rng.standard_normal((len(sel), 3))
        for _ in range(1000):
            fast = np.linalg.norm(v, axis=1) > vmax
            if not fast.any():
                break
            v[fast] = sigma[fast, None] * rng.standard_normal((int(fast.sum()), 3))
        s = np.linalg.norm(v, axis=1)
        over = s > vmax
        v[over] *= (vmax[over] / s[over])[:, None]
        vel[sel] = v

    if disk is not None:
        sel = np.nonzero(typ == DISK)[0]
        nR = 200
        dR = m.disk_rmax / nR
        Rg = dR * np.arange(1, nR + 1)
        # midplane field: the spheroids' enclosed mass plus the thin
        # exponential disk's own field (Freeman 1970, y = R / 2h):
        # v_c^2 = 4 pi G Sigma0 h y^2 [I0(y) K0(y) - I1(y) K1(y)]
        F = G * sum(c.enclosed(Rg) for c in comps if c is not disk) / Rg ** 2
        y = Rg / (2 * m.disk_h)
        F = F + 4 * np.pi * G * disk.sigma0 * m.disk_h * y * y * (
            special.i0(y) * special.k0(y) - special.i1(y) * special.k1(y)) / Rg
        om2 = np.maximum(F / Rg, 1e-30)
        kap2 = np.clip(np.gradient(F, dR) + 3 * F / Rg, om2, 4 * om2)
        kq = np.sqrt(np.interp(m.disk_Q_radius, Rg, kap2))
        sRq = m.disk_Q * 3.36 * G * float(disk.surface(np.array(m.disk_Q_radius))) / kq
        x, y = pos[sel, 0], pos[sel, 1]
        R = np.hypot(x, y)
        o2, k2 = np.interp(R, Rg, om2), np.interp(R, Rg, kap2)
        sR2 = sRq ** 2 * np.exp(-(R - m.disk_Q_radius) / m.disk_h)
        ratio = k2 / (4 * o2)
        sZ2 = np.pi * G * disk.surface(R) * m.disk_z0
        vbar = np.sqrt(np.maximum(0.0, o2 * R * R + sR2 * (1 - ratio - 2 * R / m.disk_h)))
        g = rng.standard_normal((len(sel), 3))
        vR = np.sqrt(sR2) * g[:, 0]
        vphi = vbar + np.sqrt(sR2 * ratio) * g[:, 1]
        Rs = np.where(R > 0, R, 1.0)
        c, s = np.where(R > 0, x / Rs, 1.0), np.where(R > 0, y / Rs, 0.0)
        vel[sel, 0] = vR * c - vphi * s
        vel[sel, 1] = vR * s + vphi * c
        vel[sel, 2] = np.sqrt(sZ2) * g[:, 2]
    return vel


def orient(pos, vel, incl_deg, omega_deg=0.0):
    """Rotates positions and velocities (in place) by incl_deg about x, then
    omega_deg about z: the disk's spin axis tilts by incl_deg."""
    i, w = np.radians(incl_deg), np.radians(omega_deg)
    rx = np.array([[1, 0, 0], [0, np.cos(i), -np.sin(i)], [0, np.sin(i), np.cos(i)]])
    rz = np.array([[np.cos(w), -np.sin(w), 0], [np.sin(w), np.cos(w), 0], [0, 0, 1]])
    rot = rz @ rx
    pos[:] = pos @ rot.T
    vel[:] = vel @ rot.T


def parabolic_orbit(G, m1, m2, rp, r0):
    """Relative position and velocity (dx, dv) of body 2 about body 1 on a
    parabolic Kepler orbit of pericentre rp, at separation r0 on the way in,
    in the x-y plane with the pericentre on +x."""
    if not (rp > 0 and r0 >= rp):
        raise ValueError("parabolic_orbit: start separation below pericentre")
    mu = G * (m1 + m2)
    # r = 2 rp / (1 + cos f); before pericentre the true anomaly is negative
    f = -np.arccos(np.clip(2 * rp / r0 - 1, -1.0, 1.0))
    ell = np.sqrt(2 * mu * rp)            # specific angular momentum
    rhat = np.array([np.cos(f), np.sin(f), 0.0])
    that = np.array([-np.sin(f), np.cos(f), 0.0])
    vr = mu / ell * np.sin(f)             # negative: approaching
    return r0 * rhat, vr * rhat + (ell / r0) * that


def make_encounter(n_each, seed=1, incl1=30.0, incl2=60.0, rp=2.0, r0=15.0, omega1=0.0,
                   omega2=0.0, **fields):
    """Two galaxies of n_each bodies (seeds seed and seed + 1), inclined
    incl1 / incl2 degrees, on a parabolic orbit of pericentre rp from
    separation r0, centre of mass at rest at the origin -> pos, vel, mass,
    type (galaxy 1 first)."""
    p1, v1, m1, t1 = make_galaxy(model=galaxy_model(n_each, seed, **fields))
    p2, v2, m2, t2 = make_galaxy(model=galaxy_model(n_each, seed + 1, **fields))
    orient(p1, v1, incl1, omega1)
    orient(p2, v2, incl2, omega2)
    M1, M2 = m1.sum(), m2.sum()
    dx, dv = parabolic_orbit(fields.get("G", 1.0), M1, M2, rp, r0)
    f1, f2 = -M2 / (M1 + M2), M1 / (M1 + M2)
    pos = np.concatenate([p1 + f1 * dx, p2 + f2 * dx])
    vel = np.concatenate([v1 + f1 * dv, v2 + f2 * dv])
    return pos, vel, np.concatenate([m1, m2]), np.concatenate([t1, t2])
