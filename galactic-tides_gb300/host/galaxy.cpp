// Hernquist (1993) disk + bulge + halo galaxy: the benchmark input.
// Positions restate src/hernquist_ics.cpp:142-204 draw for draw; velocities
// use the same moment equations (hernquist_ics.cpp:207-378) on analytic
// enclosed-mass forces. See galaxy.h.
//
// Compiled with -ffp-contract=off so every expression rounds as in the
// reference's x86-64 build.

#include "galaxy.h"

#include <algorithm>
#include <cmath>
#include <functional>
#include <numeric>
#include <random>
#include <vector>

namespace {

using Rng = std::mt19937_64;

// Linear interpolation in a monotonic table, clamped at both ends
// (hernquist_ics.cpp:16-23).
double lookup(const std::vector<double> &x, const std::vector<double> &y, double v) {
  if (v <= x.front()) return y.front();
  if (v >= x.back()) return y.back();
  const std::size_t j = static_cast<std::size_t>(std::upper_bound(x.begin(), x.end(), v) - x.begin());
  const double t = (v - x[j - 1]) / (x[j] - x[j - 1]);
  return y[j - 1] + t * (y[j] - y[j - 1]);
}

// n points evenly spaced in log r (hernquist_ics.cpp:25-30).
std::vector<double> log_spaced(double lo, double hi, std::size_t n) {
  std::vector<double> g(n);
  const double a = std::log(lo), b = std::log(hi);
  for (std::size_t i = 0; i < n; ++i) g[i] = std::exp(a + (b - a) * double(i) / double(n - 1));
  return g;
}

// A truncated spherical profile normalised to `mass`, with its cumulative
// mass tabulated by the trapezoidal rule on r = 0 plus 4000 log-spaced radii
// (hernquist_ics.cpp:34-56).
class Spheroid {
 public:
  Spheroid(std::function<double(double)> shape, double rmax, double mass, double rmin)
      : shape_(std::move(shape)), rmax_(rmax), mass_(mass) {
    r_.push_back(0.0);
    for (double r : log_spaced(rmin, rmax, 4000)) r_.push_back(r);
    m_.assign(r_.size(), 0.0);
    auto shell = [&](double r) { return r > 0 ? 4 * M_PI * r * r * shape_(r) : 0.0; };
    for (std::size_t i = 1; i < r_.size(); ++i)
      m_[i] = m_[i - 1] + 0.5 * (shell(r_[i - 1]) + shell(r_[i])) * (r_[i] - r_[i - 1]);
    scale_ = mass_ / m_.back();
    for (double &m : m_) m *= scale_;
  }
  double density(double r) const { return (r > rmax_ || r <= 0) ? 0.0 : scale_ * shape_(r); }
  double enclosed(double r) const { return r >= rmax_ ? mass_ : lookup(r_, m_, r); }
  double radius_of(double u) const { return lookup(m_, r_, u * mass_); }

 private:
  std::function<double(double)> shape_;
  double rmax_, mass_, scale_ = 1.0;
  std::vector<double> r_, m_;
};

struct Dir {
  double x, y, z;
};

// Isotropic unit vector: cos(theta) then azimuth (hernquist_ics.cpp:58-62).
Dir isotropic(Rng &rng) {
  std::uniform_real_distribution<double> u(0.0, 1.0);
  const double cz = 2 * u(rng) - 1;
  const double ph = 2 * M_PI * u(rng);
  const double s = std::sqrt(1 - cz * cz);
  return {s * std::cos(ph), s * std::sin(ph), cz};
}

double disk_fraction(double x) { return 1.0 - (1.0 + x) * std::exp(-x); }  // :65

}  // namespace

extern "C" {

void gtc_galaxy_default(gtc_galaxy_model *m, uint64_t n, uint64_t seed) {
  m->G = 1.0;
  m->disk_n = n * 40 / 100;
  m->bulge_n = n * 13 / 100;
  m->halo_n = n - m->disk_n - m->bulge_n;
  m->disk_mass = 1.0;
  m->disk_h = 1.0;
  m->disk_z0 = 0.1;
  m->disk_rmax = 10.0;
  m->disk_Q = 1.5;
  m->disk_Q_radius = 2.43;
  m->bulge_mass = 0.33;
  m->bulge_a = 0.2;
  m->bulge_rmax = 4.0;
  m->halo_mass = 5.8;
  m->halo_core = 1.0;
  m->halo_cutoff = 10.0;
  m->halo_rmax = 30.0;
  m->vesc_fraction = 0.95;
  m->seed = seed;
}

int gtc_make_galaxy(const gtc_galaxy_model *mp, double *pos, double *vel, double *mass,
                    int32_t *type) {
  const gtc_galaxy_model &m = *mp;
  const bool disk = m.disk_n > 0, bulge = m.bulge_n > 0, halo = m.halo_n > 0;
  if ((disk && !(m.disk_mass > 0)) || (bulge && !(m.bulge_mass > 0)) ||
      (halo && !(m.halo_mass > 0)) || (!disk && !bulge && !halo))
    return 1;
  Rng rng(m.seed);
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  std::normal_distribution<double> gauss(0.0, 1.0);
  auto open01 = [&]() {
    double u;
    do u = uni(rng);
    while (u <= 0.0 || u >= 1.0);
    return u;
  };
  const double h = m.disk_h, gamma = m.halo_core, rc = m.halo_cutoff, a = m.bulge_a;
  const Spheroid halo_p([=](double r) { return std::exp(-r * r / (rc * rc)) / (r * r + gamma * gamma); },
                        m.halo_rmax, halo ? m.halo_mass : 0.0,
                        1e-4 * (gamma > 0 ? std::min(gamma, rc) : rc));
  const Spheroid bulge_p([=](double r) { return a / (r * std::pow(r + a, 3)); }, m.bulge_rmax,
                         bulge ? m.bulge_mass : 0.0, 1e-4 * a);
  const double xmax = m.disk_rmax / h;
  const double dnorm = disk_fraction(xmax);
  const double sigma0 = disk ? m.disk_mass / (2 * M_PI * h * h * dnorm) : 0.0;
  auto surface = [&](double R) { return R > m.disk_rmax ? 0.0 : sigma0 * std::exp(-R / h); };
  auto disk_within = [&](double r) {
    return disk ? m.disk_mass * disk_fraction(std::min(r, m.disk_rmax) / h) / dnorm : 0.0;
  };

  // ---- positions: halo, disk, bulge, in the reference's draw order --------
  std::size_t k = 0;
  auto put = [&](double x, double y, double z, double mk, int32_t t) {
    pos[3 * k] = x;
    pos[3 * k + 1] = y;
    pos[3 * k + 2] = z;
    mass[k] = mk;
    type[k] = t;
    ++k;
  };
  // A spheroid body: the direction is drawn before the radius, the order
  // in which g++ evaluates `radius(u_open()) * random_direction(rng)`.
  auto spheroid_body = [&](const Spheroid &p, double mk, int32_t t) {
    const Dir d = isotropic(rng);
    const double r = p.radius_of(open01());
    put(r * d.x, r * d.y, r * d.z, mk, t);
  };
  if (halo)
    for (uint64_t i = 0; i < m.halo_n; ++i) spheroid_body(halo_p, m.halo_mass / m.halo_n, 1);
  if (disk)
    for (uint64_t i = 0; i < m.disk_n; ++i) {
      const double target = open01() * dnorm;
      double lo = 0.0, hi = xmax;
      for (int it = 0; it < 60; ++it) {
        const double mid = 0.5 * (lo + hi);
        (disk_fraction(mid) < target ? lo : hi) = mid;
      }
      const double R = 0.5 * (lo + hi) * h;
      const double phi = 2 * M_PI * uni(rng);
      const double z = m.disk_z0 * std::atanh(2 * open01() - 1);
      put(R * std::cos(phi), R * std::sin(phi), z, m.disk_mass / m.disk_n, 2);
    }
  if (bulge)
    for (uint64_t i = 0; i < m.bulge_n; ++i) spheroid_body(bulge_p, m.bulge_mass / m.bulge_n, 3);
  const std::size_t n = k;

  // ---- analytic forces for the moment equations ---------------------------
  const double rlo = 1e-4 * std::min({gamma > 0 ? gamma : rc, a, h});
  const double rhi = std::max({m.halo_rmax, m.bulge_rmax, m.disk_rmax});
  const std::vector<double> rg = log_spaced(rlo, rhi, 2000);
  const std::size_t ng = rg.size();
  std::vector<double> gr(ng), phi(ng), s2_halo(ng, 0.0), s2_bulge(ng, 0.0);
  auto menc = [&](double r) {
    return halo_p.enclosed(r) + bulge_p.enclosed(r) + disk_within(r);
  };
  for (std::size_t i = 0; i < ng; ++i) gr[i] = m.G * menc(rg[i]) / (rg[i] * rg[i]);
  const double mtot = menc(rhi);
  phi[ng - 1] = -m.G * mtot / rhi;
  for (std::size_t i = ng - 1; i-- > 0;)
    phi[i] = phi[i + 1] - 0.5 * (gr[i] + gr[i + 1]) * (rg[i + 1] - rg[i]);
  auto potential = [&](double r) {
    if (r >= rhi) return -m.G * mtot / r;
    return lookup(rg, phi, std::max(r, rlo));
  };
  auto jeans = [&](const Spheroid &c, std::vector<double> &s2) {  // hernquist_ics.cpp:250-262
    double integral = 0.0;
    for (std::size_t i = ng - 1; i-- > 0;) {
      integral += 0.5 * (c.density(rg[i]) * gr[i] + c.density(rg[i + 1]) * gr[i + 1]) *
                  (rg[i + 1] - rg[i]);
      const double rho = c.density(rg[i]);
      s2[i] = rho > 0 ? integral / rho : 0.0;
    }
  };
  if (halo) jeans(halo_p, s2_halo);
  if (bulge) jeans(bulge_p, s2_bulge);
  auto spheroid_velocity = [&](std::size_t i, const std::vector<double> &s2) {
    const double r = std::sqrt(pos[3 * i] * pos[3 * i] + pos[3 * i + 1] * pos[3 * i + 1] +
                               pos[3 * i + 2] * pos[3 * i + 2]);
    const double sigma = std::sqrt(std::max(0.0, lookup(rg, s2, std::max(r, rlo))));
    const double vmax = m.vesc_fraction * std::sqrt(std::max(0.0, -2.0 * potential(r)));
    double v[3];
    for (int tries = 0;; ++tries) {
      for (double &c : v) c = sigma * gauss(rng);
      const double s = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      if (s <= vmax) break;
      if (tries > 1000) {
        for (double &c : v) c *= vmax / s;
        break;
      }
    }
    for (int c = 0; c < 3; ++c) vel[3 * i + c] = v[c];
  };

  // disk: rotation curve, epicyclic frequency (hernquist_ics.cpp:265-345)
  const std::size_t nR = 200;
  std::vector<double> Rg(nR), F(nR), om2(nR), kap2(nR);
  const double dR = m.disk_rmax / double(nR);
  for (std::size_t i = 0; i < nR; ++i) {
    Rg[i] = (double(i) + 1.0) * dR;
    F[i] = m.G * menc(Rg[i]) / (Rg[i] * Rg[i]);
  }
  for (std::size_t i = 0; i < nR; ++i) {
    double dF;
    if (i == 0) dF = (F[1] - F[0]) / dR;
    else if (i == nR - 1) dF = (F[i] - F[i - 1]) / dR;
    else dF = (F[i + 1] - F[i - 1]) / (2 * dR);
    om2[i] = std::max(F[i] / Rg[i], 1e-30);
    kap2[i] = std::clamp(dF + 3 * F[i] / Rg[i], om2[i], 4 * om2[i]);
  }
  const double kQ = std::sqrt(lookup(Rg, kap2, m.disk_Q_radius));
  const double sRQ = m.disk_Q * 3.36 * m.G * surface(m.disk_Q_radius) / kQ;

  for (std::size_t i = 0; i < n; ++i) {
    if (type[i] == 1) {
      spheroid_velocity(i, s2_halo);
    } else if (type[i] == 3) {
      spheroid_velocity(i, s2_bulge);
    } else {
      const double x = pos[3 * i], y = pos[3 * i + 1];
      const double R = std::hypot(x, y);
      const double o2 = lookup(Rg, om2, R), k2 = lookup(Rg, kap2, R);
      const double vc2 = o2 * R * R;
      const double sZ2 = M_PI * m.G * surface(R) * m.disk_z0;
      const double sR2 = sRQ * sRQ * std::exp(-(R - m.disk_Q_radius) / h);
      const double ratio = k2 / (4 * o2);
      const double sP2 = sR2 * ratio;
      const double vbar2 = std::max(0.0, vc2 + sR2 * (1 - ratio - 2 * R / h));
      const double vR = std::sqrt(sR2) * gauss(rng);
      const double vphi = std::sqrt(vbar2) + std::sqrt(sP2) * gauss(rng);
      const double vz = std::sqrt(sZ2) * gauss(rng);
      const double c = R > 0 ? x / R : 1.0, s = R > 0 ? y / R : 0.0;
      vel[3 * i] = vR * c - vphi * s;
      vel[3 * i + 1] = vR * s + vphi * c;
      vel[3 * i + 2] = vz;
    }
  }

  // ---- centre-of-mass frame (hernquist_ics.cpp:381-388) -------------------
  double mt = 0.0, cm[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
  for (std::size_t i = 0; i < n; ++i) {
    mt += mass[i];
    for (int c = 0; c < 3; ++c) {
      cm[c] += mass[i] * pos[3 * i + c];
      cv[c] += mass[i] * vel[3 * i + c];
    }
  }
  double dx[3], dv[3];
  for (int c = 0; c < 3; ++c) {
    dx[c] = -cm[c] / mt;
    dv[c] = -cv[c] / mt;
  }
  for (std::size_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      pos[3 * i + c] += dx[c];
      vel[3 * i + c] += dv[c];
    }
  return 0;
}

void gtc_orient(double *pos, double *vel, uint64_t n, double incl_deg, double omega_deg) {
  const double i = incl_deg * M_PI / 180.0, w = omega_deg * M_PI / 180.0;
  const double ci = std::cos(i), si = std::sin(i), cw = std::cos(w), sw = std::sin(w);
  auto rot = [&](double *v) {
    // about x, then about z
    const double ax = v[0], ay = ci * v[1] - si * v[2], az = si * v[1] + ci * v[2];
    v[0] = cw * ax - sw * ay;
    v[1] = sw * ax + cw * ay;
    v[2] = az;
  };
  for (uint64_t k = 0; k < n; ++k) {
    rot(pos + 3 * k);
    rot(vel + 3 * k);
  }
}

int gtc_parabolic_orbit(double G, double m1, double m2, double rp, double r0, double dx[3],
                        double dv[3]) {
  if (!(r0 >= rp) || !(rp > 0)) return 1;
  const double M = m1 + m2;
  // true anomaly at r0 on the approaching branch: r = 2 rp / (1 + cos f)
  const double f = -std::acos(std::clamp(2 * rp / r0 - 1, -1.0, 1.0));
  const double hmom = std::sqrt(2 * G * M * rp);
  const double vr = G * M / hmom * std::sin(f), vt = hmom / r0;
  const double rh[3] = {std::cos(f), std::sin(f), 0.0}, fh[3] = {-std::sin(f), std::cos(f), 0.0};
  for (int a = 0; a < 3; ++a) {
    dx[a] = r0 * rh[a];
    dv[a] = vr * rh[a] + vt * fh[a];
  }
  return 0;
}

int gtc_make_encounter(const gtc_galaxy_model *m, double incl1, double omega1, double incl2,
                       double omega2, double rp, double r0, double *pos, double *vel,
                       double *mass, int32_t *type) {
  const uint64_t n = m->disk_n + m->bulge_n + m->halo_n;
  gtc_galaxy_model m2 = *m;
  m2.seed = m->seed + 1;
  if (gtc_make_galaxy(m, pos, vel, mass, type)) return 1;
  if (gtc_make_galaxy(&m2, pos + 3 * n, vel + 3 * n, mass + n, type + n)) return 1;
  gtc_orient(pos, vel, n, incl1, omega1);
  gtc_orient(pos + 3 * n, vel + 3 * n, n, incl2, omega2);
  double m1 = 0, mm2 = 0;
  for (uint64_t k = 0; k < n; ++k) {
    m1 += mass[k];
    mm2 += mass[n + k];
  }
  double dx[3], dv[3];
  if (gtc_parabolic_orbit(m->G, m1, mm2, rp, r0, dx, dv)) return 1;
  // centre of mass at rest at the origin
  const double f1 = -mm2 / (m1 + mm2), f2 = m1 / (m1 + mm2);
  for (uint64_t k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) {
      pos[3 * k + a] += f1 * dx[a];
      vel[3 * k + a] += f1 * dv[a];
      pos[3 * (n + k) + a] += f2 * dx[a];
      vel[3 * (n + k) + a] += f2 * dv[a];
    }
  return 0;
}

void gtc_sample_indices(uint64_t n, uint64_t m, uint64_t seed, uint64_t *out) {
  std::mt19937_64 rng(seed);
  std::vector<std::size_t> s(n);
  std::iota(s.begin(), s.end(), std::size_t{0});
  std::shuffle(s.begin(), s.end(), rng);
  for (uint64_t k = 0; k < m && k < n; ++k) out[k] = s[k];
}

}  // extern "C"
