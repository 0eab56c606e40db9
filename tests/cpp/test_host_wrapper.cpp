// The C++ wrapper (gtc.hpp) used the way the reference's code uses its
// solvers: a Particles-like container, compute(), stats, and the exception
// types for refused calls. Forces are checked against the oracle's CPU group
// solver on the same particles (median relative difference < 1e-5, as the
// reference's GPU-vs-CPU test, tests/test_metal.cpp:315-316).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <iostream>
#include <random>
#include <stdexcept>
#include <vector>

#include "gtc.hpp"

extern "C" int orc_group_force(const double *pos, const double *mass, uint64_t n, double G,
                               double theta, double eps, int quad, int group_size, int leaf_size,
                               int pack, int repeat, uint64_t parallel_threshold, double *acc,
                               double *pot, void *timings);

static int failures = 0;
#define CHECK(cond)                                                               \
  do {                                                                            \
    if (!(cond)) {                                                                \
      std::cerr << __FILE__ << ":" << __LINE__ << ": CHECK failed: " #cond "\n"; \
      ++failures;                                                                 \
    }                                                                             \
  } while (0)

struct Vec3 {
  double x = 0, y = 0, z = 0;
};
struct Particles {  // the layout of galactic_tides::Particles for these fields
  std::vector<Vec3> pos, acc;
  std::vector<double> mass, pot;
  std::size_t size() const { return pos.size(); }
};

static Particles lopsided(std::size_t n, unsigned seed) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  Particles p;
  for (std::size_t i = 0; i < n; ++i) {
    Vec3 c;
    double a = 1.0;
    if (i % 10 == 0) {
      c = (i % 20 == 0) ? Vec3{4, 0, 0} : Vec3{-1, 3, 2};
      a = 0.1;
    }
    const double x = std::sqrt(u(rng) * 0.95), r = a * x / (1 - x);
    const double cz = 2 * u(rng) - 1, ph = 2 * M_PI * u(rng), s = std::sqrt(1 - cz * cz);
    p.pos.push_back({c.x + r * s * std::cos(ph), c.y + r * s * std::sin(ph), c.z + r * cz});
    p.mass.push_back(1.0 / n);
  }
  return p;
}

int main() {
  Particles p = lopsided(4000, 42);
  const double G = 1.0, theta = 0.75, eps = 0.01;
  gtc::GroupGravity<Particles> grav(G, theta, eps, true);
  grav.compute(p);
  const gtc_stats st = grav.stats();
  CHECK(st.cell_interactions > 0 && st.body_interactions > 0 && st.n_groups > 0);

  std::vector<double> acc(3 * p.size()), pot(p.size());
  CHECK(orc_group_force(&p.pos[0].x, p.mass.data(), p.size(), G, theta, eps, 1, 32, 8, 1, 1,
                        ~0ull, acc.data(), pot.data(), nullptr) == 0);
  std::vector<double> err;
  for (std::size_t i = 0; i < p.size(); ++i) {
    const double dx = p.acc[i].x - acc[3 * i], dy = p.acc[i].y - acc[3 * i + 1],
                 dz = p.acc[i].z - acc[3 * i + 2];
    const double a = std::sqrt(acc[3 * i] * acc[3 * i] + acc[3 * i + 1] * acc[3 * i + 1] +
                               acc[3 * i + 2] * acc[3 * i + 2]);
    err.push_back(std::sqrt(dx * dx + dy * dy + dz * dz) / a);
  }
  std::sort(err.begin(), err.end());
  std::cout << "cuda group vs oracle: median " << err[err.size() / 2] << " max " << err.back()
            << "\n";
  CHECK(err[err.size() / 2] < 1e-5);
  CHECK(err.back() < 1e-3);

  // DirectGravity on the device against the group solver: same physics.
  Particles q = p;
  gtc::DirectGravity<Particles> direct(G, eps);
  direct.compute(q);
  CHECK(std::isfinite(q.acc[17].x) && q.acc[17].x != 0.0);

  // Refusals carry the reference's exception types.
  bool threw = false;
  try {
    gtc::GroupGravity<Particles> wide(G, theta, eps, true, 33);
  } catch (const std::invalid_argument &) {
    threw = true;
  }
  CHECK(threw);
  threw = false;
  try {
    gtc::Context bad(1 << 20);
  } catch (const std::invalid_argument &) {
    threw = true;
  } catch (const std::runtime_error &) {
    threw = true;
  }
  CHECK(threw);

  if (failures) {
    std::cerr << failures << " failure(s)\n";
    return 1;
  }
  std::cout << "all checks passed\n";
  return 0;
}
