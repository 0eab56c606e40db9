// C entry points over the reference implementation, for checking the oracle.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled together with the
// reference's own sources (src/octree.cpp, src/group_lists.cpp,
// src/gravity.cpp, src/gravity_backends.cpp, src/hernquist_ics.cpp, ...)
// by oracle/Makefile.ref into oracle/_ref/libgtref.so. It needs the
// reference tree on disk, so it is only built where the reference is
// present; nothing on the product path links it.
//
// Every function here calls the reference's public C++ API unchanged and
// copies the result into flat arrays that Python (ctypes) can read.

#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "galactic_tides/gravity.h"
#include "galactic_tides/gravity_backends.h"
#include "galactic_tides/group_lists.h"
#include "galactic_tides/hernquist_ics.h"
#include "galactic_tides/integrator.h"
#include "galactic_tides/octree.h"

using namespace galactic_tides;

namespace {

thread_local std::string g_error;

Particles make_particles(const double *pos, const double *mass, std::uint64_t n) {
  Particles p;
  p.resize(n);
  for (std::uint64_t i = 0; i < n; ++i) {
    p.pos[i] = Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    p.mass[i] = mass[i];
    p.id[i] = i;
    p.type[i] = ParticleType::Halo;
  }
  return p;
}

void copy_out(const Particles &p, double *acc, double *pot) {
  for (std::size_t i = 0; i < p.size(); ++i) {
    if (acc) {
      acc[3 * i] = p.acc[i].x;
      acc[3 * i + 1] = p.acc[i].y;
      acc[3 * i + 2] = p.acc[i].z;
    }
    if (pot) pot[i] = p.pot[i];
  }
}

GravityParams make_gp(double G, double theta, double eps, int quad) {
  GravityParams gp;
  gp.G = G;
  gp.theta = theta;
  gp.eps = eps;
  gp.quadrupole = quad != 0;
  return gp;
}

}  // namespace

extern "C" {

// Flat export of one Octree::Node (octree.h:52-63), field for field.
struct RefNode {
  double center[3];
  double half;
  double com[3];
  double mass;
  double quad[6];
  double delta;
  std::int32_t first_child, n_children;
  std::uint32_t begin, end;
};

struct RefModel {
  double G;
  std::uint64_t disk_n, bulge_n, halo_n;
  double disk_mass, disk_h, disk_z0, disk_rmax, disk_Q, disk_Q_radius;
  double bulge_mass, bulge_a, bulge_rmax;
  double halo_mass, halo_core, halo_cutoff, halo_rmax;
  double vesc_fraction;
  std::uint64_t seed;
  double eps, theta;
};

const char *ref_last_error() { return g_error.c_str(); }

// make_hernquist_galaxy (src/hernquist_ics.cpp:142) with the fields set directly.
int ref_galaxy(const RefModel *m, double *pos, double *vel, double *mass, int *type) {
  try {
    HernquistModel hm;
    hm.G = m->G;
    hm.disk_n = m->disk_n;
    hm.bulge_n = m->bulge_n;
    hm.halo_n = m->halo_n;
    hm.disk_mass = m->disk_mass;
    hm.disk_h = m->disk_h;
    hm.disk_z0 = m->disk_z0;
    hm.disk_rmax = m->disk_rmax;
    hm.disk_Q = m->disk_Q;
    hm.disk_Q_radius = m->disk_Q_radius;
    hm.bulge_mass = m->bulge_mass;
    hm.bulge_a = m->bulge_a;
    hm.bulge_rmax = m->bulge_rmax;
    hm.halo_mass = m->halo_mass;
    hm.halo_core = m->halo_core;
    hm.halo_cutoff = m->halo_cutoff;
    hm.halo_rmax = m->halo_rmax;
    hm.vesc_fraction = m->vesc_fraction;
    hm.seed = m->seed;
    hm.gravity.G = m->G;
    hm.gravity.eps = m->eps;
    hm.gravity.theta = m->theta;
    const Particles p = make_hernquist_galaxy(hm);
    for (std::size_t i = 0; i < p.size(); ++i) {
      for (int k = 0; k < 3; ++k) {
        pos[3 * i + k] = p.pos[i][k];
        vel[3 * i + k] = p.vel[i][k];
      }
      mass[i] = p.mass[i];
      type[i] = static_cast<int>(p.type[i]);
    }
    return 0;
  } catch (const std::exception &e) {
    g_error = e.what();
    return 1;
  }
}

// Octree::build (src/octree.cpp:169) -> opaque handle.
void *ref_tree_build(const double *pos, const double *mass, std::uint64_t n, int leaf_size,
                     std::uint64_t parallel_threshold) {
  try {
    auto *t = new Octree;
    std::vector<Vec3> p(n);
    std::vector<double> m(mass, mass + n);
    for (std::uint64_t i = 0; i < n; ++i) p[i] = Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    t->set_parallel_threshold(parallel_threshold);
    t->build(p, m, leaf_size);
    return t;
  } catch (const std::exception &e) {
    g_error = e.what();
    return nullptr;
  }
}

void ref_tree_free(void *h) { delete static_cast<Octree *>(h); }
std::uint64_t ref_tree_nnodes(void *h) { return static_cast<Octree *>(h)->nodes().size(); }
int ref_tree_depth(void *h) { return static_cast<Octree *>(h)->depth(); }

void ref_tree_export(void *h, RefNode *out, std::uint64_t *order) {
  const Octree &t = *static_cast<Octree *>(h);
  const auto &nodes = t.nodes();
  for (std::size_t k = 0; k < nodes.size(); ++k) {
    const auto &nd = nodes[k];
    RefNode &o = out[k];
    for (int a = 0; a < 3; ++a) {
      o.center[a] = nd.center[a];
      o.com[a] = nd.com[a];
    }
    o.half = nd.half;
    o.mass = nd.mass;
    for (int q = 0; q < 6; ++q) o.quad[q] = nd.quad[q];
    o.delta = nd.delta;
    o.first_child = nd.first_child;
    o.n_children = nd.n_children;
    o.begin = nd.begin;
    o.end = nd.end;
  }
  for (std::size_t k = 0; k < t.order().size(); ++k) order[k] = t.order()[k];
}

// Octree::accel_pot (src/octree.cpp:275) at an arbitrary point.
void ref_tree_accel_pot(void *h, const double *x, std::uint64_t self, double G, double theta,
                        double eps, int quad, double *acc, double *pot) {
  const Octree &t = *static_cast<Octree *>(h);
  Vec3 a;
  t.accel_pot(Vec3(x[0], x[1], x[2]), self == ~0ull ? Octree::kNoSelf : self,
              make_gp(G, theta, eps, quad), a, *pot);
  acc[0] = a.x;
  acc[1] = a.y;
  acc[2] = a.z;
}

struct RefListStats {
  std::uint64_t n_groups, n_cell_list, n_body_list;
  std::uint64_t cell_interactions, body_interactions, max_list;
  std::int64_t max_group;
  double origin[3];
};

// build_group_lists (src/group_lists.cpp:18) -> opaque handle.
void *ref_lists_build(void *tree, double G, double theta, double eps, int quad, int group_size,
                      int pack) {
  try {
    auto *L = new GroupLists;
    build_group_lists(*static_cast<Octree *>(tree), make_gp(G, theta, eps, quad), group_size, *L,
                      pack != 0);
    return L;
  } catch (const std::exception &e) {
    g_error = e.what();
    return nullptr;
  }
}

void ref_lists_free(void *h) { delete static_cast<GroupLists *>(h); }

void ref_lists_stats(void *h, RefListStats *s) {
  const GroupLists &L = *static_cast<GroupLists *>(h);
  s->n_groups = L.groups.size();
  s->n_cell_list = L.cell_list.size();
  s->n_body_list = L.body_list.size();
  s->cell_interactions = L.cell_interactions;
  s->body_interactions = L.body_interactions;
  s->max_list = L.max_list;
  s->max_group = L.max_group;
  for (int a = 0; a < 3; ++a) s->origin[a] = L.origin[a];
}

// bodies (n float4), cells (n_nodes x 12 floats), lists and groups (8 uint32 each).
void ref_lists_export(void *h, float *bodies, float *cells, std::uint32_t *cell_list,
                      std::uint32_t *body_list, std::uint32_t *groups) {
  const GroupLists &L = *static_cast<GroupLists *>(h);
  if (bodies) std::memcpy(bodies, L.bodies.data(), L.bodies.size() * sizeof(kern::float4));
  if (cells) std::memcpy(cells, L.cells.data(), L.cells.size() * sizeof(kern::GTCell));
  if (cell_list) std::memcpy(cell_list, L.cell_list.data(), L.cell_list.size() * 4);
  if (body_list) std::memcpy(body_list, L.body_list.data(), L.body_list.size() * 4);
  if (groups) std::memcpy(groups, L.groups.data(), L.groups.size() * sizeof(kern::GTGroup));
}

// evaluate_group_lists_cpu (src/gravity_backends.cpp:70) on a lists handle.
void ref_lists_eval(void *h, double G, double eps, int quad, float *out) {
  const GroupLists &L = *static_cast<GroupLists *>(h);
  GravityParams gp = make_gp(G, 0.5, eps, quad);
  kern::GTParams kp = make_kernel_params(gp, L.bodies.size());
  kp.n_groups = static_cast<kern::uint>(L.groups.size());
  gpu_vector<kern::float4> o;
  evaluate_group_lists_cpu(L, kp, o);
  std::memcpy(out, o.data(), o.size() * sizeof(kern::float4));
}

struct RefTimings {
  double tree, lists, evaluate;
  std::uint64_t cell_interactions, particle_interactions;
};

// GroupTreeGravity (Device::CPU) compute (src/gravity_backends.cpp:109), original order out.
int ref_group_force(const double *pos, const double *mass, std::uint64_t n, double G,
                    double theta, double eps, int quad, int group_size, int leaf_size, int pack,
                    int repeat, double *acc, double *pot, RefTimings *tm) {
  try {
    Particles p = make_particles(pos, mass, n);
    GroupTreeGravity g(make_gp(G, theta, eps, quad), Device::CPU, group_size, leaf_size, pack);
    for (int r = 0; r < (repeat < 1 ? 1 : repeat); ++r) g.compute(p);
    copy_out(p, acc, pot);
    if (tm) {
      tm->tree = g.timings().tree;
      tm->lists = g.timings().lists;
      tm->evaluate = g.timings().evaluate;
      tm->cell_interactions = g.stats().cell_interactions;
      tm->particle_interactions = g.stats().particle_interactions;
    }
    return 0;
  } catch (const std::exception &e) {
    g_error = e.what();
    return 1;
  }
}

// compute_gravity_tree (src/gravity.cpp:7).
int ref_tree_force(const double *pos, const double *mass, std::uint64_t n, double G, double theta,
                   double eps, int quad, int leaf_size, double *acc, double *pot,
                   std::uint64_t *stats) {
  try {
    Particles p = make_particles(pos, mass, n);
    Octree tree;
    const WalkStats s = compute_gravity_tree(p, make_gp(G, theta, eps, quad), tree, leaf_size);
    copy_out(p, acc, pot);
    if (stats) {
      stats[0] = s.cell_interactions;
      stats[1] = s.particle_interactions;
    }
    return 0;
  } catch (const std::exception &e) {
    g_error = e.what();
    return 1;
  }
}

// compute_gravity_direct (src/gravity.cpp:28), FP64.
void ref_direct_fp64(const double *pos, const double *mass, std::uint64_t n, double G, double eps,
                     double *acc, double *pot) {
  Particles p = make_particles(pos, mass, n);
  compute_gravity_direct(p, make_gp(G, 0.5, eps, 1));
  copy_out(p, acc, pot);
}

// pack_bodies + gt_direct_accel (gravity_backends.cpp:15; gravity_kernels.h:173), FP32.
void ref_direct_fp32(const double *pos, const double *mass, std::uint64_t n, const double *origin,
                     double G, double eps, float *bodies_out, float *out) {
  std::vector<Vec3> p(n);
  std::vector<double> m(mass, mass + n);
  for (std::uint64_t i = 0; i < n; ++i) p[i] = Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
  gpu_vector<kern::float4> bodies;
  pack_bodies(p, m, Vec3(origin[0], origin[1], origin[2]), bodies);
  const kern::GTParams kp = make_kernel_params(make_gp(G, 0.5, eps, 1), n);
  for (kern::uint i = 0; i < n; ++i) {
    const kern::GTAcc a = kern::gt_direct_accel(i, bodies.data(), kp);
    out[4 * i] = a.ax;
    out[4 * i + 1] = a.ay;
    out[4 * i + 2] = a.az;
    out[4 * i + 3] = a.pot;
  }
  if (bodies_out) std::memcpy(bodies_out, bodies.data(), n * sizeof(kern::float4));
}

// LeapfrogKDK (src/integrator.cpp:5) with a CPU group solver, `steps` steps of dt.
int ref_leapfrog_group(double *pos, double *vel, const double *mass, std::uint64_t n, double G,
                       double theta, double eps, int group_size, int leaf_size, int pack,
                       double dt, int steps, double *energy) {
  try {
    Particles p = make_particles(pos, mass, n);
    for (std::uint64_t i = 0; i < n; ++i) p.vel[i] = Vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    GroupTreeGravity g(make_gp(G, theta, eps, 1), Device::CPU, group_size, leaf_size, pack);
    LeapfrogKDK lf(g);
    lf.prime(p);
    energy[0] = compute_diagnostics(p, 0.0).total();
    for (int s = 0; s < steps; ++s) lf.step(p, dt);
    energy[1] = compute_diagnostics(p, dt * steps).total();
    for (std::uint64_t i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) {
        pos[3 * i + k] = p.pos[i][k];
        vel[3 * i + k] = p.vel[i][k];
      }
    return 0;
  } catch (const std::exception &e) {
    g_error = e.what();
    return 1;
  }
}

}  // extern "C"
