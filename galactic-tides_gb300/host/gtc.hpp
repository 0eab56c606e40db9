// C++ face of the GB300 gravity backend: RAII over the C ABI (include/gtc.h)
// with the reference's exception types, and the two solvers with the shape of
// the reference's GroupTreeGravity / DirectGravity (gravity_backends.h:33-81)
// for `device = cuda`.
//
// The solvers are templates over the particle container so this header does
// not depend on the reference's headers: any type with `pos` (a contiguous
// array of {double x, y, z}), `mass`, `acc` (like pos) and `pot` vectors and a
// size() works, which is galactic_tides::Particles (particles.h:30-45).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gtc.h"

namespace gtc {

// gtc_status -> the exception the reference throws for the same condition:
// std::invalid_argument for bad arguments (gravity_backends.cpp:93-96,
// metal_backend.mm:218-223), std::runtime_error for everything else
// (metal_backend.mm:159,206,260; metal_stub.cpp:15-19; group_lists.cpp:25-26).
inline void check(gtc_status s, const gtc_context *ctx) {
  if (s == GTC_OK) return;
  const std::string msg = gtc_last_error(ctx);
  if (s == GTC_INVALID_ARGUMENT) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

// The device context (metal::Context, metal_backend.h:25-54): owns a CUDA
// stream and the device buffers reused from call to call. Not copyable.
class Context {
 public:
  explicit Context(int device = 0) {
    gtc_context *c = nullptr;
    check(gtc_create(&c, device), nullptr);
    ctx_ = c;
  }
  ~Context() { gtc_destroy(ctx_); }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;

  // out[i] = (ax, ay, az, pot) for every body against every other.
  void direct(const std::vector<gtc_float4> &bodies, const gtc_kernel_params &p,
              std::vector<gtc_float4> &out) {
    out.resize(bodies.size());
    gtc_kernel_params q = p;
    q.n = static_cast<uint32_t>(bodies.size());
    check(gtc_direct(ctx_, bodies.data(), &q, out.data()), ctx_);
  }

  // Evaluates grouped lists: out[i] for every body i in tree order.
  void tree(const std::vector<gtc_float4> &bodies, const std::vector<gtc_cell> &cells,
            const std::vector<uint32_t> &cell_list, const std::vector<uint32_t> &body_list,
            const std::vector<gtc_group> &groups, const gtc_kernel_params &p,
            std::vector<gtc_float4> &out) {
    out.resize(bodies.size());
    check(gtc_tree(ctx_, bodies.data(), cells.data(), static_cast<uint32_t>(cells.size()),
                   cell_list.data(), cell_list.size(), body_list.data(), body_list.size(),
                   groups.data(), &p, out.data()),
          ctx_);
  }

  void group_force(const double *pos, const double *mass, uint64_t n,
                   const gtc_gravity_params &gp, double *acc, double *pot) {
    check(gtc_group_force(ctx_, pos, mass, n, &gp, acc, pot), ctx_);
  }
  void direct_force(const double *pos, const double *mass, uint64_t n,
                    const gtc_gravity_params &gp, double *acc, double *pot) {
    check(gtc_direct_force(ctx_, pos, mass, n, &gp, acc, pot), ctx_);
  }
  void tree_force(const double *pos, const double *mass, uint64_t n,
                  const gtc_gravity_params &gp, double *acc, double *pot) {
    check(gtc_tree_force(ctx_, pos, mass, n, &gp, acc, pot), ctx_);
  }

  gtc_stats stats() const {
    gtc_stats s{};
    check(gtc_get_stats(ctx_, &s), ctx_);
    return s;
  }
  // A tuning option by name (gtc_set_option; the names are listed in gtc.h).
  void set_option(const char *name, double value) {
    check(gtc_set_option(ctx_, name, value), ctx_);
  }
  gtc_context *handle() { return ctx_; }

 private:
  gtc_context *ctx_ = nullptr;
};

// Gravity parameters in the reference's terms (GravityParams, octree.h:13-18,
// plus the make_gravity keys, gravity_backends.cpp:154-160).
inline gtc_gravity_params gravity_params(double G, double theta, double eps, bool quadrupole,
                                         int group_size = 32, int leaf_size = 8,
                                         bool pack = true) {
  gtc_gravity_params p{};
  p.G = G;
  p.theta = theta;
  p.eps = eps;
  p.quadrupole = quadrupole ? 1 : 0;
  p.group_size = group_size;
  p.leaf_size = leaf_size;
  p.pack = pack ? 1 : 0;
  p.criterion = GTC_CRITERION_THETA;
  return p;
}

// GroupTreeGravity with Device::CUDA: tree, lists and evaluation all on the
// device; results land in the caller's order as in gravity_backends.cpp:132-136.
// group_size at most 32 (as on Metal, gravity_backends.cpp:94-96); packing on.
template <class Particles>
class GroupGravity {
 public:
  GroupGravity(double G, double theta, double eps, bool quadrupole, int group_size = 32,
               int leaf_size = 8, int device = 0)
      : ctx_(device), gp_(gravity_params(G, theta, eps, quadrupole, group_size, leaf_size)) {
    if (group_size < 1) throw std::invalid_argument("group_size must be at least 1");
    if (group_size > 32) throw std::invalid_argument("group_size can be at most 32 on cuda");
  }
  void compute(Particles &p) {
    const std::size_t n = p.size();
    p.acc.resize(n);
    p.pot.resize(n);
    static_assert(sizeof(p.pos[0]) == 3 * sizeof(double), "pos must hold 3 doubles per body");
    ctx_.group_force(n ? &p.pos[0].x : nullptr, p.mass.data(), n, gp_,
                     n ? &p.acc[0].x : nullptr, p.pot.data());
  }
  const gtc_stats stats() const { return ctx_.stats(); }
  Context &context() { return ctx_; }

 private:
  Context ctx_;
  gtc_gravity_params gp_;
};

// DirectGravity with Device::CUDA: the FP32 tiled kernel on bodies packed
// relative to the bounding-box centre (gravity_backends.cpp:53-68).
template <class Particles>
class DirectGravity {
 public:
  DirectGravity(double G, double eps, int device = 0)
      : ctx_(device), gp_(gravity_params(G, 0.5, eps, false)) {}
  void compute(Particles &p) {
    const std::size_t n = p.size();
    p.acc.resize(n);
    p.pot.resize(n);
    ctx_.direct_force(n ? &p.pos[0].x : nullptr, p.mass.data(), n, gp_,
                      n ? &p.acc[0].x : nullptr, p.pot.data());
  }

 private:
  Context ctx_;
  gtc_gravity_params gp_;
};

// TreeGravity with the device (gravity = tree): the per-particle walk
// (Octree::accel_pot, octree.cpp:275-344) for every body, FP64, the
// reference's forces bit for bit.
template <class Particles>
class TreeGravity {
 public:
  TreeGravity(double G, double theta, double eps, bool quadrupole, int leaf_size = 8,
              int device = 0)
      : ctx_(device), gp_(gravity_params(G, theta, eps, quadrupole, 32, leaf_size)) {}
  void compute(Particles &p) {
    const std::size_t n = p.size();
    p.acc.resize(n);
    p.pot.resize(n);
    ctx_.tree_force(n ? &p.pos[0].x : nullptr, p.mass.data(), n, gp_,
                    n ? &p.acc[0].x : nullptr, p.pot.data());
  }
  const gtc_stats stats() const { return ctx_.stats(); }

 private:
  Context ctx_;
  gtc_gravity_params gp_;
};

}  // namespace gtc
