// gravity_backends_cuda.cpp -- the `device = cuda` solvers of galactic-tides,
// built on libgtc.so (include/gtc.h) through galactic-tides_gb300/host/gtc.hpp.
#include <memory>
#include <stdexcept>
#include <string>

#include "galactic_tides/integrator.h"
#include "galactic_tides/params.h"
#include "gtc.hpp"

namespace galactic_tides {

// gravity = group, device = cuda: tree, lists and evaluation on the GPU.
class CudaGroupGravity : public ForceModel {
 public:
  CudaGroupGravity(const GravityParams &gp, int group_size, int leaf_size)
      : grav_(gp.G, gp.theta, gp.eps, gp.quadrupole, group_size, leaf_size) {}
  void compute(Particles &p) override { grav_.compute(p); }
  WalkStats stats() const override {
    const gtc_stats s = grav_.stats();
    WalkStats w;
    w.cell_interactions = s.cell_interactions;
    w.particle_interactions = s.body_interactions;
    return w;
  }

 private:
  gtc::GroupGravity<Particles> grav_;
};

// gravity = direct, device = cuda: the FP32 tiled kernel.
class CudaDirectGravity : public ForceModel {
 public:
  explicit CudaDirectGravity(const GravityParams &gp) : grav_(gp.G, gp.eps) {}
  void compute(Particles &p) override {
    grav_.compute(p);
    const std::size_t n = p.size();
    stats_.particle_interactions = n > 0 ? n * (n - 1) : 0;
  }
  WalkStats stats() const override { return stats_; }

 private:
  gtc::DirectGravity<Particles> grav_;
  WalkStats stats_;
};

// gravity = tree, device = cuda: every body's own walk, FP64, the reference's
// forces bit for bit.
class CudaTreeGravity : public ForceModel {
 public:
  CudaTreeGravity(const GravityParams &gp, int leaf_size)
      : grav_(gp.G, gp.theta, gp.eps, gp.quadrupole, leaf_size) {}
  void compute(Particles &p) override { grav_.compute(p); }
  WalkStats stats() const override {
    const gtc_stats s = grav_.stats();
    WalkStats w;
    w.cell_interactions = s.cell_interactions;
    w.particle_interactions = s.body_interactions;
    return w;
  }

 private:
  gtc::TreeGravity<Particles> grav_;
};

// Called from make_gravity when device == "cuda".
std::unique_ptr<ForceModel> make_cuda_gravity(const Params &params, const GravityParams &gp,
                                              std::string *summary) {
  const std::string kind = params.get_string("gravity", "tree");
  if (kind == "group") {
    const int group = static_cast<int>(params.get_int("group_size", 32));
    const int leaf = static_cast<int>(params.get_int("leaf_size", 8));
    if (summary)
      *summary = "tree with grouped walk (groups of up to " + std::to_string(group) +
                 ", packed), built and evaluated on cuda";
    return std::make_unique<CudaGroupGravity>(gp, group, leaf);
  }
  if (kind == "direct") {
    if (summary) *summary = "direct summation, single precision, on cuda";
    return std::make_unique<CudaDirectGravity>(gp);
  }
  if (kind == "tree") {
    const int leaf = static_cast<int>(params.get_int("leaf_size", 8));
    if (summary) *summary = "tree (per-particle walk, double precision), built and walked on cuda";
    return std::make_unique<CudaTreeGravity>(gp, leaf);
  }
  throw std::runtime_error("gravity = " + kind + " has no cuda backend");
}

}  // namespace galactic_tides
