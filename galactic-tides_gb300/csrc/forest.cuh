// A batched ensemble advanced as one forest (forest.cu).
#pragma once

#include <string>
#include <vector>

#include "pipeline.cuh"

namespace gtc {

// One system of the ensemble: caller device arrays (pos, vel, acc: n x 3;
// mass, pot: n) and its solver parameters.
struct ForestSystem {
  double *pos = nullptr, *vel = nullptr, *acc = nullptr, *pot = nullptr;
  const double *mass = nullptr;
  u64 n = 0;
  SolverParams sp{};
};

struct ForestSystemPtrs {
  double *pos, *vel, *acc, *pot;
  const double *mass;
};

struct ForestSystemStats {
  unsigned long long cell_interactions, body_interactions, groups, max_list;
};

struct ForestRun {
  Workspace ws;                 // the forest's tree, groups and lists (ws.forest set)
  std::vector<ForestSystem> sys;
  SolverParams sp{};            // the shared parameters (group size and packing per system)
  u64 n = 0;                    // bodies in all
  DeviceBuffer tables, sysid, roots, root_node, group_root, apos, amass, stats, counter,
      split_flags, sys_groups, sys_max, slot_plan, graph_slots;
  u32 *host_lists = nullptr;    // pinned: per-system group counts, then list maxima
  u32 host_systems = 0;         // systems host_lists holds
  // Memory for the systems' split tables: each gets levels 0..T-1 (3 x 2^T
  // doubles), T the most levels (up to the 21 of one key word) within it.
  static constexpr u64 kSplitBudget = 256ull << 20;
  const ForestSystemPtrs *ptrs_dev = nullptr;
  Scalars *host_sc = nullptr;   // pinned

  ForestRun() = default;
  ForestRun(const ForestRun &) = delete;
  ForestRun &operator=(const ForestRun &) = delete;
  ~ForestRun();

  // Systems can share a forest when their G, theta, eps, quadrupole flag,
  // leaf size and criterion agree (group size and packing may differ).
  static bool eligible(const std::vector<ForestSystem> &systems, std::string *why);
  // The arena and per-system tables for these systems; gathers their
  // positions and masses.
  void setup(const std::vector<ForestSystem> &systems, cudaStream_t s);
  // One force evaluation of every system into its acc and pot (with kick:
  // then v += h a); without write, the systems' arrays are left as they are
  // (a solve that only sizes the buffers).
  void solve(int kick, double h, cudaStream_t s, bool write = true);
  // One leapfrog step of every system (integrator.cpp:5-17).
  void step(double dt, cudaStream_t s);
  void kick_drift(double h, double dt, cudaStream_t s);
  // The systems' positions and masses into the arena again.
  void gather(cudaStream_t s);
  void scatter(int kick, double h, const u32 *abort, cudaStream_t s);
  // Per-system interaction counts of the current lists.
  std::vector<ForestSystemStats> system_stats(cudaStream_t s);
  // Per-system list slots for a captured step (caps: the uniform capacities
  // from the last eager solve; headroom as there), sized from each system's
  // group count and longest lists of that solve; sets caps.sys_slots and the
  // pools and sizes the list arrays. False (caps unchanged) when even
  // these do not fit 32-bit list offsets.
  bool size_graph_slots(GraphCaps &caps, double headroom, cudaStream_t s);
};

}  // namespace gtc
