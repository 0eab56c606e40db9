// The context behind the C ABI's opaque gtc_context.
#pragma once

#include <string>

#include "../../include/gtc.h"
#include "learned.cuh"
#include "pipeline.cuh"

struct gtc_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[6] = {};
  std::string error;
  gtc_stats stats{};
  gtc::Workspace ws;
  gtc::Scalars *host_sc = nullptr;  // pinned
  gtc::DeviceBuffer counter;        // evaluator work queue
  gtc::DeviceBuffer sample_scratch; // FP64 sample partial sums
  bool have_group = false;
  gtc::SolverParams last{};
  // learned opening criterion
  gtc::LearnedSet samples;          // training set
  gtc::DeviceBuffer model;          // kModelFloats floats (FP32, device)
  gtc::DeviceBuffer net;            // LearnedNet: the model in tensor-core layout
  bool have_model = false;
  float model_band = 1e30f;         // the model's band (host copy)
  float model_ymean = 0.f;          // the model's y_mean (host copy)
  gtc::DeviceBuffer train_scratch;  // per-block partial gradients, Adam moments, losses
  gtc::DeviceBuffer cfeat, gtol;    // per-node features, per-group tolerances
  gtc::LearnedScratch lscratch;     // the learned walk's rounds
  gtc::DeviceBuffer prev_amag;      // |a| per body (caller order) of the last solve
  gtc::u64 prev_n = 0;              // bodies in prev_amag (0: none)
  // the learned walk's inputs (FP32 moment estimates, node features and
  // records) run on their own stream, beside the group choice on `stream`
  cudaStream_t lstream = nullptr;
  cudaEvent_t lfork = nullptr, ldone = nullptr;
  double guard_theta = 1.5;         // options of the learned walk
  double band_override = -1.0;      // < 0: the model's band
  gtc::u32 walk_budget = gtc::kLearnedWalkBudget;  // learned walk: nodes a thread tests before
  gtc::u32 pair_budget = gtc::kLearnedPairBudget;  // a warp takes over, round 0 / later (0: all)
  bool read_every_round = false;    // learned walk: no rounds walked before the first read back
  int learned_warps = -1;           // learned walk: rounds by warps (1), threads per part (0),
                                    // or warps below the walk's group threshold (-1)
  gtc::DeviceBuffer diag;           // diagnostics partial sums
  gtc::DeviceBuffer tree_counts;    // per-particle walk: cell and particle interactions
  double graph_headroom = 0.25;     // leapfrog graphs: buffer headroom over the last sizes
};

namespace gtc {
// Builds the tree and groups of (pos, mass) (device arrays) and appends up
// to max_new labelled (group, cell) pairs to the context's training set.
void learned_add_samples(gtc_context *ctx, const double *pos, const double *mass, u64 n,
                         const SolverParams &sp, double theta_gen, double theta_guard,
                         u64 max_new, u32 max_cell_bodies, u64 *added);
void learned_set_model(gtc_context *ctx, const float *host_model);
void learned_init_model(gtc_context *ctx, u64 seed);
double learned_train_on(gtc_context *ctx, const float *feat, const float *label, u64 nsamples,
                        u64 steps, u32 batch, float lr, u64 seed, const u32 *fixed,
                        float *grad_out);
void learned_update_band(gtc_context *ctx, double quantile);
}  // namespace gtc
