// The learned opening criterion: model layout, features and the walk that
// uses it.
//
// A small MLP (6 -> 64 -> 64 -> 1, ReLU) corrects a physical error model.
// For a candidate cell and a group of targets it predicts the force error
// the cell would contribute if accepted as a multipole,
//   e = log2( max over the group's targets |a_multipole - a_exact| / (G M_tot / L^2) )
// (L = root half-size, M_tot = total mass) as
//   e = prior + y_mean + y_std * net((f - mean) / std),
//   prior = log2(2 * 3^1.5) + f3 + 3 f1 - 5 f2,
// the prior being the size of the quadrupole expansion's leading error term,
// 2 G m (sqrt(3) h)^3 / d^5. It is trained on labels from FP64 direct sums.
// In the walk a cell is accepted when e is below the group's tolerance,
// log2(alpha a_g L^2 / (G M_tot)), a_g being the smallest |a| of the group's
// targets from the previous evaluation. A geometric test with a loose
// opening angle guards the model: cells that fail it are always opened.
#pragma once

#include "pipeline.cuh"

namespace gtc {

constexpr int kFeat = 6;
constexpr int kHid = 64;
// W1 [kFeat][kHid], b1 [kHid], W2 [kHid][kHid], b2 [kHid], W3 [kHid], b3
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kFeat * kHid, kOffW2 = kOffB1 + kHid,
              kOffB2 = kOffW2 + kHid * kHid, kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid;
constexpr int kParams = kOffB3 + 1;  // 4673
// after the parameters: feature mean[6], stdev[6], y_mean, y_std, band
constexpr int kOffMean = kParams, kOffStd = kOffMean + kFeat, kOffYMean = kOffStd + kFeat,
              kOffYStd = kOffYMean + 1, kOffBand = kOffYStd + 1;
constexpr int kModelFloats = kOffBand + 1;  // 4688
constexpr float kPriorBase = 3.3773f;       // log2(2 * 3^1.5)
// Node records one thread of the learned walk tests before the rest of its
// walk goes to a warp: in round 0, and in later rounds (where each deferred
// pair costs a few dependent loads more than a node).
constexpr u32 kLearnedWalkBudget = 576, kLearnedPairBudget = 48;

// Raw features of a (group, cell) pair, all from FP32 quantities so that
// training and inference see the same numbers:
//   f0 log2(group half-extent / L)   f1 log2(cell half-size / L)
//   f2 log2(distance box->com / L)   f3 log2(cell mass / M_total)
//   f4 log2(|Q| / (M L^2))           f5 com offset / cell half-size
struct FeatScale {
  float inv_l;      // 1 / L
  float inv_mtot;   // 1 / M_total
};

__device__ __forceinline__ float safe_log2(float v) { return __log2f(fmaxf(v, 1e-30f)); }

// Per-node inputs: the guard's geometry, the node's part of the prior and
// the cell-only features (the first 16 bytes settle most tests).
struct alignas(16) CellFeat {
  float half, delta, prior, f1;
  float f3, f4, f5, pad;
};

__device__ __forceinline__ CellFeat cell_features(float half, float mass, float qnorm,
                                                  float delta, const FeatScale &s) {
  CellFeat c;
  c.f1 = safe_log2(half * s.inv_l);
  c.f3 = safe_log2(mass * s.inv_mtot);
  c.f4 = safe_log2(qnorm / fmaxf(mass, 1e-30f) * s.inv_l * s.inv_l + 1e-12f);
  c.f5 = delta / fmaxf(half, 1e-30f);
  c.half = half;
  c.delta = delta;
  c.prior = kPriorBase + c.f3 + 3.f * c.f1;
  c.pad = 0.f;
  return c;
}
__device__ __forceinline__ float group_feature(float gh_max, const FeatScale &s) {
  return safe_log2(fmaxf(gh_max * s.inv_l, 1e-9f));
}
__device__ __forceinline__ float distance_feature(float d2, const FeatScale &s) {
  return safe_log2(fmaxf(sqrtf(d2) * s.inv_l, 1e-9f));
}
__device__ __forceinline__ float prior_log2err(float node_prior, float f2) {
  return node_prior - 5.f * f2;
}

// The learned walk's node record, 48 bytes (one record, one array per
// visited node): the overlap test's centre and slack and the centre of mass
// (the walk records' FP32 values), the guard's (2 h / theta_guard + delta)^2,
// the links and the node's part of the centred prior as a distance scale.
//
// The centred prior of a (group, cell) pair is
//   e = prior + y_mean - 5 f2,  f2 = log2(d / L),
// so the walk's tests e < tau - band (accept) and e > tau + band (open) are
// tests on d^2 alone:
//   accept  d^2 > pscale * 2^(0.4 (band - tau)) L^2,
//   open    d^2 < pscale * 2^(0.4 (-band - tau)) L^2,
// with pscale = 2^(0.4 (prior + y_mean)) per node and the rest per group:
// no square root or logarithm per visited node.
struct alignas(16) LWalkRec {
  float cx, cy, cz, slack;
  float mx, my, mz, guard2;
  u32 skip, nbody_leaf, begin;
  float pscale;
};
static_assert(sizeof(LWalkRec) == 48, "three float4 loads");

// Training set held by the context.
struct LearnedSet {
  DeviceBuffer feat;    // kFeat floats per sample
  DeviceBuffer label;   // 1 float per sample
  DeviceBuffer pair;    // (group, node) of each sample in the tree it came from
  u64 count = 0, capacity = 0;
};

// The model as the walk's warp-level BF16 tensor-core inference reads it:
// mma.sync m16n8k16 B fragments in lane order, so that each lane loads its
// fragment with one shared-memory access.
struct alignas(16) LearnedNet {
  u32 w1[8 * 32];         // layer 1: per n-tile and lane, (W1[2t][n], W1[2t+1][n]), bias in row 6
  uint2 w2[4 * 8 * 32];   // layer 2: per (k-step, n-tile, lane) the two B registers
  float b2[kHid], w3[kHid];
  float mean[kFeat], inv_std[kFeat];
  float b3, y_mean, y_std, band;
};

// Device memory of the learned walk, kept between calls.
struct LearnedScratch {
  DeviceBuffer lrec;                // per node: the walk's record (LWalkRec)
  DeviceBuffer pend, pcount, roff;  // per (part, group): the pairs a round deferred, how many,
                                    // the first of their rows
  DeviceBuffer q[2], dec[2];        // deferred (group, node) rows and the network's decisions
  DeviceBuffer cont;                // round-0 walks handed on to warps
  DeviceBuffer next;                // the warp rounds' group counter
  // FP32 estimates of the moments the walk decides from (cells in GTCell
  // layout, delta), and the root's mass as rootmom[1].y
  DeviceBuffer cells32, delta32, rootmom;
  // per-group slots of the three parts of round 0 (0: not sized yet) and
  // of deferred pairs
  u32 slot_cells[3] = {0, 0, 0}, slot_bodies[3] = {0, 0, 0}, slot_pend = 0;
  // rounds the last walk ran and the row capacity for its largest round:
  // the next walk runs that many rounds before it reads anything back (0:
  // one read per round)
  u32 rounds = 0, row_cap = 0;
  void release() {
    for (DeviceBuffer *b : {&lrec, &pend, &pcount, &roff, &q[0], &q[1], &dec[0], &dec[1], &cont,
                            &next, &cells32, &delta32, &rootmom})
      b->release();
    for (int k = 0; k < 3; ++k) slot_cells[k] = slot_bodies[k] = 0;
    slot_pend = 0;
    rounds = row_cap = 0;
  }
};

// What the learned walk needs besides the tree and the groups.
struct LearnedWalk {
  const LearnedNet *net = nullptr;  // device
  const CellFeat *cfeat = nullptr;  // per node (device)
  DeviceBuffer *gtol = nullptr;     // per group (f0, tolerance), filled by build_lists
  LearnedScratch *scratch = nullptr;
  const float *prev_amag = nullptr; // |a| per body in caller order (device)
  double alpha = 0.02, G = 1.0;
  float inv_theta_guard = 1.f / 1.5f;
  float band = 3.f;                 // log2 units; 0: prior only; huge: the MLP decides all
  float y_mean = 0.f;               // the model's mean correction (centres the prior)
  u32 walk_budget = kLearnedWalkBudget;  // round 0: nodes a thread tests before a warp takes over
  u32 pair_budget = kLearnedPairBudget;  // later rounds: the same
  bool plan_rounds = true;  // walk the last call's rounds before reading anything back
  // each round by warps, one per group (1), by threads per part (0), or by
  // warps below Workspace::kWarpWalkGroups groups (-1), as the plain walk
  int warps_mode = -1;
  // recorded after the walk's inputs (learned_walk_inputs) on another
  // stream: the walk's stream waits for it first (null: same stream)
  cudaEvent_t inputs_ready = nullptr;
};

// Per-node features (after build_tree and the FP64 moments: the training
// samples' features).
void learned_node_features(Workspace &ws, DeviceBuffer &cfeat, cudaStream_t s);
// The learned walk's inputs from FP32 moment estimates (moments32), on the
// main stream while the FP64 moments may still run: scratch.cells32,
// delta32 and rootmom, the per-node features and the walk's per-node
// records (LWalkRec) for the guard angle 1 / inv_theta_guard and the model's
// y_mean.
void learned_walk_inputs(Workspace &ws, LearnedScratch &scratch, DeviceBuffer &cfeat,
                         float inv_theta_guard, float y_mean, cudaStream_t s);
// Per-group group feature and tolerance (inside build_lists, after the group boxes).
void learned_group_tolerances(Workspace &ws, const LearnedWalk &lw, u32 ng, cudaStream_t s);
// The learned walk in rounds, three threads per group (one per part of the
// root's children, later rounds each taking its own part's deferred pairs),
// each writing into its own slots: group records, cell_list, body_list and
// the interaction counters of the ng groups (inside build_lists).
void learned_build_lists(Workspace &ws, const LearnedWalk &lw, u32 ng, Scalars *host,
                         cudaStream_t s);
// The tensor-core layout of an FP32 model (kModelFloats floats, device).
void learned_prepare_net(const float *model, LearnedNet *net, cudaStream_t s);
// The walk's inference on given raw features: predicted log2 error per row.
void learned_predict(const LearnedNet *net, const float *feat, u64 n, float *pred,
                     cudaStream_t s);

}  // namespace gtc
