// The device-resident grouped solver: workspace and stage entry points.
//
// Data layout in HBM (N bodies, M tree nodes, G groups):
//   per body   pos/mass (caller order, FP64), sort keys (up to three 63-bit
//              words of octant digits), tree-order permutation, tree-order
//              FP64 positions/masses, FP32 bodies (float4), FP32 output.
//   per node   geometry (centre, half), FP64 moments (com, mass, quadrupole,
//              delta), range [begin, end), skip, parent, depth, children, and
//              the packed FP32 cell (48 B), FP32 walk record (48 B) and FP64
//              walk record (64 B) the kernels read.
//   per axis   the split table: the centres of key levels 0..20, heap order.
//   per group  target range, FP64 and FP32 boxes, and the 64 B group record
//              (counts and up to three segments of each list).
//   lists      cell_list / body_list, uint32 node / body indices: back to
//              back, or in per-group slots (one segment per walk part).
// Nodes are numbered in the reference walk's visiting order (root, then the
// children's subtrees last octant first), which makes the grouped walk a
// stackless forward scan with skip links.
#pragma once

#include "common.cuh"

namespace gtc {

constexpr int kMaxDepth = 60;     // depth cap of the reference octree (octree.cpp:18)
constexpr int kLevelsPerWord = 21;
// Levels of the per-axis split-value table of the key kernel (all of the
// first key word's), and its size per axis (heap order, index 0 unused).
constexpr int kSplitLevels = kLevelsPerWord;
constexpr u32 kSplitSize = 1u << kSplitLevels;
constexpr u32 kFewBodies = 2;     // accepted cells this small go on the body list (group_lists.h:58)
constexpr int kMaxGroupSize = 32;

// Root cube: the reference's bounding-box rule (octree.cpp:184-198) and the
// half side of a node at every depth (each child halves its parent's side).
struct TreeRoot {
  double lo[3], hi[3];
  double center[3];
  double half_at[kMaxDepth + 1];
  // first level whose node may be "tiny" for some body (from the box: no
  // body's own bound is larger), kMaxDepth + 1 when none is
  int tiny_from;
};

// What the grouped walk reads per node. The FP32 record decides almost every
// opening test; the FP64 record (the reference's exact quantities) settles
// the few tests the FP32 record cannot decide with certainty.
struct alignas(16) WalkRec32 {
  float cx, cy, cz, slack;   // centre relative to the root centre; half * 1.0001
  float mx, my, mz, crit2;   // centre of mass relative to the root centre; crit^2
  u32 skip;                  // first node after this node's subtree
  u32 nbody_leaf;            // bodies in the node | 0x80000000 for a leaf
  u32 begin;                 // first body (tree order)
  float bound;               // >= every |value| above plus slack (error bound scale)
};
struct alignas(16) WalkRec64 {
  double cx, cy, cz, slack;  // slack = half * 1.0001 (group_lists.cpp:147)
  double mx, my, mz, crit2;  // crit = 2 half / theta + delta (group_lists.cpp:59-60)
};

// Tile shape of the softened quadrupole list evaluation: staged pairs a
// lane works per inner-loop iteration (1 or 2; the forces do not depend on
// it), and a pass's fixed cost in staged entries per lane, which sets how
// many slices a group's lists are cut into (summation order).
struct EvalShape {
  int pairs = 2;
  u32 pass_cost = 24;
};

struct SolverParams {
  double G, theta, eps;
  int quadrupole, group_size, leaf_size, pack, criterion;
  double alpha;  // learned criterion's tolerance
};

// A forest's per-system list slots for the one-pass walk: system k's groups
// get slots sized from that system's own group count and longest lists (one
// size for every group would give the small systems' groups the largest
// system's slots). Group j of the system has its rest slots at rc_at + j rc
// (cells) and rb_at + j rb (bodies), its near-field slots at nc_at + j nc
// and nb_at + j nb.
struct alignas(16) SysSlots {
  u32 groups;                      // groups of the system the slots cover
  u32 rc, rb, nc, nb;              // slot sizes
  u32 rc_at, rb_at, nc_at, nb_at;  // the system's first slots
  u32 pad[3];
};

// A forest: the bodies of several independent systems back to back (system
// k at [start[k], start[k + 1])), each with its own root cube and tree, built
// and walked by the same launches as one system. Sorted by (system, key),
// system k keeps the same positions in tree order, so `sys` serves both
// orders. Nodes are numbered as for one tree over all bodies: every
// system's nodes form one contiguous range (the last system's first), its
// root first. Null (systems == 0) for one system.
struct ForestView {
  u32 systems = 0;
  const u16 *sys = nullptr;        // system of every body
  const u32 *start = nullptr;      // systems + 1 body offsets
  TreeRoot *roots = nullptr;       // per system: root cube
  u32 *root_node = nullptr;        // per system: its root's node index
  const u8 *group_size = nullptr;  // per system: group size
  const u8 *pack = nullptr;        // per system: packing (0 off, 1 a group's worth, k >= 2 threshold)
  u32 *group_root = nullptr;       // per group: its system's root node
  u32 *sys_groups = nullptr;       // per system: groups of the current choice
  u32 *sys_max = nullptr;          // per system: longest rest cells, rest bodies, near
                                   // cells, near bodies of the last walk (whole lists
                                   // after count + fill)
  u32 *host_groups = nullptr;      // pinned copies of both, read back by eager builds
  u32 *host_max = nullptr;
  uint4 *slot_plan = nullptr;      // per group: slot starts, then sizes (per-system slots)
  int split_levels = 0;            // levels T of each system's split table (2^T per axis)
  u32 *split_unsorted = nullptr;   // per system: its table's in-order values decrease somewhere
  const uint4 *bbox_blocks = nullptr;  // bounding-box blocks: (system, rank, blocks, 0)
  const uint2 *sys_blocks = nullptr;   // per system: (first bounding-box block, blocks)
  u32 bbox_nblocks = 0;
  explicit operator bool() const { return systems > 0; }
};

struct Workspace {
  ForestView forest;
  // bodies
  DeviceBuffer pos, mass;                 // staged caller input (host calls)
  DeviceBuffer acc, pot;                  // staged caller output (host calls)
  DeviceBuffer key0, key0_alt, idx, idx_alt, key1, key2, tiny;
  DeviceBuffer lcp, leafdepth, count, count_scan, flags, flags_scan;
  DeviceBuffer tpos, tmass, bodies, out;
  // deep rounds
  DeviceBuffer dpos, dkey, dkey_alt, drec, drec_alt, dseg, dtmp;
  // nodes
  DeviceBuffer geom, mom, quad, delta, nbegin, nend, skip, parent, depth, nchild, isleaf, kids,
      arrive, bucket, walk32, walk64, cells;
  // groups and lists
  DeviceBuffer tasks, gbegin, gend, gbox, gboxf, gcells, gbodies, gcell_off, gbody_off, groups, cell_list,
      body_list, spill, splitpt;
  // scalars and reductions
  DeviceBuffer root, bbox_part, scalars, split;
  DeviceBuffer scan_tmp;
  DeviceBuffer direct_part;               // direct sum: per-slice partial sums
  DeviceBuffer up_arrive;                 // bottom-up FP32 moments: children finished, per node
  int direct_targets = 2;                 // direct sum: targets per thread (2 or 4)
  EvalShape eval_shape;                   // list evaluation's tile shape
  RadixScratch radix;

  // host-side view of the last build
  u64 n = 0, n_nodes = 0, n_groups = 0, n_cell_list = 0, n_body_list = 0;
  int key_words = 1;
  int sort_levels = 0;        // key levels the next eager build sorts first (0: all 21)
  int tree_depth = 0;         // the last eager build's deepest leaf
  int walk_split_depth = 0;   // tuning: subtree depth of the walk tasks (0..2)
  // The plain walk by warps (one warp per group, 32 node tests per step) or
  // by threads (two per group in the one pass, one in count + fill). Mode
  // -1 (default) picks warps below kWarpWalkGroups groups: with fewer, the
  // thread walk leaves most of the GPU idle; with more, its neighbouring
  // groups walking the same nodes together make it the faster. walk_warps:
  // the choice of the current lists.
  int walk_mode = -1;
  bool walk_warps = true;
  static constexpr u64 kWarpWalkGroups = 40000;
  bool warps_for(u64 groups) const {
    return walk_mode > 0 || (walk_mode < 0 && groups < kWarpWalkGroups);
  }
  // The current lists hold each group's entries in walk-step order rather
  // than the reference's visiting order (exports sort them back).
  bool lists_unordered = false;
  DeviceBuffer walk_next;     // the warp walk's group counter
  // One-pass walk: group g's lists start at g * slot_cells and g *
  // slot_bodies (capacities sized from the previous walk's longest lists);
  // 0 until a walk has measured them. `gapped`: the current lists use that
  // layout (groups' ranges are not back to back).
  u32 slot_cells = 0, slot_bodies = 0, slot_near_cells = 0, slot_near_bodies = 0;
  bool gapped = false;
  u32 list_passes = 0;  // walks of the last list build (1 one pass, 2 count + fill, rounds)
  // The tree's moments and node records run on a side stream once the
  // topology is known, beside the group choice on the main stream; whoever
  // reads them first makes the main stream wait for `side_done`. The walk
  // records are ready earlier, at `side_walk` (the quadrupoles and the cells
  // follow them on the side stream).
  cudaStream_t side = nullptr;
  cudaEvent_t side_fork = nullptr, side_done = nullptr, side_walk = nullptr;
  bool side_pending = false, walk_pending = false;
  // Optional stage events (context option "stage_events"): CUDA events at
  // the boundaries of the eager build's and walk's stages, for per-stage
  // device times. Off by default.
  enum Stage { kStBuild, kStSort0, kStSort1, kStTopo, kStMom0, kStMomW, kStMom1, kStWalk0,
               kStWalk1, kStages };
  bool stage_on = false;
  cudaEvent_t stage_ev[kStages] = {};
  bool stage_hit[kStages] = {};
  int sort_passes = 0;  // 8-bit passes of the last build's first sort
  void stage(int k, cudaStream_t s);
  // Overflow pool behind n_groups slots of `slot` entries: a sixteenth of
  // the slots plus four slots.
  static u64 pool_for(u64 n_groups, u32 slot) { return n_groups * slot / 16 + 4ull * slot; }
  void release_all();
};

// Device scalars written by the stages, read back once per call.
struct Scalars {
  u32 deep;               // bodies whose leaf lies below the key words so far
  u32 n_nodes;
  u32 n_groups;
  u32 depth;              // deepest leaf
  u64 n_cell_list, n_body_list;
  unsigned long long cell_interactions, body_interactions, max_list;
  u32 max_group;
  u32 aux;
  unsigned long long fp64_tests;  // opening tests the FP32 bounds left undecided
  unsigned long long mlp_rows;    // learned walk: rows the MLP decided
  unsigned long long mlp_batches; // learned walk: warp inferences
  u32 lcont, lcont_taken; // learned walk: walks handed on to warps, and taken so far
  u32 max_rows;           // learned walk: most pairs one round deferred (all parts and groups)
  u32 list_overflow;      // learned walk: a list slot overflowed
  u32 abort;              // graph replay: the step outgrew the captured sizes (bits)
  u32 error;              // device-detected failure code (0 = none)
  u32 max_cells, max_bodies;  // longest cell and body list of a group (one-pass walk: its rest)
  u32 max_near_cells, max_near_bodies;  // one-pass walk: longest lists of a near-field walk
  // learned walk: longest lists of each part (cells, then bodies; all
  // rounds), most pairs a part deferred in a round
  u32 lmax_cells[3], lmax_bodies[3], max_pend;
  unsigned long long spill_used[2];  // one-pass walk: overflow pool entries taken (cells, bodies)
  u32 spilled;            // one-pass walk: groups that outgrew their slots
  unsigned long long walk_nodes;  // node records the walk tested
  u32 split_unsorted;     // the split table's in-order values decrease somewhere (keys step by level)
};

// The list statistics of one group per lane (valid lanes), summed and
// maximised over the warp first so that each counter takes one atomic per
// warp; every lane of the warp must call it. With `totals`, the list
// lengths are added to the list sizes too.
__device__ __forceinline__ void group_stats_warp(Scalars *sc, bool valid, u64 t, u64 nc, u64 nb,
                                                 bool totals, bool maxima = true) {
  unsigned long long ci = valid ? t * nc : 0, bi = valid ? t * nb - t : 0,
                     ml = valid ? nc + nb : 0, tc = valid ? nc : 0, tb = valid ? nb : 0;
  u32 mg = valid ? static_cast<u32>(t) : 0u;
  u32 mc = valid ? static_cast<u32>(nc < 0xffffffffull ? nc : 0xffffffffull) : 0u;
  u32 mb = valid ? static_cast<u32>(nb < 0xffffffffull ? nb : 0xffffffffull) : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ci += __shfl_xor_sync(kFullMask, ci, o);
    bi += __shfl_xor_sync(kFullMask, bi, o);
    tc += __shfl_xor_sync(kFullMask, tc, o);
    tb += __shfl_xor_sync(kFullMask, tb, o);
    const unsigned long long m = __shfl_xor_sync(kFullMask, ml, o);
    ml = m > ml ? m : ml;
  }
  mg = __reduce_max_sync(kFullMask, mg);
  mc = __reduce_max_sync(kFullMask, mc);
  mb = __reduce_max_sync(kFullMask, mb);
  const unsigned any = __ballot_sync(kFullMask, valid);  // every lane, before lane 0 alone goes on
  if ((threadIdx.x & 31) != 0 || any == 0) return;
  atomicAdd(&sc->cell_interactions, ci);
  atomicAdd(&sc->body_interactions, bi);
  atomicMax(&sc->max_list, ml);
  atomicMax(&sc->max_group, mg);
  if (maxima) {
    atomicMax(&sc->max_cells, mc);
    atomicMax(&sc->max_bodies, mb);
  }
  if (totals) {
    atomicAdd(reinterpret_cast<unsigned long long *>(&sc->n_cell_list), tc);
    atomicAdd(reinterpret_cast<unsigned long long *>(&sc->n_body_list), tb);
  }
}

// The evaluator's group record, 64 bytes (four uint4): targets [begin, end),
// the list lengths, and the cell and body lists as up to kListSegments
// segments each (start, count), concatenated in list order; empty segments
// are skipped. uint4 0: begin, end, cells, bodies; 1: cell segments 0 and 1;
// 2: cell segment 2, body segment 0; 3: body segments 1 and 2.
constexpr int kListSegments = 3;
constexpr int kGroupRecWords = 16;

struct ListSegs {
  u32 start[kListSegments], count[kListSegments];
};

__host__ __device__ inline ListSegs one_segment(u64 start, u64 count) {
  ListSegs s{};
  s.start[0] = static_cast<u32>(start);
  s.count[0] = static_cast<u32>(count);
  return s;
}

__host__ __device__ inline void store_group_rec(uint4 *groups, u64 g, u32 begin, u32 end,
                                                const ListSegs &c, const ListSegs &b) {
  const u32 nc = c.count[0] + c.count[1] + c.count[2];
  const u32 nb = b.count[0] + b.count[1] + b.count[2];
  groups[4 * g] = make_uint4(begin, end, nc, nb);
  groups[4 * g + 1] = make_uint4(c.start[0], c.count[0], c.start[1], c.count[1]);
  groups[4 * g + 2] = make_uint4(c.start[2], c.count[2], b.start[0], b.count[0]);
  groups[4 * g + 3] = make_uint4(b.start[1], b.count[1], b.start[2], b.count[2]);
}

// A group's lists as the evaluator reads them: entry e of the concatenated
// segments is at at(e).
struct SegView {
  u32 s0, n0, s1, n1, s2;
  __host__ __device__ __forceinline__ u32 at(u32 e) const {
    return e < n0 ? s0 + e : (e - n0 < n1 ? s1 + (e - n0) : s2 + (e - n0 - n1));
  }
};
__host__ __device__ __forceinline__ SegView cell_segs(const uint4 &q1, const uint4 &q2) {
  return SegView{q1.x, q1.y, q1.z, q1.w, q2.x};
}
__host__ __device__ __forceinline__ SegView body_segs(const uint4 &q2, const uint4 &q3) {
  return SegView{q2.z, q2.w, q3.x, q3.y, q3.z};
}

// Adds each lane's count to *total with one atomic per warp (every lane of
// the warp must call it).
__device__ __forceinline__ void warp_add(unsigned long long *total, unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(total, v);
}

// Stage 1: octree on the device. pos (N x 3) and mass in caller order.
// Fills geometry, moments, ranges, the tree-order permutation (idx), the
// FP32 bodies and cells and the walk records. Returns the node count.
// `host` is pinned memory the device scalars are read back into.
// The side stream and its events (made before a capture uses them).
void ensure_side(Workspace &ws);
// The side stream, started after the work queued on s so far.
cudaStream_t fork_side(Workspace &ws, cudaStream_t s);
// Work queued on the side stream so far ends before what s runs next.
void join_side(Workspace &ws, cudaStream_t s);
// The side stream's walk records (marked by mark_walk_ready) are written
// before what s runs next; its later work may still run.
void mark_walk_ready(Workspace &ws, cudaStream_t side);
void join_walk(Workspace &ws, cudaStream_t s);
// Joins the side stream when it leaves scope (every exit of a solve).
struct SideJoin {
  Workspace &ws;
  cudaStream_t s;
  ~SideJoin() { join_side(ws, s); }
};

// walk_records: pack the theta walk's node records (the learned walk has its
// own and skips them).
void build_tree(Workspace &ws, const double *pos, const double *mass, u64 n,
                const SolverParams &sp, cudaStream_t s, Scalars *host, bool walk_records = true);

struct LearnedWalk;

// Stage 2: groups (with sibling packing) and the grouped walk; fills groups,
// cell_list and body_list and the interaction counters. With `lw` the walk
// decides by the learned criterion instead of the opening angle.
void build_lists(Workspace &ws, const SolverParams &sp, cudaStream_t s, Scalars *host,
                 const LearnedWalk *lw = nullptr);

// Where an evaluation writes each target's acceleration and potential:
// always out (FP32, tree order); with acc set also acc and pot (FP64, caller
// order through `order`: the scatter of gravity_backends.cpp:132-136, done
// by the evaluation's own threads), and with amag set |a| per body (caller
// order) for the next learned solve.
struct EvalOut {
  float4 *out = nullptr;
  const u32 *order = nullptr;
  double *acc = nullptr, *pot = nullptr;
  float *amag = nullptr;
};

// Stage 3: warp-per-group evaluation of the lists into eo.
// `counter` is one device word the kernel's work queue uses; `shape` the
// tile shape of the softened quadrupole evaluation.
void evaluate_lists(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                    const u32 *body_list, const uint4 *groups, u64 n_groups, float G, float eps2,
                    bool quadrupole, const EvalOut &eo, u32 *counter, cudaStream_t s,
                    const EvalShape &shape = EvalShape{});

// Capacities of a solve replayed from a CUDA graph: the sizes of the
// buffers the graph was captured with. A replay whose tree, depth or lists
// outgrow them sets Scalars::abort, and every later kernel of the replay
// returns at once (memory stays in bounds; the step is then redone eagerly).
struct GraphCaps {
  u32 nodes;        // node arrays
  int depth;        // deepest node the per-depth moment launches cover
  u32 groups;       // groups the list slots cover
  u32 slot_cells, slot_bodies;  // each group's list slots (one-pass walk, its rest)
  u32 slot_near_cells, slot_near_bodies;  // ... and its near-field walk
  u64 pool_cells, pool_bodies;  // overflow pools behind the slots
  // a forest: per-system slots (device table; null: the sizes above for
  // every group), and where the pools start
  const SysSlots *sys_slots = nullptr;
  u64 pool_at_cells = 0, pool_at_bodies = 0;
};
// Both stages without a host synchronisation, for stream capture: grids
// sized by the capacities, counts read on the device. One key word only (a
// tree deeper than 21 levels aborts), one walk task per group, written in
// one pass into per-group slots (more groups or a longer list aborts).
void build_tree_graph(Workspace &ws, const double *pos, const double *mass, u64 n,
                      const SolverParams &sp, const GraphCaps &caps, cudaStream_t s);
void build_lists_graph(Workspace &ws, const SolverParams &sp, const GraphCaps &caps,
                       cudaStream_t s);
// The single walk task of a graph replay (the root), written before capture.
void write_root_task(Workspace &ws, cudaStream_t s);
// The evaluation of a replay: the group count from the device, nothing
// after an abort.
void evaluate_lists_graph(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                          const u32 *body_list, const uint4 *groups, u64 max_groups,
                          const Scalars *sc, float G, float eps2, bool quadrupole,
                          const EvalOut &eo, u32 *counter, cudaStream_t s,
                          const EvalShape &shape = EvalShape{});

// Direct summation kernels.
// FP32 estimates of every node's moments (GTCell layout in cells32, delta in
// delta32) from the FP32 bodies, and the root's mass as rootmom[1].y, for
// the learned walk's decisions (after an eager build_tree, on the main
// stream; the FP64 moments may still be running on the side stream).
void moments32(Workspace &ws, float4 *cells32, float *delta32, double2 *rootmom,
               cudaStream_t s);
// Octree::accel_pot for every body on the built tree (FP64, the reference's
// per-particle walk): acc (n x 3) and pot in caller order; counts[0..1] +=
// cell and particle interactions.
void tree_walk_forces(Workspace &ws, const SolverParams &sp, double *acc, double *pot,
                      unsigned long long *counts, cudaStream_t s);
// The tiled FP32 direct sum; `scratch` holds per-source-slice partial sums;
// `targets` (2 or 4) per thread, the kernel's tile shape.
void direct_fp32(const float4 *bodies, u32 n, float G, float eps2, float4 *out,
                 DeviceBuffer &scratch, cudaStream_t s, int targets);
void direct_fp64_sample(const double *pos, const double *mass, u64 n, const u64 *idx, u64 m,
                        double G, double eps, double *acc, double *pot, DeviceBuffer &scratch,
                        cudaStream_t s);
// The FP64 sample sums in two launches: per-(source slice, target) partial
// sums into `part` (2 double2 per pair), then each target's slices added in
// slice order. The plan cuts the n sources into `slices` slices of `slice`
// bodies: about 8 blocks per SM, at least one tile of bodies per slice, and
// at most max_pairs (slice, target) pairs.
struct Fp64SamplePlan {
  u64 slices, slice;
};
Fp64SamplePlan plan_fp64_sample(u64 n, u64 m, int sms, u64 max_pairs);
void launch_fp64_sample(const double *pos, const double *mass, u64 n, const u64 *idx, u64 m,
                        double G, double eps, const Fp64SamplePlan &plan, double2 *part,
                        double *acc, double *pot, cudaStream_t s);
// float4 bodies relative to the bounding-box centre (gravity_backends.cpp:15-23, :62).
void pack_bodies_bbox(Workspace &ws, const double *pos, const double *mass, u64 n,
                      cudaStream_t s);
void bbox_root(Workspace &ws, const double *pos, u64 n, cudaStream_t s);

// Throws for a device-detected failure code (Scalars::error; 0: none): bit 4
// non-finite positions (InvalidArgument), 8 the learned walk's count and fill
// passes disagree, 16 a radix-sort look-back outwaited its bound, 1 (and any
// other) an inconsistent tree.
void check_device_error(u32 code);

// FP32 FMA throughput of the device (TFLOP/s), by a dense FMA kernel on every SM.
double fp32_peak_tflops(cudaStream_t s);

}  // namespace gtc
