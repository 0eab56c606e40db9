// C ABI of the GB300 gravity backend (include/gtc.h).

#include <algorithm>
#include <atomic>
#include <memory>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "../../include/gtc.h"
#include "context.cuh"
#include "forest.cuh"
#include "integrate.cuh"

static_assert(sizeof(gtc_float4) == 16 && alignof(gtc_float4) == 16, "float4 layout");
static_assert(sizeof(gtc_kernel_params) == 32, "GTParams layout");
static_assert(sizeof(gtc_cell) == 48, "GTCell layout");
static_assert(sizeof(gtc_group) == 32, "GTGroup layout");

namespace gtc {

namespace {
std::atomic<unsigned long long> g_launches{0};
}
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

[[noreturn]] void throw_cuda(cudaError_t e, const char *what, const char *file, int line) {
  (void)cudaGetLastError();  // a failed call leaves its error for the next check to find
  std::string msg = std::string("CUDA error ") + cudaGetErrorName(e) + " (" +
                    cudaGetErrorString(e) + ") in " + what + " at " + file + ":" +
                    std::to_string(line);
  if (e == cudaErrorMemoryAllocation) throw OutOfMemory(msg);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) throw RuntimeError(msg);
  throw RuntimeError(msg);
}

void DeviceBuffer::ensure(std::size_t want) {
  if (want <= bytes && ptr) return;
  release();
  const std::size_t grown = want + want / 8 + 256;
  void *p = nullptr;
  const cudaError_t e = cudaMalloc(&p, grown);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    throw OutOfMemory("device allocation of " + std::to_string(grown) + " bytes failed: " +
                      cudaGetErrorString(e));
  }
  ptr = p;
  bytes = grown;
}

void DeviceBuffer::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

void Workspace::release_all() {
  DeviceBuffer *all[] = {&pos, &mass, &acc, &pot, &key0, &key0_alt, &idx, &idx_alt, &key1,
                         &key2, &tiny, &lcp, &leafdepth, &count, &count_scan, &flags,
                         &flags_scan, &tpos, &tmass, &bodies, &out, &dpos, &dkey, &dkey_alt,
                         &drec, &drec_alt, &dseg, &dtmp, &geom, &mom, &quad, &delta, &nbegin,
                         &nend, &skip, &parent, &depth, &nchild, &isleaf, &kids, &arrive, &bucket, &walk32, &walk64, &cells,
                         &tasks, &gbegin, &gend, &gbox, &gboxf, &gcells, &gbodies, &gcell_off, &gbody_off,
                         &groups, &cell_list, &body_list, &spill, &splitpt, &root, &bbox_part, &scalars, &split, &scan_tmp,
                         &direct_part, &up_arrive, &walk_next, &radix.counts, &radix.scan_tmp};
  for (DeviceBuffer *b : all) b->release();
  if (side) {
    cudaStreamSynchronize(side);
    cudaStreamDestroy(side);
    cudaEventDestroy(side_fork);
    cudaEventDestroy(side_done);
    cudaEventDestroy(side_walk);
  }
  side = nullptr;
  side_fork = side_done = side_walk = nullptr;
  side_pending = walk_pending = false;
  for (cudaEvent_t &e : stage_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
}

void check_device_error(u32 code) {
  if (code == 0) return;
  if (code & 4u) throw InvalidArgument("cuda: positions must be finite");
  if (code & 8u) throw RuntimeError("cuda: the learned walk's count and fill passes disagree");
  if (code & 16u) throw RuntimeError("cuda: the radix sort's look-back outwaited its bound");
  throw RuntimeError("cuda: inconsistent tree detected on the device (code " +
                     std::to_string(code) + ")");
}

void Workspace::stage(int k, cudaStream_t s) {
  if (!stage_on) return;
  if (!stage_ev[k]) GTC_CUDA(cudaEventCreate(&stage_ev[k]));
  GTC_CUDA(cudaEventRecord(stage_ev[k], s));
  stage_hit[k] = true;
}

}  // namespace gtc

namespace {

using gtc::u32;
using gtc::u64;

thread_local std::string g_create_error;

template <class F>
gtc_status guarded(gtc_context *ctx, F &&f) {
  if (!ctx) return GTC_INVALID_ARGUMENT;
  try {
    GTC_CUDA(cudaSetDevice(ctx->device));
    f();
    ctx->error.clear();
    return GTC_OK;
  } catch (const gtc::InvalidArgument &e) {
    ctx->error = e.what();
    return GTC_INVALID_ARGUMENT;
  } catch (const gtc::OutOfMemory &e) {
    ctx->error = e.what();
    return GTC_OUT_OF_MEMORY;
  } catch (const std::bad_alloc &) {
    ctx->error = "host allocation failed";
    return GTC_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    ctx->error = e.what();
    return GTC_RUNTIME_ERROR;
  }
}

gtc::SolverParams check_params(const gtc_gravity_params *gp, bool group) {
  if (!gp) throw gtc::InvalidArgument("gravity parameters are required");
  gtc::SolverParams sp{gp->G, gp->theta, gp->eps, gp->quadrupole != 0 ? 1 : 0,
                       gp->group_size, std::max(1, gp->leaf_size), gp->pack < 0 ? 1 : gp->pack,
                       gp->criterion, gp->alpha};
  if (group) {
    if (sp.group_size < 1) throw gtc::InvalidArgument("group_size must be at least 1");
    if (sp.group_size > gtc::kMaxGroupSize)
      throw gtc::InvalidArgument("group_size can be at most 32 on cuda");
    if (!(sp.theta > 0)) throw gtc::InvalidArgument("theta must be positive");
    if (sp.criterion != GTC_CRITERION_THETA && sp.criterion != GTC_CRITERION_LEARNED)
      throw gtc::InvalidArgument("unknown opening criterion");
    if (sp.criterion == GTC_CRITERION_LEARNED && !(sp.alpha > 0 && std::isfinite(sp.alpha)))
      throw gtc::InvalidArgument("the learned criterion needs a positive alpha");
  }
  return sp;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  GTC_CUDA(cudaEventElapsedTime(&ms, a, b));
  return ms;
}

// Makes `main` wait for the learned stream's work when it leaves scope, on
// every exit of a solve (the walk itself waits for it before it starts).
struct LearnedJoin {
  gtc_context *ctx;
  cudaStream_t main;
  bool active;
  ~LearnedJoin() {
    if (!active) return;
    if (cudaEventRecord(ctx->ldone, ctx->lstream) == cudaSuccess)
      cudaStreamWaitEvent(main, ctx->ldone, 0);
  }
};

// The grouped solver on device arrays (caller order in and out).
void group_force(gtc_context *ctx, const double *pos, const double *mass, u64 n,
                 const gtc::SolverParams &sp, double *acc, double *pot) {
  if (n > 0xffffffffull) throw gtc::RuntimeError("too many particles for the 32 bit GPU indices");
  cudaStream_t s = ctx->stream;
  gtc::Workspace &ws = ctx->ws;
  ctx->have_group = false;
  ctx->stats = gtc_stats{};
  const unsigned long long launches0 = gtc::launches_so_far();
  if (n == 0) {
    ws.n = ws.n_nodes = ws.n_groups = ws.n_cell_list = ws.n_body_list = 0;
    ctx->have_group = true;
    ctx->last = sp;
    return;
  }
  // The learned walk needs a model and |a| of a previous solve of the same
  // bodies; otherwise the theta walk runs (the fallback).
  const bool learned = sp.criterion == GTC_CRITERION_LEARNED && ctx->have_model &&
                       ctx->prev_n == n;
  for (bool &h : ws.stage_hit) h = false;
  GTC_CUDA(cudaEventRecord(ctx->ev[0], s));
  const gtc::SideJoin side_join{ws, s};
  gtc::build_tree(ws, pos, mass, n, sp, s, ctx->host_sc, !learned);
  GTC_CUDA(cudaEventRecord(ctx->ev[1], s));
  LearnedJoin learned_join{ctx, s, false};
  if (learned) {
    // the walk's inputs from FP32 moment estimates, on their own stream
    // beside the group choice (the walk waits for them); the walk then runs
    // while the side stream accumulates the FP64 moments the evaluation reads
    if (!ctx->lstream) {
      int least = 0, greatest = 0;
      GTC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      GTC_CUDA(cudaStreamCreateWithPriority(&ctx->lstream, cudaStreamNonBlocking, greatest));
      GTC_CUDA(cudaEventCreateWithFlags(&ctx->lfork, cudaEventDisableTiming));
      GTC_CUDA(cudaEventCreateWithFlags(&ctx->ldone, cudaEventDisableTiming));
    }
    GTC_CUDA(cudaEventRecord(ctx->lfork, s));
    GTC_CUDA(cudaStreamWaitEvent(ctx->lstream, ctx->lfork, 0));
    learned_join.active = true;
    gtc::learned_walk_inputs(ws, ctx->lscratch, ctx->cfeat,
                             static_cast<float>(1.0 / ctx->guard_theta), ctx->model_ymean,
                             ctx->lstream);
    GTC_CUDA(cudaEventRecord(ctx->ldone, ctx->lstream));
    gtc::LearnedWalk lw;
    lw.inputs_ready = ctx->ldone;
    lw.net = ctx->net.as<gtc::LearnedNet>();
    lw.cfeat = ctx->cfeat.as<gtc::CellFeat>();
    lw.gtol = &ctx->gtol;
    lw.scratch = &ctx->lscratch;
    lw.y_mean = ctx->model_ymean;
    lw.prev_amag = ctx->prev_amag.as<float>();
    lw.alpha = sp.alpha;
    lw.G = sp.G;
    lw.inv_theta_guard = static_cast<float>(1.0 / ctx->guard_theta);
    lw.band = ctx->band_override >= 0 ? static_cast<float>(ctx->band_override) : ctx->model_band;
    lw.walk_budget = ctx->walk_budget == 0 ? ~0u : ctx->walk_budget;
    lw.pair_budget = ctx->pair_budget == 0 ? ~0u : ctx->pair_budget;
    lw.plan_rounds = !ctx->read_every_round;
    lw.warps_mode = ctx->learned_warps;
    gtc::build_lists(ws, sp, s, ctx->host_sc, &lw);
  } else {
    gtc::build_lists(ws, sp, s, ctx->host_sc);
  }
  GTC_CUDA(cudaEventRecord(ctx->ev[2], s));
  if (n > 0) {
    ws.out.ensure(n * sizeof(float4));
    ctx->counter.ensure(sizeof(u32));
    if (ctx->have_model) ctx->prev_amag.ensure(n * sizeof(float));  // |a| for the next learned solve
    const gtc::EvalOut eo{ws.out.as<float4>(), ws.idx.as<u32>(), acc, pot,
                          ctx->have_model ? ctx->prev_amag.as<float>() : nullptr};
    GTC_CUDA(cudaEventRecord(ctx->ev[4], s));
    gtc::evaluate_lists(ws.bodies.as<float4>(), ws.cells.as<float4>(), ws.cell_list.as<u32>(),
                        ws.body_list.as<u32>(), ws.groups.as<uint4>(), ws.n_groups,
                        static_cast<float>(sp.G), static_cast<float>(sp.eps * sp.eps),
                        sp.quadrupole != 0, eo, ctx->counter.as<u32>(), s, ws.eval_shape);
    GTC_CUDA(cudaEventRecord(ctx->ev[5], s));
  }
  GTC_CUDA(cudaEventRecord(ctx->ev[3], s));
  GTC_CUDA(cudaMemcpyAsync(ctx->host_sc, ws.scalars.ptr, sizeof(gtc::Scalars),
                           cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
  gtc::check_device_error(ctx->host_sc->error);
  gtc_stats &st = ctx->stats;
  st.tree_ms = elapsed(ctx->ev[0], ctx->ev[1]);
  st.lists_ms = elapsed(ctx->ev[1], ctx->ev[2]);
  st.evaluate_ms = elapsed(ctx->ev[2], ctx->ev[3]);
  st.total_ms = elapsed(ctx->ev[0], ctx->ev[3]);
  st.eval_kernel_ms = elapsed(ctx->ev[4], ctx->ev[5]);
  st.kernel_launches = gtc::launches_so_far() - launches0;
  if (n > 0) {
    const gtc::Scalars &h = *ctx->host_sc;
    st.cell_interactions = h.cell_interactions;
    st.body_interactions = h.body_interactions;
    st.max_list = h.max_list;
    st.max_group = h.max_group;
    st.depth = h.depth;
    st.walk_tests_fp64 = h.fp64_tests;
    st.mlp_rows = h.mlp_rows;
    st.mlp_batches = h.mlp_batches;
  }
  st.criterion_used = learned ? GTC_CRITERION_LEARNED : GTC_CRITERION_THETA;
  st.list_passes = ws.list_passes;
  st.spilled_groups = n > 0 ? ctx->host_sc->spilled : 0;
  st.walk_nodes = n > 0 ? ctx->host_sc->walk_nodes : 0;
  ctx->prev_n = ctx->have_model ? n : 0;
  st.n_cell_list = ws.n_cell_list;
  st.n_body_list = ws.n_body_list;
  st.n_nodes = static_cast<u32>(ws.n_nodes);
  st.n_groups = static_cast<u32>(ws.n_groups);
  ctx->have_group = true;
  ctx->last = sp;
}

// The capacities of a captured solve of n bodies and the buffers they need:
// the last eager solve's sizes (hs, ws) with headroom (list slots with
// twice the headroom: the longest of many lists moves more than the totals
// do); offsets stay below 2^32 (a replay that needs more aborts).
void reserve_graph(gtc::Workspace &ws, const gtc::Scalars &hs, double headroom, u64 n,
                   gtc::GraphCaps &caps, bool sized_lists = false) {
  gtc::ensure_side(ws);  // the captured build forks the quadrupoles onto it
  const double f = 1.0 + headroom;
  const u64 pad = headroom > 0 ? 1024 : 0;
  caps.nodes = static_cast<u32>(std::min<u64>(static_cast<u64>(ws.n_nodes * f) + pad, 0xfffffff0ull));
  caps.depth = std::min<int>(gtc::kMaxDepth, static_cast<int>(hs.depth) + (pad ? 2 : 0));
  // list slots: the last walk's group count, and its longest lists with
  // twice the headroom (the longest of many lists moves more than the
  // totals do); offsets stay below 2^32 (a replay that needs more aborts)
  caps.groups = static_cast<u32>(std::min<u64>(static_cast<u64>(ws.n_groups * f) + pad, n));
  caps.groups = std::max<u32>(caps.groups, 1);
  const double fs = 1.0 + 2.0 * headroom;
  auto slot = [&](u32 longest) {
    const u64 v = (static_cast<u64>(longest * fs) + (pad ? 64 : 0) + 31) & ~31ull;
    const u64 most = (0xffffffffull / caps.groups / 2) & ~31ull;  // two slot arrays
    return static_cast<u32>(std::max<u64>(32, std::min(v, most)));
  };
  // (the last walk split: rest and near field; the two passes: whole lists)
  const bool split = ws.list_passes == 1;
  caps.slot_cells = slot(hs.max_cells);
  caps.slot_bodies = slot(hs.max_bodies);
  caps.slot_near_cells = slot(split ? hs.max_near_cells : hs.max_cells);
  caps.slot_near_bodies = slot(split ? hs.max_near_bodies : hs.max_bodies);
  auto pool = [&](u32 rest, u32 near) {
    const u64 used = static_cast<u64>(caps.groups) * (static_cast<u64>(rest) + near);
    const u64 room = used < 0xffffffffull ? 0xffffffffull - used : 0;
    return std::min<u64>(gtc::Workspace::pool_for(caps.groups, rest + near), room);
  };
  caps.pool_cells = pool(caps.slot_cells, caps.slot_near_cells);
  caps.pool_bodies = pool(caps.slot_bodies, caps.slot_near_bodies);
  const u64 m = caps.nodes;
  ws.geom.ensure(m * 2 * sizeof(double2));
  ws.mom.ensure(m * 2 * sizeof(double2));
  ws.quad.ensure(m * 3 * sizeof(double2));
  ws.delta.ensure(m * 8);
  ws.nbegin.ensure(m * 4);
  ws.nend.ensure(m * 4);
  ws.skip.ensure(m * 4);
  ws.parent.ensure(m * 4);
  ws.depth.ensure(m);
  ws.nchild.ensure(m);
  ws.kids.ensure(m * 8 * sizeof(u32));
  ws.isleaf.ensure(m);
  ws.bucket.ensure(m * 4);
  ws.walk32.ensure(m * sizeof(gtc::WalkRec32));
  ws.walk64.ensure(m * sizeof(gtc::WalkRec64));
  ws.cells.ensure(m * 3 * sizeof(float4));
  if (!ws.forest) ws.split.ensure(3ull * gtc::kSplitSize * sizeof(double));  // (a forest steps)
  ws.flags.ensure(std::max<u64>(n, m) * 4);
  ws.flags_scan.ensure(std::max<u64>(n, m) * 4);
  ws.gcells.ensure(2 * n * 8);
  ws.gbodies.ensure(2 * n * 8);
  ws.gcell_off.ensure((n + 1) * 8);
  ws.gbody_off.ensure((n + 1) * 8);
  ws.groups.ensure(n * gtc::kGroupRecWords * 4);
  caps.sys_slots = nullptr;
  if (!ws.forest || !sized_lists) {  // (a forest sizes them per system, when it can)
    ws.cell_list.ensure((static_cast<u64>(caps.groups) * (caps.slot_cells + caps.slot_near_cells) +
                         caps.pool_cells) * 4);
    ws.body_list.ensure((static_cast<u64>(caps.groups) * (caps.slot_bodies + caps.slot_near_bodies) +
                         caps.pool_bodies) * 4);
  }
  ws.spill.ensure(2 * n * sizeof(u32));
  ws.splitpt.ensure(2 * n * sizeof(u32));
  ws.out.ensure(n * sizeof(float4));
  gtc::reserve_scans(ws.scan_tmp, std::max<u64>(n, m));
}

// One system's leapfrog step inside a captured CUDA graph: kick and drift,
// the whole grouped solve (tree, groups, walk, evaluation, scatter) and the
// closing kick, with no host synchronisation inside. reserve() sizes the
// buffers from the system's last eager solve with headroom; record() issues
// the step on a capturing stream; finish() reads the replay's scalars: a
// replay that outgrew its buffers aborted (its kernels returned), so the
// step's evaluation and closing kick are redone eagerly and the graph must
// be captured again for the new sizes.
struct GraphStep {
  gtc_context *ctx = nullptr;
  double *pos = nullptr, *vel = nullptr, *acc = nullptr, *pot = nullptr;
  const double *mass = nullptr;
  u64 n = 0;
  gtc::SolverParams sp{};
  gtc::GraphCaps caps{};

  void reserve() {
    gtc::Workspace &ws = ctx->ws;
    reserve_graph(ws, *ctx->host_sc, ctx->graph_headroom, n, caps);
    ctx->counter.ensure(sizeof(u32));
    if (ctx->have_model) ctx->prev_amag.ensure(n * sizeof(float));
    gtc::write_root_task(ws, ctx->stream);
  }

  // Events are recorded as external nodes so that their times can be read.
  void mark(int k, cudaStream_t s) const {
    GTC_CUDA(cudaEventRecordWithFlags(ctx->ev[k], s, cudaEventRecordExternal));
  }

  void record(double dt, cudaStream_t s) const {
    gtc::Workspace &ws = ctx->ws;
    gtc::Scalars *sc = ws.scalars.as<gtc::Scalars>();
    const double h = 0.5 * dt;
    gtc::kick_drift(pos, vel, acc, n, h, dt, s);
    mark(0, s);
    gtc::build_tree_graph(ws, pos, mass, n, sp, caps, s);
    mark(1, s);
    gtc::build_lists_graph(ws, sp, caps, s);
    gtc::join_side(ws, s);  // the cells
    mark(2, s);
    mark(4, s);
    const gtc::EvalOut eo{ws.out.as<float4>(), ws.idx.as<u32>(), acc, pot,
                          ctx->have_model ? ctx->prev_amag.as<float>() : nullptr};
    gtc::evaluate_lists_graph(ws.bodies.as<float4>(), ws.cells.as<float4>(),
                              ws.cell_list.as<u32>(), ws.body_list.as<u32>(),
                              ws.groups.as<uint4>(), n, sc, static_cast<float>(sp.G),
                              static_cast<float>(sp.eps * sp.eps), sp.quadrupole != 0, eo,
                              ctx->counter.as<u32>(), s, ws.eval_shape);
    mark(5, s);
    gtc::kick(vel, acc, n, h, s, &sc->abort);
    mark(3, s);
  }

  // After the replay and the copy of its scalars into host_sc: true if the
  // graph must be captured again (the step was redone eagerly).
  bool finish(double dt) {
    gtc::Workspace &ws = ctx->ws;
    const gtc::Scalars &hs = *ctx->host_sc;
    gtc::check_device_error(hs.error);
    if (hs.abort) {
      group_force(ctx, pos, mass, n, sp, acc, pot);
      gtc::kick(vel, acc, n, 0.5 * dt, ctx->stream);
      GTC_CUDA(cudaStreamSynchronize(ctx->stream));
      return true;
    }
    ws.n_nodes = hs.n_nodes;
    ws.n_groups = hs.n_groups;
    ws.n_cell_list = hs.n_cell_list;
    ws.n_body_list = hs.n_body_list;
    ws.gapped = true;  // replays walk once into the captured slots
    ws.lists_unordered = ws.walk_warps;
    gtc_stats &st = ctx->stats;
    const u32 replays = st.graph_steps;
    st = gtc_stats{};
    st.tree_ms = elapsed(ctx->ev[0], ctx->ev[1]);
    st.lists_ms = elapsed(ctx->ev[1], ctx->ev[2]);
    st.evaluate_ms = elapsed(ctx->ev[2], ctx->ev[3]);
    st.total_ms = elapsed(ctx->ev[0], ctx->ev[3]);
    st.eval_kernel_ms = elapsed(ctx->ev[4], ctx->ev[5]);
    st.cell_interactions = hs.cell_interactions;
    st.body_interactions = hs.body_interactions;
    st.max_list = hs.max_list;
    st.max_group = hs.max_group;
    st.depth = hs.depth;
    st.walk_tests_fp64 = hs.fp64_tests;
    st.n_cell_list = hs.n_cell_list;
    st.n_body_list = hs.n_body_list;
    st.n_nodes = hs.n_nodes;
    st.n_groups = hs.n_groups;
    st.criterion_used = GTC_CRITERION_THETA;
    st.list_passes = 1;
    st.spilled_groups = hs.spilled;
    st.walk_nodes = hs.walk_nodes;
    st.kernel_launches = 0;  // one graph launch (its kernels were counted at capture)
    st.graph_steps = replays + 1;
    ctx->have_group = true;
    ctx->last = sp;
    return false;
  }
};

// A captured step graph of one or more systems.
struct StepGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void drop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
  // Captures every system's step on `main`: each system on its own stream
  // (forked from main and joined back), then the copies of their scalars.
  void capture(std::vector<GraphStep> &steps, double dt, cudaStream_t main, cudaEvent_t fork,
               std::vector<cudaEvent_t> &joins) {
    for (GraphStep &g : steps) g.reserve();
    GTC_CUDA(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal));
    try {
      GTC_CUDA(cudaEventRecord(fork, main));
      for (std::size_t k = 0; k < steps.size(); ++k) {
        cudaStream_t s = steps[k].ctx->stream;
        if (s != main) GTC_CUDA(cudaStreamWaitEvent(s, fork, 0));
        steps[k].record(dt, s);
        GTC_CUDA(cudaMemcpyAsync(steps[k].ctx->host_sc, steps[k].ctx->ws.scalars.ptr,
                                 sizeof(gtc::Scalars), cudaMemcpyDeviceToHost, s));
        if (s != main) {
          GTC_CUDA(cudaEventRecord(joins[k], s));
          GTC_CUDA(cudaStreamWaitEvent(main, joins[k], 0));
        }
      }
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(main, &g);
      if (g) cudaGraphDestroy(g);
      (void)cudaGetLastError();
      throw;
    }
    GTC_CUDA(cudaStreamEndCapture(main, &graph));
    GTC_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  }
};

// The leapfrog of one or more systems with every step replayed from one
// CUDA graph. An eager solve of each system sizes its buffers first (with
// prime, it is the priming evaluation; without, it goes to scratch and the
// caller's forces stay). Returns the steps replayed.
u64 leapfrog_graph_systems(std::vector<GraphStep> &sys, double dt, u64 steps, bool prime,
                           cudaStream_t main, cudaEvent_t fork, std::vector<cudaEvent_t> &joins) {
  for (GraphStep &g : sys) {
    gtc::Workspace &ws = g.ctx->ws;
    if (prime) {
      group_force(g.ctx, g.pos, g.mass, g.n, g.sp, g.acc, g.pot);
    } else {
      ws.acc.ensure(g.n * 24);
      ws.pot.ensure(g.n * 8);
      group_force(g.ctx, g.pos, g.mass, g.n, g.sp, ws.acc.as<double>(), ws.pot.as<double>());
    }
    g.ctx->stats.graph_steps = 0;
  }
  StepGraph graph;
  u64 replays = 0;
  try {
    for (u64 k = 0; k < steps; ++k) {
      if (!graph.exec) graph.capture(sys, dt, main, fork, joins);
      GTC_CUDA(cudaGraphLaunch(graph.exec, main));
      GTC_CUDA(cudaStreamSynchronize(main));
      bool again = false;
      for (GraphStep &g : sys) again |= g.finish(dt);
      if (again) graph.drop();
      else ++replays;
    }
  } catch (...) {
    graph.drop();
    throw;
  }
  graph.drop();
  return replays;
}

u64 leapfrog_graph(gtc_context *ctx, double *pos, double *vel, const double *mass, double *acc,
                   double *pot, u64 n, const gtc::SolverParams &sp, double dt, u64 steps,
                   bool prime) {
  std::vector<GraphStep> sys(1);
  sys[0].ctx = ctx;
  sys[0].pos = pos;
  sys[0].vel = vel;
  sys[0].mass = mass;
  sys[0].acc = acc;
  sys[0].pot = pot;
  sys[0].n = n;
  sys[0].sp = sp;
  std::vector<cudaEvent_t> joins(1, nullptr);
  cudaEvent_t fork = nullptr;
  GTC_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  try {
    const u64 r = leapfrog_graph_systems(sys, dt, steps, prime, ctx->stream, fork, joins);
    cudaEventDestroy(fork);
    return r;
  } catch (...) {
    cudaEventDestroy(fork);
    throw;
  }
}

void direct_force(gtc_context *ctx, const double *pos, const double *mass, u64 n,
                  const gtc::SolverParams &sp, double *acc, double *pot) {
  if (n > 0xffffffffull) throw gtc::RuntimeError("too many particles for the CUDA kernels");
  cudaStream_t s = ctx->stream;
  gtc::Workspace &ws = ctx->ws;
  ctx->stats = gtc_stats{};
  const unsigned long long launches0 = gtc::launches_so_far();
  GTC_CUDA(cudaEventRecord(ctx->ev[0], s));
  if (n > 0) {
    gtc::pack_bodies_bbox(ws, pos, mass, n, s);
    ws.out.ensure(n * sizeof(float4));
    GTC_CUDA(cudaEventRecord(ctx->ev[2], s));
    gtc::direct_fp32(ws.bodies.as<float4>(), static_cast<u32>(n), static_cast<float>(sp.G),
                     static_cast<float>(sp.eps * sp.eps), ws.out.as<float4>(), ws.direct_part, s,
                     ws.direct_targets);
  } else {
    GTC_CUDA(cudaEventRecord(ctx->ev[2], s));
  }
  GTC_CUDA(cudaEventRecord(ctx->ev[3], s));
  GTC_CUDA(cudaStreamSynchronize(s));
  ctx->stats.evaluate_ms = elapsed(ctx->ev[2], ctx->ev[3]);
  ctx->stats.eval_kernel_ms = ctx->stats.evaluate_ms;
  ctx->stats.total_ms = elapsed(ctx->ev[0], ctx->ev[3]);
  ctx->stats.body_interactions = n > 0 ? n * (n - 1) : 0;
  ctx->stats.kernel_launches = gtc::launches_so_far() - launches0;
}

// compute_gravity_tree (src/gravity.cpp:7-26) on device arrays: the tree,
// then every body's own walk (Octree::accel_pot).
void tree_force(gtc_context *ctx, const double *pos, const double *mass, u64 n,
                const gtc::SolverParams &sp, double *acc, double *pot) {
  if (n > 0xffffffffull) throw gtc::RuntimeError("too many particles for the 32 bit GPU indices");
  cudaStream_t s = ctx->stream;
  gtc::Workspace &ws = ctx->ws;
  ctx->have_group = false;
  ctx->stats = gtc_stats{};
  const unsigned long long launches0 = gtc::launches_so_far();
  if (n == 0) return;
  GTC_CUDA(cudaEventRecord(ctx->ev[0], s));
  {
    const gtc::SideJoin side_join{ws, s};
    gtc::build_tree(ws, pos, mass, n, sp, s, ctx->host_sc);
    gtc::join_side(ws, s);  // the walk reads the moments
  }
  GTC_CUDA(cudaEventRecord(ctx->ev[1], s));
  ctx->tree_counts.ensure(2 * sizeof(unsigned long long));
  GTC_CUDA(cudaMemsetAsync(ctx->tree_counts.ptr, 0, 2 * sizeof(unsigned long long), s));
  GTC_CUDA(cudaEventRecord(ctx->ev[4], s));
  gtc::tree_walk_forces(ws, sp, acc, pot, ctx->tree_counts.as<unsigned long long>(), s);
  GTC_CUDA(cudaEventRecord(ctx->ev[5], s));
  unsigned long long counts[2] = {0, 0};
  GTC_CUDA(cudaMemcpyAsync(counts, ctx->tree_counts.ptr, sizeof counts, cudaMemcpyDeviceToHost,
                           s));
  GTC_CUDA(cudaMemcpyAsync(ctx->host_sc, ws.scalars.ptr, sizeof(gtc::Scalars),
                           cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
  gtc::check_device_error(ctx->host_sc->error);
  gtc_stats &st = ctx->stats;
  st.tree_ms = elapsed(ctx->ev[0], ctx->ev[1]);
  st.evaluate_ms = st.eval_kernel_ms = elapsed(ctx->ev[4], ctx->ev[5]);
  st.total_ms = elapsed(ctx->ev[0], ctx->ev[5]);
  st.cell_interactions = counts[0];
  st.body_interactions = counts[1];
  st.depth = ctx->host_sc->depth;
  st.n_nodes = static_cast<u32>(ws.n_nodes);
  st.kernel_launches = gtc::launches_so_far() - launches0;
}

}  // namespace

namespace gtc {
void set_contextless_error(const std::string &msg) { g_create_error = msg; }

// Caller-order scatter for the direct path (identity order).
__global__ void k_unpack_direct(const float4 *out, u32 n, double *acc, double *pot) {
  const u32 i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const float4 o = out[i];
  acc[3ull * i] = o.x;
  acc[3ull * i + 1] = o.y;
  acc[3ull * i + 2] = o.z;
  pot[i] = o.w;
}
}  // namespace gtc

namespace {
struct ForestGraph;
}

// Independent systems advanced together. As one forest (every stage one
// launch for all systems, forest.cu) when their shared parameters agree, or
// with one context (stream, workspace) per system and every system's step
// in one captured graph.
struct gtc_ensemble {
  int device = 0;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  std::vector<gtc_context *> ctx;
  std::vector<GraphStep> sys;
  std::string error;
  int forest_mode = -1;  // option "forest": 1 always, 0 never, -1 when eligible
  int forest_walk = -1;  // option "walk_warps" of the forest's walk
  double forest_headroom = 0.25;  // option "graph_headroom" of the forest's step graph
  std::unique_ptr<gtc::ForestRun> forest;
  // The forest's step graph, kept for the next call on the same systems,
  // parameters and dt (forest_key): that call replays it at once.
  std::unique_ptr<ForestGraph> forest_graph;
  std::vector<u64> forest_key;
  ~gtc_ensemble();
};

namespace {
template <class F>
gtc_status ensemble_guarded(gtc_ensemble *e, F &&f) {
  if (!e) return GTC_INVALID_ARGUMENT;
  try {
    GTC_CUDA(cudaSetDevice(e->device));
    f();
    e->error.clear();
    return GTC_OK;
  } catch (const gtc::InvalidArgument &ex) {
    e->error = ex.what();
    return GTC_INVALID_ARGUMENT;
  } catch (const gtc::OutOfMemory &ex) {
    e->error = ex.what();
    return GTC_OUT_OF_MEMORY;
  } catch (const std::exception &ex) {
    e->error = ex.what();
    return GTC_RUNTIME_ERROR;
  }
}

// The forest's leapfrog step inside a captured CUDA graph, as GraphStep
// for one system: kick and drift of every system, the forest's build,
// walk, evaluation and scatter with the closing kick, no host
// synchronisation inside. A replay that outgrew the captured sizes (or
// needs a second key word) aborts: its step is redone eagerly and the
// graph captured again.
struct ForestGraph {
  gtc::ForestRun *f = nullptr;
  double headroom = 0.25;
  gtc::GraphCaps caps{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;

  ForestGraph() = default;
  ForestGraph(const ForestGraph &) = delete;
  ForestGraph &operator=(const ForestGraph &) = delete;
  ~ForestGraph() { drop(); }

  void drop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }

  void record(double dt, cudaStream_t s) {
    gtc::Workspace &ws = f->ws;
    gtc::Scalars *sc = ws.scalars.as<gtc::Scalars>();
    const double h = 0.5 * dt;
    f->kick_drift(h, dt, s);
    gtc::build_tree_graph(ws, f->apos.as<double>(), f->amass.as<double>(), f->n, f->sp, caps, s);
    gtc::build_lists_graph(ws, f->sp, caps, s);
    gtc::join_side(ws, s);  // the cells
    gtc::evaluate_lists_graph(ws.bodies.as<float4>(), ws.cells.as<float4>(),
                              ws.cell_list.as<u32>(), ws.body_list.as<u32>(),
                              ws.groups.as<uint4>(), f->n, sc, static_cast<float>(f->sp.G),
                              static_cast<float>(f->sp.eps * f->sp.eps), f->sp.quadrupole != 0,
                              gtc::EvalOut{ws.out.as<float4>()}, f->counter.as<u32>(), s,
                              ws.eval_shape);
    f->scatter(1, h, &sc->abort, s);
    GTC_CUDA(cudaMemcpyAsync(f->host_sc, sc, sizeof(gtc::Scalars), cudaMemcpyDeviceToHost, s));
  }

  void capture(double dt, cudaStream_t s) {
    // the list slots per system when they fit 32-bit offsets, else one size
    // for every group
    gtc::GraphCaps probe{};
    const bool per_system = f->size_graph_slots(probe, headroom, s);
    reserve_graph(f->ws, *f->host_sc, headroom, f->n, caps, per_system);
    if (per_system) {
      caps.sys_slots = probe.sys_slots;
      caps.pool_at_cells = probe.pool_at_cells;
      caps.pool_at_bodies = probe.pool_at_bodies;
      caps.pool_cells = probe.pool_cells;
      caps.pool_bodies = probe.pool_bodies;
    }
    GTC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      record(dt, s);
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      (void)cudaGetLastError();
      throw;
    }
    GTC_CUDA(cudaStreamEndCapture(s, &graph));
    GTC_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  }

  // After a replay and its synchronisation: true if the step was redone
  // eagerly (the graph must be captured again).
  bool finish(double dt, cudaStream_t s) {
    gtc::Workspace &ws = f->ws;
    const gtc::Scalars &hs = *f->host_sc;
    gtc::check_device_error(hs.error);
    if (hs.abort) {
      f->solve(1, 0.5 * dt, s);
      return true;
    }
    ws.n_nodes = hs.n_nodes;
    ws.n_groups = hs.n_groups;
    ws.n_cell_list = hs.n_cell_list;
    ws.n_body_list = hs.n_body_list;
    ws.gapped = true;  // replays walk once into the captured slots
    ws.lists_unordered = ws.walk_warps;
    ws.list_passes = 1;
    return false;
  }
};

// What a kept forest graph depends on: the systems' arrays, sizes and
// parameters, dt and the forest options.
std::vector<u64> forest_key(const gtc_ensemble *e, const std::vector<gtc::ForestSystem> &fs,
                            double dt) {
  std::vector<u64> k;
  auto d = [&](double v) {
    u64 b;
    std::memcpy(&b, &v, sizeof b);
    k.push_back(b);
  };
  d(dt);
  d(e->forest_headroom);
  k.push_back(static_cast<u64>(static_cast<int64_t>(e->forest_walk)));
  for (const gtc::ForestSystem &f : fs) {
    for (const void *p : {static_cast<const void *>(f.pos), static_cast<const void *>(f.vel),
                          static_cast<const void *>(f.acc), static_cast<const void *>(f.pot),
                          static_cast<const void *>(f.mass)})
      k.push_back(reinterpret_cast<std::uintptr_t>(p));
    k.push_back(f.n);
    d(f.sp.G);
    d(f.sp.theta);
    d(f.sp.eps);
    k.push_back((static_cast<u64>(f.sp.quadrupole) << 48) ^ (static_cast<u64>(f.sp.group_size) << 32) ^
                (static_cast<u64>(f.sp.leaf_size) << 16) ^ static_cast<u64>(f.sp.pack));
  }
  return k;
}

// The ensemble's leapfrog as one forest, eager or with every step replayed
// from one CUDA graph; afterwards each system's context holds its
// interaction counts of the last step's lists. A graph is kept for the next
// call: one on the same systems, parameters and dt without priming replays
// it at once (its positions and masses gathered again); any eager solve
// first drops it, as the buffers it points into may be reallocated.
void leapfrog_forest(gtc_ensemble *e, const std::vector<gtc::ForestSystem> &fs, double dt,
                     u64 steps, bool prime, bool graph) {
  if (!e->forest) e->forest = std::make_unique<gtc::ForestRun>();
  gtc::ForestRun &f = *e->forest;
  cudaStream_t s = e->main;
  std::vector<u64> key = forest_key(e, fs, dt);
  const bool kept = graph && !prime && e->forest_graph && e->forest_graph->exec &&
                    e->forest_key == key;
  if (!kept) {
    e->forest_graph.reset();
    e->forest_key.clear();
    f.setup(fs, s);
    f.ws.walk_mode = e->forest_walk;
  } else {
    f.gather(s);
  }
  u64 replays = 0;
  if (!graph) {
    if (prime) f.solve(0, 0.0, s);
    for (u64 k = 0; k < steps; ++k) f.step(dt, s);
  } else {
    if (!kept) {
      // an eager solve sizes the buffers (with prime, the priming forces)
      f.solve(0, 0.0, s, prime);
      e->forest_graph = std::make_unique<ForestGraph>();
      e->forest_graph->f = &f;
      e->forest_graph->headroom = e->forest_headroom;
      e->forest_key = std::move(key);
    }
    ForestGraph &fg = *e->forest_graph;
    try {
      for (u64 k = 0; k < steps; ++k) {
        if (!fg.exec) fg.capture(dt, s);
        GTC_CUDA(cudaGraphLaunch(fg.exec, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        if (fg.finish(dt, s)) fg.drop();
        else ++replays;
      }
    } catch (...) {
      e->forest_graph.reset();
      e->forest_key.clear();
      throw;
    }
  }
  const std::vector<gtc::ForestSystemStats> st = f.system_stats(s);
  for (std::size_t k = 0; k < e->ctx.size(); ++k) {
    gtc_stats &c = e->ctx[k]->stats;
    c = gtc_stats{};
    c.cell_interactions = st[k].cell_interactions;
    c.body_interactions = st[k].body_interactions;
    c.n_groups = static_cast<u32>(st[k].groups);
    c.max_list = st[k].max_list;
    c.criterion_used = GTC_CRITERION_THETA;
    c.list_passes = f.ws.list_passes;
    c.graph_steps = static_cast<u32>(replays);
    e->ctx[k]->have_group = false;  // the lists are the forest's
  }
}

}  // namespace

extern "C" {

void gtc_sample_indices(uint64_t n, uint64_t m, uint64_t seed, uint64_t *out) {
  std::vector<std::size_t> s(n);
  std::iota(s.begin(), s.end(), std::size_t{0});
  std::mt19937_64 engine(seed);
  std::shuffle(s.begin(), s.end(), engine);
  for (uint64_t k = 0; k < std::min(m, n); ++k) out[k] = s[k];
}

const char *gtc_status_name(gtc_status s) {
  switch (s) {
    case GTC_OK: return "ok";
    case GTC_INVALID_ARGUMENT: return "invalid argument";
    case GTC_RUNTIME_ERROR: return "runtime error";
    case GTC_NO_DEVICE: return "no device";
    case GTC_OUT_OF_MEMORY: return "out of memory";
  }
  return "unknown";
}

gtc_status gtc_create(gtc_context **out, int device) {
  if (!out) return GTC_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    (void)cudaGetLastError();
    g_create_error = std::string("cuda: no GPU device available") +
                     (e != cudaSuccess ? std::string(" (") + cudaGetErrorString(e) + ")" : "");
    return GTC_NO_DEVICE;
  }
  if (device < 0 || device >= count) {
    g_create_error = "cuda: device index out of range";
    return GTC_INVALID_ARGUMENT;
  }
  gtc_context *ctx = new (std::nothrow) gtc_context;
  if (!ctx) return GTC_OUT_OF_MEMORY;
  ctx->device = device;
  try {
    GTC_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop{};
    GTC_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10)
      throw gtc::RuntimeError(std::string("cuda: this build needs an sm_103 GPU, found ") +
                              prop.name);
    // The context's stream at the greatest priority: work it queues runs
    // before its side stream's (the FP64 moments, which a learned walk on
    // this stream need not wait for) when both have blocks ready.
    int least = 0, greatest = 0;
    GTC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    GTC_CUDA(cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, greatest));
    for (auto &ev : ctx->ev) GTC_CUDA(cudaEventCreate(&ev));
    GTC_CUDA(cudaHostAlloc(&ctx->host_sc, sizeof(gtc::Scalars), cudaHostAllocDefault));
    std::memset(ctx->host_sc, 0, sizeof(gtc::Scalars));
  } catch (const std::exception &ex) {
    g_create_error = ex.what();
    gtc_destroy(ctx);
    return GTC_RUNTIME_ERROR;
  }
  *out = ctx;
  return GTC_OK;
}

void gtc_destroy(gtc_context *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->ws.release_all();
  ctx->counter.release();
  ctx->sample_scratch.release();
  for (gtc::DeviceBuffer *b : {&ctx->samples.feat, &ctx->samples.label, &ctx->samples.pair,
                               &ctx->model, &ctx->net,
                               &ctx->train_scratch, &ctx->cfeat, &ctx->gtol, &ctx->prev_amag})
    b->release();
  ctx->lscratch.release();
  ctx->diag.release();
  for (auto &ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->host_sc) cudaFreeHost(ctx->host_sc);
  if (ctx->lstream) {
    cudaStreamSynchronize(ctx->lstream);
    cudaStreamDestroy(ctx->lstream);
    cudaEventDestroy(ctx->lfork);
    cudaEventDestroy(ctx->ldone);
  }
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *gtc_last_error(const gtc_context *ctx) {
  return ctx ? ctx->error.c_str() : g_create_error.c_str();
}

void *gtc_stream(gtc_context *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

gtc_status gtc_direct(gtc_context *ctx, const gtc_float4 *bodies, const gtc_kernel_params *p,
                      gtc_float4 *out) {
  return guarded(ctx, [&] {
    if (!p) throw gtc::InvalidArgument("kernel parameters are required");
    const u64 n = p->n;
    if (n == 0) return;
    if (!bodies || !out) throw gtc::InvalidArgument("bodies and out are required");
    cudaStream_t s = ctx->stream;
    gtc::Workspace &ws = ctx->ws;
    ws.bodies.ensure(n * 16);
    ws.out.ensure(n * 16);
    GTC_CUDA(cudaMemcpyAsync(ws.bodies.ptr, bodies, n * 16, cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaEventRecord(ctx->ev[2], s));
    gtc::direct_fp32(ws.bodies.as<float4>(), static_cast<u32>(n), p->G, p->eps2,
                     ws.out.as<float4>(), ws.direct_part, s, ws.direct_targets);
    GTC_CUDA(cudaEventRecord(ctx->ev[3], s));
    GTC_CUDA(cudaMemcpyAsync(out, ws.out.ptr, n * 16, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    ctx->stats = gtc_stats{};
    ctx->stats.evaluate_ms = elapsed(ctx->ev[2], ctx->ev[3]);
    ctx->stats.total_ms = ctx->stats.evaluate_ms;
    ctx->stats.body_interactions = n * (n - 1);
  });
}

gtc_status gtc_tree(gtc_context *ctx, const gtc_float4 *bodies, const gtc_cell *cells,
                    uint32_t n_cells, const uint32_t *cell_list, uint64_t n_cell_list,
                    const uint32_t *body_list, uint64_t n_body_list, const gtc_group *groups,
                    const gtc_kernel_params *p, gtc_float4 *out) {
  return guarded(ctx, [&] {
    if (!p) throw gtc::InvalidArgument("kernel parameters are required");
    const u64 n = p->n, ng = p->n_groups;
    if (n == 0 || ng == 0) return;
    if (!bodies || !groups || !out || (n_cells && !cells) || (n_cell_list && !cell_list) ||
        (n_body_list && !body_list))
      throw gtc::InvalidArgument("cuda tree: missing array");
    // The checks the reference makes (metal_backend.mm:218-223), plus bounds
    // on every index, so that no kernel reads outside the arrays.
    for (u64 g = 0; g < ng; ++g) {
      const gtc_group &G = groups[g];
      if (G.end < G.begin || G.end > n)
        throw gtc::InvalidArgument("cuda tree: a group's targets are out of range");
      if (G.end - G.begin > static_cast<u32>(gtc::kMaxGroupSize))
        throw gtc::InvalidArgument("cuda tree: a group has more than 32 targets");
      if (G.cell_end < G.cell_begin || G.cell_end > n_cell_list || G.body_end < G.body_begin ||
          G.body_end > n_body_list)
        throw gtc::InvalidArgument("cuda tree: a group's list range is out of range");
    }
    for (u64 k = 0; k < n_cell_list; ++k)
      if (cell_list[k] >= n_cells) throw gtc::InvalidArgument("cuda tree: cell index out of range");
    for (u64 k = 0; k < n_body_list; ++k)
      if (body_list[k] >= n) throw gtc::InvalidArgument("cuda tree: body index out of range");
    cudaStream_t s = ctx->stream;
    gtc::Workspace &ws = ctx->ws;
    ws.bodies.ensure(n * 16);
    ws.out.ensure(n * 16);
    ws.cells.ensure(std::max<u64>(1, n_cells) * 48);
    ws.cell_list.ensure(std::max<u64>(1, n_cell_list) * 4);
    ws.body_list.ensure(std::max<u64>(1, n_body_list) * 4);
    ws.groups.ensure(ng * gtc::kGroupRecWords * 4);
    GTC_CUDA(cudaMemcpyAsync(ws.bodies.ptr, bodies, n * 16, cudaMemcpyHostToDevice, s));
    if (n_cells) GTC_CUDA(cudaMemcpyAsync(ws.cells.ptr, cells, n_cells * 48ull, cudaMemcpyHostToDevice, s));
    if (n_cell_list)
      GTC_CUDA(cudaMemcpyAsync(ws.cell_list.ptr, cell_list, n_cell_list * 4, cudaMemcpyHostToDevice, s));
    if (n_body_list)
      GTC_CUDA(cudaMemcpyAsync(ws.body_list.ptr, body_list, n_body_list * 4, cudaMemcpyHostToDevice, s));
    std::vector<uint4> rec(4 * ng);
    for (u64 g = 0; g < ng; ++g) {
      const gtc_group &G = groups[g];
      gtc::store_group_rec(rec.data(), g, G.begin, G.end,
                           gtc::one_segment(G.cell_begin, G.cell_end - G.cell_begin),
                           gtc::one_segment(G.body_begin, G.body_end - G.body_begin));
    }
    GTC_CUDA(cudaMemcpyAsync(ws.groups.ptr, rec.data(), ng * 64, cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaStreamSynchronize(s));  // rec is released at the end of scope
    GTC_CUDA(cudaMemsetAsync(ws.out.ptr, 0, n * 16, s));
    ctx->counter.ensure(sizeof(u32));
    GTC_CUDA(cudaEventRecord(ctx->ev[2], s));
    gtc::evaluate_lists(ws.bodies.as<float4>(), ws.cells.as<float4>(), ws.cell_list.as<u32>(),
                        ws.body_list.as<u32>(), ws.groups.as<uint4>(), ng, p->G, p->eps2,
                        p->quadrupole != 0, gtc::EvalOut{ws.out.as<float4>()},
                        ctx->counter.as<u32>(), s);
    GTC_CUDA(cudaEventRecord(ctx->ev[3], s));
    GTC_CUDA(cudaMemcpyAsync(out, ws.out.ptr, n * 16, cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    ctx->have_group = false;
    ws.gapped = false;
    ctx->stats = gtc_stats{};
    ctx->stats.evaluate_ms = elapsed(ctx->ev[2], ctx->ev[3]);
    ctx->stats.total_ms = ctx->stats.evaluate_ms;
  });
}

gtc_status gtc_group_force_device(gtc_context *ctx, const double *pos, const double *mass,
                                  uint64_t n, const gtc_gravity_params *gp, double *acc,
                                  double *pot) {
  return guarded(ctx, [&] {
    const gtc::SolverParams sp = check_params(gp, true);
    if (n > 0 && (!pos || !mass || !acc || !pot))
      throw gtc::InvalidArgument("pos, mass, acc and pot are required");
    group_force(ctx, pos, mass, n, sp, acc, pot);
  });
}

gtc_status gtc_group_force(gtc_context *ctx, const double *pos, const double *mass, uint64_t n,
                           const gtc_gravity_params *gp, double *acc, double *pot) {
  return guarded(ctx, [&] {
    const gtc::SolverParams sp = check_params(gp, true);
    if (n > 0 && (!pos || !mass || !acc || !pot))
      throw gtc::InvalidArgument("pos, mass, acc and pot are required");
    gtc::Workspace &ws = ctx->ws;
    cudaStream_t s = ctx->stream;
    const u64 nn = std::max<u64>(n, 1);
    ws.pos.ensure(nn * 24);
    ws.mass.ensure(nn * 8);
    ws.acc.ensure(nn * 24);
    ws.pot.ensure(nn * 8);
    if (n) {
      GTC_CUDA(cudaMemcpyAsync(ws.pos.ptr, pos, n * 24, cudaMemcpyHostToDevice, s));
      GTC_CUDA(cudaMemcpyAsync(ws.mass.ptr, mass, n * 8, cudaMemcpyHostToDevice, s));
    }
    group_force(ctx, ws.pos.as<double>(), ws.mass.as<double>(), n, sp, ws.acc.as<double>(),
                ws.pot.as<double>());
    if (n) {
      GTC_CUDA(cudaMemcpyAsync(acc, ws.acc.ptr, n * 24, cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaMemcpyAsync(pot, ws.pot.ptr, n * 8, cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaStreamSynchronize(s));
    }
  });
}

gtc_status gtc_direct_force_device(gtc_context *ctx, const double *pos, const double *mass,
                                   uint64_t n, const gtc_gravity_params *gp, double *acc,
                                   double *pot) {
  return guarded(ctx, [&] {
    const gtc::SolverParams sp = check_params(gp, false);
    if (n > 0 && (!pos || !mass || !acc || !pot))
      throw gtc::InvalidArgument("pos, mass, acc and pot are required");
    direct_force(ctx, pos, mass, n, sp, acc, pot);
    if (n) {
      gtc::k_unpack_direct<<<gtc::ceil_div(n, 256), 256, 0, ctx->stream>>>(
          ctx->ws.out.as<float4>(), static_cast<u32>(n), acc, pot);
      GTC_LAUNCH_CHECK();
      GTC_CUDA(cudaStreamSynchronize(ctx->stream));
    }
  });
}

gtc_status gtc_direct_force(gtc_context *ctx, const double *pos, const double *mass, uint64_t n,
                            const gtc_gravity_params *gp, double *acc, double *pot) {
  return guarded(ctx, [&] {
    const gtc::SolverParams sp = check_params(gp, false);
    if (n > 0 && (!pos || !mass || !acc || !pot))
      throw gtc::InvalidArgument("pos, mass, acc and pot are required");
    gtc::Workspace &ws = ctx->ws;
    cudaStream_t s = ctx->stream;
    const u64 nn = std::max<u64>(n, 1);
    ws.pos.ensure(nn * 24);
    ws.mass.ensure(nn * 8);
    ws.acc.ensure(nn * 24);
    ws.pot.ensure(nn * 8);
    if (n) {
      GTC_CUDA(cudaMemcpyAsync(ws.pos.ptr, pos, n * 24, cudaMemcpyHostToDevice, s));
      GTC_CUDA(cudaMemcpyAsync(ws.mass.ptr, mass, n * 8, cudaMemcpyHostToDevice, s));
    }
    direct_force(ctx, ws.pos.as<double>(), ws.mass.as<double>(), n, sp, ws.acc.as<double>(),
                 ws.pot.as<double>());
    if (n) {
      gtc::k_unpack_direct<<<gtc::ceil_div(n, 256), 256, 0, s>>>(
          ws.out.as<float4>(), static_cast<u32>(n), ws.acc.as<double>(), ws.pot.as<double>());
      GTC_LAUNCH_CHECK();
      GTC_CUDA(cudaMemcpyAsync(acc, ws.acc.ptr, n * 24, cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaMemcpyAsync(pot, ws.pot.ptr, n * 8, cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaStreamSynchronize(s));
    }
  });
}

gtc_status gtc_tree_force_device(gtc_context *ctx, const double *pos, const double *mass,
                                 uint64_t n, const gtc_gravity_params *gp, double *acc,
                                 double *pot) {
  return guarded(ctx, [&] {
    const gtc::SolverParams sp = check_params(gp, false);
    if (!(sp.theta > 0)) throw gtc::InvalidArgument("theta must be positive");
    if (n > 0 && (!pos || !mass || !acc || !pot))
      throw gtc::InvalidArgument("pos, mass, acc and pot are required");
    tree_force(ctx, pos, mass, n, sp, acc, pot);
  });
}

gtc_status gtc_tree_force(gtc_context *ctx, const double *pos, const double *mass, uint64_t n,
                          const gtc_gravity_params *gp, double *acc, double *pot) {
  return guarded(ctx, [&] {
    const gtc::SolverParams sp = check_params(gp, false);
    if (!(sp.theta > 0)) throw gtc::InvalidArgument("theta must be positive");
    if (n > 0 && (!pos || !mass || !acc || !pot))
      throw gtc::InvalidArgument("pos, mass, acc and pot are required");
    gtc::Workspace &ws = ctx->ws;
    cudaStream_t s = ctx->stream;
    const u64 nn = std::max<u64>(n, 1);
    ws.pos.ensure(nn * 24);
    ws.mass.ensure(nn * 8);
    ws.acc.ensure(nn * 24);
    ws.pot.ensure(nn * 8);
    if (n) {
      GTC_CUDA(cudaMemcpyAsync(ws.pos.ptr, pos, n * 24, cudaMemcpyHostToDevice, s));
      GTC_CUDA(cudaMemcpyAsync(ws.mass.ptr, mass, n * 8, cudaMemcpyHostToDevice, s));
    }
    tree_force(ctx, ws.pos.as<double>(), ws.mass.as<double>(), n, sp, ws.acc.as<double>(),
               ws.pot.as<double>());
    if (n) {
      GTC_CUDA(cudaMemcpyAsync(acc, ws.acc.ptr, n * 24, cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaMemcpyAsync(pot, ws.pot.ptr, n * 8, cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaStreamSynchronize(s));
    }
  });
}

gtc_status gtc_direct_fp64_device(gtc_context *ctx, const double *pos, const double *mass,
                                  uint64_t n, const uint64_t *idx, uint64_t m, double G,
                                  double eps, double *acc, double *pot) {
  return guarded(ctx, [&] {
    if (m > 0 && (!pos || !mass || !idx || !acc || !pot))
      throw gtc::InvalidArgument("pos, mass, idx, acc and pot are required");
    gtc::direct_fp64_sample(pos, mass, n, idx, m, G, eps, acc, pot, ctx->sample_scratch,
                            ctx->stream);
    GTC_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

gtc_status gtc_set_option(gtc_context *ctx, const char *name, double value) {
  return guarded(ctx, [&] {
    const std::string key = name ? name : "";
    if (!std::isfinite(value)) throw gtc::InvalidArgument("option values must be finite");
    if (key == "walk_split_depth") {
      if (value != std::floor(value) || value < 0 || value > 2)
        throw gtc::InvalidArgument("walk_split_depth must be 0, 1 or 2");
      ctx->ws.walk_split_depth = static_cast<int>(value);
    } else if (key == "learned_guard_theta") {
      if (!(value > 0)) throw gtc::InvalidArgument("learned_guard_theta must be positive");
      ctx->guard_theta = value;
    } else if (key == "learned_band") {
      ctx->band_override = value;
    } else if (key == "learned_walk_budget" || key == "learned_pair_budget") {
      if (value != std::floor(value) || value < 0 || value > 4294967295.0)
        throw gtc::InvalidArgument(key + " must be a whole number of nodes >= 0");
      (key == "learned_walk_budget" ? ctx->walk_budget : ctx->pair_budget) =
          static_cast<gtc::u32>(value);
    } else if (key == "learned_read_every_round") {
      if (value != 0 && value != 1)
        throw gtc::InvalidArgument("learned_read_every_round must be 0 or 1");
      ctx->read_every_round = value != 0;
    } else if (key == "graph_headroom") {
      if (!(value >= 0) || value > 4) throw gtc::InvalidArgument("graph_headroom must be 0..4");
      ctx->graph_headroom = value;
    } else if (key == "learned_warps") {
      if (value != 0 && value != 1 && value != -1)
        throw gtc::InvalidArgument("learned_warps must be -1, 0 or 1");
      ctx->learned_warps = static_cast<int>(value);
      ctx->lscratch.release();  // slots sized for the other layout
    } else if (key == "walk_warps") {
      if (value != 0 && value != 1 && value != -1)
        throw gtc::InvalidArgument("walk_warps must be -1, 0 or 1");
      ctx->ws.walk_mode = static_cast<int>(value);
      ctx->ws.slot_cells = 0;  // slots sized by the other walk would not fit: count first
    } else if (key == "eval_pairs") {
      if (value != 1 && value != 2) throw gtc::InvalidArgument("eval_pairs must be 1 or 2");
      ctx->ws.eval_shape.pairs = static_cast<int>(value);
    } else if (key == "eval_pass_cost") {
      if (!(value >= 1 && value <= 256 && value == static_cast<double>(static_cast<int>(value))))
        throw gtc::InvalidArgument("eval_pass_cost must be a whole number in 1..256");
      ctx->ws.eval_shape.pass_cost = static_cast<gtc::u32>(value);
    } else if (key == "direct_targets") {
      if (value != 2 && value != 4) throw gtc::InvalidArgument("direct_targets must be 2 or 4");
      ctx->ws.direct_targets = static_cast<int>(value);
    } else if (key == "stage_events") {
      if (value != 0 && value != 1) throw gtc::InvalidArgument("stage_events must be 0 or 1");
      ctx->ws.stage_on = value != 0;
    } else {
      throw gtc::InvalidArgument("unknown option '" + key + "'");
    }
  });
}

gtc_status gtc_measure_fp32_peak(gtc_context *ctx, double *tflops) {
  return guarded(ctx, [&] {
    if (!tflops) throw gtc::InvalidArgument("tflops is required");
    *tflops = gtc::fp32_peak_tflops(ctx->stream);
  });
}

// ---------------------------------------------------- time integration

gtc_status gtc_leapfrog_device(gtc_context *ctx, double *pos, double *vel, const double *mass,
                               double *acc, double *pot, uint64_t n,
                               const gtc_gravity_params *gp, int solver, double dt,
                               uint64_t steps, int prime, int graph) {
  return guarded(ctx, [&] {
    if (solver != GTC_SOLVER_GROUP && solver != GTC_SOLVER_DIRECT)
      throw gtc::InvalidArgument("unknown solver");
    const gtc::SolverParams sp = check_params(gp, solver == GTC_SOLVER_GROUP);
    if (!std::isfinite(dt)) throw gtc::InvalidArgument("dt must be finite");
    if (n == 0) return;
    if (!pos || !vel || !mass || !acc || !pot)
      throw gtc::InvalidArgument("pos, vel, mass, acc and pot are required");
    cudaStream_t s = ctx->stream;
    auto forces = [&] {
      if (solver == GTC_SOLVER_GROUP) {
        group_force(ctx, pos, mass, n, sp, acc, pot);
      } else {
        direct_force(ctx, pos, mass, n, sp, acc, pot);
        gtc::k_unpack_direct<<<gtc::ceil_div(n, 256), 256, 0, s>>>(ctx->ws.out.as<float4>(),
                                                                  static_cast<u32>(n), acc, pot);
        GTC_LAUNCH_CHECK();
      }
    };
    if (graph && solver == GTC_SOLVER_GROUP && sp.criterion == GTC_CRITERION_THETA) {
      leapfrog_graph(ctx, pos, vel, mass, acc, pot, n, sp, dt, steps, prime != 0);
      return;
    }
    if (prime) forces();
    const double h = 0.5 * dt;
    for (u64 k = 0; k < steps; ++k) {
      gtc::kick_drift(pos, vel, acc, n, h, dt, s);
      forces();
      gtc::kick(vel, acc, n, h, s);
    }
    GTC_CUDA(cudaStreamSynchronize(s));
  });
}

gtc_status gtc_diagnostics_device(gtc_context *ctx, const double *pos, const double *vel,
                                  const double *mass, const double *pot, uint64_t n,
                                  double time, gtc_diagnostics *out) {
  return guarded(ctx, [&] {
    if (!out) throw gtc::InvalidArgument("out is required");
    if (n > 0 && (!pos || !vel || !mass || !pot))
      throw gtc::InvalidArgument("pos, vel, mass and pot are required");
    const size_t bytes = gtc::diagnostics_blocks() * gtc::kDiagTerms * sizeof(double);
    ctx->diag.ensure(bytes);
    std::vector<double> part(bytes / sizeof(double));
    if (n > 0) {
      gtc::diagnostics_launch(pos, vel, mass, pot, n, ctx->diag.as<double>(), ctx->stream);
      GTC_CUDA(cudaMemcpyAsync(part.data(), ctx->diag.ptr, bytes, cudaMemcpyDeviceToHost,
                               ctx->stream));
      GTC_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    gtc::diagnostics_finish(part.data(), time, out);
  });
}

// ---------------------------------------------------- learned criterion

gtc_status gtc_learned_add_samples(gtc_context *ctx, const double *pos, const double *mass,
                                   uint64_t n, const gtc_gravity_params *gp, double theta_gen,
                                   double theta_guard, uint64_t max_new,
                                   uint32_t max_cell_bodies, uint64_t *added) {
  return guarded(ctx, [&] {
    if (!added) throw gtc::InvalidArgument("added is required");
    *added = 0;
    if (!gp) throw gtc::InvalidArgument("gravity parameters are required");
    gtc_gravity_params p = *gp;
    p.criterion = GTC_CRITERION_THETA;  // the groups come from the theta walk's set-up
    const gtc::SolverParams sp = check_params(&p, true);
    if (!(theta_gen > 0) || !(theta_guard > 0))
      throw gtc::InvalidArgument("theta_gen and theta_guard must be positive");
    if (n > 0xffffffffull) throw gtc::RuntimeError("too many particles for the 32 bit GPU indices");
    if (n == 0) return;
    if (!pos || !mass) throw gtc::InvalidArgument("pos and mass are required");
    gtc::Workspace &ws = ctx->ws;
    cudaStream_t s = ctx->stream;
    ws.pos.ensure(n * 24);
    ws.mass.ensure(n * 8);
    GTC_CUDA(cudaMemcpyAsync(ws.pos.ptr, pos, n * 24, cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaMemcpyAsync(ws.mass.ptr, mass, n * 8, cudaMemcpyHostToDevice, s));
    ctx->have_group = false;
    gtc::learned_add_samples(ctx, ws.pos.as<double>(), ws.mass.as<double>(), n, sp, theta_gen,
                             theta_guard, max_new, max_cell_bodies, added);
    if (ctx->host_sc->error & 4u) throw gtc::InvalidArgument("cuda: positions must be finite");
  });
}

gtc_status gtc_learned_sample_count(const gtc_context *ctx, uint64_t *count) {
  if (!ctx || !count) return GTC_INVALID_ARGUMENT;
  *count = ctx->samples.count;
  return GTC_OK;
}

gtc_status gtc_learned_export_samples(gtc_context *ctx, uint64_t first, uint64_t count,
                                      float *feat, float *label, uint32_t *pairs) {
  return guarded(ctx, [&] {
    const gtc::LearnedSet &set = ctx->samples;
    if (first > set.count || count > set.count - first)
      throw gtc::InvalidArgument("sample range out of bounds");
    if (count == 0) return;
    cudaStream_t s = ctx->stream;
    if (feat)
      GTC_CUDA(cudaMemcpyAsync(feat, set.feat.as<float>() + first * gtc::kFeat,
                               count * gtc::kFeat * sizeof(float), cudaMemcpyDeviceToHost, s));
    if (label)
      GTC_CUDA(cudaMemcpyAsync(label, set.label.as<float>() + first, count * sizeof(float),
                               cudaMemcpyDeviceToHost, s));
    if (pairs)
      GTC_CUDA(cudaMemcpyAsync(pairs, set.pair.as<uint2>() + first, count * sizeof(uint2),
                               cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
  });
}

gtc_status gtc_learned_clear_samples(gtc_context *ctx) {
  return guarded(ctx, [&] { ctx->samples.count = 0; });
}

gtc_status gtc_learned_train(gtc_context *ctx, uint64_t steps, uint32_t batch, float lr,
                             uint64_t seed, int init, double *loss) {
  return guarded(ctx, [&] {
    const gtc::LearnedSet &set = ctx->samples;
    if (set.count == 0) throw gtc::InvalidArgument("no training samples");
    if (batch == 0 || batch > (1u << 20)) throw gtc::InvalidArgument("batch must be 1..2^20");
    if (!(lr >= 0) || !std::isfinite(lr)) throw gtc::InvalidArgument("lr must be finite and >= 0");
    if (init || !ctx->have_model) gtc::learned_init_model(ctx, seed);
    const double l = gtc::learned_train_on(ctx, set.feat.as<float>(), set.label.as<float>(),
                                           set.count, steps, batch, lr, seed, nullptr, nullptr);
    gtc::learned_update_band(ctx, 0.99);
    if (loss) *loss = l;
  });
}

gtc_status gtc_learned_gradient(gtc_context *ctx, const float *model, const float *feat,
                                const float *label, uint32_t n, float *grad, double *loss) {
  return guarded(ctx, [&] {
    if (!model || !grad || (n && (!feat || !label)))
      throw gtc::InvalidArgument("model, feat, label and grad are required");
    if (n == 0 || n > (1u << 20)) throw gtc::InvalidArgument("n must be 1..2^20");
    cudaStream_t s = ctx->stream;
    std::vector<float> saved;
    const bool had = ctx->have_model;
    if (had) {
      saved.resize(gtc::kModelFloats);
      GTC_CUDA(cudaMemcpyAsync(saved.data(), ctx->model.ptr, gtc::kModelFloats * sizeof(float),
                               cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaStreamSynchronize(s));
    }
    gtc::DeviceBuffer f, l, idx;
    struct Release {
      gtc::DeviceBuffer *b[3];
      ~Release() {
        for (gtc::DeviceBuffer *x : b) x->release();
      }
    } release{{&f, &l, &idx}};
    f.ensure(static_cast<u64>(n) * gtc::kFeat * sizeof(float));
    l.ensure(static_cast<u64>(n) * sizeof(float));
    idx.ensure(static_cast<u64>(n) * sizeof(u32));
    std::vector<u32> order(n);
    for (u32 i = 0; i < n; ++i) order[i] = i;
    GTC_CUDA(cudaMemcpyAsync(f.ptr, feat, static_cast<u64>(n) * gtc::kFeat * sizeof(float),
                             cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaMemcpyAsync(l.ptr, label, static_cast<u64>(n) * sizeof(float),
                             cudaMemcpyHostToDevice, s));
    GTC_CUDA(cudaMemcpyAsync(idx.ptr, order.data(), static_cast<u64>(n) * sizeof(u32),
                             cudaMemcpyHostToDevice, s));
    gtc::learned_set_model(ctx, model);
    double lv = 0;
    try {
      lv = gtc::learned_train_on(ctx, f.as<float>(), l.as<float>(), n, 1, n, 0.f, 0,
                                 idx.as<u32>(), grad);
    } catch (...) {
      if (had) gtc::learned_set_model(ctx, saved.data());
      else ctx->have_model = false;
      throw;
    }
    if (had) gtc::learned_set_model(ctx, saved.data());
    else ctx->have_model = false;
    if (loss) *loss = lv;
  });
}

gtc_status gtc_learned_set_model(gtc_context *ctx, const float *model) {
  return guarded(ctx, [&] {
    if (!model) throw gtc::InvalidArgument("model is required");
    gtc::learned_set_model(ctx, model);
  });
}

gtc_status gtc_learned_get_model(gtc_context *ctx, float *model) {
  return guarded(ctx, [&] {
    if (!model) throw gtc::InvalidArgument("model is required");
    if (!ctx->have_model) throw gtc::InvalidArgument("the context has no model");
    GTC_CUDA(cudaMemcpyAsync(model, ctx->model.ptr, gtc::kModelFloats * sizeof(float),
                             cudaMemcpyDeviceToHost, ctx->stream));
    GTC_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

gtc_status gtc_learned_predict(gtc_context *ctx, const float *feat, uint64_t n, float *pred) {
  return guarded(ctx, [&] {
    if (n == 0) return;
    if (!feat || !pred) throw gtc::InvalidArgument("feat and pred are required");
    if (!ctx->have_model) throw gtc::InvalidArgument("the context has no model");
    cudaStream_t s = ctx->stream;
    gtc::DeviceBuffer f, p;
    struct Release {
      gtc::DeviceBuffer *b[2];
      ~Release() {
        for (gtc::DeviceBuffer *x : b) x->release();
      }
    } release{{&f, &p}};
    f.ensure(n * gtc::kFeat * sizeof(float));
    p.ensure(n * sizeof(float));
    GTC_CUDA(cudaMemcpyAsync(f.ptr, feat, n * gtc::kFeat * sizeof(float), cudaMemcpyHostToDevice, s));
    gtc::learned_predict(ctx->net.as<gtc::LearnedNet>(), f.as<float>(), n, p.as<float>(), s);
    GTC_CUDA(cudaMemcpyAsync(pred, p.ptr, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
  });
}

// ---------------------------------------------------- ensembles and tuning

gtc_ensemble::~gtc_ensemble() = default;

void gtc_ensemble_destroy(gtc_ensemble *e) {
  if (!e) return;
  cudaSetDevice(e->device);
  if (e->main) cudaStreamSynchronize(e->main);
  e->forest_graph.reset();  // before the forest whose buffers it points into
  for (gtc_context *c : e->ctx) gtc_destroy(c);
  for (cudaEvent_t ev : e->joins)
    if (ev) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->main) cudaStreamDestroy(e->main);
  delete e;
}

gtc_status gtc_ensemble_create(gtc_ensemble **out, int device, uint32_t systems) {
  if (!out) return GTC_INVALID_ARGUMENT;
  *out = nullptr;
  if (systems == 0 || systems > 4096) {
    g_create_error = "an ensemble holds 1..4096 systems";
    return GTC_INVALID_ARGUMENT;
  }
  gtc_ensemble *e = new (std::nothrow) gtc_ensemble;
  if (!e) return GTC_OUT_OF_MEMORY;
  e->device = device;
  for (uint32_t k = 0; k < systems; ++k) {
    gtc_context *c = nullptr;
    const gtc_status st = gtc_create(&c, device);
    if (st != GTC_OK) {
      gtc_ensemble_destroy(e);
      return st;
    }
    e->ctx.push_back(c);
  }
  try {
    GTC_CUDA(cudaSetDevice(device));
    GTC_CUDA(cudaStreamCreateWithFlags(&e->main, cudaStreamNonBlocking));
    GTC_CUDA(cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming));
    e->joins.assign(systems, nullptr);
    for (auto &ev : e->joins) GTC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  } catch (const std::exception &ex) {
    g_create_error = ex.what();
    gtc_ensemble_destroy(e);
    return GTC_RUNTIME_ERROR;
  }
  e->sys.assign(systems, GraphStep{});
  for (uint32_t k = 0; k < systems; ++k) e->sys[k].ctx = e->ctx[k];
  *out = e;
  return GTC_OK;
}

const char *gtc_ensemble_last_error(const gtc_ensemble *e) {
  return e ? e->error.c_str() : g_create_error.c_str();
}

gtc_context *gtc_ensemble_context(gtc_ensemble *e, uint32_t i) {
  return e && i < e->ctx.size() ? e->ctx[i] : nullptr;
}

gtc_status gtc_ensemble_set_system(gtc_ensemble *e, uint32_t i, double *pos, double *vel,
                                   const double *mass, double *acc, double *pot, uint64_t n,
                                   const gtc_gravity_params *gp) {
  return ensemble_guarded(e, [&] {
    if (i >= e->sys.size()) throw gtc::InvalidArgument("system index out of range");
    const gtc::SolverParams sp = check_params(gp, true);
    if (sp.criterion != GTC_CRITERION_THETA)
      throw gtc::InvalidArgument("ensembles use the theta criterion");
    if (n == 0 || !pos || !vel || !mass || !acc || !pot)
      throw gtc::InvalidArgument("every system needs bodies and pos, vel, mass, acc, pot");
    if (n > 0xffffffffull) throw gtc::RuntimeError("too many particles for the 32 bit GPU indices");
    GraphStep &g = e->sys[i];
    g.pos = pos;
    g.vel = vel;
    g.mass = mass;
    g.acc = acc;
    g.pot = pot;
    g.n = n;
    g.sp = sp;
  });
}

gtc_status gtc_ensemble_set_option(gtc_ensemble *e, const char *name, double value) {
  return ensemble_guarded(e, [&] {
    if (!name) throw gtc::InvalidArgument("option name is required");
    const std::string opt(name);
    if (opt == "forest") {
      if (value != -1 && value != 0 && value != 1)
        throw gtc::InvalidArgument("forest is -1 (when eligible), 0 or 1");
      e->forest_mode = static_cast<int>(value);
    } else if (opt == "walk_warps") {
      if (value != -1 && value != 0 && value != 1)
        throw gtc::InvalidArgument("walk_warps is -1 (by group count), 0 or 1");
      e->forest_walk = static_cast<int>(value);
    } else if (opt == "graph_headroom") {
      if (!(value >= 0 && value <= 4)) throw gtc::InvalidArgument("graph_headroom is 0..4");
      e->forest_headroom = value;
    } else {
      throw gtc::InvalidArgument("unknown ensemble option: " + opt);
    }
  });
}

gtc_status gtc_ensemble_leapfrog(gtc_ensemble *e, double dt, uint64_t steps, int prime,
                                 int graph) {
  return ensemble_guarded(e, [&] {
    if (!std::isfinite(dt)) throw gtc::InvalidArgument("dt must be finite");
    for (const GraphStep &g : e->sys)
      if (g.n == 0) throw gtc::InvalidArgument("every system must be set before stepping");
    std::vector<gtc::ForestSystem> fs;
    for (const GraphStep &g : e->sys) {
      gtc::ForestSystem f;
      f.pos = g.pos;
      f.vel = g.vel;
      f.acc = g.acc;
      f.pot = g.pot;
      f.mass = g.mass;
      f.n = g.n;
      f.sp = g.sp;
      fs.push_back(f);
    }
    std::string why;
    const bool can = gtc::ForestRun::eligible(fs, &why);
    if (e->forest_mode == 1 && !can) throw gtc::InvalidArgument("forest: " + why);
    if (e->forest_mode != 0 && can) {
      leapfrog_forest(e, fs, dt, steps, prime != 0, graph != 0);
      return;
    }
    if (graph) {
      leapfrog_graph_systems(e->sys, dt, steps, prime != 0, e->main, e->fork, e->joins);
      return;
    }
    for (GraphStep &g : e->sys)
      if (prime) group_force(g.ctx, g.pos, g.mass, g.n, g.sp, g.acc, g.pot);
    const double h = 0.5 * dt;
    for (u64 k = 0; k < steps; ++k)
      for (GraphStep &g : e->sys) {
        gtc::kick_drift(g.pos, g.vel, g.acc, g.n, h, dt, g.ctx->stream);
        group_force(g.ctx, g.pos, g.mass, g.n, g.sp, g.acc, g.pot);
        gtc::kick(g.vel, g.acc, g.n, h, g.ctx->stream);
      }
    for (GraphStep &g : e->sys) GTC_CUDA(cudaStreamSynchronize(g.ctx->stream));
  });
}

gtc_status gtc_autotune_group(gtc_context *ctx, const double *pos, const double *mass,
                              uint64_t n, const gtc_gravity_params *base,
                              gtc_gravity_params *best, double *best_ms, int *walk_warps) {
  return guarded(ctx, [&] {
    if (!base || !best) throw gtc::InvalidArgument("base and best parameters are required");
    if (n == 0 || !pos || !mass) throw gtc::InvalidArgument("pos and mass are required");
    check_params(base, true);
    gtc::Workspace &ws = ctx->ws;
    ws.acc.ensure(n * 24);
    ws.pot.ensure(n * 8);
    double best_t = 1e300;
    gtc_gravity_params pick = *base;
    int pick_walk = ws.walk_mode;
    const int mode0 = ws.walk_mode;
    for (int gs : {8, 16, 24, 32})
      for (int pack : {0, gs / 2, (3 * gs) / 4, 1})  // off, thresholds, a group's worth
        for (int walk : {0, 1}) {
          gtc_gravity_params p = *base;
          p.group_size = gs;
          p.pack = pack;
          p.criterion = GTC_CRITERION_THETA;
          const gtc::SolverParams sp = check_params(&p, true);
          ws.walk_mode = walk;
          ws.slot_cells = 0;  // slots of another walk or layout: count first
          double t = 0;
          for (int rep = 0; rep < 3; ++rep) {
            group_force(ctx, pos, mass, n, sp, ws.acc.as<double>(), ws.pot.as<double>());
            if (rep > 0) t += ctx->stats.total_ms;  // the first warms up
          }
          if (t / 2 < best_t) {
            best_t = t / 2;
            pick = p;
            pick_walk = walk;
          }
        }
    ws.walk_mode = mode0;
    ws.slot_cells = 0;
    pick.criterion = base->criterion;
    *best = pick;
    if (best_ms) *best_ms = best_t;
    if (walk_warps) *walk_warps = pick_walk;
  });
}

gtc_status gtc_autotune_direct(gtc_context *ctx, const double *pos, const double *mass,
                               uint64_t n, const gtc_gravity_params *gp, int *targets,
                               double *best_ms) {
  return guarded(ctx, [&] {
    if (n == 0 || !pos || !mass || !gp) throw gtc::InvalidArgument("pos, mass and gp are required");
    const gtc::SolverParams sp = check_params(gp, false);
    gtc::Workspace &ws = ctx->ws;
    ws.acc.ensure(n * 24);
    ws.pot.ensure(n * 8);
    double best_t = 1e300;
    int pick = ws.direct_targets;
    for (int k : {2, 4}) {
      ws.direct_targets = k;
      double t = 0;
      for (int rep = 0; rep < 3; ++rep) {
        direct_force(ctx, pos, mass, n, sp, ws.acc.as<double>(), ws.pot.as<double>());
        if (rep > 0) t += ctx->stats.eval_kernel_ms;
      }
      if (t / 2 < best_t) {
        best_t = t / 2;
        pick = k;
      }
    }
    ws.direct_targets = pick;  // the context keeps the winner
    if (targets) *targets = pick;
    if (best_ms) *best_ms = best_t;
  });
}

gtc_status gtc_autotune_eval(gtc_context *ctx, const double *pos, const double *mass,
                             uint64_t n, const gtc_gravity_params *gp, int *pairs,
                             int *pass_cost, double *best_ms) {
  return guarded(ctx, [&] {
    if (n == 0 || !pos || !mass || !gp) throw gtc::InvalidArgument("pos, mass and gp are required");
    const gtc::SolverParams sp = check_params(gp, true);
    if (!sp.quadrupole || !(sp.eps > 0))
      throw gtc::InvalidArgument("the evaluation's tile shape applies to softened quadrupoles");
    gtc::Workspace &ws = ctx->ws;
    ws.acc.ensure(n * 24);
    ws.pot.ensure(n * 8);
    // the lists first (and the one-pass walk's slots): a solve with the
    // current shape, untimed
    group_force(ctx, pos, mass, n, sp, ws.acc.as<double>(), ws.pot.as<double>());
    double best_t = 1e300;
    gtc::EvalShape pick = ws.eval_shape;
    for (int k : {2, 1})
      for (gtc::u32 c : {24u, 8u, 16u, 32u, 48u}) {
        ws.eval_shape = gtc::EvalShape{k, c};
        double t = 0;
        for (int rep = 0; rep < 3; ++rep) {
          group_force(ctx, pos, mass, n, sp, ws.acc.as<double>(), ws.pot.as<double>());
          if (rep > 0) t += ctx->stats.eval_kernel_ms;  // the first warms up
        }
        if (t / 2 < best_t) {
          best_t = t / 2;
          pick = ws.eval_shape;
        }
      }
    ws.eval_shape = pick;  // the context keeps the winner
    if (pairs) *pairs = pick.pairs;
    if (pass_cost) *pass_cost = static_cast<int>(pick.pass_cost);
    if (best_ms) *best_ms = best_t;
  });
}

gtc_status gtc_get_stats(const gtc_context *ctx, gtc_stats *out) {
  if (!ctx || !out) return GTC_INVALID_ARGUMENT;
  *out = ctx->stats;
  return GTC_OK;
}

gtc_status gtc_get_stage_times(gtc_context *ctx, gtc_stage_times *out) {
  return guarded(ctx, [&] {
    if (!out) throw gtc::InvalidArgument("out is required");
    const gtc::Workspace &ws = ctx->ws;
    auto span = [&](int a, int b) -> double {
      if (!ws.stage_hit[a] || !ws.stage_hit[b]) return -1.0;
      return elapsed(ws.stage_ev[a], ws.stage_ev[b]);
    };
    using W = gtc::Workspace;
    *out = gtc_stage_times{};
    out->build_ms = span(W::kStBuild, W::kStMomW);
    out->keys_ms = span(W::kStBuild, W::kStSort0);
    out->sort_ms = span(W::kStSort0, W::kStSort1);
    out->topology_ms = span(W::kStSort1, W::kStTopo);
    out->moments_ms = span(W::kStMom0, W::kStMomW);
    out->quad_ms = span(W::kStMomW, W::kStMom1);
    out->walk_ms = span(W::kStWalk0, W::kStWalk1);
    out->sort_passes = static_cast<uint32_t>(ws.sort_passes);
  });
}

gtc_status gtc_group_sizes(const gtc_context *ctx, uint64_t *n_bodies, uint64_t *n_nodes,
                           uint64_t *n_groups, uint64_t *n_cell_list, uint64_t *n_body_list) {
  if (!ctx) return GTC_INVALID_ARGUMENT;
  const bool ok = ctx->have_group;
  if (n_bodies) *n_bodies = ok ? ctx->ws.n : 0;
  if (n_nodes) *n_nodes = ok ? ctx->ws.n_nodes : 0;
  if (n_groups) *n_groups = ok ? ctx->ws.n_groups : 0;
  if (n_cell_list) *n_cell_list = ok ? ctx->ws.n_cell_list : 0;
  if (n_body_list) *n_body_list = ok ? ctx->ws.n_body_list : 0;
  return ok ? GTC_OK : GTC_INVALID_ARGUMENT;
}

gtc_status gtc_group_export(gtc_context *ctx, gtc_node *nodes, uint64_t *order,
                            gtc_float4 *bodies, gtc_cell *cells, gtc_group *groups,
                            uint32_t *cell_list, uint32_t *body_list, gtc_float4 *out) {
  return guarded(ctx, [&] {
    if (!ctx->have_group) throw gtc::InvalidArgument("no grouped solve to export");
    gtc::Workspace &ws = ctx->ws;
    const u64 n = ws.n, m = ws.n_nodes;
    auto get = [&](void *dst, const gtc::DeviceBuffer &src, u64 bytes) {
      if (dst && bytes) GTC_CUDA(cudaMemcpy(dst, src.ptr, bytes, cudaMemcpyDeviceToHost));
    };
    GTC_CUDA(cudaStreamSynchronize(ctx->stream));
    if (nodes && m) {
      std::vector<double2> geom(2 * m), mom(2 * m);
      std::vector<double2> quad(3 * m);
      std::vector<double> delta(m);
      std::vector<u32> nb(m), ne(m), sk(m), par(m);
      std::vector<gtc::u8> dep(m), nch(m);
      get(geom.data(), ws.geom, 2 * m * sizeof(double2));
      get(mom.data(), ws.mom, 2 * m * sizeof(double2));
      get(quad.data(), ws.quad, 3 * m * sizeof(double2));
      get(delta.data(), ws.delta, m * 8);
      get(nb.data(), ws.nbegin, m * 4);
      get(ne.data(), ws.nend, m * 4);
      get(sk.data(), ws.skip, m * 4);
      get(par.data(), ws.parent, m * 4);
      get(dep.data(), ws.depth, m);
      get(nch.data(), ws.nchild, m);
      for (u64 p = 0; p < m; ++p) {
        gtc_node &o = nodes[p];
        o.center[0] = geom[2 * p].x;
        o.center[1] = geom[2 * p].y;
        o.center[2] = geom[2 * p + 1].x;
        o.half = geom[2 * p + 1].y;
        o.com[0] = mom[2 * p].x;
        o.com[1] = mom[2 * p].y;
        o.com[2] = mom[2 * p + 1].x;
        o.mass = mom[2 * p + 1].y;
        o.quad[0] = quad[3 * p].x;
        o.quad[1] = quad[3 * p].y;
        o.quad[2] = quad[3 * p + 1].x;
        o.quad[3] = quad[3 * p + 1].y;
        o.quad[4] = quad[3 * p + 2].x;
        o.quad[5] = quad[3 * p + 2].y;
        o.delta = delta[p];
        o.begin = nb[p];
        o.end = ne[p];
        o.skip = sk[p];
        o.parent = par[p];
        o.depth = dep[p];
        o.n_children = nch[p];
      }
    }
    if (order && n) {
      std::vector<u32> idx(n);
      get(idx.data(), ws.idx, n * 4);
      for (u64 k = 0; k < n; ++k) order[k] = idx[k];
    }
    get(bodies, ws.bodies, n * 16);
    get(cells, ws.cells, m * 48);
    if (groups || cell_list || body_list) {
      // the lists as the reference lays them out: each group's segments
      // concatenated, the groups back to back
      const u64 ng = ws.n_groups;
      std::vector<uint4> rec(4 * ng);
      get(rec.data(), ws.groups, ng * 64);
      u64 cext = 0, bext = 0;
      for (u64 g = 0; g < ng; ++g) {
        const gtc::SegView c = gtc::cell_segs(rec[4 * g + 1], rec[4 * g + 2]);
        const gtc::SegView b = gtc::body_segs(rec[4 * g + 2], rec[4 * g + 3]);
        const uint4 q3 = rec[4 * g + 3];
        cext = std::max<u64>({cext, u64{c.s0} + c.n0, u64{c.s1} + c.n1,
                              u64{c.s2} + rec[4 * g + 2].y});
        bext = std::max<u64>({bext, u64{b.s0} + b.n0, u64{b.s1} + b.n1, u64{b.s2} + q3.w});
      }
      std::vector<u32> cl(cell_list ? cext : 0), bl(body_list ? bext : 0);
      get(cl.data(), ws.cell_list, cl.size() * 4);
      get(bl.data(), ws.body_list, bl.size() * 4);
      u64 c = 0, b = 0;
      for (u64 g = 0; g < ng; ++g) {
        const uint4 q0 = rec[4 * g];
        const gtc::SegView cs = gtc::cell_segs(rec[4 * g + 1], rec[4 * g + 2]);
        const gtc::SegView bs = gtc::body_segs(rec[4 * g + 2], rec[4 * g + 3]);
        if (cell_list) {
          for (u32 e = 0; e < q0.z; ++e) cell_list[c + e] = cl[cs.at(e)];
          // the reference visits nodes in increasing index (node numbering)
          if (ws.lists_unordered) std::sort(cell_list + c, cell_list + c + q0.z);
        }
        if (body_list) {
          for (u32 e = 0; e < q0.w; ++e) body_list[b + e] = bl[bs.at(e)];
          // the walk by warps reaches bodies in its own order: canonical
          if (ws.lists_unordered) std::sort(body_list + b, body_list + b + q0.w);
        }
        if (groups) {
          gtc_group &o = groups[g];
          o.begin = q0.x;
          o.end = q0.y;
          o.cell_begin = static_cast<uint32_t>(c);
          o.cell_end = static_cast<uint32_t>(c + q0.z);
          o.body_begin = static_cast<uint32_t>(b);
          o.body_end = static_cast<uint32_t>(b + q0.w);
          o.pad0 = o.pad1 = 0;
        }
        c += q0.z;
        b += q0.w;
      }
    }
    get(out, ws.out, n * 16);
  });
}

}  // extern "C"
