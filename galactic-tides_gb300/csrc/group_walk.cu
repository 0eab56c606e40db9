// Group choice and grouped walk on the device, producing the reference's
// lists exactly (src/group_lists.cpp:65-207). Compiled with -fmad=false: the
// FP64 opening test rounds every product and sum separately, as the
// reference's x86-64 build does, so every accept/open decision matches.
//
// Groups. The reference visits the tree depth first and emits, for every
// node with more than group_size bodies, its children in order: small ones
// (merged with their preceding small siblings while the run fits, when
// packing), large leaves cut into chunks, large inner nodes recursed into.
// Each such node's contribution depends only on its own children, so one
// thread per node marks where its groups start in tree order; a scan turns
// the marks into the group array, which comes out in tree order as in the
// reference.
//
// Walk. One thread per group traverses the nodes in their stored order
// (the order the reference's stack pops them): accept -> record and jump to
// the node's skip link, leaf -> record its bodies and jump, otherwise step
// to the next node (its last child). A counting pass sizes the lists; after
// the offsets are scanned a second pass writes them. Once a walk has
// measured the longest lists, later walks run once, writing each group's
// lists into fixed per-group slots (half as long again), and fall back to the
// two passes when a list outgrows its slot.

#include <algorithm>

#include "learned.cuh"
#include "pipeline.cuh"

namespace gtc {
namespace {

constexpr int kT = 256;

// Graph replays pass the abort word of their Scalars and counts on the
// device; eager calls pass null and their host-known sizes.
__device__ __forceinline__ bool aborted(const u32 *abort) { return abort && *abort; }
__device__ __forceinline__ u32 bounded(u32 cap, const u32 *dev) {
  return dev ? min(cap, *dev) : cap;
}

struct NodeView {
  const u32 *nbegin, *nend, *skip;
  const u8 *isleaf;
};

__global__ void __launch_bounds__(kT)
    k_group_marks(NodeView nv, u32 m, u32 n, u32 gs, int pack, u32 *mark,
                  const u32 *m_dev = nullptr, const u32 *abort = nullptr) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || p >= bounded(m, m_dev)) return;
  const u32 size = nv.nend[p] - nv.nbegin[p];
  if (p == 0 && (size <= gs || nv.isleaf[0])) {
    for (u32 c = 0; c < n; c += gs) mark[c] = 1;
    return;
  }
  if (nv.isleaf[p] || size <= gs) return;
  // children, last octant first
  u32 ch[8];
  int nc = 0;
  for (u32 c = p + 1; c < nv.skip[p] && nc < 8; c = nv.skip[c]) ch[nc++] = c;
  bool open = false;
  u32 run_begin = 0, run_end = 0;
  for (int j = nc - 1; j >= 0; --j) {
    const u32 c = ch[j];
    const u32 cb = nv.nbegin[c], ce = nv.nend[c], cc = ce - cb;
    if (cc <= gs) {
      if (pack && open && (run_end - run_begin) + cc <= gs) {
        run_end = ce;
      } else {
        if (open) mark[run_begin] = 1;
        run_begin = cb;
        run_end = ce;
        open = true;
      }
    } else {
      if (open) mark[run_begin] = 1;
      open = false;
      if (nv.isleaf[c])
        for (u32 x = cb; x < ce; x += gs) mark[x] = 1;
    }
  }
  if (open) mark[run_begin] = 1;
}

__global__ void __launch_bounds__(kT)
    k_group_ranges(const u32 *mark, const u32 *scan, u32 n, u32 *gbegin, u32 *gend,
                   const u32 *abort = nullptr) {
  const u32 b = blockIdx.x * kT + threadIdx.x;
  if (b >= n || aborted(abort) || !mark[b]) return;
  const u32 g = scan[b];
  gbegin[g] = b;
  if (g > 0) gend[g - 1] = b;
}

__global__ void k_last_end(const Scalars *sc, u32 n, u32 *gend) {
  if (sc->abort) return;
  if (sc->n_groups > 0 && sc->n_groups <= n) gend[sc->n_groups - 1] = n;
}

// A graph replay's checks around the one-pass walk (bit 8): more groups
// than the captured slots cover (before), overflow pools too small for the
// lists that outgrew their slots (after).
__global__ void k_check_groups_graph(Scalars *sc, u32 groups) {
  if (sc->n_groups > groups) sc->abort |= 8u;
}
__global__ void k_check_slots_graph(Scalars *sc) {
  if (sc->list_overflow) sc->abort |= 8u;
}

// Group bounding box (group_lists.cpp:125-131): centre and half-extent in
// FP64, and the same in FP32 with the centre taken relative to the root
// centre (the frame of the FP32 walk records).
__global__ void __launch_bounds__(kT)
    k_group_box(const u32 *gbegin, const u32 *gend, u32 ng, const double *tpos,
                const TreeRoot *root, double *gbox, float *gboxf, const u32 *ng_dev = nullptr,
                const u32 *abort = nullptr) {
  // gboxf per group: centre (3), half-extent (3), magnitude bound, pad
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || g >= bounded(ng, ng_dev)) return;
  const u32 b0 = gbegin[g], b1 = gend[g];
  double lo[3], hi[3];
  for (int a = 0; a < 3; ++a) lo[a] = hi[a] = tpos[3ull * b0 + a];
  for (u32 k = b0; k < b1; ++k)
    for (int a = 0; a < 3; ++a) {
      const double v = tpos[3ull * k + a];
      lo[a] = v < lo[a] ? v : lo[a];
      hi[a] = hi[a] < v ? v : hi[a];
    }
  float gmax = 0.f, hmax = 0.f;
  for (int a = 0; a < 3; ++a) {
    const double c = (lo[a] + hi[a]) * 0.5, h = (hi[a] - lo[a]) * 0.5;
    gbox[6ull * g + a] = c;
    gbox[6ull * g + 3 + a] = h;
    const float cf = static_cast<float>(c - root->center[a]), hf = static_cast<float>(h);
    gboxf[8ull * g + a] = cf;
    gboxf[8ull * g + 3 + a] = hf;
    gmax = fmaxf(gmax, fabsf(cf));
    hmax = fmaxf(hmax, hf);
  }
  gboxf[8ull * g + 6] = (gmax + hmax) * (1.0f + 1.0f / (1 << 20));
  gboxf[8ull * g + 7] = 0.f;
}

// The opening test of group_lists.cpp:145-154 for one node, in FP64 exactly
// as the reference computes it.
__device__ __forceinline__ bool accept64(const WalkRec64 &r, const double *gc, const double *gh) {
  bool overlap = true;
  double d2 = 0.0;
  if (fabs(r.cx - gc[0]) > r.slack + gh[0]) overlap = false;
  double d = fabs(r.mx - gc[0]) - gh[0];
  if (d > 0) d2 += d * d;
  if (fabs(r.cy - gc[1]) > r.slack + gh[1]) overlap = false;
  d = fabs(r.my - gc[1]) - gh[1];
  if (d > 0) d2 += d * d;
  if (fabs(r.cz - gc[2]) > r.slack + gh[2]) overlap = false;
  d = fabs(r.mz - gc[2]) - gh[2];
  if (d > 0) d2 += d * d;
  return !overlap && d2 > r.crit2;
}

// The same test in FP32 with a rigorous error band. Every FP32 input is the
// FP64 quantity (relative to the root centre) rounded once; the node record
// carries B_n >= all its |values| + slack and the group B_g >= max|centre| +
// max half-extent, so every quantity compared below is at most ~2 (B_n + B_g)
// in size and each FP32 result is within 5 * 2^-24 (B_n + B_g) of the value
// from the exact inputs (more than the FP64 roundings too). The band
// E = 2^-20 (B_n + B_g) is over three times that: a comparison whose sides
// differ by more than E has the FP64 outcome; otherwise the caller runs the
// FP64 test. Returns 1 accept, 0 open, 2 undecided (NaNs end up undecided).
constexpr float kBand = 1.0f / (1 << 20);

__device__ __forceinline__ int accept32(const WalkRec32 &r, const float *gf, const float *hf,
                                        float gbound) {
  const float e = kBand * (r.bound + gbound);
  bool separated = false, within = true;
  float lo2 = 0.f, hi2 = 0.f;
  const float c[3] = {r.cx, r.cy, r.cz}, mm[3] = {r.mx, r.my, r.mz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    // overlap: on every axis |c - g| <= slack + gh (group_lists.cpp:147)
    const float x = fabsf(c[a] - gf[a]), y = r.slack + hf[a];
    separated |= x > y + e;
    within &= x < y - e;
    // distance from the box to the centre of mass (group_lists.cpp:150-151)
    const float d = fabsf(mm[a] - gf[a]) - hf[a];
    const float dl = fmaxf(d - e, 0.f), dh = fmaxf(d + e, 0.f);
    lo2 = fmaf(dl, dl, lo2);
    hi2 = fmaf(dh, dh, hi2);
  }
  const float c2 = r.crit2;
  if (within) return 0;                                      // overlaps: opened
  if (hi2 * (1.f + 4.f * kBand) < c2 * (1.f - 4.f * kBand)) return 0;  // too close
  if (separated && lo2 * (1.f - 4.f * kBand) > c2 * (1.f + 4.f * kBand)) return 1;
  return 2;
}

__device__ __forceinline__ WalkRec32 load32(const WalkRec32 *w, u32 i) {
  const float4 *p = reinterpret_cast<const float4 *>(w + i);
  const float4 a = __ldg(p), b = __ldg(p + 1);
  const uint4 c = __ldg(reinterpret_cast<const uint4 *>(p + 2));
  WalkRec32 r;
  r.cx = a.x;
  r.cy = a.y;
  r.cz = a.z;
  r.slack = a.w;
  r.mx = b.x;
  r.my = b.y;
  r.mz = b.z;
  r.crit2 = b.w;
  r.skip = c.x;
  r.nbody_leaf = c.y;
  r.begin = c.z;
  r.bound = __uint_as_float(c.w);
  return r;
}

__device__ __forceinline__ WalkRec64 load64(const WalkRec64 *w, u32 i) {
  const double2 *p = reinterpret_cast<const double2 *>(w + i);
  const double2 a0 = __ldg(p), a1 = __ldg(p + 1), b0 = __ldg(p + 2), b1 = __ldg(p + 3);
  return WalkRec64{a0.x, a0.y, a1.x, a1.y, b0.x, b0.y, b1.x, b1.y};
}

// One walk task: the subtree under `root`, reached through `anc` (the root's
// ancestor at depth 1, or kNone when root is shallower). The reference's
// walk visits the subtrees in node order, so a group's list is its tasks'
// lists concatenated in task order. When the ancestor is accepted the
// subtree is never entered and only the task first under the ancestor in
// node order (root == anc + 1, the ancestor's last-octant child) emits it.
struct Task {
  u32 root, anc, first, pad;
};
constexpr u32 kNone = 0xffffffffu;

struct WalkOut {
  u64 *ncells, *nbodies;          // count and one-pass walks, [group * ntasks + task]
  const u64 *cell_off, *body_off; // fill pass, same indexing
  u32 *cell_list, *body_list;
  u32 slot_cells, slot_bodies;    // one-pass walk: each group's capacities
  u32 *spill_cells, *spill_bodies;  // where an outgrown group's lists go (kNoSpill: its slot)
  u64 pool_cells_at, pool_cells;    // overflow pools: first entry and size
  u64 pool_bodies_at, pool_bodies;
};

// Walk modes: count the lists; write them at scanned offsets; both in one
// pass into fixed per-group slots (one task per group; an outgrown slot
// keeps counting, and its group then takes a place in the overflow pools
// for its whole lists, or flags the lists as overflowing when the pools are
// too small); or write again, whole, the lists of the groups that outgrew
// their slots, into their places in the pools.
constexpr int kCount = 0, kFill = 1, kSlots = 2, kSpill = 3;
constexpr u32 kNoSpill = 0xffffffffu;

__device__ __forceinline__ int decide(const WalkRec32 &r, const WalkRec64 *walk64, u32 i,
                                      const float *gf, const float *hf, float gbound,
                                      const double *gbox, u32 g, u32 &exact) {
  int verdict = accept32(r, gf, hf, gbound);
  if (verdict == 2) {
    double gc[3], gh[3];
    for (int a = 0; a < 3; ++a) {
      gc[a] = gbox[6ull * g + a];
      gh[a] = gbox[6ull * g + 3 + a];
    }
    verdict = accept64(load64(walk64, i), gc, gh) ? 1 : 0;
    ++exact;
  }
  return verdict;
}

template <int kMode>
__global__ void __launch_bounds__(kT)
    k_walk(const WalkRec32 *walk32, const WalkRec64 *walk64, const double *gbox,
           const float *gboxf, u32 ng_cap, const Task *tasks, u32 ntasks, WalkOut out,
           Scalars *sc, const u32 *ng_dev = nullptr, const u32 *abort = nullptr) {
  const u64 tid = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  if (aborted(abort)) return;
  const u32 ng = bounded(ng_cap, ng_dev);
  if (tid >= static_cast<u64>(ng) * ntasks) return;
  // consecutive threads: consecutive groups on the same task (similar walks)
  const u32 t = static_cast<u32>(tid / ng), g = static_cast<u32>(tid % ng);
  const u64 slot = static_cast<u64>(g) * ntasks + t;
  const float4 b0 = reinterpret_cast<const float4 *>(gboxf)[2ull * g],
               b1 = reinterpret_cast<const float4 *>(gboxf)[2ull * g + 1];
  const float gf[3] = {b0.x, b0.y, b0.z}, hf[3] = {b0.w, b1.x, b1.y};
  const float gbound = b1.z;
  u32 *cl = nullptr, *bl = nullptr;
  if (kMode == kFill) {
    cl = out.cell_list + out.cell_off[slot];
    bl = out.body_list + out.body_off[slot];
  } else if (kMode == kSlots) {
    cl = out.cell_list + static_cast<u64>(g) * out.slot_cells;
    bl = out.body_list + static_cast<u64>(g) * out.slot_bodies;
  } else if (kMode == kSpill) {
    if (out.spill_cells[g] == kNoSpill) return;
    cl = out.cell_list + out.spill_cells[g];
    bl = out.body_list + out.spill_bodies[g];
  }
  u32 nc = 0, nb = 0, exact = 0, visits = 0;
  const Task task = tasks[t];
  auto take = [&](const WalkRec32 &r, u32 i, int verdict) {
    const u32 nbody = r.nbody_leaf & 0x7fffffffu;
    if (verdict == 1 && nbody > kFewBodies) {
      if (kMode == kFill || kMode == kSpill || (kMode == kSlots && nc < out.slot_cells)) cl[nc] = i;
      ++nc;
    } else {
      if (kMode == kFill || kMode == kSpill)
        for (u32 j = 0; j < nbody; ++j) bl[nb + j] = r.begin + j;
      if (kMode == kSlots)
        for (u32 j = 0; j < nbody && nb + j < out.slot_bodies; ++j) bl[nb + j] = r.begin + j;
      nb += nbody;
    }
  };
  bool enter = true;
  if (task.anc != kNone) {
    ++visits;
    const WalkRec32 a = load32(walk32, task.anc);
    if (decide(a, walk64, task.anc, gf, hf, gbound, gbox, g, exact) == 1) {
      if (task.first) take(a, task.anc, 1);
      enter = false;
    }
  }
  if (enter) {
    u32 i = task.root;
    const u32 end = load32(walk32, task.root).skip;
    while (i < end) {
      const WalkRec32 r = load32(walk32, i);
      ++visits;
      const int verdict = decide(r, walk64, i, gf, hf, gbound, gbox, g, exact);
      if (verdict == 1 || (r.nbody_leaf >> 31)) {
        take(r, i, verdict);
        if (r.skip <= i) {  // malformed tree: never loop
          atomicOr(&sc->error, 1u);
          break;
        }
        i = r.skip;
      } else {
        ++i;
      }
    }
  }
  if (kMode == kCount || kMode == kSlots) {
    out.ncells[slot] = nc;
    out.nbodies[slot] = nb;
    if (exact) atomicAdd(&sc->fp64_tests, static_cast<unsigned long long>(exact));
    // visited nodes: one atomic per set of converged lanes
    const unsigned mask = __activemask();
    const u32 sum = __reduce_add_sync(mask, visits);
    if ((threadIdx.x & 31) == static_cast<unsigned>(__ffs(mask) - 1))
      atomicAdd(&sc->walk_nodes, static_cast<unsigned long long>(sum));
  }
  if (kMode == kSlots) {
    u32 oc = kNoSpill, ob = kNoSpill;
    if (nc > out.slot_cells || nb > out.slot_bodies) {
      const u64 c = atomicAdd(&sc->spill_used[0], static_cast<unsigned long long>(nc));
      const u64 b = atomicAdd(&sc->spill_used[1], static_cast<unsigned long long>(nb));
      if (c + nc <= out.pool_cells && b + nb <= out.pool_bodies) {
        oc = static_cast<u32>(out.pool_cells_at + c);
        ob = static_cast<u32>(out.pool_bodies_at + b);
      } else {
        atomicOr(&sc->list_overflow, 1u);
      }
      atomicAdd(&sc->spilled, 1u);
    }
    out.spill_cells[g] = oc;
    out.spill_bodies[g] = ob;
  }
}


// Walk tasks: nodes at depth `split` (0..2), and leaves above it, in node
// order. The root is never accepted (every group lies inside it), so only a
// depth-2 task has an ancestor to test.
__global__ void __launch_bounds__(kT)
    k_task_flags(const u8 *depth, const u8 *isleaf, u32 m, int split, u32 *flag) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p >= m) return;
  flag[p] = (depth[p] == split || (isleaf[p] && depth[p] < split)) ? 1u : 0u;
}

__global__ void __launch_bounds__(kT)
    k_task_fill(const u32 *flag, const u32 *scan, const u8 *depth, const u32 *parent, u32 m,
                Task *tasks) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p >= m || !flag[p]) return;
  Task t{p, kNone, 0u, 0u};
  if (depth[p] == 2) {
    t.anc = parent[p];
    t.first = p == t.anc + 1 ? 1u : 0u;
  }
  tasks[scan[p]] = t;
}

// GTGroup records from the per-task offsets, and the list counters.
__global__ void __launch_bounds__(kT)
    k_group_records(const u32 *gbegin, const u32 *gend, u32 ng, u32 ntasks, const u64 *cell_off,
                    const u64 *body_off, uint4 *groups, Scalars *sc,
                    const u32 *ng_dev = nullptr) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (sc->abort) return;
  const bool valid = g < bounded(ng, ng_dev);
  u64 t = 0, nc = 0, nb = 0;
  if (valid) {
    const u64 c0 = cell_off[static_cast<u64>(g) * ntasks],
              c1 = cell_off[static_cast<u64>(g + 1) * ntasks];
    const u64 b0 = body_off[static_cast<u64>(g) * ntasks],
              b1 = body_off[static_cast<u64>(g + 1) * ntasks];
    store_group_rec(groups, g, gbegin[g], gend[g], one_segment(c0, c1 - c0),
                    one_segment(b0, b1 - b0));
    t = gend[g] - gbegin[g];
    nc = c1 - c0;
    nb = b1 - b0;
  }
  group_stats_warp(sc, valid, t, nc, nb, false);
}

// Group records of a one-pass walk: group g's lists start at its slots.
__global__ void __launch_bounds__(kT)
    k_slot_records(const u32 *gbegin, const u32 *gend, u32 ng, const u64 *ncells,
                   const u64 *nbodies, u32 slot_cells, u32 slot_bodies, const u32 *spill_cells,
                   const u32 *spill_bodies, uint4 *groups, Scalars *sc,
                   const u32 *ng_dev = nullptr, const u32 *abort = nullptr) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort)) return;
  const bool valid = g < bounded(ng, ng_dev);
  u64 t = 0, nc = 0, nb = 0;
  if (valid) {
    nc = ncells[g];
    nb = nbodies[g];
    t = gend[g] - gbegin[g];
    u64 c0 = static_cast<u64>(g) * slot_cells, b0 = static_cast<u64>(g) * slot_bodies;
    u64 kc = nc < slot_cells ? nc : slot_cells, kb = nb < slot_bodies ? nb : slot_bodies;
    if (spill_cells[g] != kNoSpill) {  // the whole lists, in the pools
      c0 = spill_cells[g];
      b0 = spill_bodies[g];
      kc = nc;
      kb = nb;
    }
    store_group_rec(groups, g, gbegin[g], gend[g], one_segment(c0, kc), one_segment(b0, kb));
  }
  group_stats_warp(sc, valid, t, nc, nb, true);
}

void read_scalars(Workspace &ws, Scalars *host, cudaStream_t s) {
  GTC_CUDA(cudaMemcpyAsync(host, ws.scalars.ptr, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
}

// Slots for the next one-pass walk: this walk's longest lists plus a half
// and 64, in multiples of 32 entries (each slot starts on 128 bytes). The
// longest of many groups' lists moves from one step to the next, so the
// margin is wide; slots cost only memory.
void size_slots(Workspace &ws, const Scalars &h) {
  auto slot = [](u64 longest) {
    const u64 v = (longest + longest / 2 + 64 + 31) & ~31ull;
    return static_cast<u32>(std::min<u64>(v, 0x7fffffe0ull));
  };
  ws.slot_cells = slot(h.max_cells);
  ws.slot_bodies = slot(h.max_bodies);
}

}  // namespace

void build_lists(Workspace &ws, const SolverParams &sp, cudaStream_t s, Scalars *host,
                 const LearnedWalk *lw) {
  const u64 n = ws.n;
  const u64 prev_entries = ws.n_cell_list + ws.n_body_list;
  ws.n_groups = ws.n_cell_list = ws.n_body_list = 0;
  ws.gapped = false;
  ws.list_passes = 0;
  if (n == 0) return;
  const u32 n32 = static_cast<u32>(n), m = static_cast<u32>(ws.n_nodes);
  const u32 gs = static_cast<u32>(sp.group_size);
  Scalars *sc = ws.scalars.as<Scalars>();
  GTC_CUDA(cudaMemsetAsync(&sc->spilled, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->walk_nodes, 0, sizeof(unsigned long long), s));
  ws.flags.ensure(std::max<u64>(n, m) * 4);
  ws.flags_scan.ensure(std::max<u64>(n, m) * 4);
  u32 *mark = ws.flags.as<u32>(), *mscan = ws.flags_scan.as<u32>();
  const u32 mb = ceil_div(m, kT);

  // walk tasks (their count is read back with the group count)
  ws.tasks.ensure(m * sizeof(Task));
  // (the learned walk splits each group's walk along its own path instead)
  if (!lw) {
    k_task_flags<<<mb, kT, 0, s>>>(ws.depth.as<u8>(), ws.isleaf.as<u8>(), m, ws.walk_split_depth,
                                   mark);
    GTC_LAUNCH_CHECK();
    exclusive_scan_u32(mark, mscan, m, &sc->aux, ws.scan_tmp, s);
    k_task_fill<<<mb, kT, 0, s>>>(mark, mscan, ws.depth.as<u8>(), ws.parent.as<u32>(), m,
                                  ws.tasks.as<Task>());
    GTC_LAUNCH_CHECK();
  }

  // groups
  GTC_CUDA(cudaMemsetAsync(mark, 0, n * 4, s));
  NodeView nv{ws.nbegin.as<u32>(), ws.nend.as<u32>(), ws.skip.as<u32>(), ws.isleaf.as<u8>()};
  k_group_marks<<<mb, kT, 0, s>>>(nv, m, n32, gs, sp.pack, mark);
  GTC_LAUNCH_CHECK();
  exclusive_scan_u32(mark, mscan, n, &sc->n_groups, ws.scan_tmp, s);
  ws.gbegin.ensure(n * 4);
  ws.gend.ensure(n * 4);
  ws.gbox.ensure(n * 48);
  ws.gboxf.ensure(n * 32);
  ws.groups.ensure(n * kGroupRecWords * 4);
  u32 *gbegin = ws.gbegin.as<u32>(), *gend = ws.gend.as<u32>();
  k_group_ranges<<<ceil_div(n, kT), kT, 0, s>>>(mark, mscan, n32, gbegin, gend);
  GTC_LAUNCH_CHECK();
  k_last_end<<<1, 1, 0, s>>>(sc, n32, gend);
  GTC_LAUNCH_CHECK();
  GTC_CUDA(cudaMemsetAsync(&sc->cell_interactions, 0, 3 * sizeof(unsigned long long), s));
  GTC_CUDA(cudaMemsetAsync(&sc->max_group, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->fp64_tests, 0, 3 * sizeof(unsigned long long), s));
  read_scalars(ws, host, s);
  const u32 ng = host->n_groups, ntasks = host->aux;
  ws.n_groups = ng;
  const u32 gb = ceil_div(ng, kT);
  k_group_box<<<gb, kT, 0, s>>>(gbegin, gend, ng, ws.tpos.as<double>(), ws.root.as<TreeRoot>(),
                                ws.gbox.as<double>(), ws.gboxf.as<float>());
  GTC_LAUNCH_CHECK();
  if (lw) {
    learned_group_tolerances(ws, *lw, ng, s);
    learned_build_lists(ws, *lw, ng, host, s);
    return;
  }

  const WalkRec32 *w32 = ws.walk32.as<WalkRec32>();
  const WalkRec64 *w64 = ws.walk64.as<WalkRec64>();
  const double *gbox = ws.gbox.as<double>();
  const float *gboxf = ws.gboxf.as<float>();
  const Task *tasks = ws.tasks.as<Task>();
  const u64 slots = static_cast<u64>(ng) * ntasks;
  ws.gcells.ensure(slots * 8);
  ws.gbodies.ensure(slots * 8);
  GTC_CUDA(cudaMemsetAsync(&sc->max_cells, 0, 2 * sizeof(u32), s));
  const u32 tb = ceil_div(slots, kT);

  // One pass into per-group slots when the last walk sized them and they
  // fit 32-bit offsets and eight times the lists' own size (the slots of
  // the benchmark galaxy take about four times). Groups whose
  // lists outgrow their slots are walked again into the overflow pools;
  // pools too small fall back to the two passes below.
  const u32 sl_c = ws.slot_cells, sl_b = ws.slot_bodies;
  const u64 pool_c = Workspace::pool_for(ng, sl_c), pool_b = Workspace::pool_for(ng, sl_b);
  const u64 ext_c = static_cast<u64>(ng) * sl_c + pool_c, ext_b = static_cast<u64>(ng) * sl_b + pool_b;
  if (sl_c > 0 && ntasks == 1 && ext_c <= 0xffffffffull && ext_b <= 0xffffffffull &&
      ext_c + ext_b <= std::max<u64>(8 * prev_entries, 1ull << 26)) {
    ws.cell_list.ensure(ext_c * 4);
    ws.body_list.ensure(ext_b * 4);
    ws.spill.ensure(2ull * ng * sizeof(u32));
    u32 *spill_c = ws.spill.as<u32>(), *spill_b = spill_c + ng;
    GTC_CUDA(cudaMemsetAsync(&sc->n_cell_list, 0, 2 * sizeof(u64), s));
    GTC_CUDA(cudaMemsetAsync(&sc->list_overflow, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(sc->spill_used, 0, 2 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->spilled, 0, sizeof(u32), s));
    WalkOut wo{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), nullptr, nullptr,
               ws.cell_list.as<u32>(), ws.body_list.as<u32>(), sl_c, sl_b, spill_c, spill_b,
               static_cast<u64>(ng) * sl_c, pool_c, static_cast<u64>(ng) * sl_b, pool_b};
    k_walk<kSlots><<<tb, kT, 0, s>>>(w32, w64, gbox, gboxf, ng, tasks, 1, wo, sc);
    GTC_LAUNCH_CHECK();
    k_walk<kSpill><<<tb, kT, 0, s>>>(w32, w64, gbox, gboxf, ng, tasks, 1, wo, sc);
    GTC_LAUNCH_CHECK();
    k_slot_records<<<gb, kT, 0, s>>>(gbegin, gend, ng, ws.gcells.as<u64>(), ws.gbodies.as<u64>(),
                                     sl_c, sl_b, spill_c, spill_b, ws.groups.as<uint4>(), sc);
    GTC_LAUNCH_CHECK();
    read_scalars(ws, host, s);
    size_slots(ws, *host);
    if (!host->list_overflow) {
      ws.n_cell_list = host->n_cell_list;
      ws.n_body_list = host->n_body_list;
      ws.gapped = true;
      ws.list_passes = 1;
      return;
    }
    // the pools were too small: the counters start again for the two passes
    GTC_CUDA(cudaMemsetAsync(&sc->walk_nodes, 0, sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->cell_interactions, 0, 3 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_group, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(&sc->fp64_tests, 0, sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_cells, 0, 2 * sizeof(u32), s));
  }

  // count pass, offsets, fill pass
  ws.gcell_off.ensure((slots + 1) * 8);
  ws.gbody_off.ensure((slots + 1) * 8);
  u64 *cell_off = ws.gcell_off.as<u64>(), *body_off = ws.gbody_off.as<u64>();
  WalkOut wo{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), cell_off, body_off, nullptr, nullptr,
             0, 0, nullptr, nullptr, 0, 0, 0, 0};
  k_walk<kCount><<<tb, kT, 0, s>>>(w32, w64, gbox, gboxf, ng, tasks, ntasks, wo, sc);
  GTC_LAUNCH_CHECK();
  exclusive_scan_u64(ws.gcells.as<u64>(), cell_off, slots, cell_off + slots, ws.scan_tmp, s);
  exclusive_scan_u64(ws.gbodies.as<u64>(), body_off, slots, body_off + slots, ws.scan_tmp, s);
  GTC_CUDA(cudaMemcpyAsync(&sc->n_cell_list, cell_off + slots, 8, cudaMemcpyDeviceToDevice, s));
  GTC_CUDA(cudaMemcpyAsync(&sc->n_body_list, body_off + slots, 8, cudaMemcpyDeviceToDevice, s));
  k_group_records<<<gb, kT, 0, s>>>(gbegin, gend, ng, ntasks, cell_off, body_off,
                                    ws.groups.as<uint4>(), sc);
  GTC_LAUNCH_CHECK();
  read_scalars(ws, host, s);
  if (host->n_cell_list > 0xffffffffull || host->n_body_list > 0xffffffffull)
    throw RuntimeError("interaction lists too long for 32 bit offsets");
  size_slots(ws, *host);
  ws.n_cell_list = host->n_cell_list;
  ws.n_body_list = host->n_body_list;
  ws.cell_list.ensure(std::max<u64>(1, ws.n_cell_list) * 4);
  ws.body_list.ensure(std::max<u64>(1, ws.n_body_list) * 4);
  wo.cell_list = ws.cell_list.as<u32>();
  wo.body_list = ws.body_list.as<u32>();
  k_walk<kFill><<<tb, kT, 0, s>>>(w32, w64, gbox, gboxf, ng, tasks, ntasks, wo, sc);
  GTC_LAUNCH_CHECK();
  ws.list_passes = 2;
}

void build_lists_graph(Workspace &ws, const SolverParams &sp, const GraphCaps &caps,
                       cudaStream_t s) {
  const u64 n = ws.n;
  const u32 n32 = static_cast<u32>(n), mcap = caps.nodes;
  const u32 gs = static_cast<u32>(sp.group_size);
  Scalars *sc = ws.scalars.as<Scalars>();
  u32 *mark = ws.flags.as<u32>(), *mscan = ws.flags_scan.as<u32>();
  const u32 *abort = &sc->abort;
  const u32 nb = ceil_div(n, kT), mb = ceil_div(mcap, kT);
  // groups (the one walk task, the root, was written before capture)
  GTC_CUDA(cudaMemsetAsync(mark, 0, n * 4, s));
  NodeView nv{ws.nbegin.as<u32>(), ws.nend.as<u32>(), ws.skip.as<u32>(), ws.isleaf.as<u8>()};
  k_group_marks<<<mb, kT, 0, s>>>(nv, mcap, n32, gs, sp.pack, mark, &sc->n_nodes, abort);
  GTC_LAUNCH_CHECK();
  exclusive_scan_u32(mark, mscan, n, &sc->n_groups, ws.scan_tmp, s);
  u32 *gbegin = ws.gbegin.as<u32>(), *gend = ws.gend.as<u32>();
  k_group_ranges<<<nb, kT, 0, s>>>(mark, mscan, n32, gbegin, gend, abort);
  GTC_LAUNCH_CHECK();
  k_last_end<<<1, 1, 0, s>>>(sc, n32, gend);
  GTC_LAUNCH_CHECK();
  GTC_CUDA(cudaMemsetAsync(&sc->cell_interactions, 0, 3 * sizeof(unsigned long long), s));
  GTC_CUDA(cudaMemsetAsync(&sc->max_group, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->fp64_tests, 0, 3 * sizeof(unsigned long long), s));
  k_group_box<<<nb, kT, 0, s>>>(gbegin, gend, n32, ws.tpos.as<double>(), ws.root.as<TreeRoot>(),
                                ws.gbox.as<double>(), ws.gboxf.as<float>(), &sc->n_groups, abort);
  GTC_LAUNCH_CHECK();
  // one pass into the captured slots, outgrown groups again into the pools
  k_check_groups_graph<<<1, 1, 0, s>>>(sc, caps.groups);
  GTC_LAUNCH_CHECK();
  GTC_CUDA(cudaMemsetAsync(&sc->n_cell_list, 0, 2 * sizeof(u64), s));
  GTC_CUDA(cudaMemsetAsync(&sc->list_overflow, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->max_cells, 0, 2 * sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(sc->spill_used, 0, 2 * sizeof(unsigned long long), s));
  GTC_CUDA(cudaMemsetAsync(&sc->spilled, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->walk_nodes, 0, sizeof(unsigned long long), s));
  u32 *spill_c = ws.spill.as<u32>(), *spill_b = spill_c + n;
  WalkOut wo{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), nullptr, nullptr,
             ws.cell_list.as<u32>(), ws.body_list.as<u32>(), caps.slot_cells, caps.slot_bodies,
             spill_c, spill_b, static_cast<u64>(caps.groups) * caps.slot_cells, caps.pool_cells,
             static_cast<u64>(caps.groups) * caps.slot_bodies, caps.pool_bodies};
  const Task *tasks = ws.tasks.as<Task>();
  k_walk<kSlots><<<nb, kT, 0, s>>>(ws.walk32.as<WalkRec32>(), ws.walk64.as<WalkRec64>(),
                                   ws.gbox.as<double>(), ws.gboxf.as<float>(), n32, tasks, 1, wo,
                                   sc, &sc->n_groups, abort);
  GTC_LAUNCH_CHECK();
  k_walk<kSpill><<<nb, kT, 0, s>>>(ws.walk32.as<WalkRec32>(), ws.walk64.as<WalkRec64>(),
                                   ws.gbox.as<double>(), ws.gboxf.as<float>(), n32, tasks, 1, wo,
                                   sc, &sc->n_groups, abort);
  GTC_LAUNCH_CHECK();
  k_slot_records<<<nb, kT, 0, s>>>(gbegin, gend, n32, ws.gcells.as<u64>(), ws.gbodies.as<u64>(),
                                   caps.slot_cells, caps.slot_bodies, spill_c, spill_b,
                                   ws.groups.as<uint4>(), sc, &sc->n_groups, abort);
  GTC_LAUNCH_CHECK();
  k_check_slots_graph<<<1, 1, 0, s>>>(sc);
  GTC_LAUNCH_CHECK();
}

void write_root_task(Workspace &ws, cudaStream_t s) {
  ws.tasks.ensure(sizeof(Task));
  const Task t{0u, kNone, 0u, 0u};
  GTC_CUDA(cudaMemcpyAsync(ws.tasks.ptr, &t, sizeof(Task), cudaMemcpyHostToDevice, s));
  GTC_CUDA(cudaStreamSynchronize(s));
}

}  // namespace gtc
