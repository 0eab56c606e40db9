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
  // a forest: node depths (its roots are at depth 0), the system of each
  // body, and each system's group size and packing
  const u8 *depth = nullptr;
  const u16 *sys = nullptr;
  const u8 *gsize = nullptr, *gpack = nullptr;
};

__global__ void __launch_bounds__(kT)
    k_group_marks(NodeView nv, u32 m, u32 gs, int pack, u32 *mark,
                  const u32 *m_dev = nullptr, const u32 *abort = nullptr) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || p >= bounded(m, m_dev)) return;
  const u32 b0 = nv.nbegin[p], b1 = nv.nend[p];
  bool root = p == 0;
  if (nv.sys) {
    const u16 k = nv.sys[b0];
    gs = nv.gsize[k];
    pack = nv.gpack[k];
    root = nv.depth[p] == 0;
  }
  const u32 size = b1 - b0;
  if (root && (size <= gs || nv.isleaf[p])) {
    for (u32 c = b0; c < b1; c += gs) mark[c] = 1;
    return;
  }
  if (nv.isleaf[p] || size <= gs) return;
  // children, last octant first
  u32 ch[8];
  int nc = 0;
  for (u32 c = p + 1; c < nv.skip[p] && nc < 8; c = nv.skip[c]) ch[nc++] = c;
  // the packing threshold: runs of small siblings hold at most `limit`
  // bodies (pack 1: a group's worth, the reference's rule)
  const u32 limit = pack <= 1 ? gs : min(static_cast<u32>(pack), gs);
  bool open = false;
  u32 run_begin = 0, run_end = 0;
  for (int j = nc - 1; j >= 0; --j) {
    const u32 c = ch[j];
    const u32 cb = nv.nbegin[c], ce = nv.nend[c], cc = ce - cb;
    if (cc <= gs) {
      if (pack && open && (run_end - run_begin) + cc <= limit) {
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
// Order-preserving image of a finite double with +0 and -0 equal: a < b as
// doubles exactly when key(a) < key(b).
__device__ __forceinline__ u64 zero_equal_key(double v) {
  u64 b = static_cast<u64>(__double_as_longlong(v));
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void __launch_bounds__(kT)
    k_group_box(const u32 *gbegin, const u32 *gend, u32 ng, const double *tpos,
                const TreeRoot *root, double *gbox, float *gboxf, const u32 *ng_dev,
                const u32 *abort, ForestView fv) {
  // gboxf per group: centre (3), half-extent (3), magnitude bound, pad
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || g >= bounded(ng, ng_dev)) return;
  const u32 b0 = gbegin[g], b1 = gend[g];
  if (fv.sys) {  // a forest: the group's system's root
    const u16 k = fv.sys[b0];
    root += k;
    fv.group_root[g] = fv.root_node[k];
  }
  // the reference's running min and max (v < lo, hi < v: the first of equal
  // values stays), compared on integer images of the doubles (+0 and -0
  // equal) instead of on the FP64 pipe
  double lo[3], hi[3];
  u64 klo[3], khi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = hi[a] = tpos[3ull * b0 + a];
    klo[a] = khi[a] = zero_equal_key(lo[a]);
  }
  for (u32 k = b0; k < b1; ++k)
    for (int a = 0; a < 3; ++a) {
      const double v = tpos[3ull * k + a];
      const u64 kv = zero_equal_key(v);
      if (kv < klo[a]) {
        klo[a] = kv;
        lo[a] = v;
      }
      if (khi[a] < kv) {
        khi[a] = kv;
        hi[a] = v;
      }
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
  u64 *ncells, *nbodies;          // count pass, [group * ntasks + task]
  const u64 *cell_off, *body_off; // fill pass, same indexing
  u32 *cell_list, *body_list;
  const u32 *spill_cells, *spill_bodies;  // spill walk: where an outgrown group's lists go
};

// Walk modes: count the lists; write them at scanned offsets; or write
// again, whole, the lists of the groups whose one-pass walk (k_walk_split)
// outgrew their slots, into their places in the overflow pools.
constexpr int kCount = 0, kFill = 1, kSpill = 3;
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
           Scalars *sc, const u32 *ng_dev, const u32 *abort, const u32 *group_root) {
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
  } else if (kMode == kSpill) {
    if (out.spill_cells[g] == kNoSpill) return;
    cl = out.cell_list + out.spill_cells[g];
    bl = out.body_list + out.spill_bodies[g];
  }
  u32 nc = 0, nb = 0, exact = 0, visits = 0;
  // (a forest has one task, its group's own root)
  const Task task = group_root ? Task{group_root[g], kNone, 0u, 0u} : tasks[t];
  auto take = [&](const WalkRec32 &r, u32 i, int verdict) {
    const u32 nbody = r.nbody_leaf & 0x7fffffffu;
    if (verdict == 1 && nbody > kFewBodies) {
      if (kMode == kFill || kMode == kSpill) cl[nc] = i;
      ++nc;
    } else {
      if (kMode == kFill || kMode == kSpill)
        for (u32 j = 0; j < nbody; ++j) bl[nb + j] = r.begin + j;
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
  if (kMode == kCount) {
    out.ncells[slot] = nc;
    out.nbodies[slot] = nb;
    if (exact) atomicAdd(&sc->fp64_tests, static_cast<unsigned long long>(exact));
    // visited nodes: one atomic per set of converged lanes
    const unsigned mask = __activemask();
    const u32 sum = __reduce_add_sync(mask, visits);
    if ((threadIdx.x & 31) == static_cast<unsigned>(__ffs(mask) - 1))
      atomicAdd(&sc->walk_nodes, static_cast<unsigned long long>(sum));
  }
}


// The one-pass walk, split in two per group. A long walk spends about half
// its nodes inside the root child that holds the group (its near field),
// and one thread per group leaves the others idle while the longest walks
// finish. So thread `rest` walks from the root but jumps over that child,
// noting how much it had written when it did, and thread `near` walks the
// child. The group's lists are then [rest before | near | rest after]: the
// reference's order. Each part writes into its own slots; a group whose
// part outgrows its slot is walked again whole into the overflow pools.
struct SplitOut {
  u64 *ncells, *nbodies;   // [part * cap + group]: part 0 the rest, 1 the near field
  u32 *split;              // per group: the rest's cells and bodies before the near field
  u32 *cell_list, *body_list;
  u64 near_cells_at, near_bodies_at;  // the near parts' slots start here (the rest's at 0)
  u32 slot_cells, slot_bodies, slot_near_cells, slot_near_bodies;
  u32 cap;                 // groups the count arrays hold per part
  // a forest: per-group slots (starts, then sizes; null: the uniform slots
  // above), and the per-system maxima the records keep (with the body
  // systems they are indexed by)
  const uint4 *plan = nullptr;
  const u16 *sys = nullptr;
  u32 *sys_max = nullptr;
};

// Group g's slots: starts (rest cells, rest bodies, near cells, near
// bodies) and sizes, from the plan or the uniform layout.
struct GroupSlots {
  u64 rc_at, rb_at, nc_at, nb_at;
  u32 rc, rb, nc, nb;
};
__device__ __forceinline__ GroupSlots group_slots(const SplitOut &o, u32 g) {
  if (o.plan) {
    const uint4 st = o.plan[2ull * g], cp = o.plan[2ull * g + 1];
    return GroupSlots{st.x, st.y, st.z, st.w, cp.x, cp.y, cp.z, cp.w};
  }
  return GroupSlots{static_cast<u64>(g) * o.slot_cells, static_cast<u64>(g) * o.slot_bodies,
                    o.near_cells_at + static_cast<u64>(g) * o.slot_near_cells,
                    o.near_bodies_at + static_cast<u64>(g) * o.slot_near_bodies, o.slot_cells,
                    o.slot_bodies, o.slot_near_cells, o.slot_near_bodies};
}

// A forest's group count of each system: its groups are contiguous, and
// the group choice's scan at its first body is its first group.
__global__ void __launch_bounds__(kT)
    k_sys_groups(const u32 *mscan, const u32 *start, u32 systems, const Scalars *sc,
                 u32 *groups) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= systems) return;
  const u32 next = k + 1 < systems ? mscan[start[k + 1]] : sc->n_groups;
  groups[k] = next - mscan[start[k]];
}

// Each group's slots from its system's table; a group past the system's
// capacity gets none (its lists go to the overflow pools).
__global__ void __launch_bounds__(kT)
    k_slot_plan(const u32 *gbegin, u32 ng_cap, const u32 *ng_dev, const u32 *abort,
                const u16 *sys, const u32 *start, const u32 *mscan, const SysSlots *slots,
                uint4 *plan) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || g >= bounded(ng_cap, ng_dev)) return;
  const u16 k = sys[gbegin[g]];
  const SysSlots S = slots[k];
  const u32 j = g - mscan[start[k]];
  if (j < S.groups) {
    plan[2ull * g] = make_uint4(S.rc_at + j * S.rc, S.rb_at + j * S.rb, S.nc_at + j * S.nc,
                                S.nb_at + j * S.nb);
    plan[2ull * g + 1] = make_uint4(S.rc, S.rb, S.nc, S.nb);
  } else {
    plan[2ull * g] = make_uint4(0u, 0u, 0u, 0u);
    plan[2ull * g + 1] = make_uint4(0u, 0u, 0u, 0u);
  }
}

// A forest's per-system maxima of four list lengths (every lane of the
// warp calls it): one atomic per value when the warp's valid lanes share a
// system, the usual case (a system's groups are contiguous), else one per
// lane.
__device__ __forceinline__ void sys_max_warp(u32 *sys_max, const u16 *sys, bool valid, u32 b0,
                                             u32 a, u32 b, u32 c, u32 d) {
  const u32 key = valid ? sys[b0] : 0xffffffffu;
  const unsigned vm = __ballot_sync(kFullMask, valid);
  if (vm == 0) return;
  const u32 key0 = __shfl_sync(kFullMask, key, __ffs(vm) - 1);
  if (__all_sync(kFullMask, !valid || key == key0)) {
    const u32 ma = __reduce_max_sync(kFullMask, valid ? a : 0u),
              mb = __reduce_max_sync(kFullMask, valid ? b : 0u),
              mc = __reduce_max_sync(kFullMask, valid ? c : 0u),
              md = __reduce_max_sync(kFullMask, valid ? d : 0u);
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&sys_max[4ull * key0], ma);
      atomicMax(&sys_max[4ull * key0 + 1], mb);
      atomicMax(&sys_max[4ull * key0 + 2], mc);
      atomicMax(&sys_max[4ull * key0 + 3], md);
    }
  } else if (valid) {
    atomicMax(&sys_max[4ull * key], a);
    atomicMax(&sys_max[4ull * key + 1], b);
    atomicMax(&sys_max[4ull * key + 2], c);
    atomicMax(&sys_max[4ull * key + 3], d);
  }
}

// The child of `root` that holds targets [b0, b1), or kNone.
__device__ __forceinline__ u32 near_child(u32 root, u32 b0, u32 b1, const uint4 *kids,
                                          const u8 *nchild, const u32 *nbegin, const u32 *nend) {
  const int k = nchild[root];
  const uint4 k0 = kids[2ull * root], k1 = kids[2ull * root + 1];
  const u32 ch[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
  for (int j = 0; j < k && j < 8; ++j)
    if (nbegin[ch[j]] <= b0 && b1 <= nend[ch[j]]) return ch[j];
  return kNone;
}

// Small blocks for the one-pass walk: its blocks run for very different
// times (the central groups walk longest), and small ones even out the SMs.
constexpr u32 kWalkThreads = 128;

__global__ void __launch_bounds__(kWalkThreads)
    k_walk_split(const WalkRec32 *walk32, const WalkRec64 *walk64, const double *gbox,
                 const float *gboxf, const u32 *gbegin, const u32 *gend, const uint4 *kids,
                 const u8 *nchild, const u32 *nbegin, const u32 *nend, u32 ng_cap, SplitOut out,
                 Scalars *sc, const u32 *ng_dev, const u32 *abort, const u32 *group_root) {
  const u64 tid = static_cast<u64>(blockIdx.x) * kWalkThreads + threadIdx.x;
  if (aborted(abort)) return;
  const u32 ng = bounded(ng_cap, ng_dev);
  if (tid >= 2ull * ng) return;
  const u32 part = tid >= ng ? 1u : 0u;
  const u32 g = static_cast<u32>(part ? tid - ng : tid);
  const float4 b0 = reinterpret_cast<const float4 *>(gboxf)[2ull * g],
               b1 = reinterpret_cast<const float4 *>(gboxf)[2ull * g + 1];
  const float gf[3] = {b0.x, b0.y, b0.z}, hf[3] = {b0.w, b1.x, b1.y};
  const float gbound = b1.z;
  const u32 root = group_root ? group_root[g] : 0u;
  // (a leaf root has no children: nchild 0)
  const u32 near = near_child(root, gbegin[g], gend[g], kids, nchild, nbegin, nend);
  const u32 near_end = near == kNone ? 0u : load32(walk32, near).skip;
  const GroupSlots gsl = group_slots(out, g);
  const u32 cap_c = part ? gsl.nc : gsl.rc;
  const u32 cap_b = part ? gsl.nb : gsl.rb;
  u32 *cl = out.cell_list + (part ? gsl.nc_at : gsl.rc_at);
  u32 *bl = out.body_list + (part ? gsl.nb_at : gsl.rb_at);
  u32 nc = 0, nb = 0, exact = 0, visits = 0, split_c = 0, split_b = 0;
  bool jumped = false;
  u32 i = 0, end = 0;
  if (part == 0) {
    i = root;
    end = load32(walk32, root).skip;
  } else if (near != kNone) {
    i = near;
    end = near_end;
  }
  while (i < end) {
    if (part == 0 && i == near) {  // the near field is the other thread's
      split_c = nc;
      split_b = nb;
      jumped = true;
      i = near_end;
      continue;
    }
    const WalkRec32 r = load32(walk32, i);
    ++visits;
    const int verdict = decide(r, walk64, i, gf, hf, gbound, gbox, g, exact);
    if (verdict == 1 || (r.nbody_leaf >> 31)) {
      const u32 nbody = r.nbody_leaf & 0x7fffffffu;
      if (verdict == 1 && nbody > kFewBodies) {
        if (nc < cap_c) cl[nc] = i;
        ++nc;
      } else {
        for (u32 j = 0; j < nbody && nb + j < cap_b; ++j) bl[nb + j] = r.begin + j;
        nb += nbody;
      }
      if (r.skip <= i) {  // malformed tree: never loop
        atomicOr(&sc->error, 1u);
        break;
      }
      i = r.skip;
    } else {
      ++i;
    }
  }
  if (part == 0 && !jumped) {
    split_c = nc;
    split_b = nb;
  }
  out.ncells[static_cast<u64>(part) * out.cap + g] = nc;
  out.nbodies[static_cast<u64>(part) * out.cap + g] = nb;
  if (part == 0) {
    out.split[2ull * g] = split_c;
    out.split[2ull * g + 1] = split_b;
  }
  if (exact) atomicAdd(&sc->fp64_tests, static_cast<unsigned long long>(exact));
  const unsigned mask = __activemask();
  const u32 sum = __reduce_add_sync(mask, visits);
  if ((threadIdx.x & 31) == static_cast<unsigned>(__ffs(mask) - 1))
    atomicAdd(&sc->walk_nodes, static_cast<unsigned long long>(sum));
}

// The walk by warps: one warp per group, 32 node tests per step. The
// warp keeps the nodes still to visit as a stack of index ranges in shared
// memory, each a run of whole subtrees [i, end) (i, skip[i], ... before
// end). Each step the lanes take the ranges on top, test each range's first
// node, and push back the rest of its range and, when the node is opened,
// its children's range (children on top: depth first). The same nodes are
// tested, with the same verdicts, as by the reference's walk; only the order
// the entries reach the lists differs (step order, lane order within a
// step; fixed for given inputs). Exports put each group's lists back in the
// reference's order (increasing node and body index, which is its visiting
// order). Modes: count the lists (kCount); write them at scanned offsets
// (kFill); write them into per-group slots, counting past a slot that
// overflows (kSlots, the one-pass walk, whose counts and records then go
// through the split walk's spill and record kernels as one part); write the
// lists of the groups that outgrew their slots again, whole, into their
// places in the overflow pools (kSpill).
constexpr int kSlots = 2;
constexpr int kWarpWalkWarps = 4;
constexpr int kWarpStack = 1024;  // ranges per warp
constexpr u32 kWarpWalkThreads = kWarpWalkWarps * 32;

struct WarpWalkOut {
  u64 *ncells, *nbodies;          // kCount: per group; kSlots: SplitOut's part 0 (cap: its stride)
  const u64 *cell_off, *body_off; // kFill
  u32 *cell_list, *body_list;
  const u32 *spill_cells, *spill_bodies;  // kSpill
  u32 *split;                     // kSlots: the split walk's split points (all lists: part 0)
  u32 slot_cells, slot_bodies, cap;
  const uint4 *plan = nullptr;    // kSlots, a forest: per-group slots (starts, sizes)
};

__device__ __forceinline__ u32 warp_excl_scan(u32 v, int lane, u32 &total) {
  u32 s = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const u32 y = __shfl_up_sync(kFullMask, s, o);
    if (lane >= o) s += y;
  }
  total = __shfl_sync(kFullMask, s, 31);
  return s - v;
}

// Walks the ranges on a warp's stack (stk[0..top), each a run of whole
// subtrees [i, end)) to the end for group g: each step the lanes take the
// ranges on top, test each range's first node, and push back the rest of
// its range and, when the node is opened, its children's range (children
// on top). Cells and bodies go to cl / bl from nc / nb on (kWrite; counting
// past cap_c / cap_b), in step order, lane order within a step. When the
// stack is nearly full, lane 0 walks the top range alone, so no step can
// overflow it. Every lane of the warp calls it; nc and nb are warp-uniform.
template <bool kWrite>
__device__ __forceinline__ void walk_ranges_warp(uint2 *stk, u32 top, const WalkRec32 *walk32,
                                                 const WalkRec64 *walk64, const float *gf,
                                                 const float *hf, float gbound,
                                                 const double *gbox, u32 g, u32 *cl, u32 *bl,
                                                 u64 cap_c, u64 cap_b, u64 &nc, u64 &nb,
                                                 u32 &exact, u32 &visits, Scalars *sc) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  while (top > 0) {
    if (top > kWarpStack - 2 * 32) {
      // nearly full: lane 0 walks the top range alone, without a stack
      const uint2 e = stk[top - 1];
      --top;
      __syncwarp();
      if (lane == 0) {
        u32 i = e.x;
        while (i < e.y) {
          const WalkRec32 r = load32(walk32, i);
          ++visits;
          const int verdict = decide(r, walk64, i, gf, hf, gbound, gbox, g, exact);
          const u32 nbody = r.nbody_leaf & 0x7fffffffu;
          const bool leaf = (r.nbody_leaf >> 31) != 0;
          if (verdict == 1 && nbody > kFewBodies) {
            if (kWrite && nc < cap_c) cl[nc] = i;
            ++nc;
          } else if (verdict == 1 || leaf) {
            for (u32 j = 0; j < nbody; ++j)
              if (kWrite && nb + j < cap_b) bl[nb + j] = r.begin + j;
            nb += nbody;
          }
          if (verdict == 1 || leaf) {
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
      nc = __shfl_sync(kFullMask, nc, 0);
      nb = __shfl_sync(kFullMask, nb, 0);
      continue;
    }
    const u32 take = min(32u, top);
    const bool has = static_cast<u32>(lane) < take;
    const uint2 e = has ? stk[top - 1 - lane] : make_uint2(0u, 0u);
    top -= take;
    __syncwarp();
    WalkRec32 r{};
    int verdict = 0;
    if (has) {
      r = load32(walk32, e.x);
      ++visits;
      verdict = decide(r, walk64, e.x, gf, hf, gbound, gbox, g, exact);
    }
    const u32 nbody = r.nbody_leaf & 0x7fffffffu;
    const bool leaf = (r.nbody_leaf >> 31) != 0;
    const bool bad = has && r.skip <= e.x;  // malformed tree: never loop
    if (bad) atomicOr(&sc->error, 1u);
    const bool cell = has && verdict == 1 && nbody > kFewBodies;
    const bool bod = has && !cell && (verdict == 1 || leaf);
    const bool kids = has && !bad && verdict == 0 && !leaf;
    const bool rest = has && !bad && r.skip < e.y;
    // cells: one slot per accepting lane, in lane order
    const unsigned mc = __ballot_sync(kFullMask, cell);
    if (kWrite && cell) {
      const u64 pos = nc + __popc(mc & below);
      if (pos < cap_c) cl[pos] = e.x;
    }
    nc += __popc(mc);
    // bodies: each lane's run after the runs of the lanes before it
    u32 bt = 0;
    const u32 boff = warp_excl_scan(bod ? nbody : 0u, lane, bt);
    if (kWrite && bod)
      for (u32 j = 0; j < nbody; ++j)
        if (nb + boff + j < cap_b) bl[nb + boff + j] = r.begin + j;
    nb += bt;
    // pushes: each lane its rest, then its children's range (on top)
    u32 pt = 0;
    const u32 poff = warp_excl_scan(static_cast<u32>(rest) + static_cast<u32>(kids), lane, pt);
    if (rest) stk[top + poff] = make_uint2(r.skip, e.y);
    if (kids) stk[top + poff + (rest ? 1u : 0u)] = make_uint2(e.x + 1, r.skip);
    top += pt;
    __syncwarp();
  }
}

template <int kMode>
__global__ void __launch_bounds__(kWarpWalkThreads)
    k_walk_warp(const WalkRec32 *walk32, const WalkRec64 *walk64, const double *gbox,
                const float *gboxf, u32 ng_cap, WarpWalkOut out, u32 *next_group, Scalars *sc,
                const u32 *ng_dev, const u32 *abort, const u32 *group_root) {
  __shared__ uint2 stack_all[kWarpWalkWarps][kWarpStack];
  if (aborted(abort)) return;
  const u32 ng = bounded(ng_cap, ng_dev);
  const int lane = threadIdx.x & 31;
  uint2 *stk = stack_all[threadIdx.x >> 5];
  u32 exact = 0, visits = 0;
  for (;;) {
    u32 g = 0;
    if (lane == 0) g = atomicAdd(next_group, 1u);
    g = __shfl_sync(kFullMask, g, 0);
    if (g >= ng) break;
    u32 *cl = nullptr, *bl = nullptr;
    u64 cap_c = ~0ull, cap_b = ~0ull;
    if (kMode == kFill) {
      cl = out.cell_list + out.cell_off[g];
      bl = out.body_list + out.body_off[g];
    } else if (kMode == kSlots) {
      if (out.plan) {
        const uint4 st = out.plan[2ull * g], cp = out.plan[2ull * g + 1];
        cap_c = cp.x;
        cap_b = cp.y;
        cl = out.cell_list + st.x;
        bl = out.body_list + st.y;
      } else {
        cap_c = out.slot_cells;
        cap_b = out.slot_bodies;
        cl = out.cell_list + static_cast<u64>(g) * cap_c;
        bl = out.body_list + static_cast<u64>(g) * cap_b;
      }
    } else if (kMode == kSpill) {
      if (out.spill_cells[g] == kNoSpill) continue;
      cl = out.cell_list + out.spill_cells[g];
      bl = out.body_list + out.spill_bodies[g];
    }
    const float4 b0 = reinterpret_cast<const float4 *>(gboxf)[2ull * g],
                 b1 = reinterpret_cast<const float4 *>(gboxf)[2ull * g + 1];
    const float gf[3] = {b0.x, b0.y, b0.z}, hf[3] = {b0.w, b1.x, b1.y};
    const float gbound = b1.z;
    u64 nc = 0, nb = 0;  // warp-uniform
    // the root contains every group and is opened, unless it is a leaf
    const u32 root = group_root ? group_root[g] : 0u;
    const WalkRec32 rr = load32(walk32, root);
    const bool root_leaf = (rr.nbody_leaf >> 31) != 0;
    if (lane == 0) stk[0] = make_uint2(root_leaf ? root : root + 1, rr.skip);
    u32 top = 1;
    __syncwarp();
    walk_ranges_warp<kMode != kCount>(stk, top, walk32, walk64, gf, hf, gbound, gbox, g, cl, bl,
                                      cap_c, cap_b, nc, nb, exact, visits, sc);
    if (lane == 0) {
      if (kMode == kCount) {
        out.ncells[g] = nc;
        out.nbodies[g] = nb;
      } else if (kMode == kSlots) {
        out.ncells[g] = nc;
        out.nbodies[g] = nb;
        out.ncells[static_cast<u64>(out.cap) + g] = 0;
        out.nbodies[static_cast<u64>(out.cap) + g] = 0;
        out.split[2ull * g] = static_cast<u32>(nc < 0xffffffffull ? nc : 0xffffffffull);
        out.split[2ull * g + 1] = static_cast<u32>(nb < 0xffffffffull ? nb : 0xffffffffull);
      }
    }
  }
  if (kMode == kCount || kMode == kSlots) {
    const u32 ex = __reduce_add_sync(kFullMask, exact), vs = __reduce_add_sync(kFullMask, visits);
    if (lane == 0) {
      if (ex) atomicAdd(&sc->fp64_tests, static_cast<unsigned long long>(ex));
      atomicAdd(&sc->walk_nodes, static_cast<unsigned long long>(vs));
    }
  }
}

// Places in the overflow pools for the groups one of whose parts outgrew its
// slot (their whole lists, walked again by one thread); pools too small flag
// the lists as overflowing.
__global__ void __launch_bounds__(kT)
    k_split_spill(const SplitOut out, u32 ng, u64 pool_cells_at, u64 pool_cells,
                  u64 pool_bodies_at, u64 pool_bodies, u32 *spill_cells, u32 *spill_bodies,
                  Scalars *sc, const u32 *ng_dev = nullptr, const u32 *abort = nullptr) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || g >= bounded(ng, ng_dev)) return;
  const u64 rc = out.ncells[g], rb = out.nbodies[g];
  const u64 nc = out.ncells[static_cast<u64>(out.cap) + g], nb = out.nbodies[static_cast<u64>(out.cap) + g];
  u32 oc = kNoSpill, ob = kNoSpill;
  const GroupSlots gsl = group_slots(out, g);
  if (rc > gsl.rc || rb > gsl.rb || nc > gsl.nc || nb > gsl.nb) {
    const u64 tc = rc + nc, tb = rb + nb;
    const u64 c = atomicAdd(&sc->spill_used[0], static_cast<unsigned long long>(tc));
    const u64 b = atomicAdd(&sc->spill_used[1], static_cast<unsigned long long>(tb));
    if (c + tc <= pool_cells && b + tb <= pool_bodies) {
      oc = static_cast<u32>(pool_cells_at + c);
      ob = static_cast<u32>(pool_bodies_at + b);
    } else {
      atomicOr(&sc->list_overflow, 1u);
    }
    atomicAdd(&sc->spilled, 1u);
  }
  spill_cells[g] = oc;
  spill_bodies[g] = ob;
}

// Group records of a split one-pass walk: three segments per list (one, in
// the pools, for a spilled group), the statistics, and the longest lists of
// either part.
__global__ void __launch_bounds__(kT)
    k_split_records(const u32 *gbegin, const u32 *gend, u32 ng, const SplitOut out,
                    const u32 *spill_cells, const u32 *spill_bodies, uint4 *groups, Scalars *sc,
                    const u32 *ng_dev = nullptr, const u32 *abort = nullptr) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort)) return;
  const bool valid = g < bounded(ng, ng_dev);
  // (a replay's grid covers every body: warps past the groups leave at once)
  if (__ballot_sync(kFullMask, valid) == 0) return;
  u64 t = 0, rc = 0, rb = 0, nc = 0, nb = 0;
  if (valid) {
    rc = out.ncells[g];
    rb = out.nbodies[g];
    nc = out.ncells[static_cast<u64>(out.cap) + g];
    nb = out.nbodies[static_cast<u64>(out.cap) + g];
    t = gend[g] - gbegin[g];
    ListSegs cs, bs;
    if (spill_cells[g] != kNoSpill) {
      cs = one_segment(spill_cells[g], rc + nc);
      bs = one_segment(spill_bodies[g], rb + nb);
    } else {
      const u32 sc_ = out.split[2ull * g], sb_ = out.split[2ull * g + 1];
      const GroupSlots gsl = group_slots(out, g);
      const u64 r0 = gsl.rc_at, q0 = gsl.rb_at, n0 = gsl.nc_at, m0 = gsl.nb_at;
      cs.start[0] = static_cast<u32>(r0);
      cs.count[0] = sc_;
      cs.start[1] = static_cast<u32>(n0);
      cs.count[1] = static_cast<u32>(nc);
      cs.start[2] = static_cast<u32>(r0 + sc_);
      cs.count[2] = static_cast<u32>(rc - sc_);
      bs.start[0] = static_cast<u32>(q0);
      bs.count[0] = sb_;
      bs.start[1] = static_cast<u32>(m0);
      bs.count[1] = static_cast<u32>(nb);
      bs.start[2] = static_cast<u32>(q0 + sb_);
      bs.count[2] = static_cast<u32>(rb - sb_);
    }
    store_group_rec(groups, g, gbegin[g], gend[g], cs, bs);
  }
  group_stats_warp(sc, valid, t, rc + nc, rb + nb, true, false);
  auto clamp = [](u64 v) { return static_cast<u32>(v < 0xffffffffull ? v : 0xffffffffull); };
  const u32 m_rc = __reduce_max_sync(kFullMask, clamp(rc)), m_rb = __reduce_max_sync(kFullMask, clamp(rb));
  const u32 m_nc = __reduce_max_sync(kFullMask, clamp(nc)), m_nb = __reduce_max_sync(kFullMask, clamp(nb));
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&sc->max_cells, m_rc);
    atomicMax(&sc->max_bodies, m_rb);
    atomicMax(&sc->max_near_cells, m_nc);
    atomicMax(&sc->max_near_bodies, m_nb);
  }
  if (out.sys_max)
    sys_max_warp(out.sys_max, out.sys, valid, valid ? gbegin[g] : 0u, clamp(rc), clamp(rb),
                 clamp(nc), clamp(nb));
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
                    const u64 *body_off, uint4 *groups, Scalars *sc, const u32 *ng_dev = nullptr,
                    const u16 *sys = nullptr, u32 *sys_max = nullptr) {
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
  if (sys_max) {  // whole lists: they size both parts' slots
    const u32 c = static_cast<u32>(nc < 0xffffffffull ? nc : 0xffffffffull);
    const u32 b = static_cast<u32>(nb < 0xffffffffull ? nb : 0xffffffffull);
    sys_max_warp(sys_max, sys, valid, valid ? gbegin[g] : 0u, c, b, c, b);
  }
}


void read_scalars(Workspace &ws, Scalars *host, cudaStream_t s) {
  GTC_CUDA(cudaMemcpyAsync(host, ws.scalars.ptr, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
}

// Slots for the next one-pass walk: this walk's longest lists plus a half
// and 64, in multiples of 32 entries (each slot starts on 128 bytes). The
// longest of many groups' lists moves from one step to the next, so the
// margin is wide; slots cost only memory.
// After a split walk max_cells / max_bodies are the rest's longest lists and
// max_near_* the near field's; after the two passes they are whole lists,
// which size both parts' slots.
void size_slots(Workspace &ws, const Scalars &h, bool split) {
  auto slot = [](u64 longest) {
    const u64 v = (longest + longest / 2 + 64 + 31) & ~31ull;
    return static_cast<u32>(std::min<u64>(v, 0x7fffffe0ull));
  };
  ws.slot_cells = slot(h.max_cells);
  ws.slot_bodies = slot(h.max_bodies);
  // the warp walk writes a group's whole lists into the first slots
  ws.slot_near_cells = slot(ws.walk_warps ? 0 : split ? h.max_near_cells : h.max_cells);
  ws.slot_near_bodies = slot(ws.walk_warps ? 0 : split ? h.max_near_bodies : h.max_bodies);
}

// The warp walk over ng groups: enough warps to fill the GPU, groups taken
// from a counter.
template <int kMode>
void launch_warp_walk(Workspace &ws, const WarpWalkOut &out, u32 ng_cap, Scalars *sc,
                      cudaStream_t s, const u32 *ng_dev = nullptr, const u32 *abort = nullptr) {
  int dev = 0, sms = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  ws.walk_next.ensure(sizeof(u32));
  GTC_CUDA(cudaMemsetAsync(ws.walk_next.ptr, 0, sizeof(u32), s));
  const u32 blocks = static_cast<u32>(std::max<u64>(
      1, std::min<u64>(ceil_div(ng_cap, kWarpWalkWarps), 8ull * static_cast<u64>(sms))));
  k_walk_warp<kMode><<<blocks, kWarpWalkThreads, 0, s>>>(
      ws.walk32.as<WalkRec32>(), ws.walk64.as<WalkRec64>(), ws.gbox.as<double>(),
      ws.gboxf.as<float>(), ng_cap, out, ws.walk_next.as<u32>(), sc, ng_dev, abort,
      ws.forest.group_root);
  GTC_LAUNCH_CHECK();
}

// The node arrays the group choice reads (a forest's per-system fields too).
NodeView node_view(const Workspace &ws) {
  NodeView nv{ws.nbegin.as<u32>(), ws.nend.as<u32>(), ws.skip.as<u32>(), ws.isleaf.as<u8>()};
  if (ws.forest) {
    nv.depth = ws.depth.as<u8>();
    nv.sys = ws.forest.sys;
    nv.gsize = ws.forest.group_size;
    nv.gpack = ws.forest.pack;
  }
  return nv;
}

}  // namespace

void build_lists(Workspace &ws, const SolverParams &sp, cudaStream_t s, Scalars *host,
                 const LearnedWalk *lw) {
  const u64 n = ws.n;
  const u64 prev_entries = ws.n_cell_list + ws.n_body_list;
  ws.n_groups = ws.n_cell_list = ws.n_body_list = 0;
  ws.gapped = false;
  ws.lists_unordered = false;
  ws.list_passes = 0;
  if (n == 0) return;
  const u32 n32 = static_cast<u32>(n), m = static_cast<u32>(ws.n_nodes);
  const u32 gs = static_cast<u32>(sp.group_size);
  Scalars *sc = ws.scalars.as<Scalars>();
  ws.walk_next.ensure(sizeof(u32));  // before any graph capture reuses the walk
  GTC_CUDA(cudaMemsetAsync(&sc->spilled, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->walk_nodes, 0, sizeof(unsigned long long), s));
  ws.flags.ensure(std::max<u64>(n, m) * 4);
  ws.flags_scan.ensure(std::max<u64>(n, m) * 4);
  u32 *mark = ws.flags.as<u32>(), *mscan = ws.flags_scan.as<u32>();
  const u32 mb = ceil_div(m, kT);

  // walk tasks (their count is read back with the group count)
  ws.tasks.ensure(m * sizeof(Task));
  // (the learned walk splits each group's walk along its own path instead;
  // a forest's groups walk their own system's tree whole, one task each)
  const ForestView &fv = ws.forest;
  if (!lw && !fv) {
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
  const NodeView nv = node_view(ws);
  k_group_marks<<<mb, kT, 0, s>>>(nv, m, gs, sp.pack, mark);
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
  if (fv) {  // each system's group count, read back with the total
    k_sys_groups<<<ceil_div(fv.systems, kT), kT, 0, s>>>(mscan, fv.start, fv.systems, sc,
                                                         fv.sys_groups);
    GTC_LAUNCH_CHECK();
    GTC_CUDA(cudaMemcpyAsync(fv.host_groups, fv.sys_groups, fv.systems * sizeof(u32),
                             cudaMemcpyDeviceToHost, s));
  }
  GTC_CUDA(cudaMemsetAsync(&sc->cell_interactions, 0, 3 * sizeof(unsigned long long), s));
  GTC_CUDA(cudaMemsetAsync(&sc->max_group, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->fp64_tests, 0, 3 * sizeof(unsigned long long), s));
  read_scalars(ws, host, s);
  const u32 ng = host->n_groups, ntasks = fv ? 1u : host->aux;
  ws.n_groups = ng;
  ws.walk_warps = ws.warps_for(ng);
  const u32 gb = ceil_div(ng, kT);
  k_group_box<<<gb, kT, 0, s>>>(gbegin, gend, ng, ws.tpos.as<double>(),
                                fv ? fv.roots : ws.root.as<TreeRoot>(), ws.gbox.as<double>(),
                                ws.gboxf.as<float>(), nullptr, nullptr, fv);
  GTC_LAUNCH_CHECK();
  if (lw) {
    // the learned walk decides from FP32 moment estimates: the FP64 moments
    // go on on the side stream, and are joined for the evaluation after it
    ws.stage(Workspace::kStWalk0, s);
    if (lw->inputs_ready) GTC_CUDA(cudaStreamWaitEvent(s, lw->inputs_ready, 0));
    learned_group_tolerances(ws, *lw, ng, s);
    learned_build_lists(ws, *lw, ng, host, s);
    ws.stage(Workspace::kStWalk1, s);
    join_side(ws, s);
    return;
  }
  join_walk(ws, s);  // the walk reads the node records (the cells follow on the side stream)
  ws.stage(Workspace::kStWalk0, s);

  const WalkRec32 *w32 = ws.walk32.as<WalkRec32>();
  const WalkRec64 *w64 = ws.walk64.as<WalkRec64>();
  const double *gbox = ws.gbox.as<double>();
  const float *gboxf = ws.gboxf.as<float>();
  const Task *tasks = ws.tasks.as<Task>();
  const u64 slots = static_cast<u64>(ng) * ntasks;
  ws.gcells.ensure(slots * 8);
  ws.gbodies.ensure(slots * 8);
  GTC_CUDA(cudaMemsetAsync(&sc->max_cells, 0, 4 * sizeof(u32), s));
  const u32 tb = ceil_div(slots, kT);
  // a forest's per-system maxima of the lists, read back after the walk
  auto clear_sys_max = [&] {
    if (fv) GTC_CUDA(cudaMemsetAsync(fv.sys_max, 0, 4ull * fv.systems * sizeof(u32), s));
  };
  auto read_sys_max = [&] {
    if (fv)
      GTC_CUDA(cudaMemcpyAsync(fv.host_max, fv.sys_max, 4ull * fv.systems * sizeof(u32),
                               cudaMemcpyDeviceToHost, s));
  };
  clear_sys_max();

  // One pass into per-group slots when the last walk sized them and they
  // fit 32-bit offsets and sixteen times the lists' own size or 2^28
  // entries, whichever is more (slots sized
  // by a two-pass walk's whole lists take about eight times for the
  // benchmark galaxy, those of a split walk about four): two threads per group, the
  // near field and the rest. Groups whose lists outgrow their slots are
  // walked again into the overflow pools; pools too small fall back to the
  // two passes below.
  const u32 sl_c = ws.slot_cells, sl_b = ws.slot_bodies;
  const u32 sn_c = ws.slot_near_cells, sn_b = ws.slot_near_bodies;
  const u64 near_c = static_cast<u64>(ng) * sl_c, near_b = static_cast<u64>(ng) * sl_b;
  const u64 pool_at_c = near_c + static_cast<u64>(ng) * sn_c;
  const u64 pool_at_b = near_b + static_cast<u64>(ng) * sn_b;
  const u64 pool_c = Workspace::pool_for(ng, sl_c + sn_c), pool_b = Workspace::pool_for(ng, sl_b + sn_b);
  const u64 ext_c = pool_at_c + pool_c, ext_b = pool_at_b + pool_b;
  if (sl_c > 0 && ntasks == 1 && ext_c <= 0xffffffffull && ext_b <= 0xffffffffull &&
      ext_c + ext_b <= std::max<u64>(16 * prev_entries, 1ull << 28)) {
    ws.cell_list.ensure(ext_c * 4);
    ws.body_list.ensure(ext_b * 4);
    ws.spill.ensure(2ull * ng * sizeof(u32));
    ws.splitpt.ensure(2ull * ng * sizeof(u32));
    ws.gcells.ensure(2ull * ng * 8);
    ws.gbodies.ensure(2ull * ng * 8);
    u32 *spill_c = ws.spill.as<u32>(), *spill_b = spill_c + ng;
    GTC_CUDA(cudaMemsetAsync(&sc->n_cell_list, 0, 2 * sizeof(u64), s));
    GTC_CUDA(cudaMemsetAsync(&sc->list_overflow, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(sc->spill_used, 0, 2 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->spilled, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_cells, 0, 4 * sizeof(u32), s));
    SplitOut so{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), ws.splitpt.as<u32>(),
                ws.cell_list.as<u32>(), ws.body_list.as<u32>(), near_c, near_b,
                sl_c, sl_b, sn_c, sn_b, ng};
    so.sys = fv.sys;
    so.sys_max = fv.sys_max;
    const WarpWalkOut wwo{so.ncells, so.nbodies, nullptr, nullptr, ws.cell_list.as<u32>(),
                          ws.body_list.as<u32>(), spill_c, spill_b, so.split, sl_c, sl_b, ng};
    if (ws.walk_warps) {
      launch_warp_walk<kSlots>(ws, wwo, ng, sc, s);
    } else {
      k_walk_split<<<ceil_div(2ull * ng, kWalkThreads), kWalkThreads, 0, s>>>(
          w32, w64, gbox, gboxf, gbegin, gend, ws.kids.as<uint4>(), ws.nchild.as<u8>(),
          ws.nbegin.as<u32>(), ws.nend.as<u32>(), ng, so, sc, nullptr, nullptr, fv.group_root);
      GTC_LAUNCH_CHECK();
    }
    k_split_spill<<<gb, kT, 0, s>>>(so, ng, pool_at_c, pool_c, pool_at_b, pool_b, spill_c, spill_b,
                                    sc);
    GTC_LAUNCH_CHECK();
    if (ws.walk_warps) {
      launch_warp_walk<kSpill>(ws, wwo, ng, sc, s);
    } else {
      WalkOut wo{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), nullptr, nullptr,
                 ws.cell_list.as<u32>(), ws.body_list.as<u32>(), spill_c, spill_b};
      k_walk<kSpill><<<tb, kT, 0, s>>>(w32, w64, gbox, gboxf, ng, tasks, 1, wo, sc, nullptr,
                                       nullptr, fv.group_root);
      GTC_LAUNCH_CHECK();
    }
    k_split_records<<<gb, kT, 0, s>>>(gbegin, gend, ng, so, spill_c, spill_b,
                                      ws.groups.as<uint4>(), sc);
    GTC_LAUNCH_CHECK();
    ws.stage(Workspace::kStWalk1, s);
    read_sys_max();
    read_scalars(ws, host, s);
    size_slots(ws, *host, true);
    if (!host->list_overflow) {
      join_side(ws, s);  // the lists' readers read the cells too
      ws.n_cell_list = host->n_cell_list;
      ws.n_body_list = host->n_body_list;
      ws.gapped = true;
      ws.lists_unordered = ws.walk_warps;
      ws.list_passes = 1;
      return;
    }
    // the pools were too small: the counters start again for the two passes
    GTC_CUDA(cudaMemsetAsync(&sc->walk_nodes, 0, sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->cell_interactions, 0, 3 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_group, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(&sc->fp64_tests, 0, sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_cells, 0, 4 * sizeof(u32), s));
    clear_sys_max();
  }

  // count pass, offsets, fill pass
  ws.gcell_off.ensure((slots + 1) * 8);
  ws.gbody_off.ensure((slots + 1) * 8);
  u64 *cell_off = ws.gcell_off.as<u64>(), *body_off = ws.gbody_off.as<u64>();
  WalkOut wo{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), cell_off, body_off, nullptr, nullptr,
             nullptr, nullptr};
  const bool warps = ws.walk_warps && ntasks == 1;
  WarpWalkOut wwo{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), cell_off, body_off, nullptr, nullptr,
                  nullptr, nullptr, nullptr, 0u, 0u, ng};
  if (warps) {
    launch_warp_walk<kCount>(ws, wwo, ng, sc, s);
  } else {
    k_walk<kCount><<<tb, kT, 0, s>>>(w32, w64, gbox, gboxf, ng, tasks, ntasks, wo, sc, nullptr,
                                     nullptr, fv.group_root);
    GTC_LAUNCH_CHECK();
  }
  exclusive_scan_u64(ws.gcells.as<u64>(), cell_off, slots, cell_off + slots, ws.scan_tmp, s);
  exclusive_scan_u64(ws.gbodies.as<u64>(), body_off, slots, body_off + slots, ws.scan_tmp, s);
  GTC_CUDA(cudaMemcpyAsync(&sc->n_cell_list, cell_off + slots, 8, cudaMemcpyDeviceToDevice, s));
  GTC_CUDA(cudaMemcpyAsync(&sc->n_body_list, body_off + slots, 8, cudaMemcpyDeviceToDevice, s));
  k_group_records<<<gb, kT, 0, s>>>(gbegin, gend, ng, ntasks, cell_off, body_off,
                                    ws.groups.as<uint4>(), sc, nullptr, fv.sys, fv.sys_max);
  GTC_LAUNCH_CHECK();
  read_sys_max();
  read_scalars(ws, host, s);
  if (host->n_cell_list > 0xffffffffull || host->n_body_list > 0xffffffffull)
    throw RuntimeError("interaction lists too long for 32 bit offsets");
  size_slots(ws, *host, false);
  ws.n_cell_list = host->n_cell_list;
  ws.n_body_list = host->n_body_list;
  ws.cell_list.ensure(std::max<u64>(1, ws.n_cell_list) * 4);
  ws.body_list.ensure(std::max<u64>(1, ws.n_body_list) * 4);
  wo.cell_list = ws.cell_list.as<u32>();
  wo.body_list = ws.body_list.as<u32>();
  if (warps) {
    wwo.cell_list = wo.cell_list;
    wwo.body_list = wo.body_list;
    launch_warp_walk<kFill>(ws, wwo, ng, sc, s);
  } else {
    k_walk<kFill><<<tb, kT, 0, s>>>(w32, w64, gbox, gboxf, ng, tasks, ntasks, wo, sc, nullptr,
                                    nullptr, fv.group_root);
    GTC_LAUNCH_CHECK();
  }
  ws.stage(Workspace::kStWalk1, s);
  ws.lists_unordered = warps;
  ws.list_passes = 2;
  join_side(ws, s);
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
  const ForestView &fv = ws.forest;
  const NodeView nv = node_view(ws);
  k_group_marks<<<mb, kT, 0, s>>>(nv, mcap, gs, sp.pack, mark, &sc->n_nodes, abort);
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
  k_group_box<<<nb, kT, 0, s>>>(gbegin, gend, n32, ws.tpos.as<double>(),
                                fv ? fv.roots : ws.root.as<TreeRoot>(), ws.gbox.as<double>(),
                                ws.gboxf.as<float>(), &sc->n_groups, abort, fv);
  GTC_LAUNCH_CHECK();
  // one pass into the captured slots (near field and rest), outgrown groups
  // again into the pools
  if (!caps.sys_slots) {  // (per-system slots: a system past its capacity spills)
    k_check_groups_graph<<<1, 1, 0, s>>>(sc, caps.groups);
    GTC_LAUNCH_CHECK();
  }
  GTC_CUDA(cudaMemsetAsync(&sc->n_cell_list, 0, 2 * sizeof(u64), s));
  GTC_CUDA(cudaMemsetAsync(&sc->list_overflow, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->max_cells, 0, 4 * sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(sc->spill_used, 0, 2 * sizeof(unsigned long long), s));
  GTC_CUDA(cudaMemsetAsync(&sc->spilled, 0, sizeof(u32), s));
  GTC_CUDA(cudaMemsetAsync(&sc->walk_nodes, 0, sizeof(unsigned long long), s));
  u32 *spill_c = ws.spill.as<u32>(), *spill_b = spill_c + n;
  ws.walk_warps = ws.warps_for(caps.groups);  // the replays' walk, chosen at capture
  const u64 near_c = static_cast<u64>(caps.groups) * caps.slot_cells;
  const u64 near_b = static_cast<u64>(caps.groups) * caps.slot_bodies;
  u64 pool_at_c = near_c + static_cast<u64>(caps.groups) * caps.slot_near_cells;
  u64 pool_at_b = near_b + static_cast<u64>(caps.groups) * caps.slot_near_bodies;
  SplitOut so{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), ws.splitpt.as<u32>(),
              ws.cell_list.as<u32>(), ws.body_list.as<u32>(), near_c, near_b,
              caps.slot_cells, caps.slot_bodies, caps.slot_near_cells,
              caps.slot_near_bodies, n32};
  WarpWalkOut wwo{so.ncells, so.nbodies, nullptr, nullptr, ws.cell_list.as<u32>(),
                  ws.body_list.as<u32>(), spill_c, spill_b, so.split, caps.slot_cells,
                  caps.slot_bodies, n32};
  if (fv) {
    so.sys = fv.sys;
    so.sys_max = fv.sys_max;
    GTC_CUDA(cudaMemsetAsync(fv.sys_max, 0, 4ull * fv.systems * sizeof(u32), s));
    if (caps.sys_slots) {  // each system's own slots (and the pools after them)
      k_slot_plan<<<nb, kT, 0, s>>>(gbegin, n32, &sc->n_groups, abort, fv.sys, fv.start, mscan,
                                    caps.sys_slots, fv.slot_plan);
      GTC_LAUNCH_CHECK();
      so.plan = fv.slot_plan;
      wwo.plan = fv.slot_plan;
      pool_at_c = caps.pool_at_cells;
      pool_at_b = caps.pool_at_bodies;
    }
  }
  if (ws.walk_warps) {
    launch_warp_walk<kSlots>(ws, wwo, n32, sc, s, &sc->n_groups, abort);
  } else {
    k_walk_split<<<ceil_div(2ull * n, kWalkThreads), kWalkThreads, 0, s>>>(
        ws.walk32.as<WalkRec32>(), ws.walk64.as<WalkRec64>(), ws.gbox.as<double>(),
        ws.gboxf.as<float>(), gbegin, gend, ws.kids.as<uint4>(), ws.nchild.as<u8>(),
        ws.nbegin.as<u32>(), ws.nend.as<u32>(), n32, so, sc, &sc->n_groups, abort,
        fv.group_root);
    GTC_LAUNCH_CHECK();
  }
  k_split_spill<<<nb, kT, 0, s>>>(so, n32, pool_at_c, caps.pool_cells, pool_at_b,
                                  caps.pool_bodies, spill_c, spill_b, sc, &sc->n_groups, abort);
  GTC_LAUNCH_CHECK();
  if (ws.walk_warps) {
    launch_warp_walk<kSpill>(ws, wwo, n32, sc, s, &sc->n_groups, abort);
  } else {
    WalkOut wo{ws.gcells.as<u64>(), ws.gbodies.as<u64>(), nullptr, nullptr,
               ws.cell_list.as<u32>(), ws.body_list.as<u32>(), spill_c, spill_b};
    const Task *tasks = ws.tasks.as<Task>();
    k_walk<kSpill><<<nb, kT, 0, s>>>(ws.walk32.as<WalkRec32>(), ws.walk64.as<WalkRec64>(),
                                     ws.gbox.as<double>(), ws.gboxf.as<float>(), n32, tasks, 1,
                                     wo, sc, &sc->n_groups, abort, fv.group_root);
    GTC_LAUNCH_CHECK();
  }
  k_split_records<<<nb, kT, 0, s>>>(gbegin, gend, n32, so, spill_c, spill_b,
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
