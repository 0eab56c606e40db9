// A batched ensemble as one forest: every system's bodies back to back in
// one arena, one tree per system, and each stage of the step -- kick and
// drift, bounding boxes, keys, sort, topology, moments, groups, walk,
// evaluation, scatter and closing kick -- one launch (or one chain of
// launches) for all systems together instead of one per system.
//
// The forest's trees, lists and forces are each system's own: a body's key
// is stepped from its own system's root cube, two systems share no node,
// the group choice uses the system's own group size and packing, and a
// group walks only its own system's tree, with positions relative to its
// own root centre. So a forest step moves every system to the same doubles
// as that system's own step (the same lists in the same order give the
// same FP32 sums). FP64 kicks and drifts compiled -fmad=false, as in
// integrate.cu (src/integrator.cpp:5-17).

#include <algorithm>
#include <cstring>
#include <vector>

#include "forest.cuh"

namespace gtc {
namespace {

constexpr int kT = 256;

// The arena's system of body i: start[k] <= i < start[k + 1].
__global__ void __launch_bounds__(kT)
    k_forest_sys(const u32 *start, u32 systems, u32 n, u16 *sys) {
  const u32 i = blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  u32 lo = 0, hi = systems;  // start[lo] <= i < start[hi]
  while (hi - lo > 1) {
    const u32 mid = (lo + hi) / 2;
    if (start[mid] <= i) lo = mid;
    else hi = mid;
  }
  sys[i] = static_cast<u16>(lo);
}

// Positions and masses of every system into the arena.
__global__ void __launch_bounds__(kT)
    k_forest_gather_bodies(const ForestSystemPtrs *sp, const u16 *sys, const u32 *start, u32 n,
                           double *apos, double *amass) {
  const u32 i = blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  const u16 k = sys[i];
  const ForestSystemPtrs p = sp[k];
  const u64 j = i - start[k];
  apos[3ull * i] = p.pos[3 * j];
  apos[3ull * i + 1] = p.pos[3 * j + 1];
  apos[3ull * i + 2] = p.pos[3 * j + 2];
  amass[i] = p.mass[j];
}

// v += h a; x += dt v (integrator.cpp:10-13) for every body of every
// system, the new positions also into the arena.
__global__ void __launch_bounds__(kT)
    k_forest_kick_drift(const ForestSystemPtrs *sp, const u16 *sys, const u32 *start, u32 n,
                        double h, double dt, double *apos) {
  const u32 i = blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  const u16 k = sys[i];
  const ForestSystemPtrs p = sp[k];
  const u64 j = i - start[k];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double v = p.vel[3 * j + a] + h * p.acc[3 * j + a];
    p.vel[3 * j + a] = v;
    const double x = p.pos[3 * j + a] + dt * v;
    p.pos[3 * j + a] = x;
    apos[3ull * i + a] = x;
  }
}

// The evaluation's results (tree order) into each system's acc and pot,
// then, with kick, v += h a (integrator.cpp:16) on the stored doubles. A
// graph replay that aborted writes nothing.
__global__ void __launch_bounds__(kT)
    k_forest_scatter(const float4 *out, const u32 *order, u32 n, const ForestSystemPtrs *sp,
                     const u16 *sys, const u32 *start, int kick, double h, const u32 *abort) {
  const u32 t = blockIdx.x * kT + threadIdx.x;
  if (t >= n || (abort && *abort)) return;
  const float4 o = out[t];
  const u32 i = order[t];
  const u16 k = sys[i];
  const ForestSystemPtrs p = sp[k];
  const u64 j = i - start[k];
  const double a[3] = {o.x, o.y, o.z};
  for (int c = 0; c < 3; ++c) p.acc[3 * j + c] = a[c];
  p.pot[j] = o.w;
  if (kick)
    for (int c = 0; c < 3; ++c) p.vel[3 * j + c] = p.vel[3 * j + c] + h * a[c];
}

// Per-system list statistics of the current lists (group records).
__global__ void __launch_bounds__(kT)
    k_forest_stats(const uint4 *groups, u32 ng, const u16 *sys, ForestSystemStats *st) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (g >= ng) return;
  const uint4 r = groups[4ull * g];  // begin, end, cells, bodies
  const u64 t = r.y - r.x;
  ForestSystemStats *s = st + sys[r.x];
  atomicAdd(&s->cell_interactions, static_cast<unsigned long long>(t * r.z));
  atomicAdd(&s->body_interactions, static_cast<unsigned long long>(t * r.w - t));
  atomicAdd(&s->groups, 1ull);
  atomicMax(&s->max_list, static_cast<unsigned long long>(r.z) + r.w);
}

}  // namespace

ForestRun::~ForestRun() {
  ws.release_all();
  DeviceBuffer *own[] = {&tables, &sysid, &roots, &root_node, &group_root, &apos, &amass, &stats,
                         &counter, &split_flags, &sys_groups, &sys_max, &slot_plan, &graph_slots};
  for (DeviceBuffer *b : own) b->release();
  if (host_sc) cudaFreeHost(host_sc);
  if (host_lists) cudaFreeHost(host_lists);
}

bool ForestRun::eligible(const std::vector<ForestSystem> &systems, std::string *why) {
  auto no = [&](const char *w) {
    if (why) *why = w;
    return false;
  };
  if (systems.empty()) return no("no systems");
  if (systems.size() > 0xffffu) return no("more than 65535 systems");
  u64 total = 0;
  const SolverParams &a = systems[0].sp;
  for (const ForestSystem &s : systems) {
    total += s.n;
    const SolverParams &b = s.sp;
    if (b.G != a.G || b.theta != a.theta || b.eps != a.eps || b.quadrupole != a.quadrupole ||
        b.leaf_size != a.leaf_size || b.criterion != a.criterion)
      return no("the systems' G, theta, eps, quadrupole and leaf_size differ");
  }
  if (total > 0xffffffffull) return no("more than 2^32 - 1 bodies in all");
  return true;
}

void ForestRun::setup(const std::vector<ForestSystem> &systems, cudaStream_t s) {
  std::string why;
  if (!eligible(systems, &why)) throw InvalidArgument("forest: " + why);
  sys = systems;
  const u32 k = static_cast<u32>(systems.size());
  std::vector<u32> start(k + 1, 0);
  std::vector<u8> gsize(k), pack(k);
  std::vector<ForestSystemPtrs> ptrs(k);
  // bounding-box blocks: about one per 8192 bodies, 1..64 per system
  std::vector<uint4> blk;
  std::vector<uint2> sys_blk(k);
  for (u32 j = 0; j < k; ++j) {
    const ForestSystem &f = systems[j];
    start[j + 1] = start[j] + static_cast<u32>(f.n);
    gsize[j] = static_cast<u8>(f.sp.group_size);
    pack[j] = static_cast<u8>(std::min(f.sp.pack, 255));
    ptrs[j] = ForestSystemPtrs{f.pos, f.vel, f.acc, f.pot, f.mass};
    const u32 nb = static_cast<u32>(std::min<u64>(64, std::max<u64>(1, (f.n + 8191) / 8192)));
    sys_blk[j] = make_uint2(static_cast<u32>(blk.size()), nb);
    for (u32 r = 0; r < nb; ++r) blk.push_back(make_uint4(j, r, nb, 0u));
  }
  n = start[k];
  sp = systems[0].sp;
  // one upload of the small per-system tables
  const u64 off_start = 0, off_gsize = off_start + 4ull * (k + 1);
  const u64 off_pack = off_gsize + k, off_ptrs = (off_pack + k + 15) & ~15ull;
  const u64 off_blk = (off_ptrs + sizeof(ForestSystemPtrs) * k + 15) & ~15ull;  // uint4 loads
  const u64 off_sblk = off_blk + sizeof(uint4) * blk.size();
  const u64 bytes = off_sblk + sizeof(uint2) * k;
  std::vector<char> h(bytes, 0);
  std::memcpy(h.data() + off_start, start.data(), 4ull * (k + 1));
  std::memcpy(h.data() + off_gsize, gsize.data(), k);
  std::memcpy(h.data() + off_pack, pack.data(), k);
  std::memcpy(h.data() + off_ptrs, ptrs.data(), sizeof(ForestSystemPtrs) * k);
  std::memcpy(h.data() + off_blk, blk.data(), sizeof(uint4) * blk.size());
  std::memcpy(h.data() + off_sblk, sys_blk.data(), sizeof(uint2) * k);
  tables.ensure(bytes);
  GTC_CUDA(cudaMemcpyAsync(tables.ptr, h.data(), bytes, cudaMemcpyHostToDevice, s));
  sysid.ensure(std::max<u64>(1, n) * sizeof(u16));
  roots.ensure(k * sizeof(TreeRoot));
  root_node.ensure(k * sizeof(u32));
  group_root.ensure(std::max<u64>(1, n) * sizeof(u32));
  apos.ensure(std::max<u64>(1, n) * 24);
  amass.ensure(std::max<u64>(1, n) * 8);
  stats.ensure(k * sizeof(ForestSystemStats));
  split_flags.ensure(k * sizeof(u32));
  sys_groups.ensure(k * sizeof(u32));
  sys_max.ensure(4ull * k * sizeof(u32));
  slot_plan.ensure(std::max<u64>(1, n) * 2 * sizeof(uint4));
  graph_slots.ensure(k * sizeof(SysSlots));
  if (host_systems < k) {
    if (host_lists) cudaFreeHost(host_lists);
    host_lists = nullptr;
    host_systems = 0;
    GTC_CUDA(cudaMallocHost(reinterpret_cast<void **>(&host_lists), 5ull * k * sizeof(u32)));
    host_systems = k;
  }
  int T = kLevelsPerWord;
  while (T > 1 && 3ull * k * (1ull << T) * sizeof(double) > kSplitBudget) --T;
  counter.ensure(sizeof(u32));
  if (!host_sc) GTC_CUDA(cudaMallocHost(reinterpret_cast<void **>(&host_sc), sizeof(Scalars)));
  char *t = tables.as<char>();
  ForestView &fv = ws.forest;
  fv.systems = k;
  fv.sys = sysid.as<u16>();
  fv.start = reinterpret_cast<const u32 *>(t + off_start);
  fv.roots = roots.as<TreeRoot>();
  fv.root_node = root_node.as<u32>();
  fv.group_size = reinterpret_cast<const u8 *>(t + off_gsize);
  fv.pack = reinterpret_cast<const u8 *>(t + off_pack);
  fv.group_root = group_root.as<u32>();
  fv.bbox_blocks = reinterpret_cast<const uint4 *>(t + off_blk);
  fv.sys_blocks = reinterpret_cast<const uint2 *>(t + off_sblk);
  fv.bbox_nblocks = static_cast<u32>(blk.size());
  fv.split_levels = T;
  fv.split_unsorted = split_flags.as<u32>();
  fv.sys_groups = sys_groups.as<u32>();
  fv.sys_max = sys_max.as<u32>();
  fv.host_groups = host_lists;
  fv.host_max = host_lists + k;
  fv.slot_plan = slot_plan.as<uint4>();
  ptrs_dev = reinterpret_cast<const ForestSystemPtrs *>(t + off_ptrs);
  if (n == 0) return;
  k_forest_sys<<<ceil_div(n, kT), kT, 0, s>>>(fv.start, k, static_cast<u32>(n), sysid.as<u16>());
  GTC_LAUNCH_CHECK();
  k_forest_gather_bodies<<<ceil_div(n, kT), kT, 0, s>>>(ptrs_dev, fv.sys, fv.start,
                                                        static_cast<u32>(n), apos.as<double>(),
                                                        amass.as<double>());
  GTC_LAUNCH_CHECK();
}

void ForestRun::gather(cudaStream_t s) {
  if (n == 0) return;
  k_forest_gather_bodies<<<ceil_div(n, kT), kT, 0, s>>>(ptrs_dev, ws.forest.sys, ws.forest.start,
                                                        static_cast<u32>(n), apos.as<double>(),
                                                        amass.as<double>());
  GTC_LAUNCH_CHECK();
}

void ForestRun::kick_drift(double h, double dt, cudaStream_t s) {
  if (n == 0) return;
  k_forest_kick_drift<<<ceil_div(n, kT), kT, 0, s>>>(ptrs_dev, ws.forest.sys, ws.forest.start,
                                                     static_cast<u32>(n), h, dt,
                                                     apos.as<double>());
  GTC_LAUNCH_CHECK();
}

void ForestRun::scatter(int kick, double h, const u32 *abort, cudaStream_t s) {
  if (n == 0) return;
  k_forest_scatter<<<ceil_div(n, kT), kT, 0, s>>>(ws.out.as<float4>(), ws.idx.as<u32>(),
                                                  static_cast<u32>(n), ptrs_dev, ws.forest.sys,
                                                  ws.forest.start, kick, h, abort);
  GTC_LAUNCH_CHECK();
}

void ForestRun::solve(int kick, double h, cudaStream_t s, bool write) {
  if (n == 0) return;
  {
    const SideJoin side_join{ws, s};
    build_tree(ws, apos.as<double>(), amass.as<double>(), n, sp, s, host_sc);
    build_lists(ws, sp, s, host_sc);
  }
  ws.out.ensure(n * sizeof(float4));
  evaluate_lists(ws.bodies.as<float4>(), ws.cells.as<float4>(), ws.cell_list.as<u32>(),
                 ws.body_list.as<u32>(), ws.groups.as<uint4>(), ws.n_groups,
                 static_cast<float>(sp.G), static_cast<float>(sp.eps * sp.eps),
                 sp.quadrupole != 0, EvalOut{ws.out.as<float4>()}, counter.as<u32>(), s,
                 ws.eval_shape);
  if (write) scatter(kick, h, nullptr, s);
  GTC_CUDA(cudaMemcpyAsync(host_sc, ws.scalars.ptr, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
  check_device_error(host_sc->error);
}

void ForestRun::step(double dt, cudaStream_t s) {
  const double h = 0.5 * dt;
  kick_drift(h, dt, s);
  solve(1, h, s);
}

bool ForestRun::size_graph_slots(GraphCaps &caps, double headroom, cudaStream_t s) {
  const ForestView &fv = ws.forest;
  const u32 k = fv.systems;
  const double f = 1.0 + headroom, fs = 1.0 + 2.0 * headroom;
  const bool pad = headroom > 0;
  auto slot = [&](u32 longest) {
    const u64 v = (static_cast<u64>(longest * fs) + (pad ? 64 : 0) + 31) & ~31ull;
    return std::max<u64>(32, v);
  };
  std::vector<SysSlots> tab(k);
  u64 at_c = 0, at_b = 0, most_c = 0, most_b = 0;
  for (u32 j = 0; j < k; ++j) {
    const u32 *mx = fv.host_max + 4ull * j;
    const u64 groups = std::min<u64>(sys[j].n, static_cast<u64>(fv.host_groups[j] * f) +
                                                   (pad ? 16 : 0));
    const u64 rc = slot(mx[0]), rb = slot(mx[1]), nc = slot(mx[2]), nb = slot(mx[3]);
    if (rc + nc > 0xffffffffull || rb + nb > 0xffffffffull) return false;
    SysSlots &S = tab[j];
    S = SysSlots{};
    S.groups = static_cast<u32>(std::max<u64>(groups, 1));
    S.rc = static_cast<u32>(rc);
    S.rb = static_cast<u32>(rb);
    S.nc = static_cast<u32>(nc);
    S.nb = static_cast<u32>(nb);
    // rest slots of every group, then near slots, per system
    const u64 rc_at = at_c, nc_at = at_c + S.groups * rc;
    const u64 rb_at = at_b, nb_at = at_b + S.groups * rb;
    at_c = nc_at + S.groups * nc;
    at_b = nb_at + S.groups * nb;
    if (at_c > 0xffffffffull || at_b > 0xffffffffull) return false;
    S.rc_at = static_cast<u32>(rc_at);
    S.nc_at = static_cast<u32>(nc_at);
    S.rb_at = static_cast<u32>(rb_at);
    S.nb_at = static_cast<u32>(nb_at);
    most_c = std::max(most_c, rc + nc);
    most_b = std::max(most_b, rb + nb);
  }
  const u64 pool_c = at_c / 16 + 4 * most_c, pool_b = at_b / 16 + 4 * most_b;
  if (at_c + pool_c > 0xffffffffull || at_b + pool_b > 0xffffffffull) return false;
  GTC_CUDA(cudaMemcpyAsync(graph_slots.ptr, tab.data(), k * sizeof(SysSlots),
                           cudaMemcpyHostToDevice, s));
  GTC_CUDA(cudaStreamSynchronize(s));
  ws.cell_list.ensure((at_c + pool_c) * 4);
  ws.body_list.ensure((at_b + pool_b) * 4);
  caps.sys_slots = graph_slots.as<SysSlots>();
  caps.pool_at_cells = at_c;
  caps.pool_at_bodies = at_b;
  caps.pool_cells = pool_c;
  caps.pool_bodies = pool_b;
  return true;
}

std::vector<ForestSystemStats> ForestRun::system_stats(cudaStream_t s) {
  const u32 k = ws.forest.systems;
  std::vector<ForestSystemStats> out(k);
  if (k == 0) return out;
  GTC_CUDA(cudaMemsetAsync(stats.ptr, 0, k * sizeof(ForestSystemStats), s));
  if (ws.n_groups > 0) {
    k_forest_stats<<<ceil_div(ws.n_groups, kT), kT, 0, s>>>(
        ws.groups.as<uint4>(), static_cast<u32>(ws.n_groups), ws.forest.sys,
        stats.as<ForestSystemStats>());
    GTC_LAUNCH_CHECK();
  }
  GTC_CUDA(cudaMemcpyAsync(out.data(), stats.ptr, k * sizeof(ForestSystemStats),
                           cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
  return out;
}

}  // namespace gtc
