// CPU oracle for the grouped-walk and direct gravity path.
//
// TEST INFRASTRUCTURE ONLY. This is a restatement, in plain C++17 + OpenMP,
// of the reference's CPU algorithm for the hot path. It is the checker for
// the CUDA library and the timed CPU baseline; nothing on the product path
// links or calls it. Parity is pinned: tests/test_oracle_golden.py checks it
// against fixtures generated by the reference itself (tests/golden/), and
// tests/test_oracle_vs_ref.py against the live reference where its sources
// are present.
//
// Every floating-point expression below keeps the reference's operand order
// and grouping, and the file is compiled with -ffp-contract=off, so results
// are bit-identical to the reference's x86-64 build (which has no FMA):
//   tree build          src/octree.cpp:169-273
//   leaf/node moments   src/octree.cpp:46-102
//   per-particle walk   src/octree.cpp:275-344, src/gravity.cpp:7-26
//   direct FP64         src/gravity.cpp:28-45
//   grouped lists       src/group_lists.cpp:18-207
//   list evaluation     include/galactic_tides/kernels/gravity_kernels.h:71-182,
//                       src/gravity_backends.cpp:70-84, :109-137

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using u32 = std::uint32_t;
using u64 = std::uint64_t;

thread_local std::string g_error;

struct D3 {
  double v[3];
};

// One tree node; field order equals the flat export used by the tests.
struct Node {
  double center[3];
  double half;
  double com[3];
  double mass;
  double quad[6];
  double delta;
  std::int32_t first_child, n_children;
  u32 begin, end;
};
static_assert(sizeof(Node) == 136, "node export layout");

constexpr int kDepthCap = 60;           // octree.cpp:18
constexpr u32 kFewBodies = 2;           // group_lists.h:58 (accepted cells this small -> bodies)

struct Tree {
  std::vector<Node> nodes;
  std::vector<u64> order;       // tree position -> original index
  std::vector<D3> tpos;         // positions in tree order
  std::vector<double> tmass;    // masses in tree order
  int depth = 0;
};

// ---------------------------------------------------------------- tree build

bool is_terminal(const Node &nd, u32 leaf_size, int depth) {  // octree.cpp:40-44
  const double s = std::fabs(nd.center[0]) + std::fabs(nd.center[1]) + std::fabs(nd.center[2]);
  return nd.end - nd.begin <= leaf_size || depth >= kDepthCap || nd.half < 1e-12 * (s + 1e-300);
}

int octant_of(const D3 &p, const double *c) {  // octree.cpp:20-22
  int o = 0;
  if (p.v[0] >= c[0]) o |= 1;
  if (p.v[1] >= c[1]) o |= 2;
  if (p.v[2] >= c[2]) o |= 4;
  return o;
}

struct Builder {
  const std::vector<D3> &pos;
  const double *mass;
  std::vector<u64> &index;
  std::vector<u64> &tmp;
  u32 leaf_size;
};

// Mass, centre of mass and traceless quadrupole from the bodies of a leaf.
void moments_from_bodies(const Builder &b, Node &nd) {  // octree.cpp:46-72
  double m = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
  for (u32 k = nd.begin; k < nd.end; ++k) {
    const u64 i = b.index[k];
    const double mi = b.mass[i];
    m += mi;
    cx += mi * b.pos[i].v[0];
    cy += mi * b.pos[i].v[1];
    cz += mi * b.pos[i].v[2];
  }
  if (m > 0) {
    cx /= m;
    cy /= m;
    cz /= m;
  } else {
    cx = nd.center[0];
    cy = nd.center[1];
    cz = nd.center[2];
  }
  double q[6] = {0, 0, 0, 0, 0, 0};
  for (u32 k = nd.begin; k < nd.end; ++k) {
    const u64 i = b.index[k];
    const double mi = b.mass[i];
    const double dx = b.pos[i].v[0] - cx, dy = b.pos[i].v[1] - cy, dz = b.pos[i].v[2] - cz;
    const double r2 = dx * dx + dy * dy + dz * dz;
    q[0] += mi * (3 * dx * dx - r2);
    q[1] += mi * (3 * dy * dy - r2);
    q[2] += mi * (3 * dz * dz - r2);
    q[3] += mi * 3 * dx * dy;
    q[4] += mi * 3 * dx * dz;
    q[5] += mi * 3 * dy * dz;
  }
  nd.mass = m;
  nd.com[0] = cx;
  nd.com[1] = cy;
  nd.com[2] = cz;
  std::memcpy(nd.quad, q, sizeof q);
  const double ex = cx - nd.center[0], ey = cy - nd.center[1], ez = cz - nd.center[2];
  nd.delta = std::sqrt(ex * ex + ey * ey + ez * ez);
}

// The same moments from a node's children, by the parallel axis theorem.
void moments_from_children(std::vector<Node> &nodes, std::size_t ni) {  // octree.cpp:75-102
  Node &nd = nodes[ni];
  const std::size_t c0 = static_cast<std::size_t>(nd.first_child);
  const std::size_t c1 = c0 + static_cast<std::size_t>(nd.n_children);
  double m = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
  for (std::size_t k = c0; k < c1; ++k) {
    const Node &ch = nodes[k];
    m += ch.mass;
    cx += ch.mass * ch.com[0];
    cy += ch.mass * ch.com[1];
    cz += ch.mass * ch.com[2];
  }
  if (m > 0) {
    cx /= m;
    cy /= m;
    cz /= m;
  } else {
    cx = nd.center[0];
    cy = nd.center[1];
    cz = nd.center[2];
  }
  double q[6] = {0, 0, 0, 0, 0, 0};
  for (std::size_t k = c0; k < c1; ++k) {
    const Node &ch = nodes[k];
    const double dx = ch.com[0] - cx, dy = ch.com[1] - cy, dz = ch.com[2] - cz;
    const double r2 = dx * dx + dy * dy + dz * dz;
    q[0] += ch.quad[0] + ch.mass * (3 * dx * dx - r2);
    q[1] += ch.quad[1] + ch.mass * (3 * dy * dy - r2);
    q[2] += ch.quad[2] + ch.mass * (3 * dz * dz - r2);
    q[3] += ch.quad[3] + ch.mass * 3 * dx * dy;
    q[4] += ch.quad[4] + ch.mass * 3 * dx * dz;
    q[5] += ch.quad[5] + ch.mass * 3 * dy * dz;
  }
  nd.mass = m;
  nd.com[0] = cx;
  nd.com[1] = cy;
  nd.com[2] = cz;
  std::memcpy(nd.quad, q, sizeof q);
  const double ex = cx - nd.center[0], ey = cy - nd.center[1], ez = cz - nd.center[2];
  nd.delta = std::sqrt(ex * ex + ey * ey + ez * ez);
}

// Stable partition of a node's bodies into octants; the non-empty children
// are appended to `nodes` as one block, in octant order.  octree.cpp:106-140
void divide(const Builder &b, std::vector<Node> &nodes, std::size_t ni) {
  const u32 lo = nodes[ni].begin, hi = nodes[ni].end;
  double c[3];
  std::memcpy(c, nodes[ni].center, sizeof c);
  const double h = nodes[ni].half;
  u32 start[9] = {0};
  for (u32 k = lo; k < hi; ++k) ++start[octant_of(b.pos[b.index[k]], c) + 1];
  start[0] = lo;
  for (int o = 1; o <= 8; ++o) start[o] += start[o - 1];
  u32 cursor[8];
  std::copy(start, start + 8, cursor);
  for (u32 k = lo; k < hi; ++k) {
    const u64 i = b.index[k];
    b.tmp[cursor[octant_of(b.pos[i], c)]++] = i;
  }
  std::copy(b.tmp.begin() + lo, b.tmp.begin() + hi, b.index.begin() + lo);

  const double hc = 0.5 * h;
  const std::size_t first = nodes.size();
  int kids = 0;
  for (int o = 0; o < 8; ++o) {
    if (start[o + 1] == start[o]) continue;
    Node ch{};
    ch.half = hc;
    ch.center[0] = c[0] + ((o & 1) ? hc : -hc);
    ch.center[1] = c[1] + ((o & 2) ? hc : -hc);
    ch.center[2] = c[2] + ((o & 4) ? hc : -hc);
    ch.first_child = -1;
    ch.begin = start[o];
    ch.end = start[o + 1];
    nodes.push_back(ch);
    ++kids;
  }
  nodes[ni].first_child = static_cast<std::int32_t>(first);
  nodes[ni].n_children = kids;
}

// Builds the subtree below node `top` (geometry and range set) in the
// serial layout: children blocks in the order their parents are divided,
// depth first. Moments are then filled from the highest index down, since
// children always sit after their parent. Returns the deepest level.
int grow(const Builder &b, std::vector<Node> &nodes, std::size_t top, int top_depth) {
  int deepest = top_depth;
  std::vector<std::pair<std::size_t, int>> todo{{top, top_depth}};
  const std::size_t mark = nodes.size();
  while (!todo.empty()) {
    const auto [ni, d] = todo.back();
    todo.pop_back();
    deepest = std::max(deepest, d);
    if (is_terminal(nodes[ni], b.leaf_size, d)) continue;
    divide(b, nodes, ni);
    const int nc = nodes[ni].n_children;
    const std::size_t fc = static_cast<std::size_t>(nodes[ni].first_child);
    for (int k = nc - 1; k >= 0; --k) todo.emplace_back(fc + k, d + 1);
  }
  auto fill = [&](std::size_t ni) {
    if (nodes[ni].n_children == 0) moments_from_bodies(b, nodes[ni]);
    else moments_from_children(nodes, ni);
  };
  for (std::size_t k = nodes.size(); k-- > mark;) fill(k);
  fill(top);
  return deepest;
}

int omp_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Octree::build. With n >= parallel_threshold the top levels are divided
// breadth first until there are 8 x threads subtrees (at most 4 levels),
// which are grown concurrently and spliced in: the reference's parallel
// layout (octree.cpp:210-266). Otherwise the serial layout.
void build_tree(Tree &t, const std::vector<D3> &pos, const double *mass, int leaf_size,
                u64 parallel_threshold) {
  const u64 n = pos.size();
  if (n > 0xffffffffull) throw std::invalid_argument("Octree::build: too many particles");
  const u32 leaf = static_cast<u32>(std::max(1, leaf_size));
  t.nodes.clear();
  t.depth = 0;
  t.order.resize(n);
  t.tpos.resize(n);
  t.tmass.resize(n);
  if (n == 0) return;
  std::vector<u64> tmp(n);
  double lo[3], hi[3];
  for (int a = 0; a < 3; ++a) lo[a] = hi[a] = pos[0].v[a];
  for (u64 k = 0; k < n; ++k) {
    t.order[k] = k;
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], pos[k].v[a]);
      hi[a] = std::max(hi[a], pos[k].v[a]);
    }
  }
  double half = 0.0;
  for (int a = 0; a < 3; ++a) half = std::max(half, 0.5 * (hi[a] - lo[a]));
  half = half * (1.0 + 1e-9) + 1e-300;
  Node root{};
  for (int a = 0; a < 3; ++a) root.center[a] = (lo[a] + hi[a]) * 0.5;
  root.half = half;
  root.first_child = -1;
  root.begin = 0;
  root.end = static_cast<u32>(n);
  t.nodes.reserve(2 * n / leaf + 16);
  t.nodes.push_back(root);
  const Builder b{pos, mass, t.order, tmp, leaf};

  if (n < parallel_threshold) {
    t.depth = grow(b, t.nodes, 0, 0);
  } else {
    const std::size_t want = 8 * static_cast<std::size_t>(omp_threads());
    std::vector<std::size_t> divided;
    std::vector<std::pair<std::size_t, int>> front{{0, 0}}, next;
    for (int d = 0; d < 4 && !front.empty() && front.size() < want; ++d) {
      next.clear();
      for (const auto &[ni, dep] : front) {
        if (is_terminal(t.nodes[ni], leaf, dep)) {
          moments_from_bodies(b, t.nodes[ni]);
          t.depth = std::max(t.depth, dep);
          continue;
        }
        divide(b, t.nodes, ni);
        divided.push_back(ni);
        for (int c = 0; c < t.nodes[ni].n_children; ++c)
          next.emplace_back(static_cast<std::size_t>(t.nodes[ni].first_child + c), dep + 1);
      }
      front.swap(next);
    }
    std::vector<std::vector<Node>> part(front.size());
    std::vector<int> deep(front.size(), 0);
#pragma omp parallel for schedule(dynamic, 1)
    for (long k = 0; k < static_cast<long>(front.size()); ++k) {
      const Node &r = t.nodes[front[k].first];
      part[k].reserve(2 * (r.end - r.begin) / leaf + 16);
      part[k].push_back(r);
      deep[k] = grow(b, part[k], 0, front[k].second);
    }
    std::vector<std::size_t> base(front.size());
    std::size_t total = t.nodes.size();
    for (std::size_t k = 0; k < front.size(); ++k) {
      base[k] = total;
      total += part[k].size() - 1;
      t.depth = std::max(t.depth, deep[k]);
    }
    t.nodes.resize(total);
#pragma omp parallel for schedule(dynamic, 1)
    for (long k = 0; k < static_cast<long>(front.size()); ++k) {
      auto moved = [&](Node nd) {
        if (nd.first_child >= 0) nd.first_child = static_cast<std::int32_t>(base[k] + nd.first_child - 1);
        return nd;
      };
      t.nodes[front[k].first] = moved(part[k][0]);
      for (std::size_t i = 1; i < part[k].size(); ++i) t.nodes[base[k] + i - 1] = moved(part[k][i]);
    }
    for (auto it = divided.rbegin(); it != divided.rend(); ++it)
      moments_from_children(t.nodes, *it);
  }
#pragma omp parallel for schedule(static)
  for (long k = 0; k < static_cast<long>(n); ++k) {
    t.tpos[k] = pos[t.order[k]];
    t.tmass[k] = mass[t.order[k]];
  }
}

// ------------------------------------------------------- per-particle walk

// Octree::accel_pot: Barnes (1994) offset criterion, quadrupoles, FP64.
void walk_one(const Tree &t, const double *x, u64 self, double G, double theta, double eps,
              bool quad, double *acc, double *pot, u64 *ncell, u64 *npart) {  // octree.cpp:275-344
  acc[0] = acc[1] = acc[2] = 0.0;
  *pot = 0.0;
  if (t.nodes.empty()) return;
  const double eps2 = eps * eps, inv_theta = 1.0 / theta;
  u64 nc = 0, np = 0;
  double ax = 0, ay = 0, az = 0, phi = 0;
  std::vector<u32> stack;
  stack.reserve(512);
  stack.push_back(0);
  while (!stack.empty()) {
    const Node &nd = t.nodes[stack.back()];
    stack.pop_back();
    const double dx = x[0] - nd.com[0], dy = x[1] - nd.com[1], dz = x[2] - nd.com[2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double crit = 2.0 * nd.half * inv_theta + nd.delta;
    const double slack = nd.half * 1.0001;
    const bool inside = std::fabs(x[0] - nd.center[0]) <= slack &&
                        std::fabs(x[1] - nd.center[1]) <= slack &&
                        std::fabs(x[2] - nd.center[2]) <= slack;
    if (!inside && r2 > crit * crit) {
      const double r2s = r2 + eps2;
      const double inv = 1.0 / std::sqrt(r2s);
      const double inv3 = inv * inv * inv;
      const double gm3 = G * nd.mass * inv3;
      ax -= gm3 * dx;
      ay -= gm3 * dy;
      az -= gm3 * dz;
      phi -= G * nd.mass * inv;
      if (quad) {
        const double *q = nd.quad;
        const double qx = q[0] * dx + q[3] * dy + q[4] * dz;
        const double qy = q[3] * dx + q[1] * dy + q[5] * dz;
        const double qz = q[4] * dx + q[5] * dy + q[2] * dz;
        const double rqr = dx * qx + dy * qy + dz * qz;
        const double inv5 = inv3 * inv * inv;
        const double inv7 = inv5 * inv * inv;
        ax += G * (qx * inv5 - 2.5 * rqr * dx * inv7);
        ay += G * (qy * inv5 - 2.5 * rqr * dy * inv7);
        az += G * (qz * inv5 - 2.5 * rqr * dz * inv7);
        phi -= 0.5 * G * rqr * inv5;
      }
      ++nc;
    } else if (nd.n_children == 0) {
      for (u32 k = nd.begin; k < nd.end; ++k) {
        if (t.order[k] == self) continue;
        const double ex = x[0] - t.tpos[k].v[0], ey = x[1] - t.tpos[k].v[1],
                     ez = x[2] - t.tpos[k].v[2];
        const double r2s = ex * ex + ey * ey + ez * ez + eps2;
        const double inv = 1.0 / std::sqrt(r2s);
        const double gm3 = G * t.tmass[k] * inv * inv * inv;
        ax -= gm3 * ex;
        ay -= gm3 * ey;
        az -= gm3 * ez;
        phi -= G * t.tmass[k] * inv;
        ++np;
      }
    } else {
      for (int c = 0; c < nd.n_children; ++c) stack.push_back(static_cast<u32>(nd.first_child + c));
    }
  }
  acc[0] = ax;
  acc[1] = ay;
  acc[2] = az;
  *pot = phi;
  if (ncell) *ncell += nc;
  if (npart) *npart += np;
}

// ------------------------------------------------------------ group lists

struct Lists {
  double origin[3];
  std::vector<float> bodies;        // 4 per body, tree order
  std::vector<float> cells;         // 12 per node
  std::vector<u32> cell_list, body_list;
  std::vector<u32> groups;          // 8 per group: begin end cb ce bb be 0 0
  u64 cell_interactions = 0, body_interactions = 0, max_list = 0;
  int max_group = 0;
};

struct WalkRec {  // group_lists.h:28-35
  double center[3], half, com[3], crit;
  std::int32_t first_child, n_children;
  u32 begin, end;
};

void build_lists(const Tree &t, double theta, int group_size, bool pack, Lists &out) {
  if (group_size < 1) throw std::invalid_argument("group_size must be at least 1");
  const auto &nodes = t.nodes;
  const u64 n = t.tpos.size();
  if (n > 0xffffffffull || nodes.size() > 0xffffffffull)
    throw std::runtime_error("too many particles for the 32 bit GPU indices");
  out.cell_interactions = out.body_interactions = out.max_list = 0;
  out.max_group = 0;
  out.bodies.assign(4 * n, 0.0f);
  out.cells.assign(12 * nodes.size(), 0.0f);
  out.groups.clear();
  out.cell_list.clear();
  out.body_list.clear();
  if (n == 0) return;

  // FP32 packing relative to the root centre; walk records.  group_lists.cpp:40-63
  for (int a = 0; a < 3; ++a) out.origin[a] = nodes[0].center[a];
  const double inv_theta = 1.0 / theta;
  std::vector<WalkRec> rec(nodes.size());
#pragma omp parallel
  {
#pragma omp for schedule(static) nowait
    for (long k = 0; k < static_cast<long>(n); ++k) {
      float *o = &out.bodies[4 * k];
      for (int a = 0; a < 3; ++a) o[a] = static_cast<float>(t.tpos[k].v[a] - out.origin[a]);
      o[3] = static_cast<float>(t.tmass[k]);
    }
#pragma omp for schedule(static)
    for (long k = 0; k < static_cast<long>(nodes.size()); ++k) {
      const Node &nd = nodes[k];
      float *c = &out.cells[12 * k];
      for (int a = 0; a < 3; ++a) c[a] = static_cast<float>(nd.com[a] - out.origin[a]);
      c[3] = static_cast<float>(nd.mass);
      for (int q = 0; q < 6; ++q) c[4 + q] = static_cast<float>(nd.quad[q]);
      WalkRec &w = rec[k];
      std::memcpy(w.center, nd.center, sizeof w.center);
      w.half = nd.half;
      std::memcpy(w.com, nd.com, sizeof w.com);
      w.crit = 2.0 * nd.half * inv_theta + nd.delta;
      w.first_child = nd.first_child;
      w.n_children = nd.n_children;
      w.begin = nd.begin;
      w.end = nd.end;
    }
  }

  // Group selection, depth first.  group_lists.cpp:65-113
  const u32 gs = static_cast<u32>(group_size);
  std::vector<std::pair<u32, u32>> spans;
  auto cut = [&](u32 b, u32 e) {
    for (u32 c = b; c < e; c += gs) spans.emplace_back(c, std::min(e, c + gs));
  };
  {
    // Explicit stack of (node, next child to look at, open run [rb, re)).
    struct Frame {
      std::size_t node;
      int next;
      u32 rb, re;
      bool open;
    };
    const Node &root = nodes[0];
    if (root.end - root.begin <= gs || root.n_children == 0) {
      cut(root.begin, root.end);
    } else {
      std::vector<Frame> st{{0, 0, 0, 0, false}};
      while (!st.empty()) {
        Frame &f = st.back();
        const Node &nd = nodes[f.node];
        if (f.next == nd.n_children) {
          if (f.open) spans.emplace_back(f.rb, f.re);
          st.pop_back();
          continue;
        }
        const std::size_t ci = static_cast<std::size_t>(nd.first_child + f.next++);
        const Node &ch = nodes[ci];
        const u32 cc = ch.end - ch.begin;
        if (cc <= gs) {
          if (pack && f.open && (f.re - f.rb) + cc <= gs) {
            f.re = ch.end;
          } else {
            if (f.open) spans.emplace_back(f.rb, f.re);
            f.rb = ch.begin;
            f.re = ch.end;
            f.open = true;
          }
        } else {
          if (f.open) spans.emplace_back(f.rb, f.re);
          f.open = false;
          if (ch.n_children == 0) cut(ch.begin, ch.end);
          else st.push_back({ci, 0, 0, 0, false});
        }
      }
    }
  }

  // One walk per group.  group_lists.cpp:115-166
  const std::size_t ng = spans.size();
  std::vector<std::vector<u32>> gcells(ng), gbodies(ng);
#pragma omp parallel for schedule(dynamic, 16)
  for (long g = 0; g < static_cast<long>(ng); ++g) {
    const u32 b0 = spans[g].first, b1 = spans[g].second;
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) lo[a] = hi[a] = t.tpos[b0].v[a];
    for (u32 k = b0; k < b1; ++k)
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], t.tpos[k].v[a]);
        hi[a] = std::max(hi[a], t.tpos[k].v[a]);
      }
    double gc[3], gh[3];
    for (int a = 0; a < 3; ++a) {
      gc[a] = (lo[a] + hi[a]) * 0.5;
      gh[a] = (hi[a] - lo[a]) * 0.5;
    }
    auto &cl = gcells[g];
    auto &bl = gbodies[g];
    auto take = [&](u32 b, u32 e) {
      for (u32 j = b; j < e; ++j) bl.push_back(j);
    };
    std::vector<u32> stack;
    stack.reserve(512);
    stack.push_back(0);
    while (!stack.empty()) {
      const u32 ni = stack.back();
      stack.pop_back();
      const WalkRec &w = rec[ni];
      bool overlap = true;
      double d2 = 0.0;
      for (int a = 0; a < 3; ++a) {
        if (std::fabs(w.center[a] - gc[a]) > w.half * 1.0001 + gh[a]) overlap = false;
        const double d = std::fabs(w.com[a] - gc[a]) - gh[a];
        if (d > 0) d2 += d * d;
      }
      if (!overlap && d2 > w.crit * w.crit) {
        if (w.end - w.begin <= kFewBodies) take(w.begin, w.end);
        else cl.push_back(ni);
      } else if (w.n_children == 0) {
        take(w.begin, w.end);
      } else {
        for (int c = 0; c < w.n_children; ++c) stack.push_back(static_cast<u32>(w.first_child + c));
      }
    }
  }

  // Flatten and count.  group_lists.cpp:168-207
  out.groups.assign(8 * ng, 0);
  u64 nc = 0, nb = 0;
  for (std::size_t g = 0; g < ng; ++g) {
    u32 *G = &out.groups[8 * g];
    G[0] = spans[g].first;
    G[1] = spans[g].second;
    G[2] = static_cast<u32>(nc);
    nc += gcells[g].size();
    G[3] = static_cast<u32>(nc);
    G[4] = static_cast<u32>(nb);
    nb += gbodies[g].size();
    G[5] = static_cast<u32>(nb);
    if (nc > 0xffffffffull || nb > 0xffffffffull)
      throw std::runtime_error("interaction lists too long for 32 bit offsets");
  }
  out.cell_list.resize(nc);
  out.body_list.resize(nb);
  u64 ci = 0, bi = 0, ml = 0;
  int mg = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : ci, bi) reduction(max : ml, mg)
  for (long g = 0; g < static_cast<long>(ng); ++g) {
    const u32 *G = &out.groups[8 * g];
    std::copy(gcells[g].begin(), gcells[g].end(), out.cell_list.begin() + G[2]);
    std::copy(gbodies[g].begin(), gbodies[g].end(), out.body_list.begin() + G[4]);
    const u64 targets = G[1] - G[0];
    ci += targets * gcells[g].size();
    bi += targets * gbodies[g].size() - targets;
    ml = std::max<u64>(ml, gcells[g].size() + gbodies[g].size());
    mg = std::max(mg, static_cast<int>(targets));
  }
  out.cell_interactions = ci;
  out.body_interactions = bi;
  out.max_list = ml;
  out.max_group = mg;
}

// ----------------------------------------------------- FP32 list arithmetic

struct Acc4 {
  float ax, ay, az, pot;
};

inline float recip_sqrt(float v) { return 1.0f / std::sqrt(v); }  // gravity_kernels.h:39

inline void add_body(Acc4 &a, float px, float py, float pz, const float *b, float G,
                     float eps2) {  // gravity_kernels.h:71-83
  const float dx = px - b[0], dy = py - b[1], dz = pz - b[2];
  const float inv = recip_sqrt(dx * dx + dy * dy + dz * dz + eps2);
  const float gm = G * b[3] * inv;
  const float gm3 = gm * inv * inv;
  a.ax -= gm3 * dx;
  a.ay -= gm3 * dy;
  a.az -= gm3 * dz;
  a.pot -= gm;
}

inline void add_cell(Acc4 &a, float px, float py, float pz, const float *c, float G, float eps2,
                     bool quad) {  // gravity_kernels.h:109-135
  const float dx = px - c[0], dy = py - c[1], dz = pz - c[2];
  const float inv = recip_sqrt(dx * dx + dy * dy + dz * dz + eps2);
  const float inv2 = inv * inv;
  const float inv3 = inv * inv2;
  const float gm = G * c[3];
  a.ax -= gm * inv3 * dx;
  a.ay -= gm * inv3 * dy;
  a.az -= gm * inv3 * dz;
  a.pot -= gm * inv;
  if (quad) {
    // c[4..9] = xx yy zz xy xz yz
    const float qx = c[4] * dx + c[7] * dy + c[8] * dz;
    const float qy = c[7] * dx + c[5] * dy + c[9] * dz;
    const float qz = c[8] * dx + c[9] * dy + c[6] * dz;
    const float rqr = dx * qx + dy * qy + dz * qz;
    const float inv5 = inv3 * inv2;
    const float inv7 = inv5 * inv2;
    a.ax += G * (qx * inv5 - 2.5f * rqr * dx * inv7);
    a.ay += G * (qy * inv5 - 2.5f * rqr * dy * inv7);
    a.az += G * (qz * inv5 - 2.5f * rqr * dz * inv7);
    a.pot -= 0.5f * G * rqr * inv5;
  }
}

// evaluate_group_lists_cpu: cells then bodies, list order, skipping self.
void eval_lists(const float *bodies, const float *cells, const u32 *cell_list,
                const u32 *body_list, const u32 *groups, u64 ng, float G, float eps2, bool quad,
                float *out) {
#pragma omp parallel for schedule(dynamic, 8)
  for (long g = 0; g < static_cast<long>(ng); ++g) {
    const u32 *grp = &groups[8 * g];
    for (u32 i = grp[0]; i < grp[1]; ++i) {
      const float *bi = &bodies[4 * i];
      Acc4 a{0.0f, 0.0f, 0.0f, 0.0f};
      for (u32 k = grp[2]; k < grp[3]; ++k)
        add_cell(a, bi[0], bi[1], bi[2], &cells[12 * static_cast<u64>(cell_list[k])], G, eps2, quad);
      for (u32 k = grp[4]; k < grp[5]; ++k) {
        const u32 j = body_list[k];
        if (j == i) continue;
        add_body(a, bi[0], bi[1], bi[2], &bodies[4 * static_cast<u64>(j)], G, eps2);
      }
      out[4 * i] = a.ax;
      out[4 * i + 1] = a.ay;
      out[4 * i + 2] = a.az;
      out[4 * i + 3] = a.pot;
    }
  }
}

std::vector<D3> to_d3(const double *pos, u64 n) {
  std::vector<D3> p(n);
  for (u64 i = 0; i < n; ++i) p[i] = D3{{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}};
  return p;
}

double seconds(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

struct GroupState {  // what GroupTreeGravity keeps between calls
  Tree tree;
  Lists lists;
  std::vector<float> out;
};

}  // namespace

extern "C" {

struct OrcListStats {
  u64 n_groups, n_cell_list, n_body_list;
  u64 cell_interactions, body_interactions, max_list;
  std::int64_t max_group;
  double origin[3];
};

struct OrcTimings {
  double tree, lists, evaluate, total;  // seconds; total includes the scatter
  u64 cell_interactions, particle_interactions;
};

const char *orc_last_error() { return g_error.c_str(); }
int orc_threads() { return omp_threads(); }

void *orc_tree_build(const double *pos, const double *mass, u64 n, int leaf_size,
                     u64 parallel_threshold) {
  try {
    auto *t = new Tree;
    build_tree(*t, to_d3(pos, n), mass, leaf_size, parallel_threshold);
    return t;
  } catch (const std::exception &e) {
    g_error = e.what();
    return nullptr;
  }
}
void orc_tree_free(void *h) { delete static_cast<Tree *>(h); }
u64 orc_tree_nnodes(void *h) { return static_cast<Tree *>(h)->nodes.size(); }
int orc_tree_depth(void *h) { return static_cast<Tree *>(h)->depth; }
void orc_tree_export(void *h, Node *nodes, u64 *order) {
  const Tree &t = *static_cast<Tree *>(h);
  if (nodes) std::memcpy(nodes, t.nodes.data(), t.nodes.size() * sizeof(Node));
  if (order) std::memcpy(order, t.order.data(), t.order.size() * sizeof(u64));
}
void orc_tree_accel_pot(void *h, const double *x, u64 self, double G, double theta, double eps,
                        int quad, double *acc, double *pot) {
  walk_one(*static_cast<Tree *>(h), x, self, G, theta, eps, quad != 0, acc, pot, nullptr, nullptr);
}

void *orc_lists_build(void *tree, double theta, int group_size, int pack) {
  try {
    auto *L = new Lists;
    build_lists(*static_cast<Tree *>(tree), theta, group_size, pack != 0, *L);
    return L;
  } catch (const std::exception &e) {
    g_error = e.what();
    return nullptr;
  }
}
void orc_lists_free(void *h) { delete static_cast<Lists *>(h); }
void orc_lists_stats(void *h, OrcListStats *s) {
  const Lists &L = *static_cast<Lists *>(h);
  s->n_groups = L.groups.size() / 8;
  s->n_cell_list = L.cell_list.size();
  s->n_body_list = L.body_list.size();
  s->cell_interactions = L.cell_interactions;
  s->body_interactions = L.body_interactions;
  s->max_list = L.max_list;
  s->max_group = L.max_group;
  std::memcpy(s->origin, L.origin, sizeof s->origin);
}
void orc_lists_export(void *h, float *bodies, float *cells, u32 *cell_list, u32 *body_list,
                      u32 *groups) {
  const Lists &L = *static_cast<Lists *>(h);
  if (bodies) std::memcpy(bodies, L.bodies.data(), L.bodies.size() * 4);
  if (cells) std::memcpy(cells, L.cells.data(), L.cells.size() * 4);
  if (cell_list) std::memcpy(cell_list, L.cell_list.data(), L.cell_list.size() * 4);
  if (body_list) std::memcpy(body_list, L.body_list.data(), L.body_list.size() * 4);
  if (groups) std::memcpy(groups, L.groups.data(), L.groups.size() * 4);
}

// The list arithmetic on arbitrary arrays in the GPU layout (bodies float4,
// cells 3 x float4, groups 8 x uint32): the checker for the CUDA evaluator.
void orc_eval_lists(const float *bodies, u64 n, const float *cells, const u32 *cell_list,
                    const u32 *body_list, const u32 *groups, u64 n_groups, double G, double eps,
                    int quad, float *out) {
  std::fill(out, out + 4 * n, 0.0f);
  eval_lists(bodies, cells, cell_list, body_list, groups, n_groups, static_cast<float>(G),
             static_cast<float>(eps * eps), quad != 0, out);
}

// GroupTreeGravity::compute on the CPU (gravity_backends.cpp:109-137):
// tree, lists, evaluation, scatter to original order. `repeat` calls, the
// timings are those of the fastest.
int orc_group_force(const double *pos, const double *mass, u64 n, double G, double theta,
                    double eps, int quad, int group_size, int leaf_size, int pack, int repeat,
                    u64 parallel_threshold, double *acc, double *pot, OrcTimings *tm) {
  try {
    using clock = std::chrono::steady_clock;
    const std::vector<D3> p = to_d3(pos, n);
    GroupState st;
    OrcTimings best{0, 0, 0, 1e300, 0, 0};
    for (int r = 0; r < std::max(1, repeat); ++r) {
      const auto t0 = clock::now();
      build_tree(st.tree, p, mass, leaf_size, parallel_threshold);
      const auto t1 = clock::now();
      build_lists(st.tree, theta, group_size, pack != 0, st.lists);
      const auto t2 = clock::now();
      st.out.assign(4 * n, 0.0f);
      eval_lists(st.lists.bodies.data(), st.lists.cells.data(), st.lists.cell_list.data(),
                 st.lists.body_list.data(), st.lists.groups.data(), st.lists.groups.size() / 8,
                 static_cast<float>(G), static_cast<float>(eps * eps), quad != 0, st.out.data());
      const auto t3 = clock::now();
      for (u64 k = 0; k < n; ++k) {
        const u64 i = st.tree.order[k];
        for (int a = 0; a < 3; ++a) acc[3 * i + a] = st.out[4 * k + a];
        pot[i] = st.out[4 * k + 3];
      }
      const auto t4 = clock::now();
      const double total = seconds(t0, t4);
      if (total < best.total)
        best = OrcTimings{seconds(t0, t1), seconds(t1, t2), seconds(t2, t3), total,
                          st.lists.cell_interactions, st.lists.body_interactions};
    }
    if (tm) *tm = best;
    return 0;
  } catch (const std::exception &e) {
    g_error = e.what();
    return 1;
  }
}

// compute_gravity_tree: build, then walk every target in tree order.
int orc_tree_force(const double *pos, const double *mass, u64 n, double G, double theta,
                   double eps, int quad, int leaf_size, u64 parallel_threshold, double *acc,
                   double *pot, u64 *stats) {
  try {
    Tree t;
    build_tree(t, to_d3(pos, n), mass, leaf_size, parallel_threshold);
    u64 ncell = 0, npart = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : ncell, npart)
    for (long k = 0; k < static_cast<long>(n); ++k) {
      const u64 i = t.order[k];
      walk_one(t, &pos[3 * i], i, G, theta, eps, quad != 0, &acc[3 * i], &pot[i], &ncell, &npart);
    }
    if (stats) {
      stats[0] = ncell;
      stats[1] = npart;
    }
    return 0;
  } catch (const std::exception &e) {
    g_error = e.what();
    return 1;
  }
}

// compute_gravity_direct restricted to targets idx[0..m): FP64 all-pairs,
// skipping j == i (gravity.cpp:28-45; the sampled form of bench:74-95).
void orc_direct_fp64(const double *pos, const double *mass, u64 n, const u64 *idx, u64 m, double G,
                     double eps, double *acc, double *pot) {
  const double eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 4)
  for (long s = 0; s < static_cast<long>(m); ++s) {
    const u64 i = idx ? idx[s] : static_cast<u64>(s);
    double ax = 0, ay = 0, az = 0, phi = 0;
    for (u64 j = 0; j < n; ++j) {
      if (j == i) continue;
      const double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1],
                   dz = pos[3 * i + 2] - pos[3 * j + 2];
      const double inv = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz + eps2);
      const double s3 = G * mass[j] * inv * inv * inv;
      ax -= s3 * dx;
      ay -= s3 * dy;
      az -= s3 * dz;
      phi -= G * mass[j] * inv;
    }
    acc[3 * s] = ax;
    acc[3 * s + 1] = ay;
    acc[3 * s + 2] = az;
    pot[s] = phi;
  }
}

// pack_bodies (gravity_backends.cpp:15-23): float4 relative to `origin`.
void orc_pack_bodies(const double *pos, const double *mass, u64 n, const double *origin,
                     float *out) {
  for (u64 i = 0; i < n; ++i) {
    for (int a = 0; a < 3; ++a) out[4 * i + a] = static_cast<float>(pos[3 * i + a] - origin[a]);
    out[4 * i + 3] = static_cast<float>(mass[i]);
  }
}

// gt_direct_accel for targets idx[0..m) (gravity_kernels.h:173-182), FP32.
void orc_direct_fp32(const float *bodies, u64 n, const u64 *idx, u64 m, double G, double eps,
                     float *out) {
  const float g = static_cast<float>(G), e2 = static_cast<float>(eps * eps);
#pragma omp parallel for schedule(dynamic, 16)
  for (long s = 0; s < static_cast<long>(m); ++s) {
    const u64 i = idx ? idx[s] : static_cast<u64>(s);
    const float *bi = &bodies[4 * i];
    Acc4 a{0.0f, 0.0f, 0.0f, 0.0f};
    for (u64 j = 0; j < n; ++j) {
      if (j == i) continue;
      add_body(a, bi[0], bi[1], bi[2], &bodies[4 * j], g, e2);
    }
    out[4 * s] = a.ax;
    out[4 * s + 1] = a.ay;
    out[4 * s + 2] = a.az;
    out[4 * s + 3] = a.pot;
  }
}

// One kick-drift-kick step sequence with the CPU group solver
// (integrator.cpp:5-16), energies before and after (integrator.cpp:18-33).
int orc_leapfrog_group(double *pos, double *vel, const double *mass, u64 n, double G,
                       double theta, double eps, int group_size, int leaf_size, int pack,
                       double dt, int steps, double *energy) {
  std::vector<double> acc(3 * n), pot(n);
  auto force = [&]() {
    return orc_group_force(pos, mass, n, G, theta, eps, 1, group_size, leaf_size, pack, 1,
                           ~0ull, acc.data(), pot.data(), nullptr);
  };
  auto total_energy = [&]() {
    double kin = 0, phi = 0;
    for (u64 i = 0; i < n; ++i) {
      const double v2 = vel[3 * i] * vel[3 * i] + vel[3 * i + 1] * vel[3 * i + 1] +
                        vel[3 * i + 2] * vel[3 * i + 2];
      kin += 0.5 * mass[i] * v2;
      phi += 0.5 * mass[i] * pot[i];
    }
    return kin + phi;
  };
  if (force()) return 1;
  energy[0] = total_energy();
  const double h = 0.5 * dt;
  for (int s = 0; s < steps; ++s) {
    for (u64 k = 0; k < 3 * n; ++k) {
      vel[k] += h * acc[k];
      pos[k] += dt * vel[k];
    }
    if (force()) return 1;
    for (u64 k = 0; k < 3 * n; ++k) vel[k] += h * acc[k];
  }
  energy[1] = total_energy();
  return 0;
}

}  // extern "C"
