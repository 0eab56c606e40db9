// Octree build on the device, bit-identical to the reference's CPU build
// (src/octree.cpp:169-273). Compiled with -fmad=false: every FP64 product
// and sum below rounds separately, as in the reference's x86-64 build.
//
// The reference splits a node at its centre c (body goes up on an axis when
// p >= c) and makes each child's centre c +- h/2, recursively, with a stable
// counting sort. Here every body replays that chain of comparisons and
// additions on its own, writing the octant of every level as a 3-bit digit
// of a key (21 levels per 64-bit word), and one stable radix sort of the
// keys reproduces the reference's tree order. The tree's shape follows from
// the sorted keys alone:
//   * lcp(a, b): the number of leading levels two bodies share;
//   * a node of depth d holds more than L = leaf_size bodies iff some run of
//     L+1 consecutive sorted bodies shares d levels, so a body's leaf depth is
//     1 + max lcp over the L+1 windows that contain it, capped by depth 60 and
//     by the reference's "tiny node" rule (octree.cpp:40-44);
//   * the nodes that end at sorted position b are the depths
//     lcp(b, b+1) < d <= leafdepth(b).
// Numbering nodes by (end descending, depth ascending) gives exactly the
// order in which the reference's group walk pops them (group_lists.cpp:
// 141-164), so each node's subtree is a contiguous index range and a
// "skip" link replaces the walk's stack. Bodies deeper than 21 levels (dense
// clumps, coincident points) get further key words in up to two more rounds,
// sorted within their depth-21 (or 42) node.
//
// Inside a leaf the reference keeps bodies in input order (its sort is
// stable and leaves are not split further), so each leaf's range is put back
// in input order before the moments are taken. Moments are FP64, leaves
// summed in tree order and parents from their children in octant order
// (octree.cpp:46-102), bottom-up with one arrival counter per node.

#include <algorithm>
#include <cstddef>
#include <cstring>

#include "pipeline.cuh"

namespace gtc {
namespace {

constexpr int kT = 256;

// Graph replays pass the abort word of their Scalars and the node count on
// the device; eager calls pass null and their host-known sizes.
__device__ __forceinline__ bool aborted(const u32 *abort) { return abort && *abort; }
__device__ __forceinline__ u32 bounded(u32 cap, const u32 *dev) {
  return dev ? min(cap, *dev) : cap;
}
constexpr u8 kNoTiny = 255;

struct Dbl4 {
  double x, y, z, w;
};
__device__ __forceinline__ Dbl4 make_dbl4(double x, double y, double z, double w) {
  return Dbl4{x, y, z, w};
}

struct KeyView {
  const u64 *w0, *w1, *w2;
  int words;
  const u16 *sys = nullptr;  // a forest: the system of each sorted position
};

__device__ __forceinline__ int word_lcp(u64 a, u64 b, int levels) {
  const u64 x = a ^ b;
  if (x == 0) return levels;
  const int q = (__clzll(static_cast<long long>(x)) - 1) / 3;
  return q < levels ? q : levels;
}

// Levels shared by the bodies at sorted positions a and b.
__device__ __forceinline__ int lcp(const KeyView &kv, u32 a, u32 b) {
  if (kv.sys && kv.sys[a] != kv.sys[b]) return -1;  // two systems share no node
  int l = word_lcp(kv.w0[a], kv.w0[b], kLevelsPerWord);
  if (l < kLevelsPerWord || kv.words == 1) return l;
  l = word_lcp(kv.w1[a], kv.w1[b], kLevelsPerWord);
  if (l < kLevelsPerWord || kv.words == 2) return kLevelsPerWord + l;
  return 2 * kLevelsPerWord + word_lcp(kv.w2[a], kv.w2[b], kMaxDepth - 2 * kLevelsPerWord);
}

// Octant digit of level `lvl` (1-based) of the body at sorted position b.
__device__ __forceinline__ int digit(const KeyView &kv, u32 b, int lvl) {
  const int w = (lvl - 1) / kLevelsPerWord, q = (lvl - 1) % kLevelsPerWord;
  const u64 word = w == 0 ? kv.w0[b] : (w == 1 ? kv.w1[b] : kv.w2[b]);
  return static_cast<int>((word >> (60 - 3 * q)) & 7u);
}

// The reference's "tiny" leaf rule (octree.cpp:43).
__device__ __forceinline__ bool tiny_node(double h, double cx, double cy, double cz) {
  return h < 1e-12 * (fabs(cx) + fabs(cy) + fabs(cz) + 1e-300);
}

__device__ __forceinline__ void step_centre(double &cx, double &cy, double &cz, int o, double h) {
  cx = cx + ((o & 1) ? h : -h);  // octree.cpp:131-132
  cy = cy + ((o & 2) ? h : -h);
  cz = cz + ((o & 4) ? h : -h);
}

// ------------------------------------------------------------ bounding box

// Order-preserving image of a double for integer comparison: a >= b exactly
// when key(a) >= key(b), for finite a, b (-0.0 is taken as +0.0).
__device__ __forceinline__ u64 order_key(double v) {
  u64 b = static_cast<u64>(__double_as_longlong(v));
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_order_key(u64 k) {
  return __longlong_as_double(static_cast<long long>((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// Per-block boxes. Min and max are taken on the order-preserving integer
// images (exact, and off the FP64 pipe); with 16-byte aligned positions a
// thread loads two bodies as three 16-byte words.
__global__ void __launch_bounds__(kT) k_bbox_partial(const double *pos, u64 n, double *part) {
  const u64 inf_lo = order_key(INFINITY), inf_hi = order_key(-INFINITY);
  u64 lo[3] = {inf_lo, inf_lo, inf_lo}, hi[3] = {inf_hi, inf_hi, inf_hi};
  auto take = [&](int a, double v) {
    const u64 k = order_key(v);
    lo[a] = k < lo[a] ? k : lo[a];
    hi[a] = k > hi[a] ? k : hi[a];
  };
  const u64 first = blockIdx.x * static_cast<u64>(kT) + threadIdx.x,
            stride = static_cast<u64>(gridDim.x) * kT;
  if ((reinterpret_cast<uintptr_t>(pos) & 15) == 0) {
    const double2 *p2 = reinterpret_cast<const double2 *>(pos);
    for (u64 q = first; q < n / 2; q += stride) {
      const double2 u = __ldg(p2 + 3 * q), v = __ldg(p2 + 3 * q + 1), w = __ldg(p2 + 3 * q + 2);
      take(0, u.x);
      take(1, u.y);
      take(2, v.x);
      take(0, v.y);
      take(1, w.x);
      take(2, w.y);
    }
    if ((n & 1) && first == 0)
      for (int a = 0; a < 3; ++a) take(a, pos[3 * (n - 1) + a]);
  } else {
    for (u64 i = first; i < n; i += stride)
      for (int a = 0; a < 3; ++a) take(a, pos[3 * i + a]);
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o > 0; o >>= 1) {
      const u64 l = __shfl_xor_sync(kFullMask, lo[a], o), h = __shfl_xor_sync(kFullMask, hi[a], o);
      lo[a] = l < lo[a] ? l : lo[a];
      hi[a] = h > hi[a] ? h : hi[a];
    }
  __shared__ u64 s[kT / 32][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int a = 0; a < 3; ++a) {
      s[warp][a] = lo[a];
      s[warp][3 + a] = hi[a];
    }
  __syncthreads();
  if (threadIdx.x < 6) {
    u64 v = s[0][threadIdx.x];
    for (int w = 1; w < kT / 32; ++w) {
      const u64 x = s[w][threadIdx.x];
      v = threadIdx.x < 3 ? (x < v ? x : v) : (x > v ? x : v);
    }
    part[6 * blockIdx.x + threadIdx.x] = from_order_key(v);
  }
}

// Root cube from the reduced box (octree.cpp:184-198); min/max are exact in
// any order, so the partial boxes are reduced by the whole block.
__device__ void root_from_parts(const double *part, int nparts, TreeRoot *root) {
  double v[6];
  for (int a = 0; a < 3; ++a) {
    v[a] = INFINITY;
    v[3 + a] = -INFINITY;
  }
  for (int p = threadIdx.x; p < nparts; p += kT)
    for (int a = 0; a < 3; ++a) {
      v[a] = fmin(v[a], part[6 * p + a]);
      v[3 + a] = fmax(v[3 + a], part[6 * p + 3 + a]);
    }
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o > 0; o >>= 1) {
      v[a] = fmin(v[a], __shfl_xor_sync(kFullMask, v[a], o));
      v[3 + a] = fmax(v[3 + a], __shfl_xor_sync(kFullMask, v[3 + a], o));
    }
  __shared__ double s[kT / 32][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int a = 0; a < 6; ++a) s[warp][a] = v[a];
  __syncthreads();
  if (threadIdx.x != 0) return;
  double lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = s[0][a];
    hi[a] = s[0][3 + a];
    for (int w = 1; w < kT / 32; ++w) {
      lo[a] = fmin(lo[a], s[w][a]);
      hi[a] = fmax(hi[a], s[w][3 + a]);
    }
  }
  double half = 0.0;
  for (int a = 0; a < 3; ++a) {
    root->lo[a] = lo[a];
    root->hi[a] = hi[a];
    root->center[a] = (lo[a] + hi[a]) * 0.5;
    const double e = 0.5 * (hi[a] - lo[a]);
    half = half < e ? e : half;
  }
  half = half * (1.0 + 1e-9) + 1e-300;
  root->half_at[0] = half;
  for (int d = 0; d < kMaxDepth; ++d) root->half_at[d + 1] = 0.5 * root->half_at[d];
  // every body's |x| + |y| + |z| is at most this sum (rounding is monotone),
  // so no body's tiny bound in k_keys exceeds this one
  double m1 = 0.0;
  for (int a = 0; a < 3; ++a) m1 = m1 + fmax(fabs(lo[a]), fabs(hi[a]));
  const long long bound = __double_as_longlong(2e-12 * (m1 + 1e-300));
  int d = 0;
  while (d <= kMaxDepth && __double_as_longlong(root->half_at[d]) >= bound) ++d;
  root->tiny_from = d;
}

__global__ void __launch_bounds__(kT) k_root(const double *part, int nparts, TreeRoot *root) {
  root_from_parts(part, nparts, root);
}

// A forest's boxes: block b covers part of system blk[b].x (rank blk[b].y of
// its blk[b].z blocks), one partial box each; then one block per system
// reduces that system's partials (sys_blk: first block, blocks) into its
// root.
__global__ void __launch_bounds__(kT)
    k_bbox_forest(const double *pos, const uint4 *blk, const u32 *start, double *part) {
  const uint4 q = blk[blockIdx.x];
  const u64 b0 = start[q.x], b1 = start[q.x + 1];
  const u64 inf_lo = order_key(INFINITY), inf_hi = order_key(-INFINITY);
  u64 lo[3] = {inf_lo, inf_lo, inf_lo}, hi[3] = {inf_hi, inf_hi, inf_hi};
  for (u64 i = b0 + static_cast<u64>(q.y) * kT + threadIdx.x; i < b1;
       i += static_cast<u64>(q.z) * kT)
    for (int a = 0; a < 3; ++a) {
      const u64 k = order_key(pos[3 * i + a]);
      lo[a] = k < lo[a] ? k : lo[a];
      hi[a] = k > hi[a] ? k : hi[a];
    }
#pragma unroll
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o > 0; o >>= 1) {
      const u64 l = __shfl_xor_sync(kFullMask, lo[a], o), h = __shfl_xor_sync(kFullMask, hi[a], o);
      lo[a] = l < lo[a] ? l : lo[a];
      hi[a] = h > hi[a] ? h : hi[a];
    }
  __shared__ u64 s[kT / 32][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int a = 0; a < 3; ++a) {
      s[warp][a] = lo[a];
      s[warp][3 + a] = hi[a];
    }
  __syncthreads();
  if (threadIdx.x < 6) {
    u64 v = s[0][threadIdx.x];
    for (int w = 1; w < kT / 32; ++w) {
      const u64 x = s[w][threadIdx.x];
      v = threadIdx.x < 3 ? (x < v ? x : v) : (x > v ? x : v);
    }
    part[6 * blockIdx.x + threadIdx.x] = from_order_key(v);
  }
}

__global__ void __launch_bounds__(kT)
    k_root_forest(const double *part, const uint2 *sys_blk, TreeRoot *roots) {
  const uint2 q = sys_blk[blockIdx.x];
  root_from_parts(part + 6ull * q.x, static_cast<int>(q.y), roots + blockIdx.x);
}

// ------------------------------------------------------------------- keys


// Split values. Along one axis the centre a body's walk compares against at
// level d depends only on the body's first d bits on that axis: the centres
// of all levels form a binary tree per axis (heap order, node 1 the root
// centre, the children of node k at level d the centre stepped down and up
// by half_at[d + 1], with the reference's FP64 addition). A body's key bits
// on an axis are then a binary search in that tree. The table holds levels
// 0..kSplitLevels - 1 (2^kSplitLevels - 1 values per axis), built once per
// tree instead of once per body; the levels below are stepped per body.
constexpr int kSplitTop = 11;                    // levels one block per axis builds

// Levels 0..kSplitTop - 1, one block per axis, level by level.
__global__ void __launch_bounds__(1024) k_split_top(const TreeRoot *root, double *split) {
  const int axis = blockIdx.x;
  double *t = split + static_cast<u64>(axis) * kSplitSize;
  if (threadIdx.x == 0) t[1] = root->center[axis];
  __syncthreads();
  for (int d = 1; d < kSplitTop; ++d) {
    const double h = root->half_at[d];
    for (u32 j = threadIdx.x; j < (1u << d); j += blockDim.x) {
      const u32 k = (1u << d) + j;
      const double c = t[k >> 1];
      t[k] = c + ((k & 1u) ? h : -h);  // step_centre's operation
    }
    __syncthreads();
  }
}

// `Levels` levels below level `from`: one thread per node of level `from`
// builds its subtree in registers, level by level, and stores it.
template <int Levels>
__global__ void __launch_bounds__(kT) k_split_sub(const TreeRoot *root, double *split, int from) {
  const u32 per_axis = 1u << from;
  const u32 tid = blockIdx.x * kT + threadIdx.x;
  if (tid >= 3 * per_axis) return;
  double *t = split + static_cast<u64>(tid / per_axis) * kSplitSize;
  const u32 base = per_axis + tid % per_axis;  // heap index at level `from`
  double v[2 << Levels];                        // v[1] the subtree's root, heap order below
  v[1] = t[base];
#pragma unroll
  for (int l = 1; l <= Levels; ++l) {
    const double h = root->half_at[from + l];
#pragma unroll
    for (int j = 0; j < (1 << l); ++j) {
      const int k = (1 << l) + j;
      v[k] = v[k >> 1] + ((k & 1) ? h : -h);
      t[(static_cast<u64>(base) << l) + j] = v[k];
    }
  }
}

// The table in order. Along an axis, the split values in in-order (heap
// node 2^d + m of level d at in-order position (2m + 1) 2^(kSplitLevels - 1
// - d) - 1). When they never decrease, a body's path through the table is
// the rank of its coordinate among them: the number of values <= x, whose
// kSplitLevels bits are the path's level-0.. bits (up iff x >= the centre),
// the path's deepest centre being the value at the rank with its last bit
// cleared.
constexpr u32 kSplitValues = kSplitSize - 1;  // per axis: heap nodes 1..kSplitSize - 1

// Heap index of in-order position p.
__device__ __forceinline__ u32 split_heap(u32 p) {
  const u32 q = p + 1;
  const int tz = __ffs(q) - 1;
  return (1u << (kSplitLevels - 1 - tz)) + (q >> (tz + 1));
}

// In-order neighbours come in (leaf, inner node) pairs, leaves at the even
// positions: each leaf against the values on either side of it.
__global__ void __launch_bounds__(kT) k_split_check(const double *split, u32 *unsorted) {
  constexpr u32 kLeaves = 1u << (kSplitLevels - 1);
  const u32 t = blockIdx.x * kT + threadIdx.x;
  if (t >= 3 * kLeaves) return;
  const double *s = split + static_cast<u64>(t / kLeaves) * kSplitSize;
  const u32 j = t % kLeaves, p = 2 * j;
  const u64 v = order_key(s[kLeaves + j]);
  bool bad = false;
  if (j > 0) bad |= order_key(s[split_heap(p - 1)]) > v;
  if (p + 1 < kSplitValues) bad |= v > order_key(s[split_heap(p + 1)]);
  if (bad) atomicOr(unsorted, 1u);
}

// Bits b of v at bit 3b (v < 2^21).
__device__ __forceinline__ u64 spread3(u64 v) {
  v &= 0x1fffffull;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

// Rank of kx among an axis's in-order values: a guess from the grid the
// values lie on (1 / inv_w apart), then moved until the values on either
// side bracket kx. False if that takes more than a few steps.
__device__ __forceinline__ bool split_rank(const double *table, u64 kx, double x,
                                           double lo_edge, float inv_w, u32 &r) {
  const float g = static_cast<float>(x - lo_edge) * inv_w;
  int v = g > 0.f ? static_cast<int>(fminf(g, static_cast<float>(kSplitValues))) : 0;
  for (int it = 0; it < 4; ++it) {
    if (v > 0 && kx < order_key(__ldg(table + split_heap(v - 1)))) {
      --v;
    } else if (v < static_cast<int>(kSplitValues) && kx >= order_key(__ldg(table + split_heap(v)))) {
      ++v;
    } else {
      r = static_cast<u32>(v);
      return true;
    }
  }
  return false;
}

// First key word: levels 1..21 from the root; records the first depth whose
// node is "tiny" (a leaf whatever its count). Digits below a tiny node are 0,
// so bodies of such a leaf stay in input order through the sort. The centres
// of the first kSplitLevels levels come from the split table; the rest are
// stepped as the reference does.
//
// A node holding body p has |centre|_1 <= |p|_1 + 3 half (plus rounding), so
// it can only be tiny once half < 1e-12 (|p|_1 + 3 half + 1e-300), i.e. once
// half < ~1.0000001e-12 (|p|_1 + 1e-300). Levels whose half is at least
// twice that bound skip the exact FP64 test; the comparison of two positive
// doubles is done on their bit patterns.
__global__ void __launch_bounds__(kT)
    k_keys(const double *pos, u32 n, const TreeRoot *root, const double *split,
           const u32 *unsorted, u64 *key, u32 *idx, u8 *tiny, u32 *error) {
  __shared__ double half_at[kLevelsPerWord + 1];
  __shared__ float inv_spacing;  // 1 / the spacing of the table's deepest values
  if (threadIdx.x <= kLevelsPerWord) half_at[threadIdx.x] = root->half_at[threadIdx.x];
  if (threadIdx.x == 0) inv_spacing = static_cast<float>(1.0 / root->half_at[kSplitLevels - 1]);
  __syncthreads();
  const bool by_rank = *unsorted == 0;
  const u32 i = blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  const double x = pos[3ull * i], y = pos[3ull * i + 1], z = pos[3ull * i + 2];
  if (!isfinite(x) || !isfinite(y) || !isfinite(z)) atomicOr(error, 4u);
  const u64 kx = order_key(x), ky = order_key(y), kz = order_key(z);
  // the first level whose node could be tiny for this body (half_at falls
  // with depth): the levels above it need no tiny test at all
  int dt = root->tiny_from;
  if (dt <= kLevelsPerWord) {
    const long long maybe_tiny =
        __double_as_longlong(2e-12 * (fabs(x) + fabs(y) + fabs(z) + 1e-300));
    dt = 0;
    while (dt <= kLevelsPerWord && __double_as_longlong(half_at[dt]) >= maybe_tiny) ++dt;
  }
  const double *tx = split, *ty = split + kSplitSize, *tz = split + 2ull * kSplitSize;
  u32 ix = 1, iy = 1, iz = 1;
  double cx = 0.0, cy = 0.0, cz = 0.0;
  u64 k = 0;
  int t = kNoTiny;
  // level d: its centre (table, or stepped below the table), the tiny test
  // where it can apply, the digit, and the next level's index or centre
  auto level = [&](int d, bool test) {
    if (d < kSplitLevels) {
      cx = __ldg(tx + ix);
      cy = __ldg(ty + iy);
      cz = __ldg(tz + iz);
    }
    if (test && t == kNoTiny && tiny_node(half_at[d], cx, cy, cz)) t = d;
    int o = (kx >= order_key(cx) ? 1 : 0) | (ky >= order_key(cy) ? 2 : 0) |
            (kz >= order_key(cz) ? 4 : 0);
    if (t != kNoTiny) o = 0;
    k = (k << 3) | static_cast<u64>(o);
    if (d + 1 < kSplitLevels) {
      ix = 2 * ix + (o & 1);
      iy = 2 * iy + ((o >> 1) & 1);
      iz = 2 * iz + (o >> 2);
    } else {
      step_centre(cx, cy, cz, o, half_at[d + 1]);
    }
  };
  int d = 0;
  if (by_rank && dt >= kSplitLevels) {
    // no tiny test within the table's levels: its levels by rank
    const float inv_w = inv_spacing;
    u32 rx, ry, rz;
    if (split_rank(tx, kx, x, root->center[0] - half_at[0], inv_w, rx) &&
        split_rank(ty, ky, y, root->center[1] - half_at[0], inv_w, ry) &&
        split_rank(tz, kz, z, root->center[2] - half_at[0], inv_w, rz)) {
      k = spread3(rx) | (spread3(ry) << 1) | (spread3(rz) << 2);
      if (dt <= kLevelsPerWord) {  // the centre below the table, for the last tiny test
        constexpr u32 kLeaves = 1u << (kSplitLevels - 1);
        cx = __ldg(tx + kLeaves + (rx >> 1));
        cy = __ldg(ty + kLeaves + (ry >> 1));
        cz = __ldg(tz + kLeaves + (rz >> 1));
        const int o = static_cast<int>((rx & 1u) | ((ry & 1u) << 1) | ((rz & 1u) << 2));
        step_centre(cx, cy, cz, o, half_at[kSplitLevels]);
      }
      d = kSplitLevels;
    }
  }
  for (; d < kLevelsPerWord && d < dt; ++d) level(d, false);
  for (; d < kLevelsPerWord; ++d) level(d, true);
  if (dt <= kLevelsPerWord && t == kNoTiny && tiny_node(half_at[kLevelsPerWord], cx, cy, cz))
    t = kLevelsPerWord;
  key[i] = k;
  idx[i] = i;
  tiny[i] = static_cast<u8>(t);
}

// A forest's split tables: per system and axis, levels 0..T-1 of the same
// table as above (heap order, 2^T entries, the system's own root), T set by
// the forest's memory budget. Built by the same operations as the
// single-system table: levels 0..min(T, kSplitTop)-1 by one block per
// (system, axis), the rest by subtrees of 4, 2 or 1 levels.
__global__ void __launch_bounds__(1024)
    k_split_top_forest(const TreeRoot *roots, double *split, u32 size, int top) {
  const u32 sa = blockIdx.x;  // system * 3 + axis
  const TreeRoot *root = roots + sa / 3;
  double *t = split + static_cast<u64>(sa) * size;
  if (threadIdx.x == 0) t[1] = root->center[sa % 3];
  __syncthreads();
  for (int d = 1; d < top; ++d) {
    const double h = root->half_at[d];
    for (u32 j = threadIdx.x; j < (1u << d); j += blockDim.x) {
      const u32 k = (1u << d) + j;
      const double c = t[k >> 1];
      t[k] = c + ((k & 1u) ? h : -h);  // step_centre's operation
    }
    __syncthreads();
  }
}

template <int Levels>
__global__ void __launch_bounds__(kT)
    k_split_sub_forest(const TreeRoot *roots, double *split, u32 size, u32 tables, int from) {
  const u32 per_axis = 1u << from;
  const u64 tid = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  if (tid >= static_cast<u64>(tables) * per_axis) return;
  const u32 sa = static_cast<u32>(tid / per_axis);
  const TreeRoot *root = roots + sa / 3;
  double *t = split + static_cast<u64>(sa) * size;
  const u32 base = per_axis + static_cast<u32>(tid % per_axis);
  double v[2 << Levels];
  v[1] = t[base];
#pragma unroll
  for (int l = 1; l <= Levels; ++l) {
    const double h = root->half_at[from + l];
#pragma unroll
    for (int j = 0; j < (1 << l); ++j) {
      const int k = (1 << l) + j;
      v[k] = v[k >> 1] + ((k & 1) ? h : -h);
      t[(static_cast<u64>(base) << l) + j] = v[k];
    }
  }
}

// Heap index of in-order position p in a table of `levels` levels.
__device__ __forceinline__ u32 split_heap_at(u32 p, int levels) {
  const u32 q = p + 1;
  const int tz = __ffs(q) - 1;
  return (1u << (levels - 1 - tz)) + (q >> (tz + 1));
}

// k_split_check per (system, axis) table; a system whose in-order values
// decrease somewhere gets its flag set (its keys then walk the table level
// by level).
__global__ void __launch_bounds__(kT)
    k_split_check_forest(const double *split, u32 size, int levels, u32 tables, u32 *unsorted) {
  const u32 leaves = 1u << (levels - 1);
  const u64 t = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  if (t >= static_cast<u64>(tables) * leaves) return;
  const u32 sa = static_cast<u32>(t / leaves);
  const double *s = split + static_cast<u64>(sa) * size;
  const u32 j = static_cast<u32>(t % leaves), p = 2 * j, values = size - 1;
  const u64 v = order_key(s[leaves + j]);
  bool bad = false;
  if (j > 0) bad |= order_key(s[split_heap_at(p - 1, levels)]) > v;
  if (p + 1 < values) bad |= v > order_key(s[split_heap_at(p + 1, levels)]);
  if (bad) atomicOr(unsorted + sa / 3, 1u);
}

// split_rank on a table of `levels` levels (values = 2^levels - 1).
__device__ __forceinline__ bool split_rank_at(const double *table, u64 kx, double x,
                                              double lo_edge, float inv_w, int levels,
                                              u32 &r) {
  const u32 values = (1u << levels) - 1;
  const float g = static_cast<float>(x - lo_edge) * inv_w;
  int v = g > 0.f ? static_cast<int>(fminf(g, static_cast<float>(values))) : 0;
  for (int it = 0; it < 4; ++it) {
    if (v > 0 && kx < order_key(__ldg(table + split_heap_at(v - 1, levels)))) {
      --v;
    } else if (v < static_cast<int>(values) &&
               kx >= order_key(__ldg(table + split_heap_at(v, levels)))) {
      ++v;
    } else {
      r = static_cast<u32>(v);
      return true;
    }
  }
  return false;
}

// A forest's first key word: k_keys with each body's own system's root and
// table of T levels (levels below T stepped as the reference does).
__global__ void __launch_bounds__(kT)
    k_keys_forest(const double *pos, u32 n, const u16 *sys, const TreeRoot *roots,
                  const double *split, u32 size, int T, const u32 *unsorted, u64 *key, u32 *idx,
                  u8 *tiny, u32 *error) {
  const u32 i = blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  const u32 s = sys[i];
  const TreeRoot *root = roots + s;
  const double *half_at = root->half_at;
  const double x = pos[3ull * i], y = pos[3ull * i + 1], z = pos[3ull * i + 2];
  if (!isfinite(x) || !isfinite(y) || !isfinite(z)) atomicOr(error, 4u);
  const u64 kx = order_key(x), ky = order_key(y), kz = order_key(z);
  int dt = root->tiny_from;
  if (dt <= kLevelsPerWord) {
    const long long maybe_tiny =
        __double_as_longlong(2e-12 * (fabs(x) + fabs(y) + fabs(z) + 1e-300));
    dt = 0;
    while (dt <= kLevelsPerWord && __double_as_longlong(half_at[dt]) >= maybe_tiny) ++dt;
  }
  const double *tx = split + 3ull * s * size, *ty = tx + size, *tz = ty + size;
  u32 ix = 1, iy = 1, iz = 1;
  double cx = 0.0, cy = 0.0, cz = 0.0;
  u64 k = 0;
  int t = kNoTiny;
  auto level = [&](int d, bool test) {
    if (d < T) {
      cx = __ldg(tx + ix);
      cy = __ldg(ty + iy);
      cz = __ldg(tz + iz);
    }
    if (test && t == kNoTiny && tiny_node(half_at[d], cx, cy, cz)) t = d;
    int o = (kx >= order_key(cx) ? 1 : 0) | (ky >= order_key(cy) ? 2 : 0) |
            (kz >= order_key(cz) ? 4 : 0);
    if (t != kNoTiny) o = 0;
    k = (k << 3) | static_cast<u64>(o);
    if (d + 1 < T) {
      ix = 2 * ix + (o & 1);
      iy = 2 * iy + ((o >> 1) & 1);
      iz = 2 * iz + (o >> 2);
    } else {
      step_centre(cx, cy, cz, o, half_at[d + 1]);
    }
  };
  int d = 0;
  if (unsorted[s] == 0 && dt >= T) {
    // no tiny test within the table's levels: its levels by rank, then the
    // centre of level T (the path's deepest table centre, stepped once)
    const float inv_w = 1.0f / static_cast<float>(half_at[T - 1]);
    u32 rx, ry, rz;
    if (split_rank_at(tx, kx, x, root->center[0] - half_at[0], inv_w, T, rx) &&
        split_rank_at(ty, ky, y, root->center[1] - half_at[0], inv_w, T, ry) &&
        split_rank_at(tz, kz, z, root->center[2] - half_at[0], inv_w, T, rz)) {
      k = spread3(rx) | (spread3(ry) << 1) | (spread3(rz) << 2);
      const u32 leaves = 1u << (T - 1);
      cx = __ldg(tx + leaves + (rx >> 1));
      cy = __ldg(ty + leaves + (ry >> 1));
      cz = __ldg(tz + leaves + (rz >> 1));
      const int o = static_cast<int>((rx & 1u) | ((ry & 1u) << 1) | ((rz & 1u) << 2));
      step_centre(cx, cy, cz, o, half_at[T]);
      d = T;
    }
  }
  for (; d < kLevelsPerWord && d < dt; ++d) level(d, false);
  for (; d < kLevelsPerWord; ++d) level(d, true);
  if (dt <= kLevelsPerWord && t == kNoTiny && tiny_node(half_at[kLevelsPerWord], cx, cy, cz))
    t = kLevelsPerWord;
  key[i] = k;
  idx[i] = i;
  tiny[i] = static_cast<u8>(t);
}

// A forest's last sort pass, by system: the system of each sorted body as
// the key, the position as the value; the key words and bodies are copied
// aside for the gather that follows the pass.
__global__ void __launch_bounds__(kT)
    k_forest_sys_keys(const u64 *key, const u32 *idx, const u16 *sys, u32 n, u64 *skey, u32 *spos,
                      u64 *key_copy, u32 *idx_copy, const u32 *abort = nullptr) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= n || aborted(abort)) return;
  const u32 i = idx[k];
  skey[k] = sys[i];
  spos[k] = k;
  key_copy[k] = key[k];
  idx_copy[k] = i;
}

__global__ void __launch_bounds__(kT)
    k_forest_gather(const u32 *spos, const u64 *key_copy, const u32 *idx_copy, u32 n, u64 *key,
                    u32 *idx, const u32 *abort = nullptr) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= n || aborted(abort)) return;
  const u32 j = spos[k];
  key[k] = key_copy[j];
  idx[k] = idx_copy[j];
}

// Per sorted position: levels shared with the next body, and the leaf depth.
__global__ void __launch_bounds__(kT)
    k_levels(KeyView kv, const u32 *idx, const u8 *tiny, u32 n, int L, signed char *lcp_next,
             u8 *leafdepth, Scalars *sc) {
  // win[i] = lcp(i, i + L) for the block's positions and the L before them,
  // each computed once; a body's w is the largest over its windows
  constexpr int kMaxWin = 64;
  __shared__ signed char win[kT + kMaxWin];
  const u32 base = blockIdx.x * kT, b = base + threadIdx.x;
  const bool shared_win = L <= kMaxWin;
  if (shared_win) {
    for (int k = threadIdx.x; k < kT + L; k += kT) {
      const long long i = static_cast<long long>(base) + k - L;
      win[k] = static_cast<signed char>(
          i >= 0 && i + L < static_cast<long long>(n) ? lcp(kv, static_cast<u32>(i), static_cast<u32>(i + L)) : -1);
    }
    __syncthreads();
  }
  int ld = 0;
  if (b < n) {
    lcp_next[b] = static_cast<signed char>(b + 1 < n ? lcp(kv, b, b + 1) : -1);
    int w = -1;
    if (n > static_cast<u32>(L)) {
      const u32 lo = b >= static_cast<u32>(L) ? b - L : 0;
      const u32 hi = min(b, n - 1 - L);
      for (u32 i = lo; i <= hi; ++i)
        w = max(w, shared_win ? static_cast<int>(win[i - base + L]) : lcp(kv, i, i + L));
    }
    ld = min(w + 1, kMaxDepth);
    ld = min(ld, static_cast<int>(tiny[idx[b]]));
    leafdepth[b] = static_cast<u8>(ld);
  }
  // one atomic per warp for each counter
  const u32 deep = __popc(__ballot_sync(kFullMask, b < n && ld > kLevelsPerWord * kv.words));
  const u32 dmax = __reduce_max_sync(kFullMask, static_cast<u32>(ld));
  if ((threadIdx.x & 31) == 0) {
    if (deep) atomicAdd(&sc->deep, deep);
    atomicMax(&sc->depth, dmax);
  }
}

// ------------------------------------------------------- deeper key words

__global__ void __launch_bounds__(kT)
    k_deep_flags(const u8 *leafdepth, u32 n, int limit, u32 *flag) {
  const u32 b = blockIdx.x * kT + threadIdx.x;
  if (b < n) flag[b] = leafdepth[b] > limit ? 1u : 0u;
}

__global__ void __launch_bounds__(kT)
    k_compact(const u32 *flag, const u32 *scan, u32 n, u32 *out) {
  const u32 b = blockIdx.x * kT + threadIdx.x;
  if (b < n && flag[b]) out[scan[b]] = b;
}

// Next key word for the deep bodies: replay the path to depth 21*words from
// the root with the existing digits, then record up to 21 more levels.
__global__ void __launch_bounds__(kT)
    k_deep_keys(KeyView kv, const u32 *dpos, u32 nd, const u32 *idx, const double *pos,
                const TreeRoot *root, u8 *tiny, u64 *word, u32 *rec, u32 *didx) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= nd) return;
  const u32 b = dpos[k];
  const u32 i = idx[b];
  if (kv.sys) root += kv.sys[b];  // a forest: the body's system's root
  const int base = kLevelsPerWord * kv.words;
  double cx = root->center[0], cy = root->center[1], cz = root->center[2];
  for (int lvl = 1; lvl <= base; ++lvl) step_centre(cx, cy, cz, digit(kv, b, lvl), root->half_at[lvl]);
  const double x = pos[3ull * i], y = pos[3ull * i + 1], z = pos[3ull * i + 2];
  const int levels = min(kLevelsPerWord, kMaxDepth - base);
  int t = tiny[i];
  u64 w = 0;
  for (int q = 0; q < levels; ++q) {
    const int d = base + q;  // depth of the node being split
    if (q > 0 && t == kNoTiny && tiny_node(root->half_at[d], cx, cy, cz)) t = d;
    int o = (x >= cx ? 1 : 0) | (y >= cy ? 2 : 0) | (z >= cz ? 4 : 0);
    if (t != kNoTiny) o = 0;
    w = (w << 3) | static_cast<u64>(o);
    step_centre(cx, cy, cz, o, root->half_at[d + 1]);
  }
  if (t == kNoTiny && tiny_node(root->half_at[base + levels], cx, cy, cz)) t = base + levels;
  w <<= 3 * (kLevelsPerWord - levels);
  tiny[i] = static_cast<u8>(t);
  word[k] = w;
  rec[k] = k;
  didx[k] = i;
}

// Segment of each deep record: a new segment starts where the existing key
// words change (a different depth-21*words node).
__global__ void __launch_bounds__(kT)
    k_deep_segments(KeyView kv, const u32 *dpos, u32 nd, u32 *flag) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= nd) return;
  bool start = k == 0;
  if (!start) {
    const u32 a = dpos[k - 1], b = dpos[k];
    start = kv.w0[a] != kv.w0[b] || (kv.words > 1 && kv.w1[a] != kv.w1[b]) ||
            (kv.sys && kv.sys[a] != kv.sys[b]);
  }
  flag[k] = start ? 1u : 0u;
}

__global__ void __launch_bounds__(kT)
    k_seg_keys(const u32 *rec, const u32 *seg_scan, const u32 *seg_flag, u32 nd, u64 *key) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= nd) return;
  const u32 r = rec[k];
  key[k] = seg_scan[r] + seg_flag[r];  // 1-based segment number
}

// Puts the deep records back into their positions, now ordered by (segment,
// new word, input order).
__global__ void __launch_bounds__(kT)
    k_deep_scatter(const u32 *dpos, const u32 *rec, const u32 *didx, const u64 *word, u32 nd,
                   u32 *idx, u64 *word_out) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= nd) return;
  const u32 r = rec[k];
  idx[dpos[k]] = didx[r];
  word_out[dpos[k]] = word[r];
}

// ------------------------------------------------------------------ nodes

__global__ void __launch_bounds__(kT)
    k_node_count(const signed char *lcp_next, const u8 *leafdepth, u32 n, u32 *count,
                 const u32 *abort = nullptr) {
  const u32 b = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort)) return;
  if (b < n) count[b] = static_cast<u32>(max(0, static_cast<int>(leafdepth[b]) - lcp_next[b]));
}

// Writes the nodes ending at sorted position b, shallowest first.
__global__ void __launch_bounds__(kT)
    k_nodes(KeyView kv, const signed char *lcp_next, const u8 *leafdepth, const u32 *count,
            const u32 *count_scan, u32 n, const Scalars *sc, const TreeRoot *root,
            const double *split, double2 *geom, u32 *nbegin, u32 *nend, u32 *skip, u8 *depth,
            u8 *isleaf, const u32 *abort = nullptr, u32 table_size = kSplitSize,
            int table_levels = kSplitLevels) {
  const u32 b = blockIdx.x * kT + threadIdx.x;
  if (b >= n || aborted(abort)) return;
  const u32 c = count[b];
  if (c == 0) return;
  const u32 total = sc->n_nodes;
  const u32 first = total - count_scan[b] - c;  // nodes ending after b come first
  const int d0 = lcp_next[b] + 1, ld = leafdepth[b];
  // centres from the split table down to its last level, stepped below it
  // (a forest: `root` and `split` hold every system's root and table)
  const bool forest = kv.sys != nullptr;
  const u32 sys = forest ? kv.sys[b] : 0u;
  root += sys;
  const double *tx = split + 3ull * sys * table_size, *ty = tx + table_size,
               *tz = ty + table_size;
  u32 ix = 1, iy = 1, iz = 1;
  double cx = 0.0, cy = 0.0, cz = 0.0;
  for (int d = 0; d <= ld; ++d) {
    if (d > 0) {
      const int o = digit(kv, b, d);
      if (d < table_levels) {
        ix = 2 * ix + (o & 1);
        iy = 2 * iy + ((o >> 1) & 1);
        iz = 2 * iz + (o >> 2);
      } else {
        if (d == table_levels) {  // the table's deepest centre on this path
          cx = __ldg(tx + ix);
          cy = __ldg(ty + iy);
          cz = __ldg(tz + iz);
        }
        step_centre(cx, cy, cz, o, root->half_at[d]);
      }
    }
    if (d < d0) continue;
    if (d < table_levels) {
      cx = __ldg(tx + ix);
      cy = __ldg(ty + iy);
      cz = __ldg(tz + iz);
    }
    const u32 p = first + static_cast<u32>(d - d0);
    geom[2 * p] = make_double2(cx, cy);
    geom[2 * p + 1] = make_double2(cz, root->half_at[d]);
    nend[p] = b + 1;
    depth[p] = static_cast<u8>(d);
    isleaf[p] = d == ld ? 1 : 0;
  }
  // First body of each node: the smallest position sharing d levels with b.
  // Deepest node first; each shallower node starts at or before the deeper
  // one, so the search gallops back from there (a few probes for the small
  // nodes that most are) and then halves the last interval.
  u32 start = b;  // shares at least d levels with b for every d here
  for (int d = ld; d >= d0; --d) {
    u32 lo = 0, hi = start;
    if (d > 0 || forest) {  // (a forest's root starts at its system's first body)
      for (u64 step = 1;; step *= 2) {  // 64-bit: never wraps to 0
        if (step > hi) break;  // lo stays 0
        const u32 cand = hi - static_cast<u32>(step);
        if (lcp(kv, cand, b) < d) {
          lo = cand + 1;
          break;
        }
        hi = cand;
      }
      while (lo < hi) {  // lcp(lo - 1, b) < d (or lo = 0), lcp(hi, b) >= d
        const u32 mid = lo + (hi - lo) / 2;
        if (lcp(kv, mid, b) >= d) hi = mid;
        else lo = mid + 1;
      }
    }
    const u32 p = first + static_cast<u32>(d - d0);
    nbegin[p] = lo;
    skip[p] = total - count_scan[lo];
    start = lo;
  }
}

// Children of a node are p+1, skip[p+1], ... (last octant first) up to skip[p].
__device__ __forceinline__ int children_of(u32 p, const u32 *skip, u32 ch[8]) {
  int k = 0;
  for (u32 c = p + 1; c < skip[p] && k < 8; c = skip[c]) ch[k++] = c;
  return k;
}

// Parents, child counts and every inner node's children (8 slots, last
// octant first), so that the moment kernels load a node's children at once
// instead of following the skip chain.
__global__ void __launch_bounds__(kT)
    k_children(const u32 *skip, const u8 *isleaf, u32 m, u32 *parent, u8 *nchild, uint4 *kids,
               const u32 *m_dev = nullptr, const u32 *abort = nullptr) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || p >= bounded(m, m_dev)) return;
  if (p == 0) parent[0] = 0xffffffffu;
  if (isleaf[p]) {
    nchild[p] = 0;
    return;
  }
  u32 ch[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
  const int k = children_of(p, skip, ch);
  nchild[p] = static_cast<u8>(k);
  for (int j = 0; j < k; ++j) parent[ch[j]] = p;
  kids[2ull * p] = make_uint4(ch[0], ch[1], ch[2], ch[3]);
  kids[2ull * p + 1] = make_uint4(ch[4], ch[5], ch[6], ch[7]);
}

// A forest's roots: system k's root is the first (shallowest) of the nodes
// ending at its last body, and has no parent.
__global__ void __launch_bounds__(kT)
    k_forest_roots(const u32 *start, u32 systems, const u32 *count, const u32 *count_scan,
                   const Scalars *sc, u32 *root_node, u32 *parent, const u32 *abort = nullptr) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= systems || aborted(abort)) return;
  const u32 last = start[k + 1] - 1;
  const u32 r = sc->n_nodes - count_scan[last] - count[last];
  root_node[k] = r;
  parent[r] = 0xffffffffu;
}

// Input order inside each leaf (the reference never splits a leaf's range).
__global__ void __launch_bounds__(kT)
    k_leaf_order(const u8 *isleaf, const u32 *nbegin, const u32 *nend, u32 m, u32 *idx,
                 const u32 *m_dev = nullptr, const u32 *abort = nullptr) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || p >= bounded(m, m_dev) || !isleaf[p]) return;
  const u32 b0 = nbegin[p], b1 = nend[p];
  for (u32 i = b0 + 1; i < b1; ++i) {
    const u32 v = idx[i];
    u32 j = i;
    while (j > b0 && idx[j - 1] > v) {
      idx[j] = idx[j - 1];
      --j;
    }
    idx[j] = v;
  }
}

__global__ void __launch_bounds__(kT)
    k_tree_order(const double *pos, const double *mass, const u32 *idx, u32 n, double *tpos,
                 double *tmass, const u32 *abort = nullptr) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= n || aborted(abort)) return;
  const u64 i = idx[k];
  tpos[3ull * k] = pos[3 * i];
  tpos[3ull * k + 1] = pos[3 * i + 1];
  tpos[3ull * k + 2] = pos[3 * i + 2];
  tmass[k] = mass[i];
}

// ---------------------------------------------------------------- moments

struct MomentArrays {
  const double2 *geom;   // 2 per node: (cx, cy), (cz, half)
  const u32 *nbegin, *nend, *skip, *parent;
  const u8 *nchild;
  const uint4 *kids;     // 2 per node: the children, last octant first
  const double *tpos, *tmass;
  double2 *mom;     // 2 per node: (mx, my), (mz, mass)
  double2 *quad;    // 3 x double2 per node: xx yy | zz xy | xz yz
  double *delta;
};

__device__ __forceinline__ Dbl4 load_pair(const double2 *a, u32 p) {
  const double2 u = a[2 * p], v = a[2 * p + 1];
  return make_dbl4(u.x, u.y, v.x, v.y);
}

__device__ __forceinline__ void store_pair(double2 *a, u32 p, double x, double y, double z,
                                           double w) {
  a[2 * p] = make_double2(x, y);
  a[2 * p + 1] = make_double2(z, w);
}

// The moments in two passes, with the reference's operations in its order:
// the centre of mass and delta first (all the walk's records need), the
// quadrupole after it, from the stored centre of mass. The walk starts
// after the first pass while the second one runs beside it.
__device__ void leaf_com(const MomentArrays &a, u32 p) {  // octree.cpp:46-54, 71
  const Dbl4 g = load_pair(a.geom, p);
  const u32 b0 = a.nbegin[p], b1 = a.nend[p];
  double m = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
  for (u32 k = b0; k < b1; ++k) {
    const double mi = a.tmass[k];
    m += mi;
    cx += mi * a.tpos[3ull * k];
    cy += mi * a.tpos[3ull * k + 1];
    cz += mi * a.tpos[3ull * k + 2];
  }
  if (m > 0) {
    cx = cx / m;
    cy = cy / m;
    cz = cz / m;
  } else {
    cx = g.x;
    cy = g.y;
    cz = g.z;
  }
  store_pair(a.mom, p, cx, cy, cz, m);
  const double ex = cx - g.x, ey = cy - g.y, ez = cz - g.z;
  a.delta[p] = sqrt(ex * ex + ey * ey + ez * ez);
}

__device__ void leaf_quad(const MomentArrays &a, u32 p) {  // octree.cpp:55-70
  const Dbl4 c = load_pair(a.mom, p);
  const double cx = c.x, cy = c.y, cz = c.z;
  const u32 b0 = a.nbegin[p], b1 = a.nend[p];
  double q0 = 0, q1 = 0, q2 = 0, q3 = 0, q4 = 0, q5 = 0;
  for (u32 k = b0; k < b1; ++k) {
    const double mi = a.tmass[k];
    const double dx = a.tpos[3ull * k] - cx, dy = a.tpos[3ull * k + 1] - cy,
                 dz = a.tpos[3ull * k + 2] - cz;
    const double r2 = dx * dx + dy * dy + dz * dz;
    q0 += mi * (3 * dx * dx - r2);
    q1 += mi * (3 * dy * dy - r2);
    q2 += mi * (3 * dz * dz - r2);
    q3 += mi * 3 * dx * dy;
    q4 += mi * 3 * dx * dz;
    q5 += mi * 3 * dy * dz;
  }
  a.quad[3 * p] = make_double2(q0, q1);
  a.quad[3 * p + 1] = make_double2(q2, q3);
  a.quad[3 * p + 2] = make_double2(q4, q5);
}

__device__ void node_com(const MomentArrays &a, u32 p) {  // octree.cpp:75-85, 101
  const Dbl4 g = load_pair(a.geom, p);
  const uint4 k0 = a.kids[2ull * p], k1 = a.kids[2ull * p + 1];
  const u32 ch[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};  // last octant first
  const int nc = a.nchild[p];
  double m = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
  for (int j = nc - 1; j >= 0; --j) {
    const Dbl4 c = load_pair(a.mom, ch[j]);
    m += c.w;
    cx += c.w * c.x;
    cy += c.w * c.y;
    cz += c.w * c.z;
  }
  if (m > 0) {
    cx = cx / m;
    cy = cy / m;
    cz = cz / m;
  } else {
    cx = g.x;
    cy = g.y;
    cz = g.z;
  }
  store_pair(a.mom, p, cx, cy, cz, m);
  const double ex = cx - g.x, ey = cy - g.y, ez = cz - g.z;
  a.delta[p] = sqrt(ex * ex + ey * ey + ez * ez);
}

__device__ void node_quad(const MomentArrays &a, u32 p) {  // octree.cpp:86-100
  const Dbl4 pc = load_pair(a.mom, p);
  const double cx = pc.x, cy = pc.y, cz = pc.z;
  const uint4 k0 = a.kids[2ull * p], k1 = a.kids[2ull * p + 1];
  const u32 ch[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
  const int nc = a.nchild[p];
  double q0 = 0, q1 = 0, q2 = 0, q3 = 0, q4 = 0, q5 = 0;
  for (int j = nc - 1; j >= 0; --j) {
    const Dbl4 c = load_pair(a.mom, ch[j]);
    const double2 qa = a.quad[3 * ch[j]], qb = a.quad[3 * ch[j] + 1], qc = a.quad[3 * ch[j] + 2];
    const double dx = c.x - cx, dy = c.y - cy, dz = c.z - cz;
    const double r2 = dx * dx + dy * dy + dz * dz;
    q0 += qa.x + c.w * (3 * dx * dx - r2);
    q1 += qa.y + c.w * (3 * dy * dy - r2);
    q2 += qb.x + c.w * (3 * dz * dz - r2);
    q3 += qb.y + c.w * 3 * dx * dy;
    q4 += qc.x + c.w * 3 * dx * dz;
    q5 += qc.y + c.w * 3 * dy * dz;
  }
  a.quad[3 * p] = make_double2(q0, q1);
  a.quad[3 * p + 1] = make_double2(q2, q3);
  a.quad[3 * p + 2] = make_double2(q4, q5);
}

// FP32 estimates of the moments, for the learned walk's decisions only: the
// same sums as the FP64 passes (leaf_com and leaf_quad, node_com and
// node_quad), in FP32 on the FP32 bodies (relative to the root centre),
// written as GTCell-layout cells plus delta.
// They take a few tens of microseconds where the FP64 moments take most of a
// millisecond, so the learned walk starts while the FP64 moments -- which
// the evaluation reads -- are still being accumulated.
struct Moment32Arrays {
  const double2 *geom;
  const u32 *nbegin, *nend;
  const u8 *nchild;
  const uint4 *kids;
  const float4 *bodies;  // tree order, relative to the root centre
  const TreeRoot *root;
  float4 *cells;         // 3 per node: (com, mass), (xx, yy, zz, xy), (xz, yz, 0, 0)
  float *delta;
};

__device__ __forceinline__ void finish_moments32(const Moment32Arrays &a, u32 p, float m, float cx,
                                                 float cy, float cz, const float *q) {
  const Dbl4 g = load_pair(a.geom, p);
  const float gx = static_cast<float>(g.x - a.root->center[0]),
              gy = static_cast<float>(g.y - a.root->center[1]),
              gz = static_cast<float>(g.z - a.root->center[2]);
  a.cells[3 * p] = make_float4(cx, cy, cz, m);
  a.cells[3 * p + 1] = make_float4(q[0], q[1], q[2], q[3]);
  a.cells[3 * p + 2] = make_float4(q[4], q[5], 0.f, 0.f);
  const float ex = cx - gx, ey = cy - gy, ez = cz - gz;
  a.delta[p] = sqrtf(ex * ex + ey * ey + ez * ez);
}

__device__ __forceinline__ float3 centre32(const Moment32Arrays &a, u32 p) {
  const Dbl4 g = load_pair(a.geom, p);
  return make_float3(static_cast<float>(g.x - a.root->center[0]),
                     static_cast<float>(g.y - a.root->center[1]),
                     static_cast<float>(g.z - a.root->center[2]));
}

__device__ void leaf_moments32(const Moment32Arrays &a, u32 p) {
  const u32 b0 = a.nbegin[p], b1 = a.nend[p];
  float m = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  for (u32 k = b0; k < b1; ++k) {
    const float4 b = a.bodies[k];
    m += b.w;
    cx += b.w * b.x;
    cy += b.w * b.y;
    cz += b.w * b.z;
  }
  if (m > 0) {
    cx /= m;
    cy /= m;
    cz /= m;
  } else {
    const float3 c = centre32(a, p);
    cx = c.x;
    cy = c.y;
    cz = c.z;
  }
  float q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (u32 k = b0; k < b1; ++k) {
    const float4 b = a.bodies[k];
    const float dx = b.x - cx, dy = b.y - cy, dz = b.z - cz;
    const float r2 = dx * dx + dy * dy + dz * dz;
    q[0] += b.w * (3.f * dx * dx - r2);
    q[1] += b.w * (3.f * dy * dy - r2);
    q[2] += b.w * (3.f * dz * dz - r2);
    q[3] += b.w * 3.f * dx * dy;
    q[4] += b.w * 3.f * dx * dz;
    q[5] += b.w * 3.f * dy * dz;
  }
  finish_moments32(a, p, m, cx, cy, cz, q);
}

// Children's cells written by other threads of the same launch are read
// from L2 (kL2): an SM's L1 may hold an older copy of the line.
template <bool kL2>
__device__ __forceinline__ float4 cell32(const float4 *p) {
  return kL2 ? __ldcg(p) : *p;
}

template <bool kL2 = false>
__device__ void node_moments32(const Moment32Arrays &a, u32 p) {
  const uint4 k0 = a.kids[2ull * p], k1 = a.kids[2ull * p + 1];
  const u32 ch[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
  const int nc = a.nchild[p];
  float m = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  for (int j = nc - 1; j >= 0; --j) {
    const float4 c = cell32<kL2>(&a.cells[3 * ch[j]]);
    m += c.w;
    cx += c.w * c.x;
    cy += c.w * c.y;
    cz += c.w * c.z;
  }
  if (m > 0) {
    cx /= m;
    cy /= m;
    cz /= m;
  } else {
    const float3 c = centre32(a, p);
    cx = c.x;
    cy = c.y;
    cz = c.z;
  }
  float q[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int j = nc - 1; j >= 0; --j) {
    const float4 c = cell32<kL2>(&a.cells[3 * ch[j]]), qa = cell32<kL2>(&a.cells[3 * ch[j] + 1]),
                 qb = cell32<kL2>(&a.cells[3 * ch[j] + 2]);
    const float dx = c.x - cx, dy = c.y - cy, dz = c.z - cz;
    const float r2 = dx * dx + dy * dy + dz * dz;
    q[0] += qa.x + c.w * (3.f * dx * dx - r2);
    q[1] += qa.y + c.w * (3.f * dy * dy - r2);
    q[2] += qa.z + c.w * (3.f * dz * dz - r2);
    q[3] += qa.w + c.w * 3.f * dx * dy;
    q[4] += qb.x + c.w * 3.f * dx * dz;
    q[5] += qb.y + c.w * 3.f * dy * dz;
  }
  finish_moments32(a, p, m, cx, cy, cz, q);
}

// Moments bottom-up, one launch per depth: leaves first (any depth), then
// the inner nodes of each depth from the deepest up, so every node's
// children are complete when it is combined. Nodes are bucketed by depth
// (bucket kLeafBucket holds the leaves); the order inside a bucket does not
// matter, each node's sums run in the reference's order.
// Buckets also split by size -- inner nodes by child count, leaves by body
// count -- so that the nodes a warp combines loop the same number of times:
// the FP64 pipe, the bound here, then issues full warps.
constexpr int kSizeClasses = 8;                          // 1..8 children
constexpr int kLeafClasses = 9;                          // 1..8 bodies, more
constexpr int kLeafBucket = (kMaxDepth + 1) * kSizeClasses;  // first leaf bucket
constexpr int kBuckets = kLeafBucket + kLeafClasses;

struct BucketView {
  const u8 *depth, *isleaf, *nchild;
  const u32 *nbegin, *nend;
};

__device__ __forceinline__ int bucket_of(const BucketView &v, u32 p) {
  if (v.isleaf[p]) {
    const u32 nb = v.nend[p] - v.nbegin[p];
    return kLeafBucket + static_cast<int>(nb < 1 ? 0u : min(nb, static_cast<u32>(kLeafClasses)) - 1);
  }
  const int c = v.nchild[p];
  return v.depth[p] * kSizeClasses + (c < 1 ? 0 : min(c, kSizeClasses) - 1);
}

// Per-block histograms in shared memory, one global atomic per bucket.
__global__ void __launch_bounds__(kT)
    k_bucket_count(BucketView v, u32 m, u32 *count, const u32 *m_dev = nullptr,
                   u32 *abort = nullptr, int depth_cap = kMaxDepth) {
  __shared__ u32 h[kBuckets];
  if (aborted(abort)) return;
  for (int b = threadIdx.x; b < kBuckets; b += kT) h[b] = 0;
  __syncthreads();
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p < bounded(m, m_dev)) {
    if (abort && !v.isleaf[p] && v.depth[p] > depth_cap) atomicOr(abort, 4u);
    atomicAdd(&h[bucket_of(v, p)], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += kT)
    if (h[b]) atomicAdd(&count[b], h[b]);
}

// offsets[b] = start of bucket b; also clears the fill counters.
constexpr int kBucketThreads = 512;  // one bucket per thread
static_assert(kBuckets <= kBucketThreads, "bucket scan covers every bucket");
__global__ void __launch_bounds__(kBucketThreads)
    k_bucket_offsets(const u32 *count, u32 *offset, u32 *fill, const u32 *abort = nullptr) {
  __shared__ u32 part[kBucketThreads / 32];
  if (aborted(abort)) return;  // the same flag for every thread
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const u32 c = t < kBuckets ? count[t] : 0u;
  u32 incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const u32 v = __shfl_up_sync(kFullMask, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) part[w] = incl;
  __syncthreads();
  if (w == 0) {
    const u32 v = lane < kBucketThreads / 32 ? part[lane] : 0u;
    u32 pi = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 x = __shfl_up_sync(kFullMask, pi, o);
      if (lane >= o) pi += x;
    }
    if (lane < kBucketThreads / 32) part[lane] = pi - v;
  }
  __syncthreads();
  if (t < kBuckets) {
    offset[t] = part[w] + incl - c;
    fill[t] = 0;
  }
}

// Each block reserves one range per bucket, then places its nodes in it.
__global__ void __launch_bounds__(kT)
    k_bucket_fill(BucketView v, u32 m, const u32 *offset, u32 *fill, u32 *bucket,
                  const u32 *m_dev = nullptr, const u32 *abort = nullptr) {
  __shared__ u32 h[kBuckets], base[kBuckets];
  if (aborted(abort)) return;
  for (int b = threadIdx.x; b < kBuckets; b += kT) h[b] = 0;
  __syncthreads();
  const u32 p = blockIdx.x * kT + threadIdx.x;
  int b = -1;
  u32 local = 0;
  if (p < bounded(m, m_dev)) {
    b = bucket_of(v, p);
    local = atomicAdd(&h[b], 1u);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kBuckets; k += kT)
    base[k] = h[k] ? offset[k] + atomicAdd(&fill[k], h[k]) : 0;
  __syncthreads();
  if (b >= 0) bucket[base[b] + local] = p;
}

// kQuad: the quadrupole pass, else the centre-of-mass pass.
template <bool kQuad>
__global__ void __launch_bounds__(kT)
    k_leaf_moments(MomentArrays a, const u32 *bucket, const u32 *meta) {
  // the leaf buckets' count and first place, from the bucket scan
  u32 count = 0;
  for (int b = kLeafBucket; b < kLeafBucket + kLeafClasses; ++b) count += meta[b];
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= count) return;
  const u32 p = bucket[meta[kBuckets + kLeafBucket] + k];
  if (kQuad) leaf_quad(a, p);
  else leaf_com(a, p);
}

// Inner-node moments of one depth: one warp per block, `per` nodes to a
// warp (lanes past it idle). A depth with few nodes spreads them over many
// SMs: the sums are FP64-bound, and one SM's FP64 rate took ~40 us for a
// block of 256 nodes whatever the depth.
constexpr int kMomentWarps = 1216;  // warps a depth is spread over (8 per SM)

__host__ __device__ __forceinline__ u32 nodes_per_warp(u32 count) {
  const u32 per = (count + kMomentWarps - 1) / kMomentWarps;
  return per < 1 ? 1u : (per > 32 ? 32u : per);
}

// Over the device counts of buckets [b0, b0 + nb) (leaves or one depth's
// inner nodes), grid-stride over kMomentWarps warps: no count is read back,
// so the launches of every depth queue at once (eager and graph replays).
template <bool kQuad>
__global__ void __launch_bounds__(32)
    k_node_moments(MomentArrays a, const u32 *bucket, const u32 *meta, int b0, int nb,
                   const u32 *abort) {
  if (*abort) return;
  u32 count = 0;
  for (int b = b0; b < b0 + nb; ++b) count += meta[b];
  const u32 off = meta[kBuckets + b0];
  const u32 per = nodes_per_warp(count);
  if (threadIdx.x >= per) return;
  for (u64 k = static_cast<u64>(blockIdx.x) * per + threadIdx.x; k < count;
       k += static_cast<u64>(gridDim.x) * per) {
    const u32 p = bucket[off + k];
    if (b0 >= kLeafBucket) {
      if (kQuad) leaf_quad(a, p);
      else leaf_com(a, p);
    } else {
      if (kQuad) node_quad(a, p);
      else node_com(a, p);
    }
  }
}

// All of the FP32 moments in one launch, bottom-up: a thread per leaf (in
// the leaf buckets' order) computes its leaf, then climbs while it is the
// last child of its parent to finish, computing that parent from its
// children in child order as node_moments32 does. So every node is computed
// once, after all its children, with the same operations as the per-depth
// launches; the climb ends at the root or at a parent a sibling will
// finish (at most kMaxDepth steps).
__global__ void __launch_bounds__(kT)
    k_moments32_up(Moment32Arrays a, const u32 *bucket, const u32 *meta, const u32 *parent,
                   u32 *arrive) {
  u32 count = 0;
  for (int b = kLeafBucket; b < kLeafBucket + kLeafClasses; ++b) count += meta[b];
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= count) return;
  u32 p = bucket[meta[kBuckets + kLeafBucket] + k];
  leaf_moments32(a, p);
  for (int step = 0; step <= kMaxDepth; ++step) {
    const u32 q = parent[p];
    if (q == 0xffffffffu) return;
    __threadfence();  // this node's values before its parent's count
    if (atomicAdd(&arrive[q], 1u) + 1u != a.nchild[q]) return;
    __threadfence();  // the siblings' values, counted before this, are visible
    node_moments32<true>(a, q);
    p = q;
  }
}

__global__ void k_root_mass(const float4 *cells32, double2 *rootmom) {
  rootmom[0] = make_double2(0.0, 0.0);
  rootmom[1] = make_double2(0.0, static_cast<double>(cells32[0].w));
}

// A graph replay's checks after the node count: deeper keys needed, or a
// leaf below the sorted levels (bit 1), or more nodes than the node arrays
// hold (bit 2).
__global__ void k_check_tree_graph(Scalars *sc, u32 cap, int sorted_levels) {
  if (sc->deep > 0 || static_cast<int>(sc->depth) > sorted_levels) sc->abort |= 1u;
  if (sc->n_nodes > cap) sc->abort |= 2u;
}

// --------------------------------------------------------------- packing

// Walk records (FP32 and FP64) of every node (group_lists.cpp:59-61): they
// need the centres of mass and deltas only, so they are packed after the
// first moment pass.
__global__ void __launch_bounds__(kT)
    k_pack_walk(const double2 *geom, const double2 *mom, const double *delta, const u32 *nbegin,
                const u32 *nend, const u32 *skip, const u8 *isleaf, u32 m, const TreeRoot *root,
                double inv_theta, WalkRec32 *walk32, WalkRec64 *walk64,
                const u32 *m_dev = nullptr, const u32 *abort = nullptr,
                const u16 *sys = nullptr) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || p >= bounded(m, m_dev)) return;
  if (sys) root += sys[nbegin[p]];  // a forest: relative to the node's system's root
  const Dbl4 g = load_pair(geom, p), c = load_pair(mom, p);
  const double crit = 2.0 * g.w * inv_theta + delta[p];
  WalkRec64 r;
  r.cx = g.x;
  r.cy = g.y;
  r.cz = g.z;
  r.slack = g.w * 1.0001;
  r.mx = c.x;
  r.my = c.y;
  r.mz = c.z;
  r.crit2 = crit * crit;
  walk64[p] = r;
  const double ox = root->center[0], oy = root->center[1], oz = root->center[2];
  WalkRec32 f;
  f.cx = static_cast<float>(g.x - ox);
  f.cy = static_cast<float>(g.y - oy);
  f.cz = static_cast<float>(g.z - oz);
  f.slack = static_cast<float>(r.slack);
  f.mx = static_cast<float>(c.x - ox);
  f.my = static_cast<float>(c.y - oy);
  f.mz = static_cast<float>(c.z - oz);
  f.crit2 = static_cast<float>(r.crit2);
  f.skip = skip[p];
  f.nbody_leaf = (nend[p] - nbegin[p]) | (isleaf[p] ? 0x80000000u : 0u);
  f.begin = nbegin[p];
  // magnitude bound of this record's FP32 values, rounded up
  const float mag = fmaxf(fmaxf(fmaxf(fabsf(f.cx), fabsf(f.cy)), fmaxf(fabsf(f.cz), fabsf(f.mx))),
                          fmaxf(fabsf(f.my), fabsf(f.mz)));
  f.bound = (mag + f.slack) * (1.0f + 1.0f / (1 << 20));
  walk32[p] = f;
}

// FP32 cell of every node, after the quadrupole pass (group_lists.cpp:52-58).
__global__ void __launch_bounds__(kT)
    k_pack_cells(const double2 *mom, const double2 *quad, const u32 *nbegin, u32 m,
                 const TreeRoot *root, float4 *cells, const u32 *m_dev = nullptr,
                 const u32 *abort = nullptr, const u16 *sys = nullptr) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (aborted(abort) || p >= bounded(m, m_dev)) return;
  if (sys) root += sys[nbegin[p]];
  const Dbl4 c = load_pair(mom, p);
  const double ox = root->center[0], oy = root->center[1], oz = root->center[2];
  const double2 qa = quad[3 * p], qb = quad[3 * p + 1], qc = quad[3 * p + 2];
  cells[3 * p] = make_float4(static_cast<float>(c.x - ox), static_cast<float>(c.y - oy),
                             static_cast<float>(c.z - oz), static_cast<float>(c.w));
  cells[3 * p + 1] = make_float4(static_cast<float>(qa.x), static_cast<float>(qa.y),
                                 static_cast<float>(qb.x), static_cast<float>(qb.y));
  cells[3 * p + 2] = make_float4(static_cast<float>(qc.x), static_cast<float>(qc.y), 0.0f, 0.0f);
}

// A forest's FP32 bodies, each relative to its system's root centre.
__global__ void __launch_bounds__(kT)
    k_pack_bodies_forest(const double *tpos, const double *tmass, u32 n, const u16 *sys,
                         const TreeRoot *roots, float4 *bodies, const u32 *abort = nullptr) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= n || aborted(abort)) return;
  const double *o = roots[sys[k]].center;
  bodies[k] = make_float4(static_cast<float>(tpos[3ull * k] - o[0]),
                          static_cast<float>(tpos[3ull * k + 1] - o[1]),
                          static_cast<float>(tpos[3ull * k + 2] - o[2]),
                          static_cast<float>(tmass[k]));
}

// FP32 bodies relative to `origin` (group_lists.cpp:46-50, gravity_backends.cpp:15-23).
__global__ void __launch_bounds__(kT)
    k_pack_bodies(const double *tpos, const double *tmass, u32 n, const double *origin,
                  float4 *bodies, const u32 *abort = nullptr) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= n || aborted(abort)) return;
  bodies[k] = make_float4(static_cast<float>(tpos[3ull * k] - origin[0]),
                          static_cast<float>(tpos[3ull * k + 1] - origin[1]),
                          static_cast<float>(tpos[3ull * k + 2] - origin[2]),
                          static_cast<float>(tmass[k]));
}

const double *root_centre(const TreeRoot *root) {
  return reinterpret_cast<const double *>(reinterpret_cast<const char *>(root) +
                                          offsetof(TreeRoot, center));
}

void read_scalars(Workspace &ws, Scalars *host, cudaStream_t s) {
  GTC_CUDA(cudaMemcpyAsync(host, ws.scalars.ptr, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

void bbox_root(Workspace &ws, const double *pos, u64 n, cudaStream_t s) {
  const u32 nparts = std::min<u32>(1024, std::max<u32>(1, ceil_div(n, kT)));
  ws.bbox_part.ensure(6 * sizeof(double) * nparts);
  ws.root.ensure(sizeof(TreeRoot));
  k_bbox_partial<<<nparts, kT, 0, s>>>(pos, n, ws.bbox_part.as<double>());
  GTC_LAUNCH_CHECK();
  k_root<<<1, kT, 0, s>>>(ws.bbox_part.as<double>(), static_cast<int>(nparts), ws.root.as<TreeRoot>());
  GTC_LAUNCH_CHECK();
}

void pack_bodies_bbox(Workspace &ws, const double *pos, const double *mass, u64 n,
                      cudaStream_t s) {
  bbox_root(ws, pos, n, s);
  ws.bodies.ensure(n * sizeof(float4));
  const TreeRoot *root = ws.root.as<TreeRoot>();
  k_pack_bodies<<<ceil_div(n, kT), kT, 0, s>>>(pos, mass, static_cast<u32>(n),
                                               root_centre(root), ws.bodies.as<float4>());
  GTC_LAUNCH_CHECK();
}

void ensure_side(Workspace &ws) {
  if (ws.side) return;
  GTC_CUDA(cudaStreamCreateWithFlags(&ws.side, cudaStreamNonBlocking));
  GTC_CUDA(cudaEventCreateWithFlags(&ws.side_fork, cudaEventDisableTiming));
  GTC_CUDA(cudaEventCreateWithFlags(&ws.side_done, cudaEventDisableTiming));
  GTC_CUDA(cudaEventCreateWithFlags(&ws.side_walk, cudaEventDisableTiming));
}

cudaStream_t fork_side(Workspace &ws, cudaStream_t s) {
  ensure_side(ws);
  GTC_CUDA(cudaEventRecord(ws.side_fork, s));
  GTC_CUDA(cudaStreamWaitEvent(ws.side, ws.side_fork, 0));
  ws.side_pending = true;
  ws.walk_pending = false;
  return ws.side;
}

void join_side(Workspace &ws, cudaStream_t s) {
  ws.walk_pending = false;
  if (!ws.side_pending) return;
  ws.side_pending = false;
  if (cudaEventRecord(ws.side_done, ws.side) == cudaSuccess)
    cudaStreamWaitEvent(s, ws.side_done, 0);
}

void mark_walk_ready(Workspace &ws, cudaStream_t side) {
  ws.stage(Workspace::kStMomW, side);
  GTC_CUDA(cudaEventRecord(ws.side_walk, side));
  ws.walk_pending = true;
}

void join_walk(Workspace &ws, cudaStream_t s) {
  if (!ws.walk_pending) {
    join_side(ws, s);  // no walk mark: all of the side stream's work
    return;
  }
  ws.walk_pending = false;
  GTC_CUDA(cudaStreamWaitEvent(s, ws.side_walk, 0));
}

namespace {
// The split table, its in-order copy and check, and the first key word of
// every body.
void make_keys(Workspace &ws, const double *pos, u32 n, cudaStream_t s) {
  const TreeRoot *root = ws.root.as<TreeRoot>();
  Scalars *sc = ws.scalars.as<Scalars>();
  ws.split.ensure(3ull * kSplitSize * sizeof(double));
  k_split_top<<<3, 1024, 0, s>>>(root, ws.split.as<double>());
  GTC_LAUNCH_CHECK();
  // levels kSplitTop..20: subtrees of 4, 4 and 2 levels
  static_assert(kSplitTop - 1 + 4 + 4 + 2 == kSplitLevels - 1, "split table levels");
  double *split = ws.split.as<double>();
  k_split_sub<4><<<ceil_div(3u << (kSplitTop - 1), kT), kT, 0, s>>>(root, split, kSplitTop - 1);
  GTC_LAUNCH_CHECK();
  k_split_sub<4><<<ceil_div(3u << (kSplitTop + 3), kT), kT, 0, s>>>(root, split, kSplitTop + 3);
  GTC_LAUNCH_CHECK();
  k_split_sub<2><<<ceil_div(3u << (kSplitTop + 7), kT), kT, 0, s>>>(root, split, kSplitTop + 7);
  GTC_LAUNCH_CHECK();
  k_split_check<<<ceil_div(3u << (kSplitLevels - 1), kT), kT, 0, s>>>(split, &sc->split_unsorted);
  GTC_LAUNCH_CHECK();
  k_keys<<<ceil_div(n, kT), kT, 0, s>>>(pos, n, root, split, &sc->split_unsorted,
                                        ws.key0.as<u64>(), ws.idx.as<u32>(), ws.tiny.as<u8>(),
                                        &sc->error);
  GTC_LAUNCH_CHECK();
}
}  // namespace

namespace {
// Sorts the (key, body) pairs on the first `levels` levels of the first key
// word, rounded up to whole 8-bit passes (21 or more: the whole word), and
// returns the levels the order is exact for. Bodies that share those levels
// keep their input order, which is all the tree needs while no leaf lies
// deeper. A forest's pairs are then sorted by system, stably: (system,
// key), each system at its own bodies' positions.
int sort_top_levels(Workspace &ws, u32 n, int levels, cudaStream_t s,
                    const u32 *abort = nullptr) {
  const int passes = levels >= kLevelsPerWord ? 8 : (3 * std::max(levels, 1) + 7) / 8;
  const int low = std::max(0, 3 * kLevelsPerWord - 8 * passes);
  ws.sort_passes = passes;
  u32 *err = &ws.scalars.as<Scalars>()->error;
  radix_sort_pairs(ws.key0.as<u64>(), ws.idx.as<u32>(), ws.key0_alt.as<u64>(),
                   ws.idx_alt.as<u32>(), n, 3 * kLevelsPerWord - low, ws.radix, s, low, err);
  if (ws.forest) {
    const ForestView &fv = ws.forest;
    ws.dkey.ensure(n * 8ull);
    ws.dkey_alt.ensure(n * 8ull);
    ws.drec.ensure(n * 4ull);
    ws.drec_alt.ensure(n * 4ull);
    u64 *skey = ws.dkey.as<u64>();
    u32 *spos = ws.drec.as<u32>();
    const u32 nb = ceil_div(n, kT);
    k_forest_sys_keys<<<nb, kT, 0, s>>>(ws.key0.as<u64>(), ws.idx.as<u32>(), fv.sys, n, skey,
                                        spos, ws.key0_alt.as<u64>(), ws.idx_alt.as<u32>(), abort);
    GTC_LAUNCH_CHECK();
    int bits = 1;
    while (bits < 16 && (1u << bits) < fv.systems) ++bits;
    radix_sort_pairs(skey, spos, ws.dkey_alt.as<u64>(), ws.drec_alt.as<u32>(), n, bits, ws.radix,
                     s, 0, err);
    k_forest_gather<<<nb, kT, 0, s>>>(spos, ws.key0_alt.as<u64>(), ws.idx_alt.as<u32>(), n,
                                      ws.key0.as<u64>(), ws.idx.as<u32>(), abort);
    GTC_LAUNCH_CHECK();
  }
  return low == 0 ? kLevelsPerWord : (3 * kLevelsPerWord - low) / 3;
}

// A forest's root cubes (one per system), split tables and first key words.
void forest_keys(Workspace &ws, const double *pos, u32 n, cudaStream_t s) {
  const ForestView &fv = ws.forest;
  ws.bbox_part.ensure(6 * sizeof(double) * fv.bbox_nblocks);
  k_bbox_forest<<<fv.bbox_nblocks, kT, 0, s>>>(pos, fv.bbox_blocks, fv.start,
                                               ws.bbox_part.as<double>());
  GTC_LAUNCH_CHECK();
  k_root_forest<<<fv.systems, kT, 0, s>>>(ws.bbox_part.as<double>(), fv.sys_blocks, fv.roots);
  GTC_LAUNCH_CHECK();
  const int T = fv.split_levels;
  const u32 size = 1u << T, tables = 3 * fv.systems;
  ws.split.ensure(static_cast<u64>(tables) * size * sizeof(double));
  double *split = ws.split.as<double>();
  const int top = std::min(T, kSplitTop);
  k_split_top_forest<<<tables, 1024, 0, s>>>(fv.roots, split, size, top);
  GTC_LAUNCH_CHECK();
  for (int lv = top; lv < T;) {  // levels lv.. below the nodes of level lv - 1
    const int L = T - lv >= 4 ? 4 : (T - lv >= 2 ? 2 : 1);
    const u32 blocks = ceil_div(static_cast<u64>(tables) << (lv - 1), kT);
    if (L == 4) k_split_sub_forest<4><<<blocks, kT, 0, s>>>(fv.roots, split, size, tables, lv - 1);
    else if (L == 2) k_split_sub_forest<2><<<blocks, kT, 0, s>>>(fv.roots, split, size, tables, lv - 1);
    else k_split_sub_forest<1><<<blocks, kT, 0, s>>>(fv.roots, split, size, tables, lv - 1);
    GTC_LAUNCH_CHECK();
    lv += L;
  }
  GTC_CUDA(cudaMemsetAsync(fv.split_unsorted, 0, fv.systems * sizeof(u32), s));
  k_split_check_forest<<<ceil_div(static_cast<u64>(tables) << (T - 1), kT), kT, 0, s>>>(
      split, size, T, tables, fv.split_unsorted);
  GTC_LAUNCH_CHECK();
  k_keys_forest<<<ceil_div(n, kT), kT, 0, s>>>(pos, n, fv.sys, fv.roots, split, size, T,
                                               fv.split_unsorted, ws.key0.as<u64>(),
                                               ws.idx.as<u32>(), ws.tiny.as<u8>(),
                                               &ws.scalars.as<Scalars>()->error);
  GTC_LAUNCH_CHECK();
}

void forest_roots(Workspace &ws, const u32 *abort, cudaStream_t s) {
  const ForestView &fv = ws.forest;
  k_forest_roots<<<ceil_div(fv.systems, kT), kT, 0, s>>>(
      fv.start, fv.systems, ws.count.as<u32>(), ws.count_scan.as<u32>(),
      ws.scalars.as<Scalars>(), fv.root_node, ws.parent.as<u32>(), abort);
  GTC_LAUNCH_CHECK();
}

void pack_bodies_tree(Workspace &ws, u32 n, const TreeRoot *root, const u32 *abort,
                      cudaStream_t s) {
  if (ws.forest) {
    k_pack_bodies_forest<<<ceil_div(n, kT), kT, 0, s>>>(ws.tpos.as<double>(), ws.tmass.as<double>(),
                                                        n, ws.forest.sys, ws.forest.roots,
                                                        ws.bodies.as<float4>(), abort);
  } else {
    k_pack_bodies<<<ceil_div(n, kT), kT, 0, s>>>(ws.tpos.as<double>(), ws.tmass.as<double>(), n,
                                                 root_centre(root), ws.bodies.as<float4>(), abort);
  }
  GTC_LAUNCH_CHECK();
}
}  // namespace

void build_tree(Workspace &ws, const double *pos, const double *mass, u64 n,
                const SolverParams &sp, cudaStream_t s, Scalars *host, bool walk_records) {
  ws.n = n;
  ws.n_nodes = 0;
  ws.key_words = 1;
  if (n == 0) return;
  const u32 n32 = static_cast<u32>(n);
  const u32 nb = ceil_div(n, kT);
  const int L = std::max(1, sp.leaf_size);

  ws.key0.ensure(n * 8);
  ws.key0_alt.ensure(n * 8);
  ws.idx.ensure(n * 4);
  ws.idx_alt.ensure(n * 4);
  ws.tiny.ensure(n);
  ws.lcp.ensure(n);
  ws.leafdepth.ensure(n);
  ws.count.ensure(n * 4);
  ws.count_scan.ensure(n * 4);
  ws.tpos.ensure(n * 24);
  ws.tmass.ensure(n * 8);
  ws.bodies.ensure(n * sizeof(float4));
  ws.scalars.ensure(sizeof(Scalars));
  join_side(ws, s);  // nothing of an earlier call may still write the buffers
  Scalars *sc = ws.scalars.as<Scalars>();
  GTC_CUDA(cudaMemsetAsync(sc, 0, sizeof(Scalars), s));

  ws.stage(Workspace::kStBuild, s);
  const ForestView &fv = ws.forest;
  if (fv) forest_keys(ws, pos, n32, s);
  else bbox_root(ws, pos, n, s);
  const TreeRoot *root = fv ? fv.roots : ws.root.as<TreeRoot>();
  u64 *key0 = ws.key0.as<u64>();
  u32 *idx = ws.idx.as<u32>();
  u8 *tiny = ws.tiny.as<u8>();
  if (!fv) make_keys(ws, pos, n32, s);
  // the levels the last tree needed first; all of them when a leaf lies
  // deeper (sorting the partly sorted pairs again gives the full order)
  ws.stage(Workspace::kStSort0, s);
  const int sorted = sort_top_levels(ws, n32, ws.sort_levels > 0 ? ws.sort_levels : kLevelsPerWord, s);
  ws.stage(Workspace::kStSort1, s);

  KeyView kv{key0, nullptr, nullptr, 1, fv.sys};
  signed char *lcp_next = ws.lcp.as<signed char>();
  u8 *leafdepth = ws.leafdepth.as<u8>();
  // Node numbering: count the nodes ending at each sorted position (with
  // the levels, so that one read back serves both).
  u32 *count = ws.count.as<u32>(), *cscan = ws.count_scan.as<u32>();
  auto count_nodes = [&] {
    k_node_count<<<nb, kT, 0, s>>>(lcp_next, leafdepth, n32, count);
    GTC_LAUNCH_CHECK();
    exclusive_scan_u32(count, cscan, n, &sc->n_nodes, ws.scan_tmp, s);
  };
  k_levels<<<nb, kT, 0, s>>>(kv, idx, tiny, n32, L, lcp_next, leafdepth, sc);
  GTC_LAUNCH_CHECK();
  count_nodes();
  read_scalars(ws, host, s);
  if (host->error & 4u) throw InvalidArgument("cuda: positions must be finite");
  if (sorted < kLevelsPerWord && static_cast<int>(host->depth) > sorted) {
    sort_top_levels(ws, n32, kLevelsPerWord, s);
    GTC_CUDA(cudaMemsetAsync(&sc->deep, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(&sc->depth, 0, sizeof(u32), s));
    k_levels<<<nb, kT, 0, s>>>(kv, idx, tiny, n32, L, lcp_next, leafdepth, sc);
    GTC_LAUNCH_CHECK();
    count_nodes();
    read_scalars(ws, host, s);
  }
  const bool had_deep = host->deep > 0;

  // Deeper key words for bodies whose leaves lie below the words so far.
  while (host->deep > 0 && kv.words < 3) {
    const int limit = kLevelsPerWord * kv.words;
    DeviceBuffer &wbuf = kv.words == 1 ? ws.key1 : ws.key2;
    wbuf.ensure(n * 8);
    GTC_CUDA(cudaMemsetAsync(wbuf.ptr, 0, n * 8, s));
    ws.flags.ensure(n * 4);
    ws.flags_scan.ensure(n * 4);
    u32 *flag = ws.flags.as<u32>(), *fscan = ws.flags_scan.as<u32>();
    k_deep_flags<<<nb, kT, 0, s>>>(leafdepth, n32, limit, flag);
    GTC_LAUNCH_CHECK();
    exclusive_scan_u32(flag, fscan, n, &sc->deep, ws.scan_tmp, s);
    read_scalars(ws, host, s);
    const u32 nd = host->deep;
    ws.dpos.ensure(nd * 4ull);
    ws.dkey.ensure(nd * 8ull);
    ws.dkey_alt.ensure(nd * 8ull);
    ws.drec.ensure(nd * 4ull);
    ws.drec_alt.ensure(nd * 4ull);
    const u64 idx_bytes = (nd * 4ull + 15) & ~15ull;
    ws.dtmp.ensure(idx_bytes + nd * 8ull);
    u32 *dpos = ws.dpos.as<u32>(), *drec = ws.drec.as<u32>();
    u32 *didx = ws.dtmp.as<u32>();
    u64 *dword = reinterpret_cast<u64 *>(ws.dtmp.as<char>() + idx_bytes);
    const u32 ndb = ceil_div(nd, kT);
    k_compact<<<nb, kT, 0, s>>>(flag, fscan, n32, dpos);
    GTC_LAUNCH_CHECK();
    k_deep_keys<<<ndb, kT, 0, s>>>(kv, dpos, nd, idx, pos, root, tiny, dword, drec, didx);
    GTC_LAUNCH_CHECK();
    // order records by (segment, new word, input order): sort by the word,
    // then stably by segment number
    u64 *dkey = ws.dkey.as<u64>();
    GTC_CUDA(cudaMemcpyAsync(dkey, dword, nd * 8ull, cudaMemcpyDeviceToDevice, s));
    radix_sort_pairs(dkey, drec, ws.dkey_alt.as<u64>(), ws.drec_alt.as<u32>(), nd, 63, ws.radix, s,
                     0, &sc->error);
    u32 *sflag = ws.flags.as<u32>(), *sscan = ws.flags_scan.as<u32>();
    k_deep_segments<<<ndb, kT, 0, s>>>(kv, dpos, nd, sflag);
    GTC_LAUNCH_CHECK();
    exclusive_scan_u32(sflag, sscan, nd, &sc->aux, ws.scan_tmp, s);
    read_scalars(ws, host, s);
    int seg_bits = 1;
    while (seg_bits < 32 && (1ull << seg_bits) <= host->aux) ++seg_bits;
    k_seg_keys<<<ndb, kT, 0, s>>>(drec, sscan, sflag, nd, dkey);
    GTC_LAUNCH_CHECK();
    radix_sort_pairs(dkey, drec, ws.dkey_alt.as<u64>(), ws.drec_alt.as<u32>(), nd, seg_bits,
                     ws.radix, s, 0, &sc->error);
    k_deep_scatter<<<ndb, kT, 0, s>>>(dpos, drec, didx, dword, nd, idx, wbuf.as<u64>());
    GTC_LAUNCH_CHECK();
    if (kv.words == 1) kv.w1 = ws.key1.as<u64>();
    else kv.w2 = ws.key2.as<u64>();
    kv.words += 1;
    GTC_CUDA(cudaMemsetAsync(&sc->deep, 0, sizeof(u32), s));
    k_levels<<<nb, kT, 0, s>>>(kv, idx, tiny, n32, L, lcp_next, leafdepth, sc);
    GTC_LAUNCH_CHECK();
    read_scalars(ws, host, s);
  }
  if (host->deep > 0) throw RuntimeError("octree deeper than the depth cap");
  ws.key_words = kv.words;
  ws.sort_levels = kv.words == 1 ? static_cast<int>(host->depth) + 1 : 0;
  if (had_deep) {  // new key words: count again
    count_nodes();
    read_scalars(ws, host, s);
  }
  const u32 m = host->n_nodes;
  ws.n_nodes = m;
  ws.tree_depth = static_cast<int>(host->depth);
  ws.geom.ensure(m * 2 * sizeof(double2));
  ws.mom.ensure(m * 2 * sizeof(double2));
  ws.quad.ensure(m * 3 * sizeof(double2));
  ws.delta.ensure(m * 8ull);
  ws.nbegin.ensure(m * 4ull);
  ws.nend.ensure(m * 4ull);
  ws.skip.ensure(m * 4ull);
  ws.parent.ensure(m * 4ull);
  ws.depth.ensure(m);
  ws.nchild.ensure(m);
  ws.isleaf.ensure(m);
  ws.arrive.ensure(3 * kBuckets * sizeof(u32));
  ws.bucket.ensure(m * 4ull);
  ws.walk32.ensure(m * sizeof(WalkRec32));
  ws.walk64.ensure(m * sizeof(WalkRec64));
  ws.cells.ensure(m * 3 * sizeof(float4));
  const u32 mb = ceil_div(m, kT);

  k_nodes<<<nb, kT, 0, s>>>(kv, lcp_next, leafdepth, count, cscan, n32, sc, root,
                            ws.split.as<double>(), ws.geom.as<double2>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(),
                            ws.skip.as<u32>(), ws.depth.as<u8>(), ws.isleaf.as<u8>(), nullptr,
                            fv ? 1u << fv.split_levels : kSplitSize,
                            fv ? fv.split_levels : kSplitLevels);
  GTC_LAUNCH_CHECK();
  ws.kids.ensure(static_cast<u64>(m) * 8 * sizeof(u32));
  k_children<<<mb, kT, 0, s>>>(ws.skip.as<u32>(), ws.isleaf.as<u8>(), m, ws.parent.as<u32>(),
                               ws.nchild.as<u8>(), ws.kids.as<uint4>());
  GTC_LAUNCH_CHECK();
  if (fv) forest_roots(ws, nullptr, s);
  k_leaf_order<<<mb, kT, 0, s>>>(ws.isleaf.as<u8>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(), m, idx);
  GTC_LAUNCH_CHECK();
  k_tree_order<<<nb, kT, 0, s>>>(pos, mass, idx, n32, ws.tpos.as<double>(), ws.tmass.as<double>());
  GTC_LAUNCH_CHECK();
  ws.stage(Workspace::kStTopo, s);

  // moments, one depth at a time from the leaves up
  u32 *meta = ws.arrive.as<u32>();  // count[kBuckets], offset[kBuckets], fill[kBuckets]
  u32 *bucket = ws.bucket.as<u32>();
  GTC_CUDA(cudaMemsetAsync(meta, 0, kBuckets * sizeof(u32), s));
  const BucketView bv{ws.depth.as<u8>(), ws.isleaf.as<u8>(), ws.nchild.as<u8>(),
                      ws.nbegin.as<u32>(), ws.nend.as<u32>()};
  k_bucket_count<<<mb, kT, 0, s>>>(bv, m, meta);
  GTC_LAUNCH_CHECK();
  k_bucket_offsets<<<1, kBucketThreads, 0, s>>>(meta, meta + kBuckets, meta + 2 * kBuckets);
  GTC_LAUNCH_CHECK();
  k_bucket_fill<<<mb, kT, 0, s>>>(bv, m, meta + kBuckets, meta + 2 * kBuckets, bucket);
  GTC_LAUNCH_CHECK();
  MomentArrays ma{ws.geom.as<double2>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(),
                  ws.skip.as<u32>(), ws.parent.as<u32>(), ws.nchild.as<u8>(),
                  ws.kids.as<uint4>(), ws.tpos.as<double>(), ws.tmass.as<double>(),
                  ws.mom.as<double2>(),
                  ws.quad.as<double2>(), ws.delta.as<double>()};
  // the moments and node records on the side stream: the FP64 moments'
  // small depths leave most SMs idle, and the group choice needs none of
  // it. Bucket sizes are read on the device: leaves (at most m), then each
  // depth's inner nodes from the deepest possible one up.
  // The centres of mass first and the walk records from them (the walk
  // waits for these only), then the quadrupoles and the cells beside the
  // walk.
  cudaStream_t ms = fork_side(ws, s);
  ws.stage(Workspace::kStMom0, ms);
  k_leaf_moments<false><<<mb, kT, 0, ms>>>(ma, bucket, meta);
  GTC_LAUNCH_CHECK();
  for (int d = static_cast<int>(host->depth) - 1; d >= 0; --d) {
    k_node_moments<false><<<kMomentWarps, 32, 0, ms>>>(ma, bucket, meta, d * kSizeClasses,
                                                        kSizeClasses, &sc->abort);
    GTC_LAUNCH_CHECK();
  }
  if (walk_records) {
    k_pack_walk<<<mb, kT, 0, ms>>>(ws.geom.as<double2>(), ws.mom.as<double2>(),
                                   ws.delta.as<double>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(),
                                   ws.skip.as<u32>(), ws.isleaf.as<u8>(), m, root,
                                   1.0 / sp.theta, ws.walk32.as<WalkRec32>(),
                                   ws.walk64.as<WalkRec64>(), nullptr, nullptr, fv.sys);
    GTC_LAUNCH_CHECK();
  }
  mark_walk_ready(ws, ms);
  k_leaf_moments<true><<<mb, kT, 0, ms>>>(ma, bucket, meta);
  GTC_LAUNCH_CHECK();
  for (int d = static_cast<int>(host->depth) - 1; d >= 0; --d) {
    k_node_moments<true><<<kMomentWarps, 32, 0, ms>>>(ma, bucket, meta, d * kSizeClasses,
                                                       kSizeClasses, &sc->abort);
    GTC_LAUNCH_CHECK();
  }
  k_pack_cells<<<mb, kT, 0, ms>>>(ws.mom.as<double2>(), ws.quad.as<double2>(),
                                  ws.nbegin.as<u32>(), m, root, ws.cells.as<float4>(), nullptr,
                                  nullptr, fv.sys);
  GTC_LAUNCH_CHECK();
  ws.stage(Workspace::kStMom1, ms);
  pack_bodies_tree(ws, n32, root, nullptr, s);
}

void moments32(Workspace &ws, float4 *cells32, float *delta32, double2 *rootmom,
               cudaStream_t s) {
  const u32 m = static_cast<u32>(ws.n_nodes);
  if (m == 0) return;
  const Moment32Arrays a{ws.geom.as<double2>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(),
                         ws.nchild.as<u8>(),   ws.kids.as<uint4>(), ws.bodies.as<float4>(),
                         ws.root.as<TreeRoot>(), cells32, delta32};
  const u32 *meta = ws.arrive.as<u32>(), *bucket = ws.bucket.as<u32>();
  ws.up_arrive.ensure(m * sizeof(u32));
  GTC_CUDA(cudaMemsetAsync(ws.up_arrive.ptr, 0, m * sizeof(u32), s));
  k_moments32_up<<<ceil_div(m, kT), kT, 0, s>>>(a, bucket, meta, ws.parent.as<u32>(),
                                                ws.up_arrive.as<u32>());
  GTC_LAUNCH_CHECK();
  k_root_mass<<<1, 1, 0, s>>>(cells32, rootmom);
  GTC_LAUNCH_CHECK();
}

void build_tree_graph(Workspace &ws, const double *pos, const double *mass, u64 n,
                      const SolverParams &sp, const GraphCaps &caps, cudaStream_t s) {
  ws.n = n;
  ws.key_words = 1;
  const u32 n32 = static_cast<u32>(n), mcap = caps.nodes;
  const u32 nb = ceil_div(n, kT), mb = ceil_div(mcap, kT);
  const int L = std::max(1, sp.leaf_size);
  Scalars *sc = ws.scalars.as<Scalars>();
  u32 *abort = &sc->abort;
  GTC_CUDA(cudaMemsetAsync(sc, 0, sizeof(Scalars), s));
  const ForestView &fv = ws.forest;
  if (fv) forest_keys(ws, pos, n32, s);
  else bbox_root(ws, pos, n, s);
  const TreeRoot *root = fv ? fv.roots : ws.root.as<TreeRoot>();
  u64 *key0 = ws.key0.as<u64>();
  u32 *idx = ws.idx.as<u32>();
  u8 *tiny = ws.tiny.as<u8>();
  if (!fv) make_keys(ws, pos, n32, s);
  // the levels the captured depth allows: a deeper tree aborts the replay
  const int sorted = sort_top_levels(ws, n32, caps.depth + 1, s);
  const KeyView kv{key0, nullptr, nullptr, 1, fv.sys};
  signed char *lcp_next = ws.lcp.as<signed char>();
  u8 *leafdepth = ws.leafdepth.as<u8>();
  k_levels<<<nb, kT, 0, s>>>(kv, idx, tiny, n32, L, lcp_next, leafdepth, sc);
  GTC_LAUNCH_CHECK();
  u32 *count = ws.count.as<u32>(), *cscan = ws.count_scan.as<u32>();
  k_node_count<<<nb, kT, 0, s>>>(lcp_next, leafdepth, n32, count);
  GTC_LAUNCH_CHECK();
  exclusive_scan_u32(count, cscan, n, &sc->n_nodes, ws.scan_tmp, s);
  k_check_tree_graph<<<1, 1, 0, s>>>(sc, mcap, sorted);
  GTC_LAUNCH_CHECK();
  const u32 *m_dev = &sc->n_nodes;
  k_nodes<<<nb, kT, 0, s>>>(kv, lcp_next, leafdepth, count, cscan, n32, sc, root,
                            ws.split.as<double>(), ws.geom.as<double2>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(),
                            ws.skip.as<u32>(), ws.depth.as<u8>(), ws.isleaf.as<u8>(), abort,
                            fv ? 1u << fv.split_levels : kSplitSize,
                            fv ? fv.split_levels : kSplitLevels);
  GTC_LAUNCH_CHECK();
  k_children<<<mb, kT, 0, s>>>(ws.skip.as<u32>(), ws.isleaf.as<u8>(), mcap, ws.parent.as<u32>(),
                               ws.nchild.as<u8>(), ws.kids.as<uint4>(), m_dev, abort);
  GTC_LAUNCH_CHECK();
  if (fv) forest_roots(ws, abort, s);
  k_leaf_order<<<mb, kT, 0, s>>>(ws.isleaf.as<u8>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(), mcap,
                                 idx, m_dev, abort);
  GTC_LAUNCH_CHECK();
  k_tree_order<<<nb, kT, 0, s>>>(pos, mass, idx, n32, ws.tpos.as<double>(), ws.tmass.as<double>(),
                                 abort);
  GTC_LAUNCH_CHECK();
  u32 *meta = ws.arrive.as<u32>();
  u32 *bucket = ws.bucket.as<u32>();
  GTC_CUDA(cudaMemsetAsync(meta, 0, kBuckets * sizeof(u32), s));
  const BucketView bv{ws.depth.as<u8>(), ws.isleaf.as<u8>(), ws.nchild.as<u8>(),
                      ws.nbegin.as<u32>(), ws.nend.as<u32>()};
  k_bucket_count<<<mb, kT, 0, s>>>(bv, mcap, meta, m_dev, abort, caps.depth);
  GTC_LAUNCH_CHECK();
  k_bucket_offsets<<<1, kBucketThreads, 0, s>>>(meta, meta + kBuckets, meta + 2 * kBuckets, abort);
  GTC_LAUNCH_CHECK();
  k_bucket_fill<<<mb, kT, 0, s>>>(bv, mcap, meta + kBuckets, meta + 2 * kBuckets, bucket, m_dev,
                                  abort);
  GTC_LAUNCH_CHECK();
  MomentArrays ma{ws.geom.as<double2>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(),
                  ws.skip.as<u32>(), ws.parent.as<u32>(), ws.nchild.as<u8>(),
                  ws.kids.as<uint4>(), ws.tpos.as<double>(), ws.tmass.as<double>(),
                  ws.mom.as<double2>(),
                  ws.quad.as<double2>(), ws.delta.as<double>()};
  // the centres of mass and the walk records in line; the quadrupoles and
  // the cells on the side stream, beside the group choice and the walk (the
  // caller joins it before the evaluation)
  k_node_moments<false><<<kMomentWarps, 32, 0, s>>>(ma, bucket, meta, kLeafBucket, kLeafClasses,
                                                     abort);
  GTC_LAUNCH_CHECK();
  for (int d = std::min(caps.depth, kMaxDepth); d >= 0; --d) {
    k_node_moments<false><<<kMomentWarps, 32, 0, s>>>(ma, bucket, meta, d * kSizeClasses,
                                                       kSizeClasses, abort);
    GTC_LAUNCH_CHECK();
  }
  k_pack_walk<<<mb, kT, 0, s>>>(ws.geom.as<double2>(), ws.mom.as<double2>(),
                                ws.delta.as<double>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(),
                                ws.skip.as<u32>(), ws.isleaf.as<u8>(), mcap, root, 1.0 / sp.theta,
                                ws.walk32.as<WalkRec32>(), ws.walk64.as<WalkRec64>(), m_dev,
                                abort, fv.sys);
  GTC_LAUNCH_CHECK();
  cudaStream_t ms = fork_side(ws, s);
  k_node_moments<true><<<kMomentWarps, 32, 0, ms>>>(ma, bucket, meta, kLeafBucket, kLeafClasses,
                                                     abort);
  GTC_LAUNCH_CHECK();
  for (int d = std::min(caps.depth, kMaxDepth); d >= 0; --d) {
    k_node_moments<true><<<kMomentWarps, 32, 0, ms>>>(ma, bucket, meta, d * kSizeClasses,
                                                      kSizeClasses, abort);
    GTC_LAUNCH_CHECK();
  }
  k_pack_cells<<<mb, kT, 0, ms>>>(ws.mom.as<double2>(), ws.quad.as<double2>(),
                                  ws.nbegin.as<u32>(), mcap, root, ws.cells.as<float4>(), m_dev,
                                  abort, fv.sys);
  GTC_LAUNCH_CHECK();
  pack_bodies_tree(ws, n32, root, abort, s);
}

}  // namespace gtc
