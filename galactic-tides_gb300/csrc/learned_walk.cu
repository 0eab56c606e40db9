// The learned criterion inside the grouped walk: per-node features, per-group
// tolerances, the walk with warp-level BF16 tensor-core inference, and the
// tensor-core layout of the model.
//
// Inference runs on the legacy warp-synchronous tensor path (mma.sync
// m16n8k16, BF16 operands, FP32 accumulators): one warp evaluates 32 rows
// (one per lane) in 80 instructions, 16 for the first layer (6 features, a
// constant 1 for the bias, zero padding to K = 16) and 64 for the second.
// The first layer's accumulators are repacked in registers as the second
// layer's A operand; the third layer is a dot product over each lane's
// accumulator columns, summed across the four lanes of a quad.

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "learned.cuh"

namespace gtc {
namespace {

constexpr int kT = 256;

__device__ __forceinline__ void mma_bf16(float (&d)[4], u32 a0, u32 a1, u32 a2, u32 a3, u32 b0,
                                         u32 b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ u32 pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const u32 *>(&v);
}

// The MLP for the 32 rows of `rows` (per row: the six normalised features
// and a constant 1 as BF16 pairs). Every lane of the warp must call it; lane
// L gets the network output (normalised units) of row L. The two 16-row
// tiles run one after the other, which keeps the walk's register count low
// (more warps in flight to hide its memory latency); the B fragments come
// from shared memory.
__device__ __forceinline__ float warp_mlp(const uint4 *rows, const u32 *w1, const uint2 *w2,
                                          const float *b2, const float *w3, float b3, int lane) {
  const int g = lane >> 2, t = lane & 3;
  float o[4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    const u32 a0 = reinterpret_cast<const u32 *>(&rows[mt * 16 + g])[t];
    const u32 a1 = reinterpret_cast<const u32 *>(&rows[mt * 16 + g + 8])[t];
    u32 A[4][4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      float c[4] = {0.f, 0.f, 0.f, 0.f}, e[4] = {0.f, 0.f, 0.f, 0.f};
      mma_bf16(c, a0, a1, 0u, 0u, w1[j * 32 + lane], 0u);
      mma_bf16(e, a0, a1, 0u, 0u, w1[(j + 1) * 32 + lane], 0u);
      A[j / 2][0] = pack_bf16(fmaxf(c[0], 0.f), fmaxf(c[1], 0.f));
      A[j / 2][1] = pack_bf16(fmaxf(c[2], 0.f), fmaxf(c[3], 0.f));
      A[j / 2][2] = pack_bf16(fmaxf(e[0], 0.f), fmaxf(e[1], 0.f));
      A[j / 2][3] = pack_bf16(fmaxf(e[2], 0.f), fmaxf(e[3], 0.f));
    }
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float2 bb = *reinterpret_cast<const float2 *>(&b2[8 * j + 2 * t]);
      float c[4] = {bb.x, bb.y, bb.x, bb.y};
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint2 b = w2[(kk * 8 + j) * 32 + lane];
        mma_bf16(c, A[kk][0], A[kk][1], A[kk][2], A[kk][3], b.x, b.y);
      }
      const float2 w = *reinterpret_cast<const float2 *>(&w3[8 * j + 2 * t]);
      s0 = fmaf(fmaxf(c[0], 0.f), w.x, fmaf(fmaxf(c[1], 0.f), w.y, s0));
      s1 = fmaf(fmaxf(c[2], 0.f), w.x, fmaf(fmaxf(c[3], 0.f), w.y, s1));
    }
    s0 += __shfl_xor_sync(kFullMask, s0, 1);
    s0 += __shfl_xor_sync(kFullMask, s0, 2);
    s1 += __shfl_xor_sync(kFullMask, s1, 1);
    s1 += __shfl_xor_sync(kFullMask, s1, 2);
    o[2 * mt] = s0;      // row mt*16 + g
    o[2 * mt + 1] = s1;  // row mt*16 + g + 8
  }
  // row L lives in quad L % 8 as o[L / 8]
  const int src = (lane & 7) << 2, h = lane >> 3;
  const float v0 = __shfl_sync(kFullMask, o[0], src), v1 = __shfl_sync(kFullMask, o[1], src),
              v2 = __shfl_sync(kFullMask, o[2], src), v3 = __shfl_sync(kFullMask, o[3], src);
  return (h == 0 ? v0 : h == 1 ? v1 : h == 2 ? v2 : v3) + b3;
}

// The block's copy of what every lane reads per inference.
struct NetShared {
  uint2 w2[4 * 8 * 32];
  u32 w1[8 * 32];
  float b2[kHid], w3[kHid];
  float mean[kFeat], inv_std[kFeat];
};

__device__ __forceinline__ void load_net(const LearnedNet *net, NetShared &s) {
  for (int k = threadIdx.x; k < 4 * 8 * 32; k += blockDim.x) s.w2[k] = net->w2[k];
  for (int k = threadIdx.x; k < 8 * 32; k += blockDim.x) s.w1[k] = net->w1[k];
  for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
    s.b2[k] = net->b2[k];
    s.w3[k] = net->w3[k];
  }
  for (int k = threadIdx.x; k < kFeat; k += blockDim.x) {
    s.mean[k] = net->mean[k];
    s.inv_std[k] = net->inv_std[k];
  }
}

__device__ __forceinline__ uint4 feature_row(const float *f, const NetShared &s) {
  float x[kFeat];
#pragma unroll
  for (int j = 0; j < kFeat; ++j) x[j] = (f[j] - s.mean[j]) * s.inv_std[j];
  return make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]),
                    pack_bf16(1.f, 0.f));
}

__device__ __forceinline__ FeatScale scale_of(const TreeRoot *root, const double2 *mom) {
  return FeatScale{static_cast<float>(1.0 / root->half_at[0]), static_cast<float>(1.0 / mom[1].y)};
}

// ------------------------------------------------------------ kernels

__global__ void __launch_bounds__(kT)
    k_prepare_net(const float *model, LearnedNet *net) {
  const int k = blockIdx.x * kT + threadIdx.x;
  const float *W1 = model + kOffW1, *B1 = model + kOffB1, *W2 = model + kOffW2;
  if (k < 8 * 32) {
    const int j = k / 32, lane = k % 32, g = lane >> 2, t = lane & 3, n = 8 * j + g;
    // rows 2t, 2t+1 of [W1; b1; 0]
    auto w1row = [&](int r) { return r < kFeat ? W1[r * kHid + n] : r == kFeat ? B1[n] : 0.f; };
    net->w1[k] = pack_bf16(w1row(2 * t), w1row(2 * t + 1));
  }
  if (k < 4 * 8 * 32) {
    const int kk = k / 256, j = (k / 32) % 8, lane = k % 32, g = lane >> 2, t = lane & 3;
    const int n = 8 * j + g, r = 16 * kk + 2 * t;
    net->w2[k] = make_uint2(pack_bf16(W2[r * kHid + n], W2[(r + 1) * kHid + n]),
                            pack_bf16(W2[(r + 8) * kHid + n], W2[(r + 9) * kHid + n]));
  }
  if (k < kHid) {
    net->b2[k] = model[kOffB2 + k];
    net->w3[k] = model[kOffW3 + k];
  }
  if (k < kFeat) {
    net->mean[k] = model[kOffMean + k];
    net->inv_std[k] = 1.f / model[kOffStd + k];
  }
  if (k == 0) {
    net->b3 = model[kOffB3];
    net->y_mean = model[kOffYMean];
    net->y_std = model[kOffYStd];
    net->band = model[kOffBand];
  }
}

__global__ void __launch_bounds__(kT)
    k_cell_feat(const double2 *geom, const double2 *mom, const double2 *quad, const double *delta,
                const TreeRoot *root, u32 m, CellFeat *out) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p >= m) return;
  const FeatScale fs = scale_of(root, mom);
  const double2 qa = quad[3 * p], qb = quad[3 * p + 1], qc = quad[3 * p + 2];
  // Frobenius norm of the symmetric tensor (off-diagonal terms twice)
  const double qn = sqrt(qa.x * qa.x + qa.y * qa.y + qb.x * qb.x +
                         2.0 * (qb.y * qb.y + qc.x * qc.x + qc.y * qc.y));
  out[p] = cell_features(static_cast<float>(geom[2 * p + 1].y), static_cast<float>(mom[2 * p + 1].y),
                         static_cast<float>(qn), static_cast<float>(delta[p]), fs);
}

__global__ void __launch_bounds__(kT)
    k_lwalk_rec(const WalkRec32 *walk32, const CellFeat *cfeat, u32 m, float inv_theta_guard,
                float y_mean, LWalkRec *out) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p >= m) return;
  const WalkRec32 w = walk32[p];
  const float4 c0 = reinterpret_cast<const float4 *>(cfeat + p)[0];
  const float crit = fmaf(2.f * c0.x, inv_theta_guard, c0.y);
  LWalkRec r;
  r.cx = w.cx;
  r.cy = w.cy;
  r.cz = w.cz;
  r.slack = w.slack;
  r.mx = w.mx;
  r.my = w.my;
  r.mz = w.mz;
  r.guard2 = crit * crit;
  r.skip = w.skip;
  r.nbody_leaf = w.nbody_leaf;
  r.begin = w.begin;
  r.pscale = exp2f(0.4f * (c0.z + y_mean));
  out[p] = r;
}

// Per group: the group feature f0 and the tolerance
// tau = log2(alpha * a_g * L^2 / (G M_tot)), with the group's force scale
// a_g = max(min |a_prev|, mean |a_prev| / 2) over its targets. The floor
// keeps a target whose forces nearly cancel (|a| -> 0, at the centre of a
// symmetric system) from forcing its whole group down to single bodies.
__global__ void __launch_bounds__(kT)
    k_group_tol(const u32 *gbegin, const u32 *gend, u32 ng, const u32 *order,
                const float *prev_amag, const float *gboxf, const TreeRoot *root,
                const double2 *mom, double alpha, double G, float2 *gtol) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (g >= ng) return;
  const FeatScale fs = scale_of(root, mom);
  float amin = 3.0e38f, asum = 0.f;
  for (u32 t = gbegin[g]; t < gend[g]; ++t) {
    const float v = prev_amag[order[t]];
    amin = fminf(amin, v);
    asum += v;
  }
  const float ag = fmaxf(amin, 0.5f * asum / static_cast<float>(max(gend[g] - gbegin[g], 1u)));
  const double L = root->half_at[0], mt = mom[1].y;
  const double v = alpha * static_cast<double>(ag) * L * L / (G * mt);
  const float tau = v > 0.0 ? static_cast<float>(log2(v)) : -1.0e30f;
  const float hmax = fmaxf(gboxf[8ull * g + 3], fmaxf(gboxf[8ull * g + 4], gboxf[8ull * g + 5]));
  gtol[g] = make_float2(group_feature(hmax, fs), tau);
}

__global__ void __launch_bounds__(kT)
    k_record_amag(const float4 *out, const u32 *order, u64 n, float *amag) {
  const u64 t = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  if (t >= n) return;
  const float4 o = out[t];
  amag[order[t]] = sqrtf(o.x * o.x + o.y * o.y + o.z * o.z);
}

__device__ __forceinline__ WalkRec32 load_rec(const WalkRec32 *w, u32 i) {
  const float4 *p = reinterpret_cast<const float4 *>(w + i);
  const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  WalkRec32 r;
  r.cx = a.x;
  r.cy = a.y;
  r.cz = a.z;
  r.slack = a.w;
  r.mx = b.x;
  r.my = b.y;
  r.mz = b.z;
  r.crit2 = b.w;
  r.skip = __float_as_uint(c.x);
  r.nbody_leaf = __float_as_uint(c.y);
  r.begin = __float_as_uint(c.z);
  r.bound = c.w;
  return r;
}

// The learned walk runs in rounds over items, (group, node) pairs: walk the
// subtree under the node for the group. Round 0's items split each group's
// walk along the group's own path from the root: for the path's first
// `split` levels, every sibling of the path node is an item, and the node
// the path reaches is the last (the group's near field, its longest walk;
// it is stored first). Only nodes that hold the group are opened for it on
// the way down, as the walk itself would, so the decisions are the unsplit
// walk's. A walk decides what the guard and the prior settle and defers the
// rest, the (group, cell) pairs whose centred prior lies within the band of
// the group's tolerance, skipping their subtrees. A dense kernel then runs
// the network on all deferred pairs at once, 32 rows per warp on the tensor
// cores, and the next round's items are those pairs with the network's
// decision: accept the cell, or walk its children (deferring again). The
// walk kernel itself carries no network and few registers, so many warps
// hide its memory latency, and the network's latency is off its path.
//
// Each lane appends what its items produce to its own region: accepted
// cells, runs of bodies (first, count) and deferred nodes. A gather pass
// concatenates a group's items in (round, item) order into the group's
// lists. Items are stored grouped by group in every round (a round's
// deferred pairs keep their items' order), with each group's range kept
// per round.
constexpr u64 kNoItem = ~0ull;
constexpr int kGrabLanes = 8;
constexpr int kMaxRounds = kMaxDepth + 4;

struct LArgs {
  const WalkRec32 *walk32;
  const CellFeat *cfeat;
  const LWalkRec *lrec;
  const float *gboxf;
  const float2 *gtol;
  u32 ng;
  u64 nitems;              // items of this round
  u64 item_base;           // global index of the round's first item
  const uint2 *qitems;     // (group, node) of each item
  const u8 *qdec;          // rounds > 0: the network's decision on the node (1: accept)
  const TreeRoot *root;
  const double2 *mom;
  float inv_theta_guard, band, y_mean;
  u32 lane_cells, lane_runs, lane_pend;  // capacity of each lane's regions
  u32 *reg_cells;
  uint2 *reg_runs;
  u32 *reg_pend;
  u32 *lane_fill;          // per lane: cells, runs, deferred used so far
  uint4 *seg;              // per item: first cell, cells, first run, runs (region indices)
  uint4 *seg2;             // per item: first deferred, deferred, bodies, 0
  u32 *pcount;             // per item of the round (storage order): deferred
  unsigned long long *gcells, *gbodies;  // per group: list entries of all its items
  Scalars *sc;
};

__global__ void __launch_bounds__(kT, 5) k_lwalk(LArgs a) {
  const int lane = threadIdx.x & 31;
  const FeatScale fs = scale_of(a.root, a.mom);
  const u64 gtid = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  u32 lc = a.lane_fill[3 * gtid], lr = a.lane_fill[3 * gtid + 1], lp = a.lane_fill[3 * gtid + 2];
  u32 *reg_c = a.reg_cells + gtid * a.lane_cells;
  uint2 *reg_r = a.reg_runs + gtid * a.lane_runs;
  u32 *reg_p = a.reg_pend + gtid * a.lane_pend;
  Scalars *sc = a.sc;

  u64 item = kNoItem, store = 0;
  u32 i = 0, end = 0, c0i = 0, r0i = 0, p0i = 0, nb = 0, grp = 0, visits = 0;
  int pre = -1;  // the network's decision on a deferred item's node
  bool exhausted = false;
  float gf[3] = {0.f, 0.f, 0.f}, hf[3] = {0.f, 0.f, 0.f};
  float acc_d2 = 0.f, open_d2 = 0.f;  // the item's group: d^2 scales of the accept and open tests
  const float l2 = 1.f / (fs.inv_l * fs.inv_l);
  while (true) {
    // idle lanes take the next items (one atomic per warp), once at least
    // kGrabLanes of them wait or no lane has work: the grab runs with its
    // lanes together instead of for one or two lanes every step
    const bool want = item == kNoItem && !exhausted;
    const unsigned wantm = __ballot_sync(kFullMask, want);
    const unsigned busym = __ballot_sync(kFullMask, item != kNoItem);
    if (wantm && (__popc(wantm) >= kGrabLanes || busym == 0)) {
      const int leader = __ffs(wantm) - 1;
      unsigned long long base = 0;
      if (lane == leader)
        base = atomicAdd(&sc->walk_items, static_cast<unsigned long long>(__popc(wantm)));
      base = __shfl_sync(kFullMask, base, leader);
      if (want) {
        const u64 k = base + __popc(wantm & ((1u << lane) - 1u));
        if (k >= a.nitems) {
          exhausted = true;
        } else {
          item = k;
          u32 &g = grp;
          const uint2 q = a.qitems[k];
          g = q.x;
          i = q.y;
          store = k;
          pre = a.qdec ? a.qdec[k] : -1;
          end = __float_as_uint(__ldg(reinterpret_cast<const float4 *>(a.lrec + i) + 2).x);
          const float4 b0 = reinterpret_cast<const float4 *>(a.gboxf)[2ull * g],
                       b1 = reinterpret_cast<const float4 *>(a.gboxf)[2ull * g + 1];
          gf[0] = b0.x;
          gf[1] = b0.y;
          gf[2] = b0.z;
          hf[0] = b0.w;
          hf[1] = b1.x;
          hf[2] = b1.y;
          const float tau = a.gtol[g].y;
          acc_d2 = exp2f(0.4f * (a.band - tau)) * l2;
          open_d2 = exp2f(0.4f * (-a.band - tau)) * l2;
          c0i = lc;
          r0i = lr;
          p0i = lp;
          nb = 0;
        }
      }
    }
    if (__ballot_sync(kFullMask, item != kNoItem) == 0) break;
    if (item == kNoItem) continue;  // the lanes meet again at the next ballot

    const float4 *rp = reinterpret_cast<const float4 *>(a.lrec + i);
    const float4 ra = __ldg(rp), rb = __ldg(rp + 1), rc = __ldg(rp + 2);
    LWalkRec r;
    r.cx = ra.x;
    r.cy = ra.y;
    r.cz = ra.z;
    r.slack = ra.w;
    r.mx = rb.x;
    r.my = rb.y;
    r.mz = rb.z;
    r.guard2 = rb.w;
    r.skip = __float_as_uint(rc.x);
    r.nbody_leaf = __float_as_uint(rc.y);
    r.begin = __float_as_uint(rc.z);
    r.pscale = rc.w;
    ++visits;
    const u32 nbody = r.nbody_leaf & 0x7fffffffu;
    int verdict;  // 0 open, 1 accept, 2 defer
    if (pre >= 0) {
      verdict = pre;
      pre = -1;
    } else {
      // the reference's overlap test (group_lists.cpp:147), in FP32
      const bool overlap = fabsf(r.cx - gf[0]) <= r.slack + hf[0] &&
                           fabsf(r.cy - gf[1]) <= r.slack + hf[1] &&
                           fabsf(r.cz - gf[2]) <= r.slack + hf[2];
      const float dx = fmaxf(fabsf(r.mx - gf[0]) - hf[0], 0.f),
                  dy = fmaxf(fabsf(r.my - gf[1]) - hf[1], 0.f),
                  dz = fmaxf(fabsf(r.mz - gf[2]) - hf[2], 0.f);
      const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      if (overlap || !(d2 > r.guard2)) {
        verdict = 0;
      } else if (nbody <= kFewBodies) {
        verdict = 1;
      } else {
        verdict = d2 > r.pscale * acc_d2 ? 1 : d2 < r.pscale * open_d2 ? 0 : 2;
      }
    }
    if (verdict == 2) {
      if (lp < a.lane_pend) reg_p[lp] = i;
      ++lp;
    } else if (verdict == 1 && nbody > kFewBodies) {
      if (lc < a.lane_cells) reg_c[lc] = i;
      ++lc;
    } else if (verdict == 1 || (r.nbody_leaf >> 31)) {
      if (lr < a.lane_runs) reg_r[lr] = make_uint2(r.begin, nbody);
      ++lr;
      nb += nbody;
    }
    if (verdict != 0 || (r.nbody_leaf >> 31)) {
      if (r.skip <= i) {  // malformed tree: never loop
        atomicOr(&sc->error, 1u);
        i = end;
      } else {
        i = r.skip;
      }
    } else {
      ++i;
    }
    if (i >= end) {  // the item is done
      const u64 gi = a.item_base + store;
      a.seg[gi] = make_uint4(static_cast<u32>(gtid * a.lane_cells + c0i), lc - c0i,
                             static_cast<u32>(gtid * a.lane_runs + r0i), lr - r0i);
      a.seg2[gi] = make_uint4(static_cast<u32>(gtid * a.lane_pend + p0i), lp - p0i, nb, 0u);
      a.pcount[store] = lp - p0i;
      if (lc > c0i) atomicAdd(&a.gcells[grp], static_cast<unsigned long long>(lc - c0i));
      if (nb) atomicAdd(&a.gbodies[grp], static_cast<unsigned long long>(nb));
      item = kNoItem;
    }
  }
  warp_add(&sc->walk_nodes, visits);  // the lanes leave the loop together
  a.lane_fill[3 * gtid] = lc;
  a.lane_fill[3 * gtid + 1] = lr;
  a.lane_fill[3 * gtid + 2] = lp;
  if (lc > a.lane_cells || lr > a.lane_runs || lp > a.lane_pend) atomicOr(&sc->list_overflow, 1u);
}

// Round 0's items of each group (kFill = false: their count): the siblings
// of the group's path nodes down `split` levels, after the node the path
// reaches. A path stops early at a leaf or where the group's targets span
// more than one child.
constexpr int kMaxSplit = 8;

template <bool kFill>
__global__ void __launch_bounds__(kT)
    k_path_items(const u32 *gbegin, const u32 *gend, u32 ng, const u32 *skip, const u32 *nbegin,
                 const u32 *nend, const u8 *isleaf, int split, u32 *count, const u32 *offset,
                 uint2 *items) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (g >= ng) return;
  const u32 b0 = gbegin[g], b1 = gend[g];
  u32 path[kMaxSplit + 1];
  int depth = 0;
  u32 p = 0;
  path[0] = 0;
  while (depth < split && !isleaf[p]) {
    u32 next = 0xffffffffu;
    for (u32 c = p + 1; c < skip[p]; c = skip[c])
      if (nbegin[c] <= b0 && b1 <= nend[c]) next = c;
    if (next == 0xffffffffu) break;
    p = next;
    path[++depth] = p;
  }
  if (!kFill) {
    u32 n = 1;
    for (int d = 0; d < depth; ++d)
      for (u32 c = path[d] + 1; c < skip[path[d]]; c = skip[c]) n += c != path[d + 1];
    count[g] = n;
    return;
  }
  u64 o = offset[g];
  items[o++] = make_uint2(g, p);  // the near field first
  for (int d = 0; d < depth; ++d)
    for (u32 c = path[d] + 1; c < skip[path[d]]; c = skip[c])
      if (c != path[d + 1]) items[o++] = make_uint2(g, c);
}

// Start of every group's deferred pairs in the next round's item order,
// from the exclusive scan of the deferred counts and the starts of the
// groups' items in this round.
__global__ void __launch_bounds__(kT)
    k_lgstart(u32 ng, const u32 *poff, const u32 *cur, u32 *next) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (g > ng) return;
  next[g] = poff[cur[g]];
}

// The deferred pairs of a round, in storage order, as the next round's items.
__global__ void __launch_bounds__(kT)
    k_lcompact(u64 nitems, u64 item_base, const uint2 *qitems, const uint4 *seg2,
               const u32 *poff, const u32 *reg_pend, uint2 *next) {
  const u64 j = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  if (j >= nitems) return;
  const uint4 s2 = seg2[item_base + j];
  if (s2.y == 0) return;
  const u32 g = qitems[j].x;
  const u32 o = poff[j];
  for (u32 m = 0; m < s2.y; ++m) next[o + m] = make_uint2(g, reg_pend[s2.x + m]);
}

// The network's decision on every deferred pair: one warp per 32 pairs.
__global__ void __launch_bounds__(kT)
    k_ldecide(const uint2 *q, u64 nq, const WalkRec32 *walk32, const CellFeat *cfeat,
              const float *gboxf, const float2 *gtol, const LearnedNet *net, const TreeRoot *root,
              const double2 *mom, u8 *dec) {
  __shared__ NetShared sn;
  __shared__ uint4 rows[kT / 32][32];
  load_net(net, sn);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const u64 k = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  float thr = 0.f;
  uint4 row = make_uint4(0u, 0u, 0u, 0u);
  if (k < nq) {
    const FeatScale fs = scale_of(root, mom);
    const uint2 qk = q[k];
    const u32 g = qk.x, p = qk.y;
    const float4 b0 = reinterpret_cast<const float4 *>(gboxf)[2ull * g],
                 b1 = reinterpret_cast<const float4 *>(gboxf)[2ull * g + 1];
    const WalkRec32 r = load_rec(walk32, p);
    const float4 c0 = __ldg(reinterpret_cast<const float4 *>(cfeat + p));
    const float4 c1 = __ldg(reinterpret_cast<const float4 *>(cfeat + p) + 1);
    const float dx = fmaxf(fabsf(r.mx - b0.x) - b0.w, 0.f),
                dy = fmaxf(fabsf(r.my - b0.y) - b1.x, 0.f),
                dz = fmaxf(fabsf(r.mz - b0.z) - b1.y, 0.f);
    const float f2 = distance_feature(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), fs);
    const float2 gt = gtol[g];
    const float e = prior_log2err(c0.z, f2) + net->y_mean;
    thr = (gt.y - e) / net->y_std;
    const float f[kFeat] = {gt.x, c0.w, f2, c1.x, c1.y, c1.z};
    row = feature_row(f, sn);
  }
  rows[warp][lane] = row;
  __syncwarp();
  const float y = warp_mlp(rows[warp], sn.w1, sn.w2, sn.b2, sn.w3, net->b3, lane);
  if (k < nq) dec[k] = y < thr ? 1 : 0;
}

struct RoundView {
  const u64 *base;         // per round: global index of its first item
  const u32 *gstart;       // per round: [ng + 1] starts of the groups' items
  u32 rounds, ng;
};

// Copies one item's cells and body runs to the group's lists at (oc, ob),
// all lanes of the warp together.
__device__ __forceinline__ void copy_item_warp(const uint4 &sg, const u32 *reg_cells,
                                               const uint2 *reg_runs, u32 *cell_list,
                                               u32 *body_list, u64 oc, u64 ob, int lane) {
  for (u32 k = lane; k < sg.y; k += 32) cell_list[oc + k] = reg_cells[sg.x + k];
  for (u32 k0 = 0; k0 < sg.w; k0 += 32) {
    const u32 k = k0 + lane;
    const uint2 run = k < sg.w ? reg_runs[sg.z + k] : make_uint2(0u, 0u);
    u32 incl = run.y;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 v = __shfl_up_sync(kFullMask, incl, o);
      if (lane >= o) incl += v;
    }
    const u64 start = ob + incl - run.y;
    for (u32 j = 0; j < run.y; ++j) body_list[start + j] = run.x + j;
    ob += __shfl_sync(kFullMask, incl, 31);
  }
}

__device__ __forceinline__ u32 warp_exclusive_scan(u32 v, int lane) {
  u32 incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const u32 x = __shfl_up_sync(kFullMask, incl, o);
    if (lane >= o) incl += x;
  }
  return incl - v;
}

constexpr u32 kSmallItem = 8;  // items with at most this many cells and runs copy by lane

// One warp per group: its items' lists in (round, item) order into the
// group's ranges of cell_list and body_list, its GTGroup record and the
// list counters. Each batch of 32 items gets its output offsets from warp
// scans; small items (most deferred ones: one cell, or a leaf's run) are
// copied by their own lane, large ones by the whole warp.
constexpr int kGatherWarps = kT / 32;

__global__ void __launch_bounds__(kT)
    k_lgather(const uint4 *seg, const uint4 *seg2, RoundView rv, const u32 *reg_cells,
              const uint2 *reg_runs, const u32 *gbegin, const u32 *gend, const u64 *cell_off,
              const u64 *body_off, u32 *cell_list, u32 *body_list, uint4 *groups, Scalars *sc) {
  const u32 g = blockIdx.x * kGatherWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (g >= rv.ng) return;
  u64 oc = cell_off[g], ob = body_off[g];
  if (lane == 0) {
    store_group_rec(groups, g, gbegin[g], gend[g], one_segment(oc, cell_off[g + 1] - oc),
                    one_segment(ob, body_off[g + 1] - ob));
  }
  for (u32 r = 0; r < rv.rounds; ++r) {
    const u32 *st = rv.gstart + static_cast<u64>(r) * (rv.ng + 1);
    const u64 first = rv.base[r] + st[g], count = st[g + 1] - st[g];
    for (u64 j0 = 0; j0 < count; j0 += 32) {
      const u64 j = j0 + lane;
      const bool have = j < count;
      const uint4 sg = have ? seg[first + j] : make_uint4(0u, 0u, 0u, 0u);
      const u32 nbj = have ? seg2[first + j].z : 0u;
      const u32 cs = warp_exclusive_scan(sg.y, lane), bs = warp_exclusive_scan(nbj, lane);
      const bool small = sg.y <= kSmallItem && sg.w <= kSmallItem;
      if (small) {
        for (u32 k = 0; k < sg.y; ++k) cell_list[oc + cs + k] = reg_cells[sg.x + k];
        u64 o = ob + bs;
        for (u32 k = 0; k < sg.w; ++k) {
          const uint2 run = reg_runs[sg.z + k];
          for (u32 q = 0; q < run.y; ++q) body_list[o + q] = run.x + q;
          o += run.y;
        }
      }
      unsigned big = __ballot_sync(kFullMask, !small);
      while (big) {
        const int src = __ffs(big) - 1;
        big &= big - 1u;
        const uint4 s4 = make_uint4(__shfl_sync(kFullMask, sg.x, src),
                                    __shfl_sync(kFullMask, sg.y, src),
                                    __shfl_sync(kFullMask, sg.z, src),
                                    __shfl_sync(kFullMask, sg.w, src));
        const u32 c_at = __shfl_sync(kFullMask, cs, src), b_at = __shfl_sync(kFullMask, bs, src);
        copy_item_warp(s4, reg_cells, reg_runs, cell_list, body_list, oc + c_at, ob + b_at, lane);
      }
      oc += __shfl_sync(kFullMask, cs + sg.y, 31);
      ob += __shfl_sync(kFullMask, bs + nbj, 31);
    }
  }
}

// The groups' list statistics, one group per lane.
__global__ void __launch_bounds__(kT)
    k_list_stats(const u32 *gbegin, const u32 *gend, const u64 *cell_off, const u64 *body_off,
                 u32 ng, Scalars *sc) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  const bool valid = g < ng;
  u64 t = 0, nc = 0, nb = 0;
  if (valid) {
    t = gend[g] - gbegin[g];
    nc = cell_off[g + 1] - cell_off[g];
    nb = body_off[g + 1] - body_off[g];
  }
  group_stats_warp(sc, valid, t, nc, nb, false);
}

// The walk's inference on given raw features (tests and diagnostics).
__global__ void __launch_bounds__(kT)
    k_predict(const LearnedNet *net, const float *feat, u64 n, float *pred) {
  __shared__ NetShared sn;
  __shared__ uint4 rows[kT / 32][32];
  load_net(net, sn);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  const u64 k = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  float f[kFeat] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (k < n)
    for (int j = 0; j < kFeat; ++j) f[j] = feat[k * kFeat + j];
  rows[warp][lane] = feature_row(f, sn);
  __syncwarp();
  const float y = warp_mlp(rows[warp], sn.w1, sn.w2, sn.b2, sn.w3, net->b3, lane);
  if (k < n) {
    const float prior = kPriorBase + f[3] + 3.f * f[1];
    pred[k] = prior_log2err(prior, f[2]) + net->y_mean + net->y_std * y;
  }
}

}  // namespace

void learned_prepare_net(const float *model, LearnedNet *net, cudaStream_t s) {
  k_prepare_net<<<4, kT, 0, s>>>(model, net);
  GTC_LAUNCH_CHECK();
}

void learned_predict(const LearnedNet *net, const float *feat, u64 n, float *pred,
                     cudaStream_t s) {
  if (n == 0) return;
  k_predict<<<ceil_div(n, kT), kT, 0, s>>>(net, feat, n, pred);
  GTC_LAUNCH_CHECK();
}

void learned_node_features(Workspace &ws, DeviceBuffer &cfeat, cudaStream_t s) {
  const u32 m = static_cast<u32>(ws.n_nodes);
  if (m == 0) return;
  cfeat.ensure(static_cast<u64>(m) * sizeof(CellFeat));
  k_cell_feat<<<ceil_div(m, kT), kT, 0, s>>>(ws.geom.as<double2>(), ws.mom.as<double2>(),
                                             ws.quad.as<double2>(), ws.delta.as<double>(),
                                             ws.root.as<TreeRoot>(), m, cfeat.as<CellFeat>());
  GTC_LAUNCH_CHECK();
}

void learned_walk_records(Workspace &ws, const CellFeat *cfeat, DeviceBuffer &lrec,
                          float inv_theta_guard, float y_mean, cudaStream_t s) {
  const u32 m = static_cast<u32>(ws.n_nodes);
  if (m == 0) return;
  lrec.ensure(static_cast<u64>(m) * sizeof(LWalkRec));
  k_lwalk_rec<<<ceil_div(m, kT), kT, 0, s>>>(ws.walk32.as<WalkRec32>(), cfeat, m, inv_theta_guard,
                                             y_mean, lrec.as<LWalkRec>());
  GTC_LAUNCH_CHECK();
}

void learned_group_tolerances(Workspace &ws, const LearnedWalk &lw, u32 ng, cudaStream_t s) {
  if (ng == 0) return;
  lw.gtol->ensure(static_cast<u64>(ng) * sizeof(float2));
  k_group_tol<<<ceil_div(ng, kT), kT, 0, s>>>(
      ws.gbegin.as<u32>(), ws.gend.as<u32>(), ng, ws.idx.as<u32>(), lw.prev_amag,
      ws.gboxf.as<float>(), ws.root.as<TreeRoot>(), ws.mom.as<double2>(), lw.alpha, lw.G,
      lw.gtol->as<float2>());
  GTC_LAUNCH_CHECK();
}

void learned_build_lists(Workspace &ws, const LearnedWalk &lw, u32 ng, Scalars *host,
                         cudaStream_t s) {
  if (ng == 0) return;
  Scalars *sc = ws.scalars.as<Scalars>();
  int dev = 0, sms = 0, per_sm = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lwalk, kT, 0));
  const u32 blocks = static_cast<u32>(std::max(1, sms * std::max(1, per_sm)));
  const u64 lanes = static_cast<u64>(blocks) * kT;
  LearnedScratch &ls = *lw.scratch;
  const int split = std::min(std::max(lw.split_depth, 0), kMaxSplit);
  ws.gcells.ensure(static_cast<u64>(ng) * 8);
  ws.gbodies.ensure(static_cast<u64>(ng) * 8);
  ws.gcell_off.ensure((static_cast<u64>(ng) + 1) * 8);
  ws.gbody_off.ensure((static_cast<u64>(ng) + 1) * 8);
  ls.gstart.ensure(static_cast<u64>(kMaxRounds + 1) * (ng + 1) * sizeof(u32));
  ls.lane_fill.ensure(lanes * 3 * sizeof(u32));
  LArgs a{};
  a.walk32 = ws.walk32.as<WalkRec32>();
  a.cfeat = lw.cfeat;
  a.lrec = ls.lrec.as<LWalkRec>();
  a.gboxf = ws.gboxf.as<float>();
  a.gtol = lw.gtol->as<float2>();
  a.ng = ng;
  a.root = ws.root.as<TreeRoot>();
  a.mom = ws.mom.as<double2>();
  a.inv_theta_guard = lw.inv_theta_guard;
  a.band = lw.band;
  a.y_mean = lw.y_mean;
  a.lane_fill = ls.lane_fill.as<u32>();
  a.gcells = reinterpret_cast<unsigned long long *>(ws.gcells.as<u64>());
  a.gbodies = reinterpret_cast<unsigned long long *>(ws.gbodies.as<u64>());
  a.sc = sc;
  std::vector<u64> base;
  for (int attempt = 0;; ++attempt) {
    // lane regions (grown and walked again if one overflows)
    const u64 reg_bytes = lanes * (static_cast<u64>(ls.lane_cells) * 4 +
                                   static_cast<u64>(ls.lane_runs) * 8 +
                                   static_cast<u64>(ls.lane_pend) * 4);
    ls.regions.ensure(reg_bytes);
    char *rb = ls.regions.as<char>();
    a.reg_runs = reinterpret_cast<uint2 *>(rb);
    a.reg_cells = reinterpret_cast<u32 *>(rb + lanes * static_cast<u64>(ls.lane_runs) * 8);
    a.reg_pend = a.reg_cells + lanes * static_cast<u64>(ls.lane_cells);
    a.lane_cells = ls.lane_cells;
    a.lane_runs = ls.lane_runs;
    a.lane_pend = ls.lane_pend;
    GTC_CUDA(cudaMemsetAsync(a.lane_fill, 0, lanes * 3 * sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(ws.gcells.ptr, 0, static_cast<u64>(ng) * 8, s));
    GTC_CUDA(cudaMemsetAsync(ws.gbodies.ptr, 0, static_cast<u64>(ng) * 8, s));
    GTC_CUDA(cudaMemsetAsync(&sc->cell_interactions, 0, 3 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_group, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(&sc->mlp_rows, 0, 2 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->list_overflow, 0, sizeof(u32), s));
    // round 0's items: each group's path split
    u32 *st0 = ls.gstart.as<u32>();
    ls.pcount.ensure((static_cast<u64>(ng) + 1) * sizeof(u32));
    k_path_items<false><<<ceil_div(ng, kT), kT, 0, s>>>(
        ws.gbegin.as<u32>(), ws.gend.as<u32>(), ng, ws.skip.as<u32>(), ws.nbegin.as<u32>(),
        ws.nend.as<u32>(), ws.isleaf.as<u8>(), split, ls.pcount.as<u32>(), nullptr, nullptr);
    GTC_LAUNCH_CHECK();
    exclusive_scan_u32(ls.pcount.as<u32>(), st0, ng, st0 + ng, ws.scan_tmp, s);
    u32 n0 = 0;
    GTC_CUDA(cudaMemcpyAsync(&n0, st0 + ng, sizeof(u32), cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    ls.q[0].ensure(static_cast<u64>(n0) * sizeof(uint2));
    k_path_items<true><<<ceil_div(ng, kT), kT, 0, s>>>(
        ws.gbegin.as<u32>(), ws.gend.as<u32>(), ng, ws.skip.as<u32>(), ws.nbegin.as<u32>(),
        ws.nend.as<u32>(), ws.isleaf.as<u8>(), split, nullptr, st0, ls.q[0].as<uint2>());
    GTC_LAUNCH_CHECK();
    base.assign(1, 0);
    u64 nitems = n0, total_items = 0, rows = 0, batches = 0;
    int qsel = 0;
    bool overflow = false;
    for (u32 round = 0;; ++round) {
      if (round >= static_cast<u32>(kMaxRounds))
        throw RuntimeError("learned walk: more rounds than the tree has levels");
      const u64 need = base.back() + nitems;
      if (need > ls.items_cap) {  // grow the item arrays, keeping what is there
        const u64 cap = std::max<u64>(need + need / 2, static_cast<u64>(n0) + 4ull * ng);
        DeviceBuffer nseg;
        nseg.ensure(cap * 2 * sizeof(uint4));
        if (ls.items_cap && base.back())
          for (int h = 0; h < 2; ++h)
            GTC_CUDA(cudaMemcpyAsync(nseg.as<uint4>() + h * cap, ls.seg.as<uint4>() + h * ls.items_cap,
                                     base.back() * sizeof(uint4), cudaMemcpyDeviceToDevice, s));
        GTC_CUDA(cudaStreamSynchronize(s));
        ls.seg.release();
        ls.seg = nseg;
        ls.items_cap = cap;
      }
      a.seg = ls.seg.as<uint4>();
      a.seg2 = a.seg + ls.items_cap;
      ls.pcount.ensure((nitems + 1) * sizeof(u32));
      ls.poff.ensure((nitems + 1) * sizeof(u32));
      a.pcount = ls.pcount.as<u32>();
      a.nitems = nitems;
      a.item_base = base.back();
      a.qitems = ls.q[qsel].as<uint2>();
      a.qdec = round ? ls.dec[qsel].as<u8>() : nullptr;
      GTC_CUDA(cudaMemsetAsync(&sc->walk_items, 0, sizeof(unsigned long long), s));
      k_lwalk<<<blocks, kT, 0, s>>>(a);
      GTC_LAUNCH_CHECK();
      u32 *poff = ls.poff.as<u32>();
      exclusive_scan_u32(a.pcount, poff, nitems, poff + nitems, ws.scan_tmp, s);
      u32 *cur = ls.gstart.as<u32>() + static_cast<u64>(round) * (ng + 1);
      k_lgstart<<<ceil_div(ng + 1, kT), kT, 0, s>>>(ng, poff, cur, cur + (ng + 1));
      GTC_LAUNCH_CHECK();
      u32 deferred = 0, flags[2] = {0, 0};
      GTC_CUDA(cudaMemcpyAsync(&deferred, poff + nitems, sizeof(u32), cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaMemcpyAsync(flags, &sc->list_overflow, sizeof(u32), cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaMemcpyAsync(flags + 1, &sc->error, sizeof(u32), cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaStreamSynchronize(s));
      total_items = base.back() + nitems;
      if (flags[1])
        throw RuntimeError("cuda: inconsistent tree detected on the device (code " +
                           std::to_string(flags[1]) + ")");
      if (flags[0]) {
        overflow = true;
        break;
      }
      if (deferred == 0) break;
      // the deferred pairs become the next round's items, with the network's decisions
      const int nq = qsel ^ 1;
      ls.q[nq].ensure(static_cast<u64>(deferred) * sizeof(uint2));
      ls.dec[nq].ensure(deferred);
      k_lcompact<<<ceil_div(nitems, kT), kT, 0, s>>>(nitems, base.back(), a.qitems, a.seg2, poff,
                                                    a.reg_pend, ls.q[nq].as<uint2>());
      GTC_LAUNCH_CHECK();
      k_ldecide<<<ceil_div(deferred, kT), kT, 0, s>>>(
          ls.q[nq].as<uint2>(), deferred, a.walk32, a.cfeat, a.gboxf, a.gtol, lw.net, a.root,
          a.mom, ls.dec[nq].as<u8>());
      GTC_LAUNCH_CHECK();
      rows += deferred;
      batches += (deferred + 31) / 32;
      qsel = nq;
      base.push_back(total_items);
      nitems = deferred;
    }
    if (!overflow) {
      host->mlp_rows = rows;
      host->mlp_batches = batches;
      ws.list_passes = static_cast<u32>(base.size());
      break;
    }
    if (attempt >= 4 || lanes * static_cast<u64>(ls.lane_cells) * 2 > 0xffffffffull ||
        lanes * static_cast<u64>(ls.lane_runs) * 2 > 0xffffffffull ||
        lanes * static_cast<u64>(ls.lane_pend) * 2 > 0xffffffffull)
      throw RuntimeError("learned walk: the lane regions keep overflowing");
    ls.lane_cells *= 2;
    ls.lane_runs *= 2;
    ls.lane_pend *= 2;
  }
  const u32 rounds = static_cast<u32>(base.size());
  ls.base.ensure(rounds * sizeof(u64));
  GTC_CUDA(cudaMemcpyAsync(ls.base.ptr, base.data(), rounds * sizeof(u64), cudaMemcpyHostToDevice, s));
  GTC_CUDA(cudaMemcpyAsync(&sc->mlp_rows, &host->mlp_rows, 2 * sizeof(unsigned long long),
                           cudaMemcpyHostToDevice, s));
  const RoundView rv{ls.base.as<u64>(), ls.gstart.as<u32>(), rounds, ng};
  u64 *cell_off = ws.gcell_off.as<u64>(), *body_off = ws.gbody_off.as<u64>();
  exclusive_scan_u64(ws.gcells.as<u64>(), cell_off, ng, cell_off + ng, ws.scan_tmp, s);
  exclusive_scan_u64(ws.gbodies.as<u64>(), body_off, ng, body_off + ng, ws.scan_tmp, s);
  GTC_CUDA(cudaMemcpyAsync(&sc->n_cell_list, cell_off + ng, 8, cudaMemcpyDeviceToDevice, s));
  GTC_CUDA(cudaMemcpyAsync(&sc->n_body_list, body_off + ng, 8, cudaMemcpyDeviceToDevice, s));
  u64 totals[2] = {0, 0};
  GTC_CUDA(cudaMemcpyAsync(totals, &sc->n_cell_list, sizeof(totals), cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
  if (totals[0] > 0xffffffffull || totals[1] > 0xffffffffull)
    throw RuntimeError("interaction lists too long for 32 bit offsets");
  ws.n_cell_list = totals[0];
  ws.n_body_list = totals[1];
  host->n_cell_list = totals[0];
  host->n_body_list = totals[1];
  ws.cell_list.ensure(std::max<u64>(1, ws.n_cell_list) * 4);
  ws.body_list.ensure(std::max<u64>(1, ws.n_body_list) * 4);
  k_lgather<<<ceil_div(ng, kGatherWarps), kT, 0, s>>>(
      a.seg, a.seg2, rv, a.reg_cells, a.reg_runs, ws.gbegin.as<u32>(), ws.gend.as<u32>(),
      cell_off, body_off, ws.cell_list.as<u32>(), ws.body_list.as<u32>(), ws.groups.as<uint4>(),
      sc);
  GTC_LAUNCH_CHECK();
  k_list_stats<<<ceil_div(ng, kT), kT, 0, s>>>(ws.gbegin.as<u32>(), ws.gend.as<u32>(), cell_off,
                                               body_off, ng, sc);
  GTC_LAUNCH_CHECK();
}


void learned_record_amag(const float4 *out, const u32 *order, u64 n, float *amag,
                         cudaStream_t s) {
  if (n == 0) return;
  k_record_amag<<<ceil_div(n, kT), kT, 0, s>>>(out, order, n, amag);
  GTC_LAUNCH_CHECK();
}

}  // namespace gtc
