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
// tiles go through the layers together: each B fragment is loaded once for
// both, and the two accumulator chains interleave.
__device__ __forceinline__ float warp_mlp(const uint4 *rows, const u32 (&w1)[8], const uint2 *w2,
                                          const float *b2, const float *w3, float b3, int lane) {
  const int g = lane >> 2, t = lane & 3;
  const u32 a00 = reinterpret_cast<const u32 *>(&rows[g])[t];
  const u32 a01 = reinterpret_cast<const u32 *>(&rows[g + 8])[t];
  const u32 a10 = reinterpret_cast<const u32 *>(&rows[16 + g])[t];
  const u32 a11 = reinterpret_cast<const u32 *>(&rows[24 + g])[t];
  u32 A0[4][4], A1[4][4];
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    float c0[4] = {0.f, 0.f, 0.f, 0.f}, e0[4] = {0.f, 0.f, 0.f, 0.f};
    float c1[4] = {0.f, 0.f, 0.f, 0.f}, e1[4] = {0.f, 0.f, 0.f, 0.f};
    mma_bf16(c0, a00, a01, 0u, 0u, w1[j], 0u);
    mma_bf16(c1, a10, a11, 0u, 0u, w1[j], 0u);
    mma_bf16(e0, a00, a01, 0u, 0u, w1[j + 1], 0u);
    mma_bf16(e1, a10, a11, 0u, 0u, w1[j + 1], 0u);
    A0[j / 2][0] = pack_bf16(fmaxf(c0[0], 0.f), fmaxf(c0[1], 0.f));
    A0[j / 2][1] = pack_bf16(fmaxf(c0[2], 0.f), fmaxf(c0[3], 0.f));
    A0[j / 2][2] = pack_bf16(fmaxf(e0[0], 0.f), fmaxf(e0[1], 0.f));
    A0[j / 2][3] = pack_bf16(fmaxf(e0[2], 0.f), fmaxf(e0[3], 0.f));
    A1[j / 2][0] = pack_bf16(fmaxf(c1[0], 0.f), fmaxf(c1[1], 0.f));
    A1[j / 2][1] = pack_bf16(fmaxf(c1[2], 0.f), fmaxf(c1[3], 0.f));
    A1[j / 2][2] = pack_bf16(fmaxf(e1[0], 0.f), fmaxf(e1[1], 0.f));
    A1[j / 2][3] = pack_bf16(fmaxf(e1[2], 0.f), fmaxf(e1[3], 0.f));
  }
  float s00 = 0.f, s01 = 0.f, s10 = 0.f, s11 = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float2 bb = *reinterpret_cast<const float2 *>(&b2[8 * j + 2 * t]);
    float c0[4] = {bb.x, bb.y, bb.x, bb.y}, c1[4] = {bb.x, bb.y, bb.x, bb.y};
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const uint2 b = w2[(kk * 8 + j) * 32 + lane];
      mma_bf16(c0, A0[kk][0], A0[kk][1], A0[kk][2], A0[kk][3], b.x, b.y);
      mma_bf16(c1, A1[kk][0], A1[kk][1], A1[kk][2], A1[kk][3], b.x, b.y);
    }
    const float2 w = *reinterpret_cast<const float2 *>(&w3[8 * j + 2 * t]);
    s00 = fmaf(fmaxf(c0[0], 0.f), w.x, fmaf(fmaxf(c0[1], 0.f), w.y, s00));
    s01 = fmaf(fmaxf(c0[2], 0.f), w.x, fmaf(fmaxf(c0[3], 0.f), w.y, s01));
    s10 = fmaf(fmaxf(c1[0], 0.f), w.x, fmaf(fmaxf(c1[1], 0.f), w.y, s10));
    s11 = fmaf(fmaxf(c1[2], 0.f), w.x, fmaf(fmaxf(c1[3], 0.f), w.y, s11));
  }
#pragma unroll
  for (int o = 1; o <= 2; o <<= 1) {
    s00 += __shfl_xor_sync(kFullMask, s00, o);
    s01 += __shfl_xor_sync(kFullMask, s01, o);
    s10 += __shfl_xor_sync(kFullMask, s10, o);
    s11 += __shfl_xor_sync(kFullMask, s11, o);
  }
  // quad q holds rows q, q + 8, 16 + q, 24 + q; row L is in quad L % 8
  const int src = (lane & 7) << 2, h = lane >> 3;
  const float v0 = __shfl_sync(kFullMask, s00, src), v1 = __shfl_sync(kFullMask, s01, src),
              v2 = __shfl_sync(kFullMask, s10, src), v3 = __shfl_sync(kFullMask, s11, src);
  return (h == 0 ? v0 : h == 1 ? v1 : h == 2 ? v2 : v3) + b3;
}

// The block's copy of what every lane reads per inference.
struct NetShared {
  uint2 w2[4 * 8 * 32];
  float b2[kHid], w3[kHid];
  float mean[kFeat], inv_std[kFeat];
};

__device__ __forceinline__ void load_net(const LearnedNet *net, NetShared &s) {
  for (int k = threadIdx.x; k < 4 * 8 * 32; k += blockDim.x) s.w2[k] = net->w2[k];
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

// Work items of the learned walk: (task, group) pairs, item k = t * ng + g.
// A task is a subtree (the nodes at the split depth, and leaves above it, in
// node order); the nodes above the split depth are opened for every group.
// Each lane appends the lists of its items to its own region (cells, and
// runs of bodies (first, count)); a gather pass concatenates a group's
// items in task order into the group's lists.
constexpr u32 kNoItem = 0xffffffffu;

struct LArgs {
  const WalkRec32 *walk32;
  const CellFeat *cfeat;
  const uint4 *tasks;      // .x = the task's root node
  u32 ntasks;
  const float *gboxf;
  const float2 *gtol;
  u32 ng;
  u64 nitems;
  const LearnedNet *net;
  const TreeRoot *root;
  const double2 *mom;
  float inv_theta_guard, band;
  int batch_min;
  u32 lane_cells, lane_runs;  // capacity of each lane's region
  u32 *reg_cells;
  uint2 *reg_runs;
  uint4 *seg;              // per item: first cell, cells, first run, runs (region indices)
  u32 *seg_bodies;         // per item: bodies
  Scalars *sc;
};

// The learned walk. Each lane walks one item at a time in the plain walk's
// node order (a forward scan with skip links) and takes the next item as
// soon as it is done (one counter), so the lanes of a warp stay busy until
// the work runs out, and no group's walk is longer than its longest task.
// Per visited node:
//   overlap, or inside the guard (2 h / theta_guard + delta) -> opened
//   guarded with two bodies or fewer                           -> accepted (bodies, exact)
//   centred prior below tau - band -> accepted; above tau + band -> opened
//   otherwise the lane waits for the network.
// A waiting lane keeps its node while the others walk on; the warp runs the
// network once `batch_min` lanes wait, or every active lane does. A row's
// result does not depend on the other rows, so the decisions do not depend
// on the schedule.
// kNet = false: band 0, the prior decides every test and the kernel carries
// no network (fewer registers, more warps in flight).
template <bool kNet>
__global__ void __launch_bounds__(kT) k_lwalk(LArgs a) {
  __shared__ NetShared sn;
  __shared__ uint4 rows[kT / 32][kNet ? 32 : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 w1[8];
  if (kNet) {
    load_net(a.net, sn);
    rows[warp][lane] = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
    for (int j = 0; j < 8; ++j) w1[j] = a.net->w1[j * 32 + lane];
  }
  const float b3 = a.net->b3, y_mean = a.net->y_mean, inv_y_std = 1.f / a.net->y_std;
  __syncthreads();
  const FeatScale fs = scale_of(a.root, a.mom);
  const u64 gtid = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  u32 *reg_c = a.reg_cells + gtid * a.lane_cells;
  uint2 *reg_r = a.reg_runs + gtid * a.lane_runs;
  Scalars *sc = a.sc;

  u64 item = kNoItem;
  u32 i = 0, end = 0, lc = 0, lr = 0, c0i = 0, r0i = 0, nb = 0;
  bool exhausted = false, waiting = false;
  float gf[3] = {0.f, 0.f, 0.f}, hf[3] = {0.f, 0.f, 0.f}, f0 = 0.f, tau = 0.f, thr = 0.f;
  WalkRec32 r{};
  unsigned long long rows_run = 0, batches = 0;
  while (true) {
    // idle lanes take the next items (one atomic per warp)
    const bool want = item == kNoItem && !exhausted;
    const unsigned wantm = __ballot_sync(kFullMask, want);
    if (wantm) {
      const int leader = __ffs(wantm) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&sc->walk_items, static_cast<unsigned long long>(__popc(wantm)));
      base = __shfl_sync(kFullMask, base, leader);
      if (want) {
        const u64 k = base + __popc(wantm & ((1u << lane) - 1u));
        if (k >= a.nitems) {
          exhausted = true;
        } else {
          item = k;
          const u32 t = static_cast<u32>(k / a.ng), g = static_cast<u32>(k % a.ng);
          const float4 b0 = reinterpret_cast<const float4 *>(a.gboxf)[2ull * g],
                       b1 = reinterpret_cast<const float4 *>(a.gboxf)[2ull * g + 1];
          gf[0] = b0.x;
          gf[1] = b0.y;
          gf[2] = b0.z;
          hf[0] = b0.w;
          hf[1] = b1.x;
          hf[2] = b1.y;
          const float2 gt = a.gtol[g];
          f0 = gt.x;
          tau = gt.y;
          i = a.tasks[t].x;
          end = __float_as_uint(__ldg(reinterpret_cast<const float4 *>(a.walk32 + i) + 2).x);
          c0i = lc;
          r0i = lr;
          nb = 0;
        }
      }
    }
    const bool active = item != kNoItem;
    const unsigned act = __ballot_sync(kFullMask, active);
    if (act == 0) break;

    int verdict = -1;
    if (active && !waiting) {
      r = load_rec(a.walk32, i);
      const float4 c0 = __ldg(reinterpret_cast<const float4 *>(a.cfeat + i));
      // the reference's overlap test (group_lists.cpp:147), in FP32
      const bool overlap = fabsf(r.cx - gf[0]) <= r.slack + hf[0] &&
                           fabsf(r.cy - gf[1]) <= r.slack + hf[1] &&
                           fabsf(r.cz - gf[2]) <= r.slack + hf[2];
      const float dx = fmaxf(fabsf(r.mx - gf[0]) - hf[0], 0.f),
                  dy = fmaxf(fabsf(r.my - gf[1]) - hf[1], 0.f),
                  dz = fmaxf(fabsf(r.mz - gf[2]) - hf[2], 0.f);
      const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const float crit = fmaf(2.f * c0.x, a.inv_theta_guard, c0.y);
      const u32 nbody = r.nbody_leaf & 0x7fffffffu;
      if (overlap || !(d2 > crit * crit)) {
        verdict = 0;
      } else if (nbody <= kFewBodies) {
        verdict = 1;
      } else {
        const float f2 = distance_feature(d2, fs);
        const float e = prior_log2err(c0.z, f2) + y_mean;  // centred prior
        if (!kNet) {
          verdict = e < tau ? 1 : 0;
        } else if (e < tau - a.band) {
          verdict = 1;
        } else if (e > tau + a.band) {
          verdict = 0;
        } else {
          const float4 c1 = __ldg(reinterpret_cast<const float4 *>(a.cfeat + i) + 1);
          const float f[kFeat] = {f0, c0.w, f2, c1.x, c1.y, c1.z};
          rows[warp][lane] = feature_row(f, sn);
          thr = (tau - e) * inv_y_std;
          waiting = true;
        }
      }
    }
    const unsigned wm = kNet ? __ballot_sync(kFullMask, waiting) : 0u;
    if (kNet && wm != 0 && (__popc(wm) >= a.batch_min || wm == act)) {
      __syncwarp();
      const float y = warp_mlp(rows[warp], w1, sn.w2, sn.b2, sn.w3, b3, lane);
      if (waiting) {
        verdict = y < thr ? 1 : 0;
        waiting = false;
      }
      rows_run += __popc(wm);
      ++batches;
      __syncwarp();
    }

    if (verdict >= 0) {
      const u32 nbody = r.nbody_leaf & 0x7fffffffu;
      if (verdict == 1 || (r.nbody_leaf >> 31)) {
        if (verdict == 1 && nbody > kFewBodies) {
          if (lc < a.lane_cells) reg_c[lc] = i;
          ++lc;
        } else {
          if (lr < a.lane_runs) reg_r[lr] = make_uint2(r.begin, nbody);
          ++lr;
          nb += nbody;
        }
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
        a.seg[item] = make_uint4(static_cast<u32>(gtid * a.lane_cells + c0i), lc - c0i,
                                 static_cast<u32>(gtid * a.lane_runs + r0i), lr - r0i);
        a.seg_bodies[item] = nb;
        item = kNoItem;
      }
    }
  }
  if (lc > a.lane_cells || lr > a.lane_runs) atomicOr(&sc->list_overflow, 1u);
  if (lane == 0 && batches) {
    atomicAdd(&sc->mlp_rows, rows_run);
    atomicAdd(&sc->mlp_batches, batches);
  }
}

// Per group: its items' cells and bodies summed, and the list counters.
__global__ void __launch_bounds__(kT)
    k_lsum(const uint4 *seg, const u32 *seg_bodies, u32 ng, u32 ntasks, const u32 *gbegin,
           const u32 *gend, u64 *ncells, u64 *nbodies, Scalars *sc) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  if (g >= ng) return;
  u64 nc = 0, nb = 0;
  for (u32 t = 0; t < ntasks; ++t) {
    const u64 k = static_cast<u64>(t) * ng + g;
    nc += seg[k].y;
    nb += seg_bodies[k];
  }
  ncells[g] = nc;
  nbodies[g] = nb;
  const u64 tg = gend[g] - gbegin[g];
  atomicAdd(&sc->cell_interactions, static_cast<unsigned long long>(tg * nc));
  atomicAdd(&sc->body_interactions, static_cast<unsigned long long>(tg * nb - tg));
  atomicMax(&sc->max_list, static_cast<unsigned long long>(nc + nb));
  atomicMax(&sc->max_group, static_cast<u32>(tg));
}

// One warp per group: its items' lists in task order, into the group's
// ranges of cell_list and body_list, and its GTGroup record.
constexpr int kGatherWarps = kT / 32;

__global__ void __launch_bounds__(kT)
    k_lgather(const uint4 *seg, u32 ng, u32 ntasks, const u32 *reg_cells, const uint2 *reg_runs,
              const u32 *gbegin, const u32 *gend, const u64 *cell_off, const u64 *body_off,
              u32 *cell_list, u32 *body_list, uint4 *groups) {
  const u32 g = blockIdx.x * kGatherWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (g >= ng) return;
  u64 oc = cell_off[g], ob = body_off[g];
  if (lane == 0) {
    groups[2ull * g] = make_uint4(gbegin[g], gend[g], static_cast<u32>(oc),
                                  static_cast<u32>(cell_off[g + 1]));
    groups[2ull * g + 1] = make_uint4(static_cast<u32>(ob), static_cast<u32>(body_off[g + 1]), 0u, 0u);
  }
  for (u32 t0 = 0; t0 < ntasks; t0 += 32) {
    // the next (up to) 32 items of the group, one per lane
    const u32 t = t0 + lane;
    const uint4 sgm = t < ntasks ? seg[static_cast<u64>(t) * ng + g] : make_uint4(0u, 0u, 0u, 0u);
    unsigned busy = __ballot_sync(kFullMask, sgm.y != 0 || sgm.w != 0);
    while (busy) {
      const int src = __ffs(busy) - 1;
      busy &= busy - 1u;
      const u32 c0 = __shfl_sync(kFullMask, sgm.x, src), nc = __shfl_sync(kFullMask, sgm.y, src);
      const u32 r0 = __shfl_sync(kFullMask, sgm.z, src), nr = __shfl_sync(kFullMask, sgm.w, src);
      for (u32 k = lane; k < nc; k += 32) cell_list[oc + k] = reg_cells[c0 + k];
      oc += nc;
      for (u32 k0 = 0; k0 < nr; k0 += 32) {
        const u32 k = k0 + lane;
        const uint2 run = k < nr ? reg_runs[r0 + k] : make_uint2(0u, 0u);
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
  }
}


// The walk's inference on given raw features (tests and diagnostics).
__global__ void __launch_bounds__(kT)
    k_predict(const LearnedNet *net, const float *feat, u64 n, float *pred) {
  __shared__ NetShared sn;
  __shared__ uint4 rows[kT / 32][32];
  load_net(net, sn);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 w1[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) w1[j] = net->w1[j * 32 + lane];
  __syncthreads();
  const u64 k = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  float f[kFeat] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (k < n)
    for (int j = 0; j < kFeat; ++j) f[j] = feat[k * kFeat + j];
  rows[warp][lane] = feature_row(f, sn);
  __syncwarp();
  const float y = warp_mlp(rows[warp], w1, sn.w2, sn.b2, sn.w3, net->b3, lane);
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

void learned_group_tolerances(Workspace &ws, const LearnedWalk &lw, u32 ng, cudaStream_t s) {
  if (ng == 0) return;
  lw.gtol->ensure(static_cast<u64>(ng) * sizeof(float2));
  k_group_tol<<<ceil_div(ng, kT), kT, 0, s>>>(
      ws.gbegin.as<u32>(), ws.gend.as<u32>(), ng, ws.idx.as<u32>(), lw.prev_amag,
      ws.gboxf.as<float>(), ws.root.as<TreeRoot>(), ws.mom.as<double2>(), lw.alpha, lw.G,
      lw.gtol->as<float2>());
  GTC_LAUNCH_CHECK();
}

void learned_build_lists(Workspace &ws, const LearnedWalk &lw, u32 ng, u32 ntasks,
                         Scalars *host, cudaStream_t s) {
  if (ng == 0) return;
  Scalars *sc = ws.scalars.as<Scalars>();
  int dev = 0, sms = 0, per_sm = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const bool net = lw.band > 0.f;
  if (net)
    GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lwalk<true>, kT, 0));
  else
    GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lwalk<false>, kT, 0));
  const u32 blocks = static_cast<u32>(std::max(1, sms * std::max(1, per_sm)));
  const u64 lanes = static_cast<u64>(blocks) * kT;
  const u64 nitems = static_cast<u64>(ng) * ntasks;
  ws.gcells.ensure(static_cast<u64>(ng) * 8);
  ws.gbodies.ensure(static_cast<u64>(ng) * 8);
  ws.gcell_off.ensure((static_cast<u64>(ng) + 1) * 8);
  ws.gbody_off.ensure((static_cast<u64>(ng) + 1) * 8);
  LArgs a{};
  a.walk32 = ws.walk32.as<WalkRec32>();
  a.cfeat = lw.cfeat;
  a.tasks = ws.tasks.as<uint4>();
  a.ntasks = ntasks;
  a.gboxf = ws.gboxf.as<float>();
  a.gtol = lw.gtol->as<float2>();
  a.ng = ng;
  a.nitems = nitems;
  a.net = lw.net;
  a.root = ws.root.as<TreeRoot>();
  a.mom = ws.mom.as<double2>();
  a.inv_theta_guard = lw.inv_theta_guard;
  a.band = lw.band;
  a.batch_min = lw.batch_min;
  a.sc = sc;
  u64 *cell_off = ws.gcell_off.as<u64>(), *body_off = ws.gbody_off.as<u64>();
  // each lane's region holds what its items append; if one outgrows it, the
  // regions double and the walk runs again
  u32 lane_cells = std::max<u32>(*lw.lane_cells, 256), lane_runs = std::max<u32>(*lw.lane_runs, 64);
  for (int attempt = 0;; ++attempt) {
    const u64 seg_bytes = nitems * (sizeof(uint4) + sizeof(u32));
    const u64 reg_bytes = lanes * (static_cast<u64>(lane_cells) * 4 + static_cast<u64>(lane_runs) * 8);
    lw.scratch->ensure(seg_bytes + reg_bytes);
    char *base = lw.scratch->as<char>();
    a.seg = reinterpret_cast<uint4 *>(base);
    a.reg_runs = reinterpret_cast<uint2 *>(base + nitems * sizeof(uint4));
    a.reg_cells = reinterpret_cast<u32 *>(base + nitems * sizeof(uint4) +
                                          lanes * static_cast<u64>(lane_runs) * 8);
    a.seg_bodies = reinterpret_cast<u32 *>(base + nitems * sizeof(uint4) + reg_bytes);
    a.lane_cells = lane_cells;
    a.lane_runs = lane_runs;
    GTC_CUDA(cudaMemsetAsync(&sc->cell_interactions, 0, 3 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_group, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(&sc->mlp_rows, 0, 3 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->list_overflow, 0, sizeof(u32), s));
    if (net)
      k_lwalk<true><<<blocks, kT, 0, s>>>(a);
    else
      k_lwalk<false><<<blocks, kT, 0, s>>>(a);
    GTC_LAUNCH_CHECK();
    k_lsum<<<ceil_div(ng, kT), kT, 0, s>>>(a.seg, a.seg_bodies, ng, ntasks, ws.gbegin.as<u32>(),
                                           ws.gend.as<u32>(), ws.gcells.as<u64>(),
                                           ws.gbodies.as<u64>(), sc);
    GTC_LAUNCH_CHECK();
    exclusive_scan_u64(ws.gcells.as<u64>(), cell_off, ng, cell_off + ng, ws.scan_tmp, s);
    exclusive_scan_u64(ws.gbodies.as<u64>(), body_off, ng, body_off + ng, ws.scan_tmp, s);
    GTC_CUDA(cudaMemcpyAsync(&sc->n_cell_list, cell_off + ng, 8, cudaMemcpyDeviceToDevice, s));
    GTC_CUDA(cudaMemcpyAsync(&sc->n_body_list, body_off + ng, 8, cudaMemcpyDeviceToDevice, s));
    GTC_CUDA(cudaMemcpyAsync(host, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    if (host->error)
      throw RuntimeError("cuda: inconsistent tree detected on the device (code " +
                         std::to_string(host->error) + ")");
    if (!host->list_overflow) break;
    if (attempt >= 4 || lanes * lane_cells * 2 > 0xffffffffull ||
        lanes * lane_runs * 2 > 0xffffffffull)
      throw RuntimeError("learned walk: the lane regions keep overflowing");
    lane_cells *= 2;
    lane_runs *= 2;
  }
  *lw.lane_cells = lane_cells;
  *lw.lane_runs = lane_runs;
  if (host->n_cell_list > 0xffffffffull || host->n_body_list > 0xffffffffull)
    throw RuntimeError("interaction lists too long for 32 bit offsets");
  ws.n_cell_list = host->n_cell_list;
  ws.n_body_list = host->n_body_list;
  ws.cell_list.ensure(std::max<u64>(1, ws.n_cell_list) * 4);
  ws.body_list.ensure(std::max<u64>(1, ws.n_body_list) * 4);
  k_lgather<<<ceil_div(ng, kGatherWarps), kT, 0, s>>>(
      a.seg, ng, ntasks, a.reg_cells, a.reg_runs, ws.gbegin.as<u32>(), ws.gend.as<u32>(),
      cell_off, body_off, ws.cell_list.as<u32>(), ws.body_list.as<u32>(), ws.groups.as<uint4>());
  GTC_LAUNCH_CHECK();
}


void learned_record_amag(const float4 *out, const u32 *order, u64 n, float *amag,
                         cudaStream_t s) {
  if (n == 0) return;
  k_record_amag<<<ceil_div(n, kT), kT, 0, s>>>(out, order, n, amag);
  GTC_LAUNCH_CHECK();
}

}  // namespace gtc
