// The learned criterion inside the grouped walk: per-node features, per-group
// tolerances, the walk in rounds (threads per group, warps for the long
// walks), the warp-level BF16 tensor-core inference on the pairs a round
// defers, and the tensor-core layout of the model.
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
#include <cstddef>
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
    k_cell_feat(const double2 *geom, const double2 *mom, const float4 *cells, const double *delta,
                const TreeRoot *root, u32 m, CellFeat *out) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p >= m) return;
  const FeatScale fs = scale_of(root, mom);
  // mass and quadrupole from the FP32 cell (as the evaluator sees them)
  const float4 cm = cells[3 * p], qa = cells[3 * p + 1], qb = cells[3 * p + 2];
  // Frobenius norm of the symmetric tensor (off-diagonal terms twice)
  const float qn = sqrtf(qa.x * qa.x + qa.y * qa.y + qa.z * qa.z +
                         2.f * (qa.w * qa.w + qb.x * qb.x + qb.y * qb.y));
  out[p] = cell_features(static_cast<float>(geom[2 * p + 1].y), cm.w, qn,
                         static_cast<float>(delta[p]), fs);
}

// The same features and records from the FP32 moment estimates (cells32,
// delta32) and the tree's topology, so that they need nothing of the FP64
// moments.
__global__ void __launch_bounds__(kT)
    k_cell_feat32(const double2 *geom, const double2 *rootmom, const float4 *cells32,
                  const float *delta32, const TreeRoot *root, u32 m, CellFeat *out) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p >= m) return;
  const FeatScale fs = scale_of(root, rootmom);
  const float4 cm = cells32[3 * p], qa = cells32[3 * p + 1], qb = cells32[3 * p + 2];
  const float qn = sqrtf(qa.x * qa.x + qa.y * qa.y + qa.z * qa.z +
                         2.f * (qa.w * qa.w + qb.x * qb.x + qb.y * qb.y));
  out[p] = cell_features(static_cast<float>(geom[2 * p + 1].y), cm.w, qn, delta32[p], fs);
}

__global__ void __launch_bounds__(kT)
    k_lwalk_rec32(const double2 *geom, const float4 *cells32, const CellFeat *cfeat,
                  const u32 *nbegin, const u32 *nend, const u32 *skip, const u8 *isleaf,
                  const TreeRoot *root, u32 m, float inv_theta_guard, float y_mean,
                  LWalkRec *out) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p >= m) return;
  const double2 g0 = geom[2 * p], g1 = geom[2 * p + 1];
  const float4 cm = cells32[3 * p];
  const float4 c0 = reinterpret_cast<const float4 *>(cfeat + p)[0];
  const float crit = fmaf(2.f * c0.x, inv_theta_guard, c0.y);
  LWalkRec r;
  r.cx = static_cast<float>(g0.x - root->center[0]);
  r.cy = static_cast<float>(g0.y - root->center[1]);
  r.cz = static_cast<float>(g1.x - root->center[2]);
  r.slack = static_cast<float>(g1.y * 1.0001);
  r.mx = cm.x;
  r.my = cm.y;
  r.mz = cm.z;
  r.guard2 = crit * crit;
  r.skip = skip[p];
  r.nbody_leaf = (nend[p] - nbegin[p]) | (isleaf[p] ? 0x80000000u : 0u);
  r.begin = nbegin[p];
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

constexpr int kMaxRounds = kMaxDepth + 4;

// Round 0 runs as kParts threads per group, each walking a range of the
// root's children (3, 3 and 2 of 8, in walk order) into its own slots: the
// groups with the longest lists, at the centre where |a| is small, set the
// round's time, and their walks spread over all the root's children. The
// parts' lists follow each other in walk order, so a group's lists are its
// parts' lists in turn; later rounds append to each part's own slot.
//
// A round-0 walk stops after a budget of node records (kLearnedWalkBudget
// by default). What is left of it
// (the nodes from where it stopped to the end of its range) goes to a
// continuation that a whole warp walks (k_lcont): the few longest walks,
// thousands of dependent record loads each, would otherwise set the round's
// time alone.
constexpr int kParts = 3;
// Small blocks for the walk rounds: their threads run for very different
// times, and small blocks even out the SMs.
constexpr u32 kRoundThreads = 128;

struct GArgs {
  const LWalkRec *lrec;
  const float *gboxf;
  const float2 *gtol;
  u32 ng;
  const TreeRoot *root;     // with mom: L, the d unit of the prior tests
  const double2 *mom;
  float band;
  u32 slot_cells[kParts], slot_bodies[kParts], slot_pend;
  u64 cells_at[kParts], bodies_at[kParts];  // part k's slots: at + g * slot
  u32 *cells, *bodies, *pend;  // deferred pairs: part k's at (k * ng + g) * slot_pend
  u64 *ncells, *nbodies;    // [part * ng + group]
  u32 *pcount;              // [part * ng + group]: pairs deferred this round
  const uint4 *kids;        // the root's children (last octant first: walk order)
  const u8 *nchild;
  const uint2 *rows;        // later rounds: the last round's deferred (group, node) pairs,
  const u8 *dec;            // the network's decisions (1 accept)
  const u32 *roff;          // and each (part, group)'s first row (kParts ng + 1)
  uint4 *cont;              // round-0 walks handed on: (part * ng + group, next node, end)
  u32 budget;               // nodes a thread tests before handing on (this round)
  u32 *next;                // the warp rounds' group counter
  Scalars *sc;
};

// The walk's test of node record (ra, rb, rc) for one group: 0 open,
// 1 accept, 2 defer to the network.
__device__ __forceinline__ int lverdict(const float4 &ra, const float4 &rb, const float4 &rc,
                                        const float *gf, const float *hf, float acc_d2,
                                        float open_d2) {
  // the reference's overlap test (group_lists.cpp:147), in FP32
  const bool overlap = fabsf(ra.x - gf[0]) <= ra.w + hf[0] && fabsf(ra.y - gf[1]) <= ra.w + hf[1] &&
                       fabsf(ra.z - gf[2]) <= ra.w + hf[2];
  const float dx = fmaxf(fabsf(rb.x - gf[0]) - hf[0], 0.f),
              dy = fmaxf(fabsf(rb.y - gf[1]) - hf[1], 0.f),
              dz = fmaxf(fabsf(rb.z - gf[2]) - hf[2], 0.f);
  const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  if (overlap || !(d2 > rb.w)) return 0;
  if ((__float_as_uint(rc.y) & 0x7fffffffu) <= kFewBodies) return 1;
  return d2 > rc.w * acc_d2 ? 1 : d2 < rc.w * open_d2 ? 0 : 2;
}

// The walk of subtrees [i, end) for one group, the first node's verdict
// given when pre >= 0; cells, bodies and deferred pairs to cl, bl, pl
// (capacities capc, capb, capp; counting goes on past them). It stops
// before the next node once it has tested `budget` nodes in all and
// returns where it stopped (end when done).
struct LWalkState {
  u64 nc, nb;
  u32 np, visits;
};

__device__ __forceinline__ u32 lwalk_range(const GArgs &a, const float *gf, const float *hf,
                                           float acc_d2, float open_d2, u32 i, u32 end, int pre,
                                           u32 *cl, u32 *bl, u32 *pl, u32 capc, u32 capb,
                                           u32 capp, u32 budget, LWalkState &w) {
  while (i < end) {
    if (w.visits >= budget) return i;
    const float4 *rp = reinterpret_cast<const float4 *>(a.lrec + i);
    const float4 ra = __ldg(rp), rb = __ldg(rp + 1), rc = __ldg(rp + 2);
    ++w.visits;
    const u32 skip = __float_as_uint(rc.x), nbody_leaf = __float_as_uint(rc.y);
    const u32 nbody = nbody_leaf & 0x7fffffffu;
    int verdict = pre;
    if (pre >= 0)
      pre = -1;
    else
      verdict = lverdict(ra, rb, rc, gf, hf, acc_d2, open_d2);
    if (verdict == 2) {
      if (w.np < capp) pl[w.np] = i;
      ++w.np;
    } else if (verdict == 1 && nbody > kFewBodies) {
      if (w.nc < capc) cl[w.nc] = i;
      ++w.nc;
    } else if (verdict == 1 || (nbody_leaf >> 31)) {
      const u32 first = __float_as_uint(rc.z);
      for (u32 j = 0; j < nbody && w.nb + j < capb; ++j) bl[w.nb + j] = first + j;
      w.nb += nbody;
    }
    if (verdict != 0 || (nbody_leaf >> 31)) {
      if (skip <= i) {  // malformed tree: never loop
        atomicOr(&a.sc->error, 1u);
        return end;
      }
      i = skip;
    } else {
      ++i;
    }
  }
  return end;
}

__device__ __forceinline__ u32 lskip(const LWalkRec *lrec, u32 i) {
  return __float_as_uint(__ldg(reinterpret_cast<const float4 *>(lrec + i) + 2).x);
}

__device__ __forceinline__ void group_scales(const GArgs &a, u32 g, float *gf, float *hf,
                                             float &acc_d2, float &open_d2) {
  const float4 b0 = reinterpret_cast<const float4 *>(a.gboxf)[2ull * g],
               b1 = reinterpret_cast<const float4 *>(a.gboxf)[2ull * g + 1];
  gf[0] = b0.x;
  gf[1] = b0.y;
  gf[2] = b0.z;
  hf[0] = b0.w;
  hf[1] = b1.x;
  hf[2] = b1.y;
  const float tau = a.gtol[g].y;
  const FeatScale fs = scale_of(a.root, a.mom);
  const float l2 = 1.f / (fs.inv_l * fs.inv_l);
  acc_d2 = exp2f(0.4f * (a.band - tau)) * l2;
  open_d2 = exp2f(0.4f * (-a.band - tau)) * l2;
}

// A part's maxima and the visits: one atomic per set of converged lanes of
// the same part (a warp can hold lanes of two parts).
__device__ __forceinline__ void lround_stats(Scalars *sc, int part, u64 nc, u64 nb, u32 np,
                                             u32 visits) {
  auto clamp = [](u64 v) { return static_cast<u32>(v < 0xffffffffull ? v : 0xffffffffull); };
  const unsigned mask = __match_any_sync(__activemask(), part);
  const u32 mc = __reduce_max_sync(mask, clamp(nc)), mb = __reduce_max_sync(mask, clamp(nb));
  const u32 mp = __reduce_max_sync(mask, np), sv = __reduce_add_sync(mask, visits);
  if ((threadIdx.x & 31) == static_cast<unsigned>(__ffs(mask) - 1)) {
    atomicMax(&sc->lmax_cells[part], mc);
    atomicMax(&sc->lmax_bodies[part], mb);
    atomicMax(&sc->max_pend, mp);
    atomicAdd(&sc->walk_nodes, static_cast<unsigned long long>(sv));
  }
}

// Round 0: thread (part, group) walks the part's range of the root's
// children (the root itself, when it is a leaf, in part 0).
__global__ void __launch_bounds__(kRoundThreads) k_lround0(GArgs a) {
  const u64 tid = static_cast<u64>(blockIdx.x) * kRoundThreads + threadIdx.x;
  if (tid >= static_cast<u64>(kParts) * a.ng) return;
  const int part = static_cast<int>(tid / a.ng);
  const u32 g = static_cast<u32>(tid % a.ng);
  float gf[3], hf[3], acc_d2, open_d2;
  group_scales(a, g, gf, hf, acc_d2, open_d2);
  const int nc = a.nchild[0];
  u32 i = 0, end = 0;
  if (nc == 0) {
    if (part == 0) end = lskip(a.lrec, 0);
  } else {
    const uint4 k0 = a.kids[0], k1 = a.kids[1];
    const u32 ch[8] = {k0.x, k0.y, k0.z, k0.w, k1.x, k1.y, k1.z, k1.w};
    const int j0 = (part * nc + kParts - 1) / kParts, j1 = ((part + 1) * nc + kParts - 1) / kParts;
    if (j0 < j1) {
      i = ch[j0];
      end = lskip(a.lrec, ch[j1 - 1]);
    }
  }
  const u32 capc = a.slot_cells[part], capb = a.slot_bodies[part];
  u32 *cl = a.cells + a.cells_at[part] + static_cast<u64>(g) * capc;
  u32 *bl = a.bodies + a.bodies_at[part] + static_cast<u64>(g) * capb;
  u32 *pl = a.pend + (static_cast<u64>(part) * a.ng + g) * a.slot_pend;
  LWalkState w{0, 0, 0, 0};
  const u32 stop = lwalk_range(a, gf, hf, acc_d2, open_d2, i, end, -1, cl, bl, pl, capc, capb,
                               a.slot_pend, a.budget, w);
  if (stop < end) {  // at most one per (part, group): the array holds kParts ng
    const u32 c = atomicAdd(&a.sc->lcont, 1u);
    a.cont[c] = make_uint4(static_cast<u32>(tid), stop, end, 0u);
  }
  a.ncells[static_cast<u64>(part) * a.ng + g] = w.nc;
  a.nbodies[static_cast<u64>(part) * a.ng + g] = w.nb;
  a.pcount[static_cast<u64>(part) * a.ng + g] = w.np;
  if (w.nc > capc || w.nb > capb || w.np > a.slot_pend) atomicOr(&a.sc->list_overflow, 1u);
  lround_stats(a.sc, part, w.nc, w.nb, w.np, w.visits);
}

// The rest of the walks that ran out of budget, one warp each. The warp
// keeps the walk's remaining nodes as a stack of index ranges, each a run of
// whole subtrees whose parents the walk opened. Each step the lanes take the
// 32 ranges on top, test each range's first node and push back its children
// (when opened) and the rest of its range, so the lanes test exactly the
// nodes the thread would have, 32 at a time. In later rounds the thread's
// remaining deferred pairs go on the stack too, as a node with the network's
// decision in place of the range's end (kPairOpen, kPairAccept), 64 at a
// time whenever fewer than 32 ranges are left. Entries are appended to the
// part's slots in step order, lane order within a step: a fixed order for
// given inputs.
constexpr int kContWarps = 4;
constexpr int kContStack = 1024;  // ranges per warp
constexpr u32 kPairOpen = 0xfffffffeu, kPairAccept = 0xffffffffu;  // node counts stay below

__global__ void __launch_bounds__(kContWarps * 32) k_lcont(GArgs a, bool later) {
  __shared__ uint2 stack_all[kContWarps][kContStack];
  const int lane = threadIdx.x & 31;
  uint2 *stk = stack_all[threadIdx.x >> 5];
  const unsigned below = (1u << lane) - 1u;
  const u32 ncont = a.sc->lcont;
  if (a.sc->list_overflow) return;  // a buffer was outgrown: the walk is redone
  for (;;) {
    u32 c = 0;
    if (lane == 0) c = atomicAdd(&a.sc->lcont_taken, 1u);
    c = __shfl_sync(kFullMask, c, 0);
    if (c >= ncont) return;
    const uint4 ct = a.cont[c];
    const u32 pg = ct.x;
    const int part = static_cast<int>(pg / a.ng);
    const u32 g = pg % a.ng;
    float gf[3], hf[3], acc_d2, open_d2;
    group_scales(a, g, gf, hf, acc_d2, open_d2);
    const u32 capc = a.slot_cells[part], capb = a.slot_bodies[part], capp = a.slot_pend;
    u32 *cl = a.cells + a.cells_at[part] + static_cast<u64>(g) * capc;
    u32 *bl = a.bodies + a.bodies_at[part] + static_cast<u64>(g) * capb;
    u32 *pl = a.pend + static_cast<u64>(pg) * capp;
    u64 nc = a.ncells[pg], nb = a.nbodies[pg];
    u32 np = a.pcount[pg], visits = 0;
    u32 kp = later ? ct.w : 0u;  // the next deferred pair, up to k1
    const u32 k1 = later ? a.roff[pg + 1] : 0u;
    int size = 0;
    if (ct.y < ct.z) {
      if (lane == 0) stk[0] = make_uint2(ct.y, ct.z);
      size = 1;
    }
    bool bad = false;
    __syncwarp();
    while ((size > 0 || kp < k1) && !bad) {
      if (size < 32 && kp < k1) {  // room: 32 + 64 ranges stay below kContStack - 32
        const u32 cnt = k1 - kp < 64u ? k1 - kp : 64u;
        for (u32 j = lane; j < cnt; j += 32)
          stk[size + cnt - 1 - j] = make_uint2(a.rows[kp + j].y, a.dec[kp + j] ? kPairAccept : kPairOpen);
        kp += cnt;
        size += static_cast<int>(cnt);
        __syncwarp();
      }
      if (size > kContStack - 32) {
        // nearly full (a step adds at most one range per lane): lane 0
        // walks the range on top alone
        if (lane == 0) {
          const uint2 r = stk[size - 1];
          const bool pair = r.y >= kPairOpen;
          LWalkState w{nc, nb, np, 0};
          lwalk_range(a, gf, hf, acc_d2, open_d2, r.x, pair ? lskip(a.lrec, r.x) : r.y,
                      pair ? static_cast<int>(r.y - kPairOpen) : -1, cl, bl, pl, capc, capb, capp,
                      ~0u, w);
          nc = w.nc;
          nb = w.nb;
          np = w.np;
          visits += w.visits;
        }
        nc = __shfl_sync(kFullMask, nc, 0);
        nb = __shfl_sync(kFullMask, nb, 0);
        np = __shfl_sync(kFullMask, np, 0);
        --size;
        __syncwarp();
        continue;
      }
      const int k = size < 32 ? size : 32;
      const bool act = lane < k;
      uint2 r = make_uint2(0u, 0u);
      if (act) r = stk[size - 1 - lane];
      __syncwarp();
      size -= k;
      int verdict = 0;
      u32 skip = 0, nbody_leaf = 0, first = 0, rend = r.y;
      if (act) {
        const float4 *rp = reinterpret_cast<const float4 *>(a.lrec + r.x);
        const float4 ra = __ldg(rp), rb = __ldg(rp + 1), rc = __ldg(rp + 2);
        ++visits;
        skip = __float_as_uint(rc.x);
        nbody_leaf = __float_as_uint(rc.y);
        first = __float_as_uint(rc.z);
        if (r.y >= kPairOpen) {  // a deferred pair: the network's decision, its subtree
          verdict = static_cast<int>(r.y - kPairOpen);
          rend = skip;
        } else {
          verdict = lverdict(ra, rb, rc, gf, hf, acc_d2, open_d2);
        }
      }
      const u32 nbody = nbody_leaf & 0x7fffffffu;
      const bool leaf = (nbody_leaf >> 31) != 0;
      const bool is_cell = act && verdict == 1 && nbody > kFewBodies;
      const bool is_pend = act && verdict == 2;
      const u32 nbo = act && ((verdict == 1 && nbody <= kFewBodies) || (verdict == 0 && leaf))
                          ? nbody : 0u;
      const unsigned bc = __ballot_sync(kFullMask, is_cell), bp = __ballot_sync(kFullMask, is_pend);
      if (is_cell) {
        const u64 at = nc + __popc(bc & below);
        if (at < capc) cl[at] = r.x;
      }
      if (is_pend) {
        const u64 at = np + __popc(bp & below);
        if (at < capp) pl[at] = r.x;
      }
      u32 incl = nbo;  // bodies: inclusive scan over the lanes
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u32 t = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += t;
      }
      for (u32 j = 0; j < nbo; ++j) {
        const u64 at = nb + (incl - nbo) + j;
        if (at < capb) bl[at] = first + j;
      }
      nc += __popc(bc);
      np += __popc(bp);
      nb += __shfl_sync(kFullMask, incl, 31);
      // the next ranges: the opened node's children [r.x + 1, skip) above
      // the rest of its range [skip, r.y)
      bool has_rest = false, has_kids = false;
      const u32 kids_end = skip < rend ? skip : rend;
      if (act) {
        if (skip <= r.x) {  // malformed tree: never loop
          bad = true;
        } else {
          has_rest = skip < rend;
          has_kids = verdict == 0 && !leaf && r.x + 1 < kids_end;
        }
      }
      const u32 npush = (has_rest ? 1u : 0u) + (has_kids ? 1u : 0u);
      u32 from = npush;  // pushes of this lane and the lanes above it
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u32 t = __shfl_down_sync(kFullMask, from, o);
        if (lane + o < 32) from += t;
      }
      const u32 base = static_cast<u32>(size) + from - npush;
      if (has_rest) stk[base] = make_uint2(skip, rend);
      if (has_kids) stk[base + (has_rest ? 1u : 0u)] = make_uint2(r.x + 1, kids_end);
      size += static_cast<int>(__shfl_sync(kFullMask, from, 0));
      bad = __any_sync(kFullMask, bad);
      __syncwarp();
    }
    const u32 sv = __reduce_add_sync(kFullMask, visits);
    if (lane == 0) {
      if (bad) atomicOr(&a.sc->error, 1u);
      a.ncells[pg] = nc;
      a.nbodies[pg] = nb;
      a.pcount[pg] = np;
      if (nc > capc || nb > capb || np > capp) atomicOr(&a.sc->list_overflow, 1u);
      auto clamp = [](u64 v) { return static_cast<u32>(v < 0xffffffffull ? v : 0xffffffffull); };
      atomicMax(&a.sc->lmax_cells[part], clamp(nc));
      atomicMax(&a.sc->lmax_bodies[part], clamp(nb));
      atomicMax(&a.sc->max_pend, np);
      atomicAdd(&a.sc->walk_nodes, static_cast<unsigned long long>(sv));
    }
    __syncwarp();
  }
}

// A round by warps: one warp per group, the group's whole walk in part 0's
// slots (parts 1 and 2 stay empty). The warp keeps the nodes still to visit
// as a stack of index ranges (as k_lcont does): round 0 starts from the
// root's children; a later round from the pairs the group deferred in the
// last round, each with the network's decision in place of the range's end
// (accepted: the cell; opened: its subtree). Each step the lanes test the
// first node of the 32 ranges on top; entries reach the lists in step order,
// lane order within a step (fixed for given inputs), and the pairs deferred
// now go to the group's pend slot for the next round.
constexpr int kLWarps = 4;
constexpr int kLStack = 1024;  // ranges per warp

__global__ void __launch_bounds__(kLWarps * 32) k_lwarp(GArgs a, u32 round) {
  __shared__ uint2 stack_all[kLWarps][kLStack];
  const int lane = threadIdx.x & 31;
  uint2 *stk = stack_all[threadIdx.x >> 5];
  const unsigned below = (1u << lane) - 1u;
  if (a.sc->list_overflow) return;  // a buffer was outgrown: the walk is redone
  const u32 root_end = lskip(a.lrec, 0);
  const bool root_leaf = a.nchild[0] == 0;
  u32 visits = 0;
  u32 mc_max = 0, mb_max = 0, mp_max = 0;
  bool bad = false;
  for (;;) {
    u32 g = 0;
    if (lane == 0) g = atomicAdd(a.next, 1u);
    g = __shfl_sync(kFullMask, g, 0);
    if (g >= a.ng) break;
    float gf[3], hf[3], acc_d2, open_d2;
    group_scales(a, g, gf, hf, acc_d2, open_d2);
    const u32 capc = a.slot_cells[0], capb = a.slot_bodies[0], capp = a.slot_pend;
    u32 *cl = a.cells + a.cells_at[0] + static_cast<u64>(g) * capc;
    u32 *bl = a.bodies + a.bodies_at[0] + static_cast<u64>(g) * capb;
    u32 *pl = a.pend + static_cast<u64>(g) * capp;  // part 0's pend slots come first
    u64 nc = round ? a.ncells[g] : 0, nb = round ? a.nbodies[g] : 0;
    u32 np = 0;
    u32 kp = round ? a.roff[g] : 0u, k1 = round ? a.roff[g + 1] : 0u;
    int size = 0;
    if (round == 0) {
      if (lane == 0) stk[0] = root_leaf ? make_uint2(0u, root_end) : make_uint2(1u, root_end);
      size = 1;
    }
    __syncwarp();
    while ((size > 0 || kp < k1) && !bad) {
      if (size < 32 && kp < k1) {  // room: 32 + 64 ranges stay below kLStack - 32
        const u32 cnt = k1 - kp < 64u ? k1 - kp : 64u;
        for (u32 j = lane; j < cnt; j += 32)
          stk[size + cnt - 1 - j] =
              make_uint2(a.rows[kp + j].y, a.dec[kp + j] ? kPairAccept : kPairOpen);
        kp += cnt;
        size += static_cast<int>(cnt);
        __syncwarp();
      }
      if (size > kLStack - 32) {
        // nearly full (a step adds at most one range per lane): lane 0
        // walks the range on top alone
        if (lane == 0) {
          const uint2 r = stk[size - 1];
          const bool pair = r.y >= kPairOpen;
          LWalkState w{nc, nb, np, 0};
          lwalk_range(a, gf, hf, acc_d2, open_d2, r.x, pair ? lskip(a.lrec, r.x) : r.y,
                      pair ? static_cast<int>(r.y - kPairOpen) : -1, cl, bl, pl, capc, capb, capp,
                      ~0u, w);
          nc = w.nc;
          nb = w.nb;
          np = w.np;
          visits += w.visits;
        }
        nc = __shfl_sync(kFullMask, nc, 0);
        nb = __shfl_sync(kFullMask, nb, 0);
        np = __shfl_sync(kFullMask, np, 0);
        --size;
        __syncwarp();
        continue;
      }
      const int k = size < 32 ? size : 32;
      const bool act = lane < k;
      uint2 r = make_uint2(0u, 0u);
      if (act) r = stk[size - 1 - lane];
      __syncwarp();
      size -= k;
      int verdict = 0;
      u32 skip = 0, nbody_leaf = 0, first = 0, rend = r.y;
      if (act) {
        const float4 *rp = reinterpret_cast<const float4 *>(a.lrec + r.x);
        const float4 ra = __ldg(rp), rb = __ldg(rp + 1), rc = __ldg(rp + 2);
        ++visits;
        skip = __float_as_uint(rc.x);
        nbody_leaf = __float_as_uint(rc.y);
        first = __float_as_uint(rc.z);
        if (r.y >= kPairOpen) {  // a deferred pair: the network's decision, its subtree
          verdict = static_cast<int>(r.y - kPairOpen);
          rend = skip;
        } else {
          verdict = lverdict(ra, rb, rc, gf, hf, acc_d2, open_d2);
        }
      }
      const u32 nbody = nbody_leaf & 0x7fffffffu;
      const bool leaf = (nbody_leaf >> 31) != 0;
      const bool is_cell = act && verdict == 1 && nbody > kFewBodies;
      const bool is_pend = act && verdict == 2;
      const u32 nbo = act && ((verdict == 1 && nbody <= kFewBodies) || (verdict == 0 && leaf))
                          ? nbody : 0u;
      const unsigned bc = __ballot_sync(kFullMask, is_cell), bp = __ballot_sync(kFullMask, is_pend);
      if (is_cell) {
        const u64 at = nc + __popc(bc & below);
        if (at < capc) cl[at] = r.x;
      }
      if (is_pend) {
        const u64 at = np + __popc(bp & below);
        if (at < capp) pl[at] = r.x;
      }
      u32 incl = nbo;  // bodies: inclusive scan over the lanes
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u32 tt = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += tt;
      }
      for (u32 j = 0; j < nbo; ++j) {
        const u64 at = nb + (incl - nbo) + j;
        if (at < capb) bl[at] = first + j;
      }
      nc += __popc(bc);
      np += __popc(bp);
      nb += __shfl_sync(kFullMask, incl, 31);
      // the next ranges: the opened node's children [r.x + 1, skip) above
      // the rest of its range [skip, r.y)
      bool has_rest = false, has_kids = false;
      const u32 kids_end = skip < rend ? skip : rend;
      if (act) {
        if (skip <= r.x) {  // malformed tree: never loop
          bad = true;
        } else {
          has_rest = skip < rend;
          has_kids = verdict == 0 && !leaf && r.x + 1 < kids_end;
        }
      }
      const u32 npush = (has_rest ? 1u : 0u) + (has_kids ? 1u : 0u);
      u32 from = npush;  // pushes of this lane and the lanes above it
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u32 tt = __shfl_down_sync(kFullMask, from, o);
        if (lane + o < 32) from += tt;
      }
      const u32 base = static_cast<u32>(size) + from - npush;
      if (has_rest) stk[base] = make_uint2(skip, rend);
      if (has_kids) stk[base + (has_rest ? 1u : 0u)] = make_uint2(r.x + 1, kids_end);
      size += static_cast<int>(__shfl_sync(kFullMask, from, 0));
      bad = __any_sync(kFullMask, bad);
      __syncwarp();
    }
    if (lane == 0) {
      a.ncells[g] = nc;
      a.nbodies[g] = nb;
      a.pcount[g] = np;
      if (round == 0) {  // parts 1 and 2 hold nothing
        for (int part = 1; part < kParts; ++part) {
          a.ncells[static_cast<u64>(part) * a.ng + g] = 0;
          a.nbodies[static_cast<u64>(part) * a.ng + g] = 0;
        }
      }
      for (int part = 1; part < kParts; ++part) a.pcount[static_cast<u64>(part) * a.ng + g] = 0;
      if (nc > capc || nb > capb || np > capp) atomicOr(&a.sc->list_overflow, 1u);
    }
    auto clamp = [](u64 v) { return static_cast<u32>(v < 0xffffffffull ? v : 0xffffffffull); };
    mc_max = max(mc_max, clamp(nc));
    mb_max = max(mb_max, clamp(nb));
    mp_max = max(mp_max, np);
    __syncwarp();
  }
  const u32 sv = __reduce_add_sync(kFullMask, visits);
  if (lane == 0) {
    if (bad) atomicOr(&a.sc->error, 1u);
    atomicMax(&a.sc->lmax_cells[0], mc_max);
    atomicMax(&a.sc->lmax_bodies[0], mb_max);
    atomicMax(&a.sc->max_pend, mp_max);
    atomicAdd(&a.sc->walk_nodes, static_cast<unsigned long long>(sv));
  }
}

// A later round, kParts threads per group: thread (part, group) takes the
// pairs its part deferred in the last round, in order, with the network's
// decisions, appends to the part's slot and defers into the part's pend
// slot, so a part's lists are its round-0 walk followed by each later
// round's.
__global__ void __launch_bounds__(kRoundThreads) k_lround(GArgs a) {
  const u64 pg = static_cast<u64>(blockIdx.x) * kRoundThreads + threadIdx.x;
  if (pg >= static_cast<u64>(kParts) * a.ng) return;
  if (a.sc->list_overflow) return;  // an earlier round outgrew a buffer: redone
  const int part = static_cast<int>(pg / a.ng);
  const u32 g = static_cast<u32>(pg % a.ng);
  const u32 k0 = a.roff[pg], k1 = a.roff[pg + 1];
  if (k0 == k1) {
    a.pcount[pg] = 0;
    return;
  }
  float gf[3], hf[3], acc_d2, open_d2;
  group_scales(a, g, gf, hf, acc_d2, open_d2);
  const u32 capc = a.slot_cells[part], capb = a.slot_bodies[part];
  u32 *cl = a.cells + a.cells_at[part] + static_cast<u64>(g) * capc;
  u32 *bl = a.bodies + a.bodies_at[part] + static_cast<u64>(g) * capb;
  u32 *pl = a.pend + pg * a.slot_pend;
  LWalkState w{a.ncells[pg], a.nbodies[pg], 0, 0};
  for (u32 k = k0; k < k1; ++k) {
    if (w.visits >= a.budget) {  // the pairs from k on go to a warp
      const u32 c = atomicAdd(&a.sc->lcont, 1u);
      a.cont[c] = make_uint4(static_cast<u32>(pg), 0u, 0u, k);
      break;
    }
    const u32 i = a.rows[k].y, end = lskip(a.lrec, i);
    const u32 stop = lwalk_range(a, gf, hf, acc_d2, open_d2, i, end, a.dec[k], cl, bl, pl, capc,
                                 capb, a.slot_pend, a.budget, w);
    if (stop < end) {  // the rest of this pair's subtree and the later pairs
      const u32 c = atomicAdd(&a.sc->lcont, 1u);
      a.cont[c] = make_uint4(static_cast<u32>(pg), stop, end, k + 1);
      break;
    }
  }
  a.ncells[pg] = w.nc;
  a.nbodies[pg] = w.nb;
  a.pcount[pg] = w.np;
  if (w.nc > capc || w.nb > capb || w.np > a.slot_pend) atomicOr(&a.sc->list_overflow, 1u);
  lround_stats(a.sc, part, w.nc, w.nb, w.np, w.visits);
}

// A round's deferred pairs as dense rows, ordered by (part, group) and, for
// each, in the order they were deferred, if the row buffer holds `cap`
// rows (else the overflow flag); also the round's rows in the statistics.
__global__ void __launch_bounds__(kT) k_lrows(const GArgs a, uint2 *rows, u64 cap) {
  const u64 pg = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  const u64 nparts = static_cast<u64>(kParts) * a.ng;
  const u32 total = a.roff[nparts];
  if (a.sc->list_overflow & 1u) return;  // a slot was outgrown: the walk is redone
  if (pg == 0) {
    atomicMax(&a.sc->max_rows, total);
    atomicAdd(&a.sc->mlp_rows, static_cast<unsigned long long>(total));
    atomicAdd(&a.sc->mlp_batches, static_cast<unsigned long long>((total + 31u) / 32u));
    if (total > cap) atomicOr(&a.sc->list_overflow, 2u);
  }
  if (pg >= nparts || total > cap) return;
  const u32 g = static_cast<u32>(pg % a.ng);
  const u32 n = a.pcount[pg], o = a.roff[pg];
  const u32 *pl = a.pend + pg * a.slot_pend;
  for (u32 j = 0; j < n; ++j) rows[o + j] = make_uint2(g, pl[j]);
}

// Group records of the learned walk (the parts' slots, one segment each) and
// the list statistics.
__global__ void __launch_bounds__(kT) k_lgroup_records(const GArgs a, const u32 *gbegin,
                                                       const u32 *gend, uint4 *groups) {
  const u32 g = blockIdx.x * kT + threadIdx.x;
  const bool valid = g < a.ng;
  u64 t = 0, nc = 0, nb = 0;
  if (valid) {
    ListSegs cs{}, bs{};  // (segments past kParts stay empty)
    for (int k = 0; k < kParts; ++k) {
      const u64 at = static_cast<u64>(k) * a.ng + g;
      cs.start[k] = static_cast<u32>(a.cells_at[k] + static_cast<u64>(g) * a.slot_cells[k]);
      cs.count[k] = static_cast<u32>(a.ncells[at]);
      bs.start[k] = static_cast<u32>(a.bodies_at[k] + static_cast<u64>(g) * a.slot_bodies[k]);
      bs.count[k] = static_cast<u32>(a.nbodies[at]);
      nc += a.ncells[at];
      nb += a.nbodies[at];
    }
    store_group_rec(groups, g, gbegin[g], gend[g], cs, bs);
    t = gend[g] - gbegin[g];
  }
  group_stats_warp(a.sc, valid, t, nc, nb, true, false);
}

// The network's decision on every deferred pair: one warp per 32 pairs.
__global__ void __launch_bounds__(kT)
    k_ldecide(const uint2 *q, u64 nq, const LWalkRec *lrec, const CellFeat *cfeat,
              const float *gboxf, const float2 *gtol, const LearnedNet *net, const TreeRoot *root,
              const double2 *mom, u8 *dec, const u32 *nq_dev = nullptr,
              const u32 *overflow = nullptr) {
  __shared__ NetShared sn;
  __shared__ uint4 rows[kT / 32][32];
  // rows counted on the device; none written when a buffer was outgrown
  if (nq_dev && *nq_dev < nq) nq = *nq_dev;
  if (overflow && *overflow) nq = 0;
  if (static_cast<u64>(blockIdx.x) * kT >= nq) return;  // the whole block
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
    const float4 rm = __ldg(reinterpret_cast<const float4 *>(lrec + p) + 1);  // com, guard
    const float4 c0 = __ldg(reinterpret_cast<const float4 *>(cfeat + p));
    const float4 c1 = __ldg(reinterpret_cast<const float4 *>(cfeat + p) + 1);
    const float dx = fmaxf(fabsf(rm.x - b0.x) - b0.w, 0.f),
                dy = fmaxf(fabsf(rm.y - b0.y) - b1.x, 0.f),
                dz = fmaxf(fabsf(rm.z - b0.z) - b1.y, 0.f);
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
                                             ws.cells.as<float4>(), ws.delta.as<double>(),
                                             ws.root.as<TreeRoot>(), m, cfeat.as<CellFeat>());
  GTC_LAUNCH_CHECK();
}

void learned_walk_inputs(Workspace &ws, LearnedScratch &ls, DeviceBuffer &cfeat,
                         float inv_theta_guard, float y_mean, cudaStream_t s) {
  const u32 m = static_cast<u32>(ws.n_nodes);
  if (m == 0) return;
  ls.cells32.ensure(static_cast<u64>(m) * 3 * sizeof(float4));
  ls.delta32.ensure(static_cast<u64>(m) * sizeof(float));
  ls.rootmom.ensure(2 * sizeof(double2));
  moments32(ws, ls.cells32.as<float4>(), ls.delta32.as<float>(), ls.rootmom.as<double2>(), s);
  cfeat.ensure(static_cast<u64>(m) * sizeof(CellFeat));
  k_cell_feat32<<<ceil_div(m, kT), kT, 0, s>>>(ws.geom.as<double2>(), ls.rootmom.as<double2>(),
                                               ls.cells32.as<float4>(), ls.delta32.as<float>(),
                                               ws.root.as<TreeRoot>(), m, cfeat.as<CellFeat>());
  GTC_LAUNCH_CHECK();
  ls.lrec.ensure(static_cast<u64>(m) * sizeof(LWalkRec));
  k_lwalk_rec32<<<ceil_div(m, kT), kT, 0, s>>>(
      ws.geom.as<double2>(), ls.cells32.as<float4>(), cfeat.as<CellFeat>(), ws.nbegin.as<u32>(),
      ws.nend.as<u32>(), ws.skip.as<u32>(), ws.isleaf.as<u8>(), ws.root.as<TreeRoot>(), m,
      inv_theta_guard, y_mean, ls.lrec.as<LWalkRec>());
  GTC_LAUNCH_CHECK();
}

void learned_group_tolerances(Workspace &ws, const LearnedWalk &lw, u32 ng, cudaStream_t s) {
  if (ng == 0) return;
  lw.gtol->ensure(static_cast<u64>(ng) * sizeof(float2));
  k_group_tol<<<ceil_div(ng, kT), kT, 0, s>>>(
      ws.gbegin.as<u32>(), ws.gend.as<u32>(), ng, ws.idx.as<u32>(), lw.prev_amag,
      ws.gboxf.as<float>(), ws.root.as<TreeRoot>(), lw.scratch->rootmom.as<double2>(), lw.alpha,
      lw.G, lw.gtol->as<float2>());
  GTC_LAUNCH_CHECK();
}

namespace {
// Slots for the next learned walk: the longest lists plus a half and 64, in
// multiples of 32 entries.
u32 learned_slot(u64 longest) {
  const u64 v = (longest + longest / 2 + 64 + 31) & ~31ull;
  return static_cast<u32>(std::min<u64>(v, 0x7fffffe0ull));
}
}  // namespace

void learned_build_lists(Workspace &ws, const LearnedWalk &lw, u32 ng, Scalars *host,
                         cudaStream_t s) {
  static_assert(kParts <= kListSegments, "one list segment per part");
  if (ng == 0) return;
  if (ws.n_nodes >= kPairOpen)
    throw RuntimeError("learned walk: too many tree nodes for 32 bit node ranges");
  Scalars *sc = ws.scalars.as<Scalars>();
  LearnedScratch &ls = *lw.scratch;
  const bool warps = lw.warps_mode > 0 || (lw.warps_mode < 0 && ng < Workspace::kWarpWalkGroups);
  if (ls.slot_cells[0] == 0) {  // the first learned walk: the theta walk's slots to start with
    for (int k = 0; k < kParts; ++k) {
      // the warp rounds write a group's whole lists into part 0
      const bool used = !warps || k == 0;
      ls.slot_cells[k] = used ? std::max<u32>(warps ? ws.slot_cells : ws.slot_cells / 2, 256)
                              : learned_slot(0);
      ls.slot_bodies[k] = used ? std::max<u32>(warps ? ws.slot_bodies : ws.slot_bodies / 2, 256)
                               : learned_slot(0);
    }
    ls.slot_pend = 256;
  }
  ws.gcells.ensure(static_cast<u64>(kParts) * ng * 8);
  ws.gbodies.ensure(static_cast<u64>(kParts) * ng * 8);
  const u64 nparts = static_cast<u64>(kParts) * ng;  // (part, group) pairs
  ls.pcount.ensure(nparts * sizeof(u32));
  ls.roff.ensure((nparts + 1) * sizeof(u32));
  GArgs a{};
  a.lrec = ls.lrec.as<LWalkRec>();
  a.gboxf = ws.gboxf.as<float>();
  a.gtol = lw.gtol->as<float2>();
  a.ng = ng;
  a.root = ws.root.as<TreeRoot>();
  a.mom = ls.rootmom.as<double2>();  // the root's mass, from the FP32 estimates
  a.band = lw.band;
  a.ncells = ws.gcells.as<u64>();
  a.nbodies = ws.gbodies.as<u64>();
  a.pcount = ls.pcount.as<u32>();
  a.kids = ws.kids.as<uint4>();
  a.nchild = ws.nchild.as<u8>();
  a.roff = ls.roff.as<u32>();
  ls.cont.ensure(nparts * sizeof(uint4));
  a.cont = ls.cont.as<uint4>();
  a.sc = sc;
  const u32 gb = ceil_div(ng, kT), pb = static_cast<u32>(ceil_div(nparts, kT));
  const u32 rb = static_cast<u32>(ceil_div(nparts, kRoundThreads));
  int dev = 0, sms = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // warps that take the handed-on walks in turn: a few per SM
  const u32 cont_blocks = static_cast<u32>(std::max(1, sms) * 4);
  // the warp rounds: enough warps to fill the GPU, groups from a counter
  const u32 warp_blocks = static_cast<u32>(
      std::max<u64>(1, std::min<u64>(ceil_div(ng, kLWarps), 8ull * std::max(1, sms))));
  ls.next.ensure(sizeof(u32));
  a.next = ls.next.as<u32>();
  u32 rounds = 0;  // rounds walked
  for (int attempt = 0;; ++attempt) {
    u64 c_at = 0, b_at = 0;
    for (int k = 0; k < kParts; ++k) {
      a.slot_cells[k] = ls.slot_cells[k];
      a.slot_bodies[k] = ls.slot_bodies[k];
      a.cells_at[k] = c_at;
      a.bodies_at[k] = b_at;
      c_at += static_cast<u64>(ng) * ls.slot_cells[k];
      b_at += static_cast<u64>(ng) * ls.slot_bodies[k];
    }
    if (c_at > 0xffffffffull || b_at > 0xffffffffull)
      throw RuntimeError("interaction lists too long for 32 bit offsets");
    ws.cell_list.ensure(std::max<u64>(1, c_at) * 4);
    ws.body_list.ensure(std::max<u64>(1, b_at) * 4);
    ls.pend.ensure(std::max<u64>(1, static_cast<u64>(kParts) * ng * ls.slot_pend) * 4);
    a.slot_pend = ls.slot_pend;
    a.cells = ws.cell_list.as<u32>();
    a.bodies = ws.body_list.as<u32>();
    a.pend = ls.pend.as<u32>();
    GTC_CUDA(cudaMemsetAsync(&sc->cell_interactions, 0, 3 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_group, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(&sc->list_overflow, 0, sizeof(u32), s));
    GTC_CUDA(cudaMemsetAsync(sc->lmax_cells, 0,
                             offsetof(Scalars, max_pend) + sizeof(u32) -
                                 offsetof(Scalars, lmax_cells),
                             s));  // lmax_cells, lmax_bodies, max_pend
    GTC_CUDA(cudaMemsetAsync(&sc->walk_nodes, 0, sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->mlp_rows, 0, 2 * sizeof(unsigned long long), s));
    GTC_CUDA(cudaMemsetAsync(&sc->max_rows, 0, sizeof(u32), s));
    u32 *roff = ls.roff.as<u32>();
    int qsel = 0;
    // one round: its walk, the warps' continuations, and the scan of the
    // pairs it deferred (their total at roff[nparts])
    auto walk_round = [&](u32 r) {
      if (r >= static_cast<u32>(kMaxRounds))
        throw RuntimeError("learned walk: more rounds than the tree has levels");
      if (r > 0) {
        a.rows = ls.q[qsel].as<uint2>();
        a.dec = ls.dec[qsel].as<u8>();
      }
      if (warps) {
        GTC_CUDA(cudaMemsetAsync(a.next, 0, sizeof(u32), s));
        k_lwarp<<<warp_blocks, kLWarps * 32, 0, s>>>(a, r);
        GTC_LAUNCH_CHECK();
      } else {
        GTC_CUDA(cudaMemsetAsync(&sc->lcont, 0, 2 * sizeof(u32), s));
        a.budget = r == 0 ? lw.walk_budget : lw.pair_budget;
        if (r == 0)
          k_lround0<<<rb, kRoundThreads, 0, s>>>(a);
        else
          k_lround<<<rb, kRoundThreads, 0, s>>>(a);
        GTC_LAUNCH_CHECK();
        k_lcont<<<cont_blocks, kContWarps * 32, 0, s>>>(a, r > 0);
        GTC_LAUNCH_CHECK();
      }
      exclusive_scan_u32(a.pcount, roff, nparts, roff + nparts, ws.scan_tmp, s);
    };
    // the round's deferred pairs as rows, and the network's decisions on
    // them: `launch_rows` rows' worth of blocks, the count read on the device
    auto decide = [&](u64 launch_rows) {
      const int nq = qsel ^ 1;
      const u64 cap = std::min<u64>(ls.q[nq].bytes / sizeof(uint2), ls.dec[nq].bytes);  // rows held
      k_lrows<<<pb, kT, 0, s>>>(a, ls.q[nq].as<uint2>(), cap);
      GTC_LAUNCH_CHECK();
      if (launch_rows > 0) {
        k_ldecide<<<ceil_div(launch_rows, kT), kT, 0, s>>>(
            ls.q[nq].as<uint2>(), launch_rows, a.lrec, lw.cfeat, a.gboxf, a.gtol, lw.net,
            ws.root.as<TreeRoot>(), a.mom, ls.dec[nq].as<u8>(), roff + nparts,
            &sc->list_overflow);
        GTC_LAUNCH_CHECK();
      }
      qsel = nq;
    };
    // the last round's deferred pairs and the flags; true on overflow
    u32 deferred = 0;
    auto read_back = [&]() {
      u32 flags[2] = {0, 0};
      GTC_CUDA(cudaMemcpyAsync(&deferred, roff + nparts, sizeof(u32), cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaMemcpyAsync(flags, &sc->list_overflow, sizeof(u32), cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaMemcpyAsync(flags + 1, &sc->error, sizeof(u32), cudaMemcpyDeviceToHost, s));
      GTC_CUDA(cudaStreamSynchronize(s));
      if (flags[1])
        throw RuntimeError("cuda: inconsistent tree detected on the device (code " +
                           std::to_string(flags[1]) + ")");
      return flags[0] != 0;
    };
    bool overflow = false;
    rounds = 0;
    if (lw.plan_rounds && ls.rounds > 0 && ls.row_cap > 0) {
      // as many rounds as the last walk, with buffers for its largest one,
      // and one read back at the end
      for (int k = 0; k < 2; ++k) {
        ls.q[k].ensure(static_cast<u64>(ls.row_cap) * sizeof(uint2));
        ls.dec[k].ensure(ls.row_cap);
      }
      for (; rounds < ls.rounds; ++rounds) {
        walk_round(rounds);
        decide(ls.row_cap);
      }
      overflow = read_back();
    }
    // then one read back per round until a round defers nothing (the last
    // planned round's pairs are decided already)
    if (!overflow && (rounds == 0 || deferred > 0)) {
      for (;;) {
        walk_round(rounds);
        ++rounds;
        overflow = read_back();
        if (overflow || deferred == 0) break;
        const int nq = qsel ^ 1;
        ls.q[nq].ensure(static_cast<u64>(deferred) * sizeof(uint2));
        ls.dec[nq].ensure(deferred);
        decide(deferred);
      }
    }
    if (!overflow) break;
    // a slot or the rows outgrew their buffers: the counts went on, so
    // buffers of their size fit; walk again from the start
    Scalars h{};
    GTC_CUDA(cudaMemcpyAsync(&h, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    GTC_CUDA(cudaStreamSynchronize(s));
    if (attempt >= 4) {
      std::string m = "learned walk: the list slots keep overflowing (round " +
                      std::to_string(rounds) + "; slot / longest:";
      for (int k = 0; k < kParts; ++k)
        m += " " + std::to_string(ls.slot_cells[k]) + "/" + std::to_string(h.lmax_cells[k]) + " " +
             std::to_string(ls.slot_bodies[k]) + "/" + std::to_string(h.lmax_bodies[k]);
      m += " pend " + std::to_string(ls.slot_pend) + "/" + std::to_string(h.max_pend) +
           "; rows " + std::to_string(ls.row_cap) + "/" + std::to_string(h.max_rows) + ")";
      throw RuntimeError(m);
    }
    for (int k = 0; k < kParts; ++k) {
      ls.slot_cells[k] = std::max<u32>(ls.slot_cells[k], learned_slot(h.lmax_cells[k]));
      ls.slot_bodies[k] = std::max<u32>(ls.slot_bodies[k], learned_slot(h.lmax_bodies[k]));
    }
    ls.slot_pend = std::max<u32>(ls.slot_pend, learned_slot(h.max_pend));
    if (h.list_overflow & 2u) ls.row_cap = std::max<u32>(ls.row_cap, learned_slot(h.max_rows));
  }
  // group records and statistics
  GTC_CUDA(cudaMemsetAsync(&sc->n_cell_list, 0, 2 * sizeof(u64), s));
  k_lgroup_records<<<gb, kT, 0, s>>>(a, ws.gbegin.as<u32>(), ws.gend.as<u32>(),
                                     ws.groups.as<uint4>());
  GTC_LAUNCH_CHECK();
  GTC_CUDA(cudaMemcpyAsync(host, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
  ws.n_cell_list = host->n_cell_list;
  ws.n_body_list = host->n_body_list;
  ws.gapped = true;
  ws.list_passes = rounds;
  // slots for the next learned walk, from this one's longest lists
  for (int k = 0; k < kParts; ++k) {
    ls.slot_cells[k] = learned_slot(host->lmax_cells[k]);
    ls.slot_bodies[k] = learned_slot(host->lmax_bodies[k]);
  }
  ls.slot_pend = learned_slot(host->max_pend);
  ls.rounds = rounds;
  ls.row_cap = learned_slot(host->max_rows);
}

}  // namespace gtc
