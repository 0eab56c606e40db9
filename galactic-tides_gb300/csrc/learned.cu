// Learned opening criterion: training samples labelled by FP64 direct sums,
// the training kernels (forward, backward, Adam) and the model's set-up.
// The walk that uses the model is in learned_walk.cu.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "context.cuh"

namespace gtc {
namespace {

constexpr int kT = 256;

__device__ __forceinline__ FeatScale scale_from(const TreeRoot *root, const double2 *mom) {
  return FeatScale{static_cast<float>(1.0 / root->half_at[0]), static_cast<float>(1.0 / mom[1].y)};
}

__device__ __forceinline__ float box_dist2(float mx, float my, float mz, const float *g,
                                           const float *h) {
  const float dx = fmaxf(fabsf(mx - g[0]) - h[0], 0.f), dy = fmaxf(fabsf(my - g[1]) - h[1], 0.f),
              dz = fmaxf(fabsf(mz - g[2]) - h[2], 0.f);
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

__device__ __forceinline__ bool boxes_overlap(const WalkRec32 &r, const float *g, const float *h) {
  return fabsf(r.cx - g[0]) <= r.slack + h[0] && fabsf(r.cy - g[1]) <= r.slack + h[1] &&
         fabsf(r.cz - g[2]) <= r.slack + h[2];
}

__device__ __forceinline__ void group_box(const float *gboxf, u32 g, float *gf, float *hf) {
  for (int a = 0; a < 3; ++a) {
    gf[a] = gboxf[8ull * g + a];
    hf[a] = gboxf[8ull * g + 3 + a];
  }
}

// Candidate (group, cell) pairs: one thread per sampled group walks the tree
// opening every node that a tight opening angle theta_gen opens, and
// records each visited cell of more than two bodies that passes the learned
// walk's guard (no overlap, beyond 2 h / theta_guard + delta): the cells a
// learned walk may have to decide about, from far and well separated to
// close to the guard.
__global__ void __launch_bounds__(kT)
    k_sample_pairs(const WalkRec32 *walk32, const CellFeat *cfeat, u32 m, const float *gboxf,
                   u32 ng, u32 group_stride, u32 group_offset, float inv_theta_gen,
                   float inv_theta_guard, uint2 *pairs, u32 capacity, u32 *count) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  const u64 g64 = static_cast<u64>(k) * group_stride + group_offset;
  if (g64 >= ng) return;
  const u32 g = static_cast<u32>(g64);
  float gf[3], hf[3];
  group_box(gboxf, g, gf, hf);
  u32 i = 0;
  while (i < m) {
    const WalkRec32 r = walk32[i];
    const CellFeat c = cfeat[i];
    const float d2 = box_dist2(r.mx, r.my, r.mz, gf, hf);
    const bool overlap = boxes_overlap(r, gf, hf);
    const float cg = fmaf(2.f * c.half, inv_theta_gen, c.delta);
    const float cq = fmaf(2.f * c.half, inv_theta_guard, c.delta);
    const u32 nbody = r.nbody_leaf & 0x7fffffffu;
    const bool leaf = r.nbody_leaf >> 31;
    if (!overlap && d2 > cq * cq && nbody > kFewBodies) {
      const u32 slot = atomicAdd(count, 1u);
      if (slot < capacity) pairs[slot] = make_uint2(g, i);
    }
    if ((!overlap && d2 > cg * cg) || leaf) {
      if (r.skip <= i) break;
      i = r.skip;
    } else {
      ++i;
    }
  }
}

// Features of each sampled pair, computed as the learned walk computes them.
__global__ void __launch_bounds__(kT)
    k_pair_features(const uint2 *pairs, u32 np, const WalkRec32 *walk32, const CellFeat *cfeat,
                    const float *gboxf, const TreeRoot *root, const double2 *mom, float *feat) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= np) return;
  const FeatScale fs = scale_from(root, mom);
  const u32 g = pairs[k].x, p = pairs[k].y;
  float gf[3], hf[3];
  group_box(gboxf, g, gf, hf);
  const WalkRec32 r = walk32[p];
  const CellFeat c = cfeat[p];
  const float f[kFeat] = {group_feature(fmaxf(hf[0], fmaxf(hf[1], hf[2])), fs), c.f1,
                          distance_feature(box_dist2(r.mx, r.my, r.mz, gf, hf), fs), c.f3, c.f4,
                          c.f5};
  for (int j = 0; j < kFeat; ++j) feat[static_cast<u64>(k) * kFeat + j] = f[j];
}

// Label of each pair, FP64: the largest |a_multipole - a_exact| over the
// group's targets, where a_exact sums the cell's bodies one by one and
// a_multipole is the cell's monopole + quadrupole field as the list
// evaluator computes it (gravity_kernels.h:109-135), softened alike.
// One warp per pair, lane = target. Cells of more than `max_bodies` bodies
// get NaN and are dropped from the set.
constexpr u32 kLabelWarps = 4;

__global__ void __launch_bounds__(32 * kLabelWarps)
    k_pair_labels(const uint2 *pairs, u32 np, const u32 *gbegin, const u32 *gend,
                  const u32 *nbegin, const u32 *nend, const double *tpos, const double *tmass,
                  const double2 *mom, const double2 *quad, const TreeRoot *root, double G,
                  double eps2, u32 max_bodies, float *label) {
  const u32 k = blockIdx.x * kLabelWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= np) return;
  const u32 g = pairs[k].x, p = pairs[k].y;
  const u32 b0 = nbegin[p], b1 = nend[p];
  if (b1 - b0 > max_bodies) {
    if (lane == 0) label[k] = __int_as_float(0x7fc00000);
    return;
  }
  const u32 t = gbegin[g] + lane;
  const bool active = t < gend[g];
  const double x = active ? tpos[3ull * t] : 0.0, y = active ? tpos[3ull * t + 1] : 0.0,
               z = active ? tpos[3ull * t + 2] : 0.0;
  double ex = 0, ey = 0, ez = 0;
  for (u32 j = b0; j < b1; ++j) {
    const double dx = x - tpos[3ull * j], dy = y - tpos[3ull * j + 1], dz = z - tpos[3ull * j + 2];
    const double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps2);
    const double s = G * tmass[j] * inv * inv * inv;
    ex -= s * dx;
    ey -= s * dy;
    ez -= s * dz;
  }
  const double2 c0 = mom[2 * p], c1 = mom[2 * p + 1];
  const double2 qa = quad[3 * p], qb = quad[3 * p + 1], qc = quad[3 * p + 2];  // xx yy | zz xy | xz yz
  const double dx = x - c0.x, dy = y - c0.y, dz = z - c1.x;
  const double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps2);
  const double inv3 = inv * inv * inv, inv5 = inv3 * inv * inv, inv7 = inv5 * inv * inv;
  const double gm3 = G * c1.y * inv3;
  const double qx = qa.x * dx + qb.y * dy + qc.x * dz;
  const double qy = qb.y * dx + qa.y * dy + qc.y * dz;
  const double qz = qc.x * dx + qc.y * dy + qb.x * dz;
  const double rqr = dx * qx + dy * qy + dz * qz;
  const double mx = -gm3 * dx + G * (qx * inv5 - 2.5 * rqr * dx * inv7);
  const double my = -gm3 * dy + G * (qy * inv5 - 2.5 * rqr * dy * inv7);
  const double mz = -gm3 * dz + G * (qz * inv5 - 2.5 * rqr * dz * inv7);
  double err = active ? sqrt((mx - ex) * (mx - ex) + (my - ey) * (my - ey) + (mz - ez) * (mz - ez))
                      : 0.0;
  for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_xor_sync(kFullMask, err, o));
  if (lane == 0) {
    const double L = root->half_at[0], unit = L * L / (G * mom[1].y);
    label[k] = static_cast<float>(log2(fmax(err * unit, 1e-30)));
  }
}

__global__ void __launch_bounds__(kT) k_finite_flags(const float *label, u32 np, u32 *flag) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k < np) flag[k] = isfinite(label[k]) ? 1u : 0u;
}

__global__ void __launch_bounds__(kT)
    k_append_samples(const u32 *flag, const u32 *scan, u32 np, const float *feat,
                     const float *label, const uint2 *pairs, u64 base, float *set_feat,
                     float *set_label, uint2 *set_pair) {
  const u32 k = blockIdx.x * kT + threadIdx.x;
  if (k >= np || !flag[k]) return;
  const u64 o = base + scan[k];
  for (int j = 0; j < kFeat; ++j) set_feat[o * kFeat + j] = feat[static_cast<u64>(k) * kFeat + j];
  set_label[o] = label[k];
  set_pair[o] = pairs[k];
}

// ------------------------------------------------------------------ training

// Training target: the label minus the prior (the network learns the
// correction), in log2 units.
__device__ __forceinline__ float residual(const float *f, float label) {
  return label - prior_log2err(kPriorBase + f[3] + 3.f * f[1], f[2]);
}

// Per-block sums and sums of squares of the six features and the residual,
// FP64 (block order kept, so the host's total is deterministic).
constexpr int kStatBlocks = 256;
constexpr int kStats = 2 * (kFeat + 1);

__global__ void __launch_bounds__(kT)
    k_stat_partials(const float *feat, const float *label, u64 n, double *part) {
  __shared__ double s[kStats][kT / 32];
  double acc[kStats] = {};
  for (u64 k = static_cast<u64>(blockIdx.x) * kT + threadIdx.x; k < n;
       k += static_cast<u64>(gridDim.x) * kT) {
    const float *f = feat + k * kFeat;
    for (int j = 0; j < kFeat; ++j) {
      acc[j] += f[j];
      acc[kFeat + 1 + j] += static_cast<double>(f[j]) * f[j];
    }
    const double y = residual(f, label[k]);
    acc[kFeat] += y;
    acc[2 * kFeat + 1] += y * y;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = 0; j < kStats; ++j) {
    double v = acc[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    if (lane == 0) s[j][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < kStats) {
    double v = 0;
    for (int w = 0; w < kT / 32; ++w) v += s[threadIdx.x][w];
    part[blockIdx.x * kStats + threadIdx.x] = v;
  }
}

// Stateless sample index for (seed, step, slot): a 64-bit mix.
__device__ __forceinline__ u64 mix64(u64 x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

constexpr int kTB = 128;        // samples per training block
constexpr int kLd = kHid + 1;   // padded row length of the shared activations

// One block: kTB samples, forward and backward of the mean squared error
// (normalised units), the block's summed gradient into part[blockIdx.x] and
// its summed squared error into loss[blockIdx.x]. With `fixed` non-null the
// samples are fixed[0..batch) instead of random draws (gradient checks).
__global__ void __launch_bounds__(kTB)
    k_train_block(const float *__restrict__ model, const float *__restrict__ feat,
                  const float *__restrict__ label, u64 nsamples, u64 seed, u64 step, u32 batch,
                  const u32 *fixed, float *part, float *loss) {
  extern __shared__ float smem[];
  float *sP = smem;                       // kModelFloats (+ padding)
  float *sZ1 = sP + kModelFloats + 4;     // kTB x kLd  (pre-activations, layer 1)
  float *sZ2 = sZ1 + kTB * kLd;           // kTB x kLd  (pre-activations, layer 2)
  float *sD1 = sZ2 + kTB * kLd;           // kTB x kLd  (dL/dz1)
  float *sD2 = sD1 + kTB * kLd;           // kTB x kLd  (dL/dz2)
  float *sX = sD2 + kTB * kLd;            // kTB x kFeat
  float *sG = sX + kTB * kFeat;           // kTB        (dL/dout)
  __shared__ float sLoss[kTB / 32];
  for (int i = threadIdx.x; i < kModelFloats; i += kTB) sP[i] = model[i];
  __syncthreads();
  const float *W1 = sP + kOffW1, *B1 = sP + kOffB1, *W2 = sP + kOffW2, *B2 = sP + kOffB2,
              *W3 = sP + kOffW3;
  const float b3 = sP[kOffB3], ymean = sP[kOffYMean], ystd = sP[kOffYStd];
  const int t = threadIdx.x;
  const u32 slot = blockIdx.x * kTB + t;
  const bool valid = slot < batch;
  u64 s = 0;
  if (valid)
    s = fixed ? fixed[slot] : mix64(seed * 0x9e3779b97f4a7c15ull + step * batch + slot) % nsamples;
  float x[kFeat], y = 0.f;
  const float *f = feat + s * kFeat;
  for (int j = 0; j < kFeat; ++j) {
    x[j] = valid ? (f[j] - sP[kOffMean + j]) / sP[kOffStd + j] : 0.f;
    sX[t * kFeat + j] = x[j];
  }
  if (valid) y = (residual(f, label[s]) - ymean) / ystd;
  float *z1 = sZ1 + t * kLd, *z2 = sZ2 + t * kLd, *d1 = sD1 + t * kLd, *d2 = sD2 + t * kLd;
  for (int h = 0; h < kHid; ++h) {
    float a = B1[h];
    for (int j = 0; j < kFeat; ++j) a = fmaf(x[j], W1[j * kHid + h], a);
    z1[h] = a;
  }
  for (int h = 0; h < kHid; ++h) {
    float a = B2[h];
    for (int i = 0; i < kHid; ++i) a = fmaf(fmaxf(z1[i], 0.f), W2[i * kHid + h], a);
    z2[h] = a;
  }
  float out = b3;
  for (int h = 0; h < kHid; ++h) out = fmaf(fmaxf(z2[h], 0.f), W3[h], out);
  const float err = valid ? out - y : 0.f;
  const float gout = 2.f * err / static_cast<float>(batch);
  sG[t] = gout;
  for (int h = 0; h < kHid; ++h) d2[h] = z2[h] > 0.f ? gout * W3[h] : 0.f;
  for (int i = 0; i < kHid; ++i) {
    float a = 0.f;
    for (int h = 0; h < kHid; ++h) a = fmaf(W2[i * kHid + h], d2[h], a);
    d1[i] = z1[i] > 0.f ? a : 0.f;
  }
  float l = err * err;
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(kFullMask, l, o);
  if ((t & 31) == 0) sLoss[t >> 5] = l;
  __syncthreads();
  float *P = part + static_cast<u64>(blockIdx.x) * kParams;
  // weight gradients: sums over the block's samples
  for (int e = t; e < kHid * kHid; e += kTB) {
    const int i = e / kHid, h = e % kHid;
    float a = 0.f;
    for (int r = 0; r < kTB; ++r) a = fmaf(fmaxf(sZ1[r * kLd + i], 0.f), sD2[r * kLd + h], a);
    P[kOffW2 + e] = a;
  }
  for (int e = t; e < kFeat * kHid; e += kTB) {
    const int j = e / kHid, h = e % kHid;
    float a = 0.f;
    for (int r = 0; r < kTB; ++r) a = fmaf(sX[r * kFeat + j], sD1[r * kLd + h], a);
    P[kOffW1 + e] = a;
  }
  if (t < kHid) {
    float a1 = 0.f, a2 = 0.f, a3 = 0.f;
    for (int r = 0; r < kTB; ++r) {
      a1 += sD1[r * kLd + t];
      a2 += sD2[r * kLd + t];
      a3 = fmaf(sG[r], fmaxf(sZ2[r * kLd + t], 0.f), a3);
    }
    P[kOffB1 + t] = a1;
    P[kOffB2 + t] = a2;
    P[kOffW3 + t] = a3;
  }
  if (t == kHid) {
    float a = 0.f;
    for (int r = 0; r < kTB; ++r) a += sG[r];
    P[kOffB3] = a;
  }
  if (t == 0) {
    float a = 0.f;
    for (int w = 0; w < kTB / 32; ++w) a += sLoss[w];
    loss[blockIdx.x] = a;
  }
}

// Sums the blocks' gradients in block order (deterministic); with lr > 0
// also takes one Adam step (beta1 0.9, beta2 0.999, eps 1e-8).
__global__ void __launch_bounds__(kT)
    k_reduce_adam(const float *part, u32 nblocks, float *grad, float *model, float *m, float *v,
                  float lr, float b1t, float b2t) {
  const u32 p = blockIdx.x * kT + threadIdx.x;
  if (p >= kParams) return;
  float g = 0.f;
  for (u32 b = 0; b < nblocks; ++b) g += part[static_cast<u64>(b) * kParams + p];
  grad[p] = g;
  if (lr > 0.f) {
    const float mm = 0.9f * m[p] + 0.1f * g, vv = 0.999f * v[p] + 0.001f * g * g;
    m[p] = mm;
    v[p] = vv;
    model[p] -= lr * (mm / (1.f - b1t)) / (sqrtf(vv / (1.f - b2t)) + 1e-8f);
  }
}

size_t train_smem_bytes() {
  return (kModelFloats + 4 + 4 * kTB * kLd + kTB * kFeat + kTB) * sizeof(float);
}

// Histogram of |y_std net(x)|, the correction about its mean y_mean, in
// 1/16 log2 units (FP32 forward), for the walk's band.
constexpr int kBandBins = 1024;

__global__ void __launch_bounds__(kT)
    k_band_hist(const float *model, const float *feat, u64 n, u64 stride, u32 *hist) {
  __shared__ float sP[kModelFloats];
  __shared__ u32 sh[kBandBins];
  for (int i = threadIdx.x; i < kModelFloats; i += kT) sP[i] = model[i];
  for (int i = threadIdx.x; i < kBandBins; i += kT) sh[i] = 0;
  __syncthreads();
  const u64 k = (static_cast<u64>(blockIdx.x) * kT + threadIdx.x) * stride;
  if (k < n) {
    float x[kFeat], z1[kHid];
    for (int j = 0; j < kFeat; ++j)
      x[j] = (feat[k * kFeat + j] - sP[kOffMean + j]) / sP[kOffStd + j];
    for (int h = 0; h < kHid; ++h) {
      float a = sP[kOffB1 + h];
      for (int j = 0; j < kFeat; ++j) a = fmaf(x[j], sP[kOffW1 + j * kHid + h], a);
      z1[h] = fmaxf(a, 0.f);
    }
    float out = sP[kOffB3];
    for (int h = 0; h < kHid; ++h) {
      float a = sP[kOffB2 + h];
      for (int i = 0; i < kHid; ++i) a = fmaf(z1[i], sP[kOffW2 + i * kHid + h], a);
      out = fmaf(fmaxf(a, 0.f), sP[kOffW3 + h], out);
    }
    const float corr = fabsf(sP[kOffYStd] * out);  // about the mean correction y_mean
    const int bin = corr < kBandBins / 16.f ? static_cast<int>(corr * 16.f) : kBandBins - 1;
    atomicAdd(&sh[bin], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kBandBins; i += kT)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

void read_back(void *dst, const void *src, size_t bytes, cudaStream_t s) {
  GTC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
  GTC_CUDA(cudaStreamSynchronize(s));
}

// Uniform in [-1, 1) from a counter (the same on every host).
double unit_uniform(u64 seed, u64 i) {
  u64 x = seed * 0x9e3779b97f4a7c15ull + i + 1;
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return static_cast<double>(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

}  // namespace

void learned_add_samples(gtc_context *ctx, const double *pos, const double *mass, u64 n,
                         const SolverParams &sp, double theta_gen, double theta_guard,
                         u64 max_new, u32 max_cell_bodies, u64 *added) {
  *added = 0;
  if (n == 0 || max_new == 0) return;
  cudaStream_t s = ctx->stream;
  Workspace &ws = ctx->ws;
  const SideJoin side_join{ws, s};
  build_tree(ws, pos, mass, n, sp, s, ctx->host_sc);
  build_lists(ws, sp, s, ctx->host_sc);
  const u32 m = static_cast<u32>(ws.n_nodes), ng = static_cast<u32>(ws.n_groups);
  learned_node_features(ws, ctx->cfeat, s);
  const CellFeat *cfeat = ctx->cfeat.as<CellFeat>();
  DeviceBuffer pairs, cnt, feat, label, flag, scan;
  struct Release {
    DeviceBuffer *b[6];
    ~Release() {
      for (DeviceBuffer *x : b) x->release();
    }
  } release{{&pairs, &cnt, &feat, &label, &flag, &scan}};
  const float igen = static_cast<float>(1.0 / theta_gen),
              iguard = static_cast<float>(1.0 / theta_guard);
  // a first pass counts every group's pairs; a group stride then keeps the
  // set near max_new
  cnt.ensure(sizeof(u32));
  pairs.ensure(sizeof(uint2));
  GTC_CUDA(cudaMemsetAsync(cnt.ptr, 0, sizeof(u32), s));
  k_sample_pairs<<<ceil_div(ng, kT), kT, 0, s>>>(ws.walk32.as<WalkRec32>(), cfeat, m,
                                                 ws.gboxf.as<float>(), ng, 1, 0, igen, iguard,
                                                 pairs.as<uint2>(), 0, cnt.as<u32>());
  GTC_LAUNCH_CHECK();
  u32 all = 0;
  read_back(&all, cnt.ptr, sizeof(u32), s);
  if (all == 0) return;
  const u32 stride = static_cast<u32>(std::max<u64>(1, (all + max_new - 1) / max_new));
  const u32 groups_used = (ng + stride - 1) / stride;
  const u32 cap = static_cast<u32>(std::min<u64>(all, 2 * max_new + 1024));
  pairs.ensure(static_cast<u64>(cap) * sizeof(uint2));
  GTC_CUDA(cudaMemsetAsync(cnt.ptr, 0, sizeof(u32), s));
  k_sample_pairs<<<ceil_div(groups_used, kT), kT, 0, s>>>(
      ws.walk32.as<WalkRec32>(), cfeat, m, ws.gboxf.as<float>(), ng, stride, stride / 2, igen,
      iguard, pairs.as<uint2>(), cap, cnt.as<u32>());
  GTC_LAUNCH_CHECK();
  u32 np = 0;
  read_back(&np, cnt.ptr, sizeof(u32), s);
  np = static_cast<u32>(std::min<u64>(std::min(np, cap), max_new));
  if (np == 0) return;
  feat.ensure(static_cast<u64>(np) * kFeat * sizeof(float));
  label.ensure(static_cast<u64>(np) * sizeof(float));
  k_pair_features<<<ceil_div(np, kT), kT, 0, s>>>(pairs.as<uint2>(), np, ws.walk32.as<WalkRec32>(),
                                                  cfeat, ws.gboxf.as<float>(),
                                                  ws.root.as<TreeRoot>(), ws.mom.as<double2>(),
                                                  feat.as<float>());
  GTC_LAUNCH_CHECK();
  k_pair_labels<<<ceil_div(np, kLabelWarps), 32 * kLabelWarps, 0, s>>>(
      pairs.as<uint2>(), np, ws.gbegin.as<u32>(), ws.gend.as<u32>(), ws.nbegin.as<u32>(),
      ws.nend.as<u32>(), ws.tpos.as<double>(), ws.tmass.as<double>(), ws.mom.as<double2>(),
      ws.quad.as<double2>(), ws.root.as<TreeRoot>(), sp.G, sp.eps * sp.eps, max_cell_bodies,
      label.as<float>());
  GTC_LAUNCH_CHECK();
  flag.ensure(static_cast<u64>(np) * 4);
  scan.ensure(static_cast<u64>(np) * 4 + 8);
  k_finite_flags<<<ceil_div(np, kT), kT, 0, s>>>(label.as<float>(), np, flag.as<u32>());
  GTC_LAUNCH_CHECK();
  u32 *kept_dev = scan.as<u32>() + np;
  exclusive_scan_u32(flag.as<u32>(), scan.as<u32>(), np, kept_dev, ws.scan_tmp, s);
  u32 kept = 0;
  read_back(&kept, kept_dev, sizeof(u32), s);
  if (kept == 0) return;
  LearnedSet &set = ctx->samples;
  const u64 need = set.count + kept;
  if (need > set.capacity) {
    const u64 cap2 = std::max<u64>(need, set.capacity + set.capacity / 2);
    DeviceBuffer nf, nl, npr;
    try {
      nf.ensure(cap2 * kFeat * sizeof(float));
      nl.ensure(cap2 * sizeof(float));
      npr.ensure(cap2 * sizeof(uint2));
    } catch (...) {
      nf.release();
      nl.release();
      npr.release();
      throw;
    }
    if (set.count) {
      GTC_CUDA(cudaMemcpyAsync(nf.ptr, set.feat.ptr, set.count * kFeat * sizeof(float),
                               cudaMemcpyDeviceToDevice, s));
      GTC_CUDA(cudaMemcpyAsync(nl.ptr, set.label.ptr, set.count * sizeof(float),
                               cudaMemcpyDeviceToDevice, s));
      GTC_CUDA(cudaMemcpyAsync(npr.ptr, set.pair.ptr, set.count * sizeof(uint2),
                               cudaMemcpyDeviceToDevice, s));
      GTC_CUDA(cudaStreamSynchronize(s));
    }
    set.feat.release();
    set.label.release();
    set.pair.release();
    set.feat = nf;
    set.label = nl;
    set.pair = npr;
    set.capacity = cap2;
  }
  k_append_samples<<<ceil_div(np, kT), kT, 0, s>>>(flag.as<u32>(), scan.as<u32>(), np,
                                                   feat.as<float>(), label.as<float>(),
                                                   pairs.as<uint2>(), set.count,
                                                   set.feat.as<float>(), set.label.as<float>(),
                                                   set.pair.as<uint2>());
  GTC_LAUNCH_CHECK();
  GTC_CUDA(cudaStreamSynchronize(s));
  set.count += kept;
  *added = kept;
}

void learned_set_model(gtc_context *ctx, const float *host_model) {
  for (int i = 0; i < kModelFloats; ++i)
    if (!std::isfinite(host_model[i]) && i != kOffBand)
      throw InvalidArgument("model value " + std::to_string(i) + " is not finite");
  for (int j = 0; j < kFeat; ++j)
    if (!(host_model[kOffStd + j] > 0.f)) throw InvalidArgument("feature scales must be positive");
  if (!(host_model[kOffYStd] > 0.f)) throw InvalidArgument("output scale must be positive");
  if (!(host_model[kOffBand] >= 0.f)) throw InvalidArgument("band must be non-negative");
  cudaStream_t s = ctx->stream;
  ctx->model.ensure(kModelFloats * sizeof(float));
  ctx->net.ensure(sizeof(LearnedNet));
  GTC_CUDA(cudaMemcpyAsync(ctx->model.ptr, host_model, kModelFloats * sizeof(float),
                           cudaMemcpyHostToDevice, s));
  learned_prepare_net(ctx->model.as<float>(), ctx->net.as<LearnedNet>(), s);
  GTC_CUDA(cudaStreamSynchronize(s));
  ctx->model_band = host_model[kOffBand];
  ctx->model_ymean = host_model[kOffYMean];
  ctx->have_model = true;
}

// Normalisation from the training set and uniform He initialisation of the
// weights (biases zero) into the context's model; the band starts open.
void learned_init_model(gtc_context *ctx, u64 seed) {
  const LearnedSet &set = ctx->samples;
  if (set.count < 2) throw InvalidArgument("the learned criterion needs training samples first");
  cudaStream_t s = ctx->stream;
  DeviceBuffer part;
  part.ensure(kStatBlocks * kStats * sizeof(double));
  k_stat_partials<<<kStatBlocks, kT, 0, s>>>(set.feat.as<float>(), set.label.as<float>(),
                                             set.count, part.as<double>());
  GTC_LAUNCH_CHECK();
  std::vector<double> hp(kStatBlocks * kStats);
  read_back(hp.data(), part.ptr, hp.size() * sizeof(double), s);
  part.release();
  double sum[kStats] = {};
  for (int b = 0; b < kStatBlocks; ++b)
    for (int j = 0; j < kStats; ++j) sum[j] += hp[b * kStats + j];
  std::vector<float> model(kModelFloats, 0.f);
  const double nn = static_cast<double>(set.count);
  for (int j = 0; j <= kFeat; ++j) {
    const double mean = sum[j] / nn;
    const double var = std::max(sum[kFeat + 1 + j] / nn - mean * mean, 0.0);
    const double sd = std::max(std::sqrt(var), 1e-3);
    if (j < kFeat) {
      model[kOffMean + j] = static_cast<float>(mean);
      model[kOffStd + j] = static_cast<float>(sd);
    } else {
      model[kOffYMean] = static_cast<float>(mean);
      model[kOffYStd] = static_cast<float>(sd);
    }
  }
  const double a1 = std::sqrt(6.0 / kFeat), a2 = std::sqrt(6.0 / kHid), a3 = std::sqrt(3.0 / kHid);
  for (int i = 0; i < kFeat * kHid; ++i)
    model[kOffW1 + i] = static_cast<float>(a1 * unit_uniform(seed, i));
  for (int i = 0; i < kHid * kHid; ++i)
    model[kOffW2 + i] = static_cast<float>(a2 * unit_uniform(seed, 10000 + i));
  for (int i = 0; i < kHid; ++i)
    model[kOffW3 + i] = static_cast<float>(a3 * unit_uniform(seed, 20000 + i));
  model[kOffBand] = 1e30f;
  learned_set_model(ctx, model.data());
}

// Adam on the mean squared error of the correction (normalised units) over
// `steps` random minibatches of the given samples (or, with `fixed`, the
// same batch every step). Returns the last step's mean loss; grad_out
// (host, kParams floats, may be null) receives the last step's gradient.
double learned_train_on(gtc_context *ctx, const float *feat, const float *label, u64 nsamples,
                        u64 steps, u32 batch, float lr, u64 seed, const u32 *fixed,
                        float *grad_out) {
  if (!ctx->have_model) throw InvalidArgument("no model to train (initialise one first)");
  if (batch == 0 || nsamples == 0) throw InvalidArgument("empty training batch");
  cudaStream_t s = ctx->stream;
  const u32 nblocks = ceil_div(batch, kTB);
  const size_t smem = train_smem_bytes();
  GTC_CUDA(cudaFuncSetAttribute(k_train_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem)));
  DeviceBuffer &scr = ctx->train_scratch;
  const u64 part_floats = static_cast<u64>(nblocks) * kParams;
  scr.ensure((part_floats + 3 * kParams + nblocks + 16) * sizeof(float));
  float *part = scr.as<float>();
  float *mom1 = part + part_floats, *mom2 = mom1 + kParams, *grad = mom2 + kParams;
  float *loss = grad + kParams;
  GTC_CUDA(cudaMemsetAsync(mom1, 0, 2 * kParams * sizeof(float), s));
  float *model = ctx->model.as<float>();
  double b1t = 1.0, b2t = 1.0;
  for (u64 k = 0; k < steps; ++k) {
    k_train_block<<<nblocks, kTB, smem, s>>>(model, feat, label, nsamples, seed, k, batch, fixed,
                                             part, loss);
    GTC_LAUNCH_CHECK();
    b1t *= 0.9;
    b2t *= 0.999;
    k_reduce_adam<<<ceil_div(kParams, kT), kT, 0, s>>>(part, nblocks, grad, model, mom1, mom2, lr,
                                                       static_cast<float>(b1t),
                                                       static_cast<float>(b2t));
    GTC_LAUNCH_CHECK();
  }
  std::vector<float> lb(nblocks);
  read_back(lb.data(), loss, nblocks * sizeof(float), s);
  if (grad_out) read_back(grad_out, grad, kParams * sizeof(float), s);
  if (lr > 0.f) {
    learned_prepare_net(model, ctx->net.as<LearnedNet>(), s);
    GTC_CUDA(cudaStreamSynchronize(s));
  }
  double l = 0;
  for (float v : lb) l += v;
  return l / batch;
}

// Band: the `quantile` of |y_std net(x)| over (a stride sample of) the
// training set, plus 1/8 for the BF16 inference, written into the model.
// Where the centred prior (prior + y_mean) lies further than this from the
// tolerance, the network would not change the decision.
void learned_update_band(gtc_context *ctx, double quantile) {
  const LearnedSet &set = ctx->samples;
  if (!ctx->have_model || set.count == 0) return;
  cudaStream_t s = ctx->stream;
  const u64 want = 4u << 20;
  const u64 stride = std::max<u64>(1, set.count / want);
  const u64 used = (set.count + stride - 1) / stride;
  DeviceBuffer hist;
  hist.ensure(kBandBins * sizeof(u32));
  GTC_CUDA(cudaMemsetAsync(hist.ptr, 0, kBandBins * sizeof(u32), s));
  k_band_hist<<<ceil_div(used, kT), kT, 0, s>>>(ctx->model.as<float>(), set.feat.as<float>(),
                                                set.count, stride, hist.as<u32>());
  GTC_LAUNCH_CHECK();
  std::vector<u32> h(kBandBins);
  read_back(h.data(), hist.ptr, kBandBins * sizeof(u32), s);
  hist.release();
  u64 total = 0;
  for (u32 v : h) total += v;
  u64 acc = 0;
  int bin = kBandBins - 1;
  for (int i = 0; i < kBandBins; ++i) {
    acc += h[i];
    if (static_cast<double>(acc) >= quantile * static_cast<double>(total)) {
      bin = i;
      break;
    }
  }
  const float band = bin == kBandBins - 1 ? 1e30f : (bin + 1) / 16.f + 0.125f;
  GTC_CUDA(cudaMemcpyAsync(ctx->model.as<float>() + kOffBand, &band, sizeof(float),
                           cudaMemcpyHostToDevice, s));
  learned_prepare_net(ctx->model.as<float>(), ctx->net.as<LearnedNet>(), s);
  GTC_CUDA(cudaStreamSynchronize(s));
  ctx->model_band = band;
}

}  // namespace gtc
