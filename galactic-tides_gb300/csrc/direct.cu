// Direct summation: the tiled FP32 kernel that replaces the reference's
// gt_direct (src/metal/gravity_kernels.metal:18-43; arithmetic of gt_body,
// gravity_kernels.h:71-83), and an FP64 kernel for a sample of targets, the
// accuracy judge of the reference bench (apps/galactic_tides_bench.cpp:74-95)
// and compute_gravity_direct (src/gravity.cpp:28-45).

#include <algorithm>

#include "pipeline.cuh"

namespace gtc {
namespace {

// ------------------------------------------------------------------ FP32

constexpr int kDT = 128;          // threads per block = sources per shared tile
constexpr float kFar = 1e15f;     // padding source: far away, zero mass, adds exactly 0

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// Two sources (one in each half of a float2) against one target: FFMA2 /
// FMUL2 / FADD2 do both at once, the two rsqrts go to the SFU. The source
// pair is (x0, x1, y0, y1), (z0, z1, Gm0, Gm1); the target's coordinates are
// negated and doubled (-x, -x). With kMask, `skip` zeroes the half whose
// source is the target itself (the reference skips j == i), before its
// singular 1/r can reach the sums.
template <bool kMask>
__device__ __forceinline__ void add_pair(const float4 s0, const float4 s1, const float2 nx,
                                         const float2 ny, const float2 nz, const float2 e2,
                                         float2 &ax, float2 &ay, float2 &az, float2 &pt,
                                         bool skip0 = false, bool skip1 = false) {
  const float2 dx = __fadd2_rn(f2(s0.x, s0.y), nx);  // source - target
  const float2 dy = __fadd2_rn(f2(s0.z, s0.w), ny);
  const float2 dz = __fadd2_rn(f2(s1.x, s1.y), nz);
  const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
  // (r^2 >= eps^2; without softening only pairs closer than ~1e-19 could
  // give a subnormal r^2, whose 1/r is meaningless either way)
  float2 inv = f2(rsqrt_normal(r2.x), rsqrt_normal(r2.y));
  if (kMask) {
    inv.x = skip0 ? 0.f : inv.x;
    inv.y = skip1 ? 0.f : inv.y;
  }
  const float2 gm = __fmul2_rn(f2(s1.z, s1.w), inv);
  const float2 gm3 = __fmul2_rn(gm, __fmul2_rn(inv, inv));
  ax = __ffma2_rn(gm3, dx, ax);
  ay = __ffma2_rn(gm3, dy, ay);
  az = __ffma2_rn(gm3, dz, az);
  pt = __fadd2_rn(pt, gm);
}

// Block (bx, by) owns targets [bx kR kDT, (bx + 1) kR kDT) -- thread t the
// targets bx kR kDT + r kDT + t, r < kR (the tile shape: more targets per
// thread reuse each staged source more, fewer leave registers for more
// warps) -- and sums the sources of slice by,
// [by len, (by + 1) len), streamed through shared memory in index order,
// kDT at a time. Even and odd sources go to the two halves of each sum.
// Only the tiles holding the block's own targets test j == i. With one
// slice the sums go straight to `out`, otherwise to part[by][target],
// added up in slice order by k_direct_sum (deterministic).
template <int kDR>
__global__ void __launch_bounds__(kDT)
    k_direct(const float4 *__restrict__ bodies, u32 n, u32 len, float G, float eps2,
             float4 *__restrict__ out) {
  constexpr u32 kDTB = kDT * kDR;  // targets per block
  __shared__ float4 tile[kDT];  // kDT / 2 source pairs, two float4 each
  const u32 t0 = blockIdx.x * kDTB;
  const u32 j0 = blockIdx.y * len, j1 = min(n, j0 + len);
  const float2 e2 = f2(eps2, eps2);
  u32 ti[kDR];
  float2 nx[kDR], ny[kDR], nz[kDR], ax[kDR], ay[kDR], az[kDR], pt[kDR];
#pragma unroll
  for (int r = 0; r < kDR; ++r) {
    ti[r] = t0 + r * kDT + threadIdx.x;
    const float4 p = ti[r] < n ? bodies[ti[r]] : make_float4(0.f, 0.f, 0.f, 0.f);
    nx[r] = f2(-p.x, -p.x);
    ny[r] = f2(-p.y, -p.y);
    nz[r] = f2(-p.z, -p.z);
    ax[r] = ay[r] = az[r] = pt[r] = f2(0.f, 0.f);
  }
  float *tf = reinterpret_cast<float *>(tile);
  const u32 pair = threadIdx.x >> 1, half = threadIdx.x & 1;
  for (u32 base = j0; base < j1; base += kDT) {
    const u32 j = base + threadIdx.x;
    const float4 b = j < j1 ? bodies[j] : make_float4(kFar, kFar, kFar, 0.f);
    tf[8 * pair + half] = b.x;
    tf[8 * pair + 2 + half] = b.y;
    tf[8 * pair + 4 + half] = b.z;
    tf[8 * pair + 6 + half] = G * b.w;
    __syncthreads();
    const bool own = base < t0 + kDTB && base + kDT > t0;
    if (!own) {
#pragma unroll 4
      for (int q = 0; q < kDT / 2; ++q) {
        const float4 s0 = tile[2 * q], s1 = tile[2 * q + 1];
#pragma unroll
        for (int r = 0; r < kDR; ++r)
          add_pair<false>(s0, s1, nx[r], ny[r], nz[r], e2, ax[r], ay[r], az[r], pt[r]);
      }
    } else {
      for (int q = 0; q < kDT / 2; ++q) {
        const float4 s0 = tile[2 * q], s1 = tile[2 * q + 1];
        const u32 js = base + 2 * q;
#pragma unroll
        for (int r = 0; r < kDR; ++r)
          add_pair<true>(s0, s1, nx[r], ny[r], nz[r], e2, ax[r], ay[r], az[r], pt[r],
                         ti[r] == js, ti[r] == js + 1);
      }
    }
    __syncthreads();
  }
  float4 *dst = out + static_cast<u64>(blockIdx.y) * n;
#pragma unroll
  for (int r = 0; r < kDR; ++r)
    if (ti[r] < n)
      dst[ti[r]] = make_float4(ax[r].x + ax[r].y, ay[r].x + ay[r].y, az[r].x + az[r].y,
                               -(pt[r].x + pt[r].y));
}

// out[i] = the sum of the slices' partial sums of target i, in slice order.
__global__ void k_direct_sum(const float4 *__restrict__ part, u32 n, u32 slices,
                             float4 *__restrict__ out) {
  const u32 i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  float4 a = part[i];
  for (u32 k = 1; k < slices; ++k) {
    const float4 v = part[static_cast<u64>(k) * n + i];
    a.x += v.x;
    a.y += v.y;
    a.z += v.z;
    a.w += v.w;
  }
  out[i] = a;
}

// ------------------------------------------------------------------ FP64

constexpr int kST = 128;   // sample targets per block

__device__ __forceinline__ u64 min_u64(u64 a, u64 b) { return a < b ? a : b; }

struct Body64 {
  double x, y, z, m;
};

// Partial sums of targets idx[blockIdx.x*kST + t] over the source slice
// blockIdx.y; slices are reduced in order afterwards (deterministic).
__global__ void __launch_bounds__(kST)
    k_direct64(const double *__restrict__ pos, const double *__restrict__ mass, u64 n,
               const u64 *__restrict__ idx, u64 m, u64 slice, double G, double eps2,
               double2 *part) {
  __shared__ Body64 tile[kST];
  const u64 s = static_cast<u64>(blockIdx.x) * kST + threadIdx.x;
  const bool active = s < m;
  const u64 i = active ? idx[s] : ~0ull;
  double px = 0, py = 0, pz = 0;
  if (active) {
    px = pos[3 * i];
    py = pos[3 * i + 1];
    pz = pos[3 * i + 2];
  }
  double ax = 0, ay = 0, az = 0, phi = 0;
  const u64 j0 = static_cast<u64>(blockIdx.y) * slice;
  const u64 j1 = min_u64(n, j0 + slice);
  for (u64 base = j0; base < j1; base += kST) {
    const u64 j = base + threadIdx.x;
    tile[threadIdx.x] = j < j1 ? Body64{pos[3 * j], pos[3 * j + 1], pos[3 * j + 2], mass[j]}
                               : Body64{0, 0, 0, 0};
    __syncthreads();
    const u64 cnt = min_u64(kST, j1 - base);
    for (u64 k = 0; k < cnt; ++k) {
      if (base + k == i) continue;
      const Body64 b = tile[k];
      const double dx = px - b.x, dy = py - b.y, dz = pz - b.z;
      const double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps2);
      const double gm = G * b.m * inv;
      const double gm3 = gm * inv * inv;
      ax -= gm3 * dx;
      ay -= gm3 * dy;
      az -= gm3 * dz;
      phi -= gm;
    }
    __syncthreads();
  }
  if (active) {
    double2 *o = part + 2 * (static_cast<u64>(blockIdx.y) * m + s);
    o[0] = make_double2(ax, ay);
    o[1] = make_double2(az, phi);
  }
}

__global__ void k_direct64_sum(const double2 *part, u64 m, u32 slices, double *acc, double *pot) {
  const u64 s = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= m) return;
  double ax = 0, ay = 0, az = 0, phi = 0;
  for (u32 k = 0; k < slices; ++k) {
    const double2 *v = part + 2 * (static_cast<u64>(k) * m + s);
    ax += v[0].x;
    ay += v[0].y;
    az += v[1].x;
    phi += v[1].y;
  }
  acc[3 * s] = ax;
  acc[3 * s + 1] = ay;
  acc[3 * s + 2] = az;
  pot[s] = phi;
}

}  // namespace

void direct_fp32(const float4 *bodies, u32 n, float G, float eps2, float4 *out,
                 DeviceBuffer &scratch, cudaStream_t s, int targets) {
  if (n == 0) return;
  if (targets != 2 && targets != 4) throw InvalidArgument("direct_targets must be 2 or 4");
  int dev = 0, sms = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // Enough (target block, source slice) units for about 16 per SM, so that
  // blocks of equal work end close together; each slice at least 8 tiles.
  const u32 tiles = ceil_div(n, kDT * static_cast<u32>(targets));
  u32 slices = std::max<u32>(1, ceil_div(16u * static_cast<u32>(sms), tiles));
  slices = std::min<u32>(slices, std::max<u32>(1, n / (8 * kDT)));
  const u32 len = ceil_div(ceil_div(n, slices), kDT) * kDT;
  slices = ceil_div(n, len);
  float4 *dst = out;
  if (slices > 1) {
    scratch.ensure(static_cast<u64>(slices) * n * sizeof(float4));
    dst = scratch.as<float4>();
  }
  if (targets == 4)
    k_direct<4><<<dim3(tiles, slices), kDT, 0, s>>>(bodies, n, len, G, eps2, dst);
  else
    k_direct<2><<<dim3(tiles, slices), kDT, 0, s>>>(bodies, n, len, G, eps2, dst);
  GTC_LAUNCH_CHECK();
  if (slices > 1) {
    k_direct_sum<<<ceil_div(n, 256), 256, 0, s>>>(dst, n, slices, out);
    GTC_LAUNCH_CHECK();
  }
}

Fp64SamplePlan plan_fp64_sample(u64 n, u64 m, int sms, u64 max_pairs) {
  const u64 tb = (m + kST - 1) / kST;
  u64 slices = std::max<u64>(1, (8ull * static_cast<u64>(sms) + tb - 1) / tb);
  slices = std::min<u64>(slices, std::max<u64>(1, n / kST));
  slices = std::min<u64>(slices, std::max<u64>(1, max_pairs / std::max<u64>(1, m)));
  const u64 slice = std::max<u64>(1, (n + slices - 1) / slices);
  return {std::max<u64>(1, (n + slice - 1) / slice), slice};
}

void launch_fp64_sample(const double *pos, const double *mass, u64 n, const u64 *idx, u64 m,
                        double G, double eps, const Fp64SamplePlan &plan, double2 *part,
                        double *acc, double *pot, cudaStream_t s) {
  dim3 grid(ceil_div(m, kST), static_cast<u32>(plan.slices));
  k_direct64<<<grid, kST, 0, s>>>(pos, mass, n, idx, m, plan.slice, G, eps * eps, part);
  GTC_LAUNCH_CHECK();
  k_direct64_sum<<<ceil_div(m, 256), 256, 0, s>>>(part, m, static_cast<u32>(plan.slices), acc,
                                                  pot);
  GTC_LAUNCH_CHECK();
}

void direct_fp64_sample(const double *pos, const double *mass, u64 n, const u64 *idx, u64 m,
                        double G, double eps, double *acc, double *pot, DeviceBuffer &scratch,
                        cudaStream_t s) {
  if (m == 0) return;
  int dev = 0, sms = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const Fp64SamplePlan plan = plan_fp64_sample(n, m, sms, ~0ull);
  scratch.ensure(plan.slices * m * 2 * sizeof(double2));
  launch_fp64_sample(pos, mass, n, idx, m, G, eps, plan, scratch.as<double2>(), acc, pot, s);
}

}  // namespace gtc

namespace gtc {
namespace {

// Eight independent FMA chains per thread, long enough to hide latency.
__global__ void __launch_bounds__(256) k_fma_peak(float *sink, int iters, float a, float b) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3f + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678f) sink[threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

double fp32_peak_tflops(cudaStream_t s) {
  int dev = 0, sms = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  DeviceBuffer sink;
  sink.ensure(256 * sizeof(float));
  const int iters = 1 << 14;
  const u32 blocks = static_cast<u32>(sms) * 8;
  cudaEvent_t a, b;
  GTC_CUDA(cudaEventCreate(&a));
  GTC_CUDA(cudaEventCreate(&b));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    GTC_CUDA(cudaEventRecord(a, s));
    k_fma_peak<<<blocks, 256, 0, s>>>(sink.as<float>(), iters, 0.999f, 1e-3f);
    GTC_LAUNCH_CHECK();
    GTC_CUDA(cudaEventRecord(b, s));
    GTC_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    GTC_CUDA(cudaEventElapsedTime(&ms, a, b));
    if (rep > 0) best = std::min(best, ms);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  sink.release();
  const double flops = 2.0 * 8.0 * iters * 256.0 * blocks;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace gtc
