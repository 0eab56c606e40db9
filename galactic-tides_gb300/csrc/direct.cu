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

constexpr int kDT = 256;   // threads per block = bodies per shared tile
constexpr int kDR = 2;     // targets per thread

// One softened body-body term, G folded into b.w.
__device__ __forceinline__ void add_body(const float4 &p, const float4 &b, float eps2, float &ax,
                                         float &ay, float &az, float &pot) {
  const float dx = p.x - b.x, dy = p.y - b.y, dz = p.z - b.z;
  const float inv = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2))));
  const float gm = b.w * inv;
  const float gm3 = gm * inv * inv;
  ax = fmaf(-gm3, dx, ax);
  ay = fmaf(-gm3, dy, ay);
  az = fmaf(-gm3, dz, az);
  pot -= gm;
}

// Block b owns targets [b*kDT*kDR, (b+1)*kDT*kDR): thread t the targets
// base + t and base + kDT + t. Bodies stream through shared memory in
// tiles of kDT, in index order (the reference's summation order); only the
// tiles holding the block's own targets test j == i.
__global__ void __launch_bounds__(kDT)
    k_direct(const float4 *__restrict__ bodies, u32 n, float G, float eps2, float4 *out) {
  __shared__ float4 tile[kDT];
  const u32 t0 = blockIdx.x * (kDT * kDR);
  u32 ti[kDR];
  float4 p[kDR];
  float ax[kDR], ay[kDR], az[kDR], pot[kDR];
#pragma unroll
  for (int r = 0; r < kDR; ++r) {
    ti[r] = t0 + r * kDT + threadIdx.x;
    p[r] = ti[r] < n ? bodies[ti[r]] : make_float4(0.f, 0.f, 0.f, 0.f);
    ax[r] = ay[r] = az[r] = pot[r] = 0.f;
  }
  for (u32 base = 0; base < n; base += kDT) {
    const u32 j = base + threadIdx.x;
    float4 b = j < n ? bodies[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    b.w *= G;
    tile[threadIdx.x] = b;
    __syncthreads();
    const u32 cnt = min(static_cast<u32>(kDT), n - base);
    const bool own = base + kDT > t0 && base < t0 + kDT * kDR;
    if (!own && cnt == kDT) {
#pragma unroll 8
      for (int k = 0; k < kDT; ++k) {
        const float4 bj = tile[k];
#pragma unroll
        for (int r = 0; r < kDR; ++r) add_body(p[r], bj, eps2, ax[r], ay[r], az[r], pot[r]);
      }
    } else {
      for (u32 k = 0; k < cnt; ++k) {
        const float4 bj = tile[k];
#pragma unroll
        for (int r = 0; r < kDR; ++r)
          if (base + k != ti[r]) add_body(p[r], bj, eps2, ax[r], ay[r], az[r], pot[r]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < kDR; ++r)
    if (ti[r] < n) out[ti[r]] = make_float4(ax[r], ay[r], az[r], pot[r]);
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

void direct_fp32(const float4 *bodies, u32 n, float G, float eps2, float4 *out, cudaStream_t s) {
  if (n == 0) return;
  k_direct<<<ceil_div(n, kDT * kDR), kDT, 0, s>>>(bodies, n, G, eps2, out);
  GTC_LAUNCH_CHECK();
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
