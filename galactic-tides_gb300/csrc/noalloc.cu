// FP64 sampled direct sums with no allocation at all.
//
// gtc_direct_fp64_device needs a context, and the context allocates its
// stream, events and a scratch buffer for the per-slice partial sums. Some
// callers cannot do that:
//   * code embedded in another framework whose caching allocator has
//     reserved the GPU's memory up front, where a cudaMalloc of our own fails
//     or fragments that pool;
//   * timing-critical loops, where cudaMalloc / cudaFree would synchronize the
//     device and stall the caller's pipeline.
// For them, this file keeps the partial sums in one fixed device array,
// g_partials (8 MiB, held by every GPU that loads libgtc.so until the
// process exits), and takes the caller's stream. It allocates nothing.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress, once per device, with that device current.
// (In host code the array's name is only a host-side stand-in, not a device
// address.) Make that first call before any stream capture.
//
// Every call shares the one array and it keeps the last call's contents.
// Nothing needs clearing: each call writes every slot before reading it.
// Calls that overlap on the GPU (for example on two streams) race on the
// array and must be ordered by the caller.

#include <mutex>
#include <string>

#include "../../include/gtc.h"
#include "pipeline.cuh"

namespace gtc {
namespace {

constexpr u64 kPartialBytes = 8ull << 20;                  // 8 MiB
constexpr u64 kMaxSlots = kPartialBytes / (2 * sizeof(double2));  // (slice, target) pairs
constexpr int kMaxDevices = 64;
constexpr int kST = 128;                                   // sample targets per block

static __device__ __align__(256) double2 g_partials[kMaxSlots * 2];

std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

struct Body64 {
  double x, y, z, m;
};

__device__ __forceinline__ u64 min_u64(u64 a, u64 b) { return a < b ? a : b; }

// Partial sums of targets idx[blockIdx.x*kST + t] over source slice
// blockIdx.y, written to part[slice][target] (two double2 per slot).
__global__ void __launch_bounds__(kST)
    k_sample_partials(const double *__restrict__ pos, const double *__restrict__ mass, u64 n,
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

// Sums the slices of every target in slice order (deterministic).
__global__ void k_sample_sum(const double2 *part, u64 m, u32 slices, double *acc, double *pot) {
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

// Device address of g_partials on the current device, looked up once.
void *partials_address(int dev) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      throw RuntimeError(std::string("cuda: cannot locate the fixed scratch array: ") +
                         cudaGetErrorString(e));
    }
    g_addr[dev] = p;
  }
  return g_addr[dev];
}

}  // namespace
}  // namespace gtc

extern "C" {

gtc_status gtc_direct_fp64_noalloc(const double *pos, const double *mass, uint64_t n,
                                   const uint64_t *idx, uint64_t m, double G, double eps,
                                   double *acc, double *pot, void *stream) {
  using namespace gtc;
  try {
    if (m == 0) return GTC_OK;
    if (!pos || !mass || !idx || !acc || !pot)
      throw InvalidArgument("pos, mass, idx, acc and pot are required");
    if (n == 0) throw InvalidArgument("no bodies to sum over (n = 0)");
    if (m > kMaxSlots)
      throw InvalidArgument("gtc_direct_fp64_noalloc: at most " + std::to_string(kMaxSlots) +
                            " sample targets (fixed 8 MiB scratch), got " + std::to_string(m));
    int dev = 0, sms = 0;
    GTC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw InvalidArgument("device index out of range");
    GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double2 *part = static_cast<double2 *>(partials_address(dev));
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const u32 tb = ceil_div(m, kST);
    // source slices: ~8 blocks per SM, at least one tile each, and all the
    // (slice, target) partial sums inside the fixed array
    u64 slices = (8ull * sms + tb - 1) / tb;
    if (slices < 1) slices = 1;
    if (slices > n / kST) slices = n / kST > 0 ? n / kST : 1;
    if (slices > kMaxSlots / m) slices = kMaxSlots / m;
    const u64 slice = (n + slices - 1) / slices;
    slices = n > 0 ? (n + slice - 1) / slice : 1;
    dim3 grid(tb, static_cast<u32>(slices));
    k_sample_partials<<<grid, kST, 0, s>>>(pos, mass, n, idx, m, slice > 0 ? slice : 1, G,
                                           eps * eps, part);
    GTC_LAUNCH_CHECK();
    k_sample_sum<<<ceil_div(m, 256), 256, 0, s>>>(part, m, static_cast<u32>(slices), acc, pot);
    GTC_LAUNCH_CHECK();
    return GTC_OK;
  } catch (const InvalidArgument &e) {
    set_contextless_error(e.what());
    return GTC_INVALID_ARGUMENT;
  } catch (const std::exception &e) {
    set_contextless_error(e.what());
    return GTC_RUNTIME_ERROR;
  }
}

}  // extern "C"
