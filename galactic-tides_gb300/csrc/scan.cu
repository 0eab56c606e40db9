// Device-wide exclusive prefix sums (reduce, scan of block totals, add back).
// Used for node numbering, group offsets, list offsets and the radix sort.

#include <algorithm>

#include "common.cuh"

namespace gtc {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr u32 kTile = kThreads * kItems;

template <class T>
__device__ T warp_inclusive(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T t = __shfl_up_sync(kFullMask, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Exclusive scan of one value per thread across the block; *total gets the sum.
template <class T>
__device__ T block_exclusive(T v, T *warp_sums, T *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T incl = warp_inclusive(v);
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T w = lane < kThreads / 32 ? warp_sums[lane] : T(0);
    w = warp_inclusive(w);
    if (lane < kThreads / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  const T before = warp > 0 ? warp_sums[warp - 1] : T(0);
  *total = warp_sums[kThreads / 32 - 1];
  __syncthreads();
  return before + incl - v;
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_tile_sums(const T *in, u64 n, T *sums) {
  __shared__ T ws[kThreads / 32];
  const u64 base = static_cast<u64>(blockIdx.x) * kTile;
  T acc = 0;
  for (int k = 0; k < kItems; ++k) {
    const u64 i = base + static_cast<u64>(k) * kThreads + threadIdx.x;
    if (i < n) acc += in[i];
  }
  T total;
  block_exclusive(acc, ws, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Scans each tile in place of out, starting from offsets[blockIdx.x].
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_tile_scan(const T *in, T *out, u64 n, const T *offsets, T *total_dev, u32 nblocks) {
  __shared__ T ws[kThreads / 32];
  const u64 base = static_cast<u64>(blockIdx.x) * kTile + static_cast<u64>(threadIdx.x) * kItems;
  T v[kItems];
  T local = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const u64 i = base + k;
    v[k] = i < n ? in[i] : T(0);
    local += v[k];
  }
  T total;
  T run = block_exclusive(local, ws, &total);
  if (offsets) run += offsets[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const u64 i = base + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
  if (total_dev && blockIdx.x == nblocks - 1 && threadIdx.x == kThreads - 1) *total_dev = run;
}

template <class T>
void scan_impl(const T *in, T *out, u64 n, T *total_dev, DeviceBuffer &tmp, u64 tmp_off,
               cudaStream_t s) {
  if (n == 0) {
    if (total_dev) GTC_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(T), s));
    return;
  }
  const u32 nb = ceil_div(n, kTile);
  if (nb == 1) {
    k_tile_scan<T><<<1, kThreads, 0, s>>>(in, out, n, nullptr, total_dev, 1);
    GTC_LAUNCH_CHECK();
    return;
  }
  // Block totals, scanned recursively, live in tmp after tmp_off.
  const u64 need = (tmp_off + 2 * static_cast<u64>(nb)) * sizeof(T);
  if (tmp.bytes < need) throw RuntimeError("scan scratch too small");
  T *sums = tmp.as<T>() + tmp_off;
  T *offs = sums + nb;
  k_tile_sums<T><<<nb, kThreads, 0, s>>>(in, n, sums);
  GTC_LAUNCH_CHECK();
  scan_impl<T>(sums, offs, nb, nullptr, tmp, tmp_off + 2 * static_cast<u64>(nb), s);
  k_tile_scan<T><<<nb, kThreads, 0, s>>>(in, out, n, offs, total_dev, nb);
  GTC_LAUNCH_CHECK();
}

template <class T>
u64 scratch_elems(u64 n) {
  u64 total = 0;
  while (n > kTile) {
    const u64 nb = (n + kTile - 1) / kTile;
    total += 2 * nb;
    n = nb;
  }
  return total + 16;
}

}  // namespace

void exclusive_scan_u32(const u32 *in, u32 *out, u64 n, u32 *total_dev, DeviceBuffer &tmp,
                        cudaStream_t s) {
  tmp.ensure(scratch_elems<u32>(n) * sizeof(u32));
  scan_impl<u32>(in, out, n, total_dev, tmp, 0, s);
}

void reserve_scans(DeviceBuffer &tmp, u64 n) {
  tmp.ensure(std::max(scratch_elems<u32>(n) * sizeof(u32), scratch_elems<u64>(n) * sizeof(u64)));
}

void exclusive_scan_u64(const u64 *in, u64 *out, u64 n, u64 *total_dev, DeviceBuffer &tmp,
                        cudaStream_t s) {
  tmp.ensure(scratch_elems<u64>(n) * sizeof(u64));
  scan_impl<u64>(in, out, n, total_dev, tmp, 0, s);
}

}  // namespace gtc
