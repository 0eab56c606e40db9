// Stable LSD radix sort of (u64 key, u32 value) pairs, 8 bits per pass.
//
// Each pass: per-tile digit histograms (digit-major, so one exclusive scan
// gives every tile's output offset per digit), then a scatter in which each
// warp ranks its keys with __match_any_sync and a warp-private histogram,
// which keeps equal digits in input order (stability); the tile is put in
// digit order in shared memory and written out in that order, so that
// consecutive threads write consecutive places of a digit's run. HBM-bound:
// one pass reads 8 B of key in the histogram and reads + writes 12 B per
// pair in the scatter.

#include <utility>

#include "common.cuh"

namespace gtc {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kPerLane = 8;                  // keys per lane per tile
constexpr u32 kTile = kThreads * kPerLane;   // 2048 keys per tile
constexpr u32 kPerWarp = 32 * kPerLane;      // contiguous keys per warp
constexpr int kBins = 256;
static_assert(kThreads == kBins, "the scatter gives each thread one digit");

__global__ void __launch_bounds__(kThreads)
    k_histogram(const u64 *keys, u32 n, int shift, u32 ntiles, u32 *counts) {
  __shared__ u32 h[kBins];
  h[threadIdx.x] = 0;
  __syncthreads();
  const u64 base = static_cast<u64>(blockIdx.x) * kTile;
  for (int k = 0; k < kPerLane; ++k) {
    const u64 i = base + static_cast<u64>(k) * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xff], 1u);
  }
  __syncthreads();
  counts[static_cast<u64>(threadIdx.x) * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kThreads)
    k_scatter(const u64 *keys, const u32 *vals, u64 *keys_out, u32 *vals_out, u32 n, int shift,
              u32 ntiles, const u32 *offsets) {
  __shared__ u32 wh[kWarps][kBins];     // per-warp running counts
  __shared__ u32 woff[kWarps][kBins];   // per-warp start within the tile's digit run
  __shared__ u32 dstart[kBins];         // start of each digit's run inside the tile
  __shared__ u32 gout[kBins];           // where each digit's run goes in the output
  __shared__ u64 skey[kTile];           // the tile, sorted by digit
  __shared__ u32 sval[kTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = lane; b < kBins; b += 32) wh[warp][b] = 0;
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  const u64 base = static_cast<u64>(blockIdx.x) * kTile + static_cast<u64>(warp) * kPerWarp;

  u64 key[kPerLane];
  u32 val[kPerLane];
  u32 rank[kPerLane];
#pragma unroll
  for (int c = 0; c < kPerLane; ++c) {
    const u64 i = base + static_cast<u64>(c) * 32 + lane;
    const bool ok = i < n;
    key[c] = ok ? keys[i] : 0;
    val[c] = ok ? vals[i] : 0;
    const u32 d = ok ? static_cast<u32>((key[c] >> shift) & 0xff) : kBins;  // kBins: no key
    const unsigned peers = __match_any_sync(kFullMask, d);
    u32 before = 0;
    if (ok) before = wh[warp][d];
    __syncwarp();
    if (ok && (peers & lt) == 0) wh[warp][d] = before + __popc(peers);
    __syncwarp();
    rank[c] = before + __popc(peers & lt);
  }
  __syncthreads();
  // Start of each warp's run of every digit inside the digit's run, the
  // digit runs' starts inside the tile (a block scan over the digits), and
  // each digit's output position.
  {
    const int d = threadIdx.x;  // kThreads == kBins
    u32 run = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      woff[w][d] = run;
      run += wh[w][d];
    }
    // exclusive scan of run over the 256 digits: warp scans, then the warp totals
    u32 incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 v = __shfl_up_sync(kFullMask, incl, o);
      if (lane >= o) incl += v;
    }
    __shared__ u32 wsum[kWarps];
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    u32 before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    dstart[d] = before + incl - run;
    gout[d] = offsets[static_cast<u64>(d) * ntiles + blockIdx.x];
  }
  __syncthreads();
  // the tile in digit order in shared memory
#pragma unroll
  for (int c = 0; c < kPerLane; ++c) {
    const u64 i = base + static_cast<u64>(c) * 32 + lane;
    if (i >= n) continue;
    const u32 d = static_cast<u32>((key[c] >> shift) & 0xff);
    const u32 local = dstart[d] + woff[warp][d] + rank[c];
    skey[local] = key[c];
    sval[local] = val[c];
  }
  __syncthreads();
  // out in order: consecutive threads write consecutive places of a digit's run
  const u64 tile0 = static_cast<u64>(blockIdx.x) * kTile;
  const u32 count = static_cast<u32>(n - tile0 < kTile ? n - tile0 : kTile);
  for (u32 j = threadIdx.x; j < count; j += kThreads) {
    const u64 k = skey[j];
    const u32 d = static_cast<u32>((k >> shift) & 0xff);
    const u32 dst = gout[d] + (j - dstart[d]);
    keys_out[dst] = k;
    vals_out[dst] = sval[j];
  }
}

}  // namespace

void radix_sort_pairs(u64 *keys, u32 *vals, u64 *alt_keys, u32 *alt_vals, u32 n, int bits,
                      RadixScratch &scratch, cudaStream_t s, int low_bit) {
  if (n <= 1 || bits <= 0) return;
  const u32 ntiles = ceil_div(n, kTile);
  const u64 ncounts = static_cast<u64>(kBins) * ntiles;
  const int passes = (bits + 7) / 8;
  scratch.counts.ensure(2 * ncounts * sizeof(u32));
  u32 *counts = scratch.counts.as<u32>();
  u32 *offsets = counts + ncounts;

  // Ping-pong between the two buffers; an odd number of passes ends with
  // one copy back.
  u64 *src_k = keys, *dst_k = alt_keys;
  u32 *src_v = vals, *dst_v = alt_vals;
  for (int p = 0; p < passes; ++p) {
    const int shift = low_bit + 8 * p;
    k_histogram<<<ntiles, kThreads, 0, s>>>(src_k, n, shift, ntiles, counts);
    GTC_LAUNCH_CHECK();
    exclusive_scan_u32(counts, offsets, ncounts, nullptr, scratch.scan_tmp, s);
    k_scatter<<<ntiles, kThreads, 0, s>>>(src_k, src_v, dst_k, dst_v, n, shift, ntiles, offsets);
    GTC_LAUNCH_CHECK();
    std::swap(src_k, dst_k);
    std::swap(src_v, dst_v);
  }
  if (src_k != keys) {
    GTC_CUDA(cudaMemcpyAsync(keys, src_k, static_cast<u64>(n) * sizeof(u64),
                             cudaMemcpyDeviceToDevice, s));
    GTC_CUDA(cudaMemcpyAsync(vals, src_v, static_cast<u64>(n) * sizeof(u32),
                             cudaMemcpyDeviceToDevice, s));
  }
}

}  // namespace gtc
