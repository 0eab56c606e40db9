// Stable LSD radix sort of (u64 key, u32 value) pairs, 8 bits per pass, in
// one sweep per pass (after Adinets and Merrill, "Onesweep: a faster least
// significant digit radix sort for GPUs", 2022).
//
// One launch counts the digits of every pass at once (the keys are read
// once for all passes) and one small launch scans them into each digit's
// start in each pass. Then each pass is a single launch: a block takes the
// next tile (2048 pairs) from a counter, ranks its keys stably (each warp
// with __match_any_sync and a warp-private histogram, equal digits in input
// order), publishes its digit counts, and finds how many pairs of each digit
// the earlier tiles hold by looking back over their published counts --
// each tile publishes first its own counts, then, once it knows them, the
// running totals up to and including it, so a look-back stops at the first
// running total it meets. The tile is put in digit order in shared memory
// and written out in that order (consecutive threads, consecutive places of
// a digit's run). Per pass a pair is read once and written once (12 B each
// way); the former per-pass histogram read (8 B) and scan launches are gone.
//
// A look-back waits only on tiles taken earlier from the counter, whose
// blocks are running or done and publish their counts before waiting
// themselves, so the waits end. Each wait is bounded all the same: past the
// limit the kernel records error bit 16 (and the pass's output is garbage).

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
constexpr int kMaxPasses = 8;
static_assert(kThreads == kBins, "the scatter gives each thread one digit");

// A tile's published word per digit: flag in the top two bits, count below.
constexpr u64 kAggregate = 1ull << 62;       // this tile's own count
constexpr u64 kInclusive = 2ull << 62;       // the count of this and every earlier tile
constexpr u64 kCountMask = (1ull << 62) - 1;
constexpr u32 kSpinLimit = 1u << 22;         // polls of one word before giving up
constexpr u32 kSortTimeout = 16u;            // error bit

__device__ __forceinline__ u64 load_relaxed(const u64 *p) {
  u64 v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void store_relaxed(u64 *p, u64 v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Digit counts of every pass: hist[p][d] += pairs whose digit p is d.
__global__ void __launch_bounds__(kThreads)
    k_digit_counts(const u64 *keys, u32 n, int low_bit, int passes, u32 *hist) {
  __shared__ u32 h[kMaxPasses][kBins];
  for (int p = 0; p < passes; ++p) h[p][threadIdx.x] = 0;
  __syncthreads();
  for (u64 i = static_cast<u64>(blockIdx.x) * kThreads + threadIdx.x; i < n;
       i += static_cast<u64>(gridDim.x) * kThreads) {
    const u64 k = keys[i];
    for (int p = 0; p < passes; ++p) atomicAdd(&h[p][(k >> (low_bit + 8 * p)) & 0xff], 1u);
  }
  __syncthreads();
  for (int p = 0; p < passes; ++p)
    if (h[p][threadIdx.x]) atomicAdd(&hist[p * kBins + threadIdx.x], h[p][threadIdx.x]);
}

// Each pass's digit starts: an exclusive scan of its 256 counts (block p).
__global__ void __launch_bounds__(kThreads) k_digit_starts(const u32 *hist, u32 *start) {
  __shared__ u32 wsum[kWarps];
  const int d = threadIdx.x, lane = d & 31, warp = d >> 5;
  const u32 c = hist[blockIdx.x * kBins + d];
  u32 incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const u32 v = __shfl_up_sync(kFullMask, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  u32 before = 0;
  for (int w = 0; w < warp; ++w) before += wsum[w];
  start[blockIdx.x * kBins + d] = before + incl - c;
}

__global__ void __launch_bounds__(kThreads)
    k_onesweep(const u64 *keys, const u32 *vals, u64 *keys_out, u32 *vals_out, u32 n, int shift,
               const u32 *digit_start, u64 *status, u32 *tile_counter, u32 *error) {
  __shared__ u32 wh[kWarps][kBins];     // per-warp running counts
  __shared__ u32 woff[kWarps][kBins];   // per-warp start within the tile's digit run
  __shared__ u32 dstart[kBins];         // start of each digit's run inside the tile
  __shared__ u64 gout[kBins];           // where each digit's run goes in the output
  __shared__ u64 skey[kTile];           // the tile, sorted by digit
  __shared__ u32 sval[kTile];
  __shared__ u32 wsum[kWarps];
  __shared__ u32 tile_s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) tile_s = atomicAdd(tile_counter, 1u);  // tiles in start order
  for (int b = lane; b < kBins; b += 32) wh[warp][b] = 0;
  __syncthreads();
  const u32 tile = tile_s;
  const unsigned lt = (1u << lane) - 1u;
  const u64 tile0 = static_cast<u64>(tile) * kTile;
  const u64 base = tile0 + static_cast<u64>(warp) * kPerWarp;

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
  {
    const int d = threadIdx.x;  // kThreads == kBins
    u32 run = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      woff[w][d] = run;
      run += wh[w][d];
    }
    // this tile's count of digit d, then the earlier tiles' by looking back
    u64 *mine = status + static_cast<u64>(tile) * kBins + d;
    store_relaxed(mine, (tile == 0 ? kInclusive : kAggregate) | run);
    u64 excl = 0;
    for (u32 t = tile; t > 0;) {
      const u64 *w = status + static_cast<u64>(t - 1) * kBins + d;
      u64 v = load_relaxed(w);
      for (u32 spin = 0; (v >> 62) == 0; ++spin) {
        if (spin == kSpinLimit) {
          atomicOr(error, kSortTimeout);
          v = kInclusive;  // give up: count 0, stop
          break;
        }
        v = load_relaxed(w);
      }
      excl += v & kCountMask;
      if ((v >> 62) == 2) break;  // a running total: done
      --t;
    }
    if (tile > 0) store_relaxed(mine, kInclusive | (excl + run));
    gout[d] = digit_start[d] + excl;
    // the digit runs' starts inside the tile: exclusive scan of run
    u32 incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const u32 v = __shfl_up_sync(kFullMask, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    u32 before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    dstart[d] = before + incl - run;
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
  const u32 count = static_cast<u32>(n - tile0 < kTile ? n - tile0 : kTile);
  for (u32 j = threadIdx.x; j < count; j += kThreads) {
    const u64 k = skey[j];
    const u32 d = static_cast<u32>((k >> shift) & 0xff);
    const u64 dst = gout[d] + (j - dstart[d]);
    keys_out[dst] = k;
    vals_out[dst] = sval[j];
  }
}

}  // namespace

void radix_sort_pairs(u64 *keys, u32 *vals, u64 *alt_keys, u32 *alt_vals, u32 n, int bits,
                      RadixScratch &scratch, cudaStream_t s, int low_bit, u32 *error) {
  if (n <= 1 || bits <= 0) return;
  const u32 ntiles = ceil_div(n, kTile);
  const int passes = (bits + 7) / 8;
  if (passes > kMaxPasses) throw InvalidArgument("radix sort: more than 64 key bits");
  // scratch, sized for the most passes whatever this call needs (so that a
  // captured sort of more levels than the eager one finds it allocated):
  // per pass the status words of every tile, then the digit counts, digit
  // starts and tile counters of every pass and an error word; the parts
  // this call uses are zeroed
  const u64 status_max = static_cast<u64>(kMaxPasses) * ntiles * kBins;
  const u64 small = 2ull * kMaxPasses * kBins + kMaxPasses + 2;
  scratch.counts.ensure(status_max * sizeof(u64) + small * sizeof(u32));
  u64 *status = scratch.counts.as<u64>();
  u32 *hist = reinterpret_cast<u32 *>(status + status_max);
  u32 *start = hist + kMaxPasses * kBins;
  u32 *tiles = start + kMaxPasses * kBins;
  u32 *own_error = tiles + kMaxPasses;
  GTC_CUDA(cudaMemsetAsync(status, 0, static_cast<u64>(passes) * ntiles * kBins * sizeof(u64), s));
  GTC_CUDA(cudaMemsetAsync(hist, 0, small * sizeof(u32), s));
  int dev = 0, sms = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const u32 hblocks = std::min<u32>(ceil_div(n, kThreads), 4u * static_cast<u32>(sms));
  k_digit_counts<<<hblocks, kThreads, 0, s>>>(keys, n, low_bit, passes, hist);
  GTC_LAUNCH_CHECK();
  k_digit_starts<<<passes, kThreads, 0, s>>>(hist, start);
  GTC_LAUNCH_CHECK();

  // Ping-pong between the two buffers; an odd number of passes ends with
  // one copy back.
  u64 *src_k = keys, *dst_k = alt_keys;
  u32 *src_v = vals, *dst_v = alt_vals;
  for (int p = 0; p < passes; ++p) {
    k_onesweep<<<ntiles, kThreads, 0, s>>>(src_k, src_v, dst_k, dst_v, n, low_bit + 8 * p,
                                           start + p * kBins,
                                           status + static_cast<u64>(p) * ntiles * kBins,
                                           tiles + p, error ? error : own_error);
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
