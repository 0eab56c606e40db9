// Shared declarations of the GB300 gravity backend (libgtc.so).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

namespace gtc {

using u8 = std::uint8_t;
using u16 = std::uint16_t;
using u32 = std::uint32_t;
using u64 = std::uint64_t;

// ----------------------------------------------------------------- errors
// Host code throws these; the C ABI layer turns them into gtc_status codes.
struct InvalidArgument : std::invalid_argument {
  using std::invalid_argument::invalid_argument;
};
struct RuntimeError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct OutOfMemory : std::runtime_error {
  using std::runtime_error::runtime_error;
};

[[noreturn]] void throw_cuda(cudaError_t e, const char *what, const char *file, int line);

#define GTC_CUDA(call)                                                       \
  do {                                                                       \
    cudaError_t gtc_e_ = (call);                                             \
    if (gtc_e_ != cudaSuccess) ::gtc::throw_cuda(gtc_e_, #call, __FILE__, __LINE__); \
  } while (0)

// Every kernel launch is followed by GTC_LAUNCH_CHECK(), which also counts it.
void count_launch();
#define GTC_LAUNCH_CHECK()            \
  do {                                \
    GTC_CUDA(cudaGetLastError());     \
    ::gtc::count_launch();            \
  } while (0)
unsigned long long launches_so_far();

// Message returned by gtc_last_error(NULL) (calls made without a context).
void set_contextless_error(const std::string &msg);

// ------------------------------------------------------- device buffers
// Grow-only device allocation, kept between calls.
struct DeviceBuffer {
  void *ptr = nullptr;
  std::size_t bytes = 0;
  void ensure(std::size_t want);
  void release();
  template <class T>
  T *as() const {
    return static_cast<T *>(ptr);
  }
};

inline u32 ceil_div(u64 a, u64 b) { return static_cast<u32>((a + b - 1) / b); }

#ifdef __CUDACC__
// 1/sqrt(x) of a positive normal float (r^2 with softening: r^2 >= eps^2):
// the SFU's rsqrt (PTX rsqrt.approx.ftz.f32) without the subnormal-input
// handling around rsqrtf, which costs FMA-pipe instructions in the
// evaluators' inner loops. It returns rsqrtf's value bit for bit on every
// positive normal float (tests/test_rsqrt_normal.py checks all of them); a
// subnormal input is taken as 0 (result +inf) where rsqrtf scales it.
__device__ __forceinline__ float rsqrt_normal(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
#endif

// --------------------------------------------------------------- scans
// Exclusive prefix sums over n elements on `s`. `tmp` is grown as needed.
// The total is written to *total_dev (device memory, may be null).
void exclusive_scan_u32(const u32 *in, u32 *out, u64 n, u32 *total_dev, DeviceBuffer &tmp,
                        cudaStream_t s);
void exclusive_scan_u64(const u64 *in, u64 *out, u64 n, u64 *total_dev, DeviceBuffer &tmp,
                        cudaStream_t s);
// Grows tmp to what scans of up to n elements need (none allocates after).
void reserve_scans(DeviceBuffer &tmp, u64 n);

// ---------------------------------------------------------- radix sort
// Stable LSD radix sort of (key, value) pairs on `bits` bits of the key from
// bit `low_bit` up, 8 bits a pass, one launch per pass. The sorted pairs end
// up back in keys/vals; alt_* are scratch of n elements each. A look-back
// that outwaits its bound sets bit 16 of *error (device word; null: a word
// of the scratch).
struct RadixScratch {
  DeviceBuffer counts, scan_tmp;
};
void radix_sort_pairs(u64 *keys, u32 *vals, u64 *alt_keys, u32 *alt_vals, u32 n, int bits,
                      RadixScratch &scratch, cudaStream_t s, int low_bit = 0,
                      u32 *error = nullptr);

// ------------------------------------------------------- warp helpers
constexpr unsigned kFullMask = 0xffffffffu;

}  // namespace gtc
