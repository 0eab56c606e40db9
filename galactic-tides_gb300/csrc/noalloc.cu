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
// process exits), and takes the caller's stream. It allocates nothing. The
// kernels are the context path's own (launch_fp64_sample, direct.cu); only
// where the partial sums live differs, and how many source slices fit.
//
// Set-up: in host code the array's name is only a host-side stand-in, not a
// device address. The first call in a CUDA context (normally a device's
// primary context) looks its device address up with cudaGetSymbolAddress,
// with that context current, and keeps it under the context's unique id
// (cuCtxGetId). A new context -- after cudaDeviceReset, or a driver-API
// context the caller made current -- has a new id and gets its own look-up,
// so a stale address is never used. Make the first call in a context before
// any stream capture.
//
// Every call shares the one array and it keeps the last call's contents.
// Nothing needs clearing: each call writes every slot before reading it.
// Calls that overlap on the GPU (for example on two streams) race on the
// array and must be ordered by the caller.

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <string>
#include <unordered_map>

#include "../../include/gtc.h"
#include "pipeline.cuh"

namespace gtc {
namespace {

constexpr u64 kPartialBytes = 8ull << 20;                          // 8 MiB
constexpr u64 kMaxPairs = kPartialBytes / (2 * sizeof(double2));  // (slice, target) pairs

static __device__ __align__(256) double2 g_partials[kMaxPairs * 2];

std::mutex g_mu;
std::unordered_map<unsigned long long, void *> g_addr;  // context id -> address
PFN_cuCtxGetCurrent_v4000 g_get_current = nullptr;
PFN_cuCtxGetId_v12000 g_get_id = nullptr;

// Unique id of the CUDA context current on this thread; false when none is.
bool current_context_id(unsigned long long *id) {
  if (!g_get_current || !g_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    GTC_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault,
                                              &q1));
    GTC_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      throw RuntimeError("cuda: the driver offers no cuCtxGetCurrent / cuCtxGetId");
    g_get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f1);
    g_get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f2);
  }
  CUcontext c = nullptr;
  if (g_get_current(&c) != CUDA_SUCCESS || !c) return false;
  return g_get_id(c, id) == CUDA_SUCCESS;
}

void *lookup_partials() {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    throw RuntimeError(std::string("cuda: cannot locate the fixed scratch array: ") +
                       cudaGetErrorString(e));
  }
  return p;
}

// Device address of g_partials in the current context, looked up once per
// context. On a thread with no context current yet, the look-up itself
// makes the device's primary context current.
double2 *partials_address() {
  std::lock_guard<std::mutex> lock(g_mu);
  unsigned long long id = 0;
  if (!current_context_id(&id)) {
    void *p = lookup_partials();
    if (!current_context_id(&id)) throw RuntimeError("cuda: no current context");
    g_addr[id] = p;
    return static_cast<double2 *>(p);
  }
  auto it = g_addr.find(id);
  if (it == g_addr.end()) it = g_addr.emplace(id, lookup_partials()).first;
  return static_cast<double2 *>(it->second);
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
    if (m > kMaxPairs)
      throw InvalidArgument("gtc_direct_fp64_noalloc: at most " + std::to_string(kMaxPairs) +
                            " sample targets (fixed 8 MiB scratch), got " + std::to_string(m));
    // An error left by the caller's own earlier work stays where it is, for
    // the caller to find: this call neither reports it as its own nor
    // clears it.
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess)
      throw RuntimeError(std::string("cuda: an earlier CUDA error is pending (left in place): ") +
                         cudaGetErrorName(pending));
    int dev = 0, sms = 0;
    GTC_CUDA(cudaGetDevice(&dev));
    GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double2 *part = partials_address();
    const Fp64SamplePlan plan = plan_fp64_sample(n, m, sms, kMaxPairs);
    launch_fp64_sample(pos, mass, n, idx, m, G, eps, plan, part, acc, pot,
                       static_cast<cudaStream_t>(stream));
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
