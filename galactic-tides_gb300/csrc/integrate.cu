// The kick-drift-kick leapfrog on the device (src/integrator.cpp:5-17) and
// its diagnostics (src/integrator.cpp:19-36), FP64 throughout. Compiled with
// -fmad=false: every product and sum rounds on its own, as in the
// reference's build, so a step given the same accelerations moves the
// particles to the same doubles.

#include <vector>

#include "integrate.cuh"

namespace gtc {
namespace {

constexpr int kT = 256;
constexpr int kDiagBlocks = 256;

// v += h a; x += dt v (integrator.cpp:10-13)
__global__ void __launch_bounds__(kT)
    k_kick_drift(double *pos, double *vel, const double *acc, u64 n3, double h, double dt) {
  const u64 k = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  if (k >= n3) return;
  const double v = vel[k] + h * acc[k];
  vel[k] = v;
  pos[k] = pos[k] + dt * v;
}

// v += h a (integrator.cpp:16); a graph replay skips it after an abort.
__global__ void __launch_bounds__(kT)
    k_kick(double *vel, const double *acc, u64 n3, double h, const u32 *abort) {
  const u64 k = static_cast<u64>(blockIdx.x) * kT + threadIdx.x;
  if (k >= n3 || (abort && *abort)) return;
  vel[k] = vel[k] + h * acc[k];
}

// Per-block sums of the diagnostics (block order kept): kinetic, potential,
// momentum (3), angular momentum (3), m x (3), mass.
__global__ void __launch_bounds__(kT)
    k_diag_partials(const double *pos, const double *vel, const double *mass, const double *pot,
                    u64 n, double *part) {
  __shared__ double s[kDiagTerms][kT / 32];
  double acc[kDiagTerms] = {};
  for (u64 i = static_cast<u64>(blockIdx.x) * kT + threadIdx.x; i < n;
       i += static_cast<u64>(gridDim.x) * kT) {
    const double m = mass[i];
    const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    const double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
    acc[0] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    acc[1] += 0.5 * m * pot[i];
    acc[2] += m * vx;
    acc[3] += m * vy;
    acc[4] += m * vz;
    acc[5] += m * (y * vz - z * vy);
    acc[6] += m * (z * vx - x * vz);
    acc[7] += m * (x * vy - y * vx);
    acc[8] += m * x;
    acc[9] += m * y;
    acc[10] += m * z;
    acc[11] += m;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = 0; j < kDiagTerms; ++j) {
    double v = acc[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    if (lane == 0) s[j][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < kDiagTerms) {
    double v = 0.0;
    for (int w = 0; w < kT / 32; ++w) v += s[threadIdx.x][w];
    part[blockIdx.x * kDiagTerms + threadIdx.x] = v;
  }
}

}  // namespace

void kick_drift(double *pos, double *vel, const double *acc, u64 n, double h, double dt,
                cudaStream_t s) {
  if (n == 0) return;
  k_kick_drift<<<ceil_div(3 * n, kT), kT, 0, s>>>(pos, vel, acc, 3 * n, h, dt);
  GTC_LAUNCH_CHECK();
}

void kick(double *vel, const double *acc, u64 n, double h, cudaStream_t s, const u32 *abort) {
  if (n == 0) return;
  k_kick<<<ceil_div(3 * n, kT), kT, 0, s>>>(vel, acc, 3 * n, h, abort);
  GTC_LAUNCH_CHECK();
}

void diagnostics_launch(const double *pos, const double *vel, const double *mass,
                        const double *pot, u64 n, double *part, cudaStream_t s) {
  k_diag_partials<<<kDiagBlocks, kT, 0, s>>>(pos, vel, mass, pot, n, part);
  GTC_LAUNCH_CHECK();
}

int diagnostics_blocks() { return kDiagBlocks; }

void diagnostics_finish(const double *part, double time, gtc_diagnostics *out) {
  double sum[kDiagTerms] = {};
  for (int b = 0; b < kDiagBlocks; ++b)
    for (int j = 0; j < kDiagTerms; ++j) sum[j] += part[b * kDiagTerms + j];
  gtc_diagnostics d{};
  d.time = time;
  d.kinetic = sum[0];
  d.potential = sum[1];
  for (int a = 0; a < 3; ++a) {
    d.momentum[a] = sum[2 + a];
    d.angular_momentum[a] = sum[5 + a];
    d.centre_of_mass[a] = sum[11] > 0 ? sum[8 + a] / sum[11] : 0.0;
  }
  d.total = d.kinetic + d.potential;
  d.virial_ratio = d.potential != 0.0 ? -2.0 * d.kinetic / d.potential : 0.0;
  *out = d;
}

}  // namespace gtc
