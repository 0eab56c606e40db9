// The device leapfrog (src/integrator.cpp) and its diagnostics.
#pragma once

#include "../../include/gtc.h"
#include "common.cuh"

namespace gtc {

constexpr int kDiagTerms = 12;

// v += h a; x += dt v, for n bodies ((x, y, z) doubles each).
void kick_drift(double *pos, double *vel, const double *acc, u64 n, double h, double dt,
                cudaStream_t s);
// v += h a (skipped when *abort is set: a graph replay that outgrew its sizes).
void kick(double *vel, const double *acc, u64 n, double h, cudaStream_t s,
          const u32 *abort = nullptr);
// Per-block FP64 partial sums of the diagnostics into part
// (diagnostics_blocks() x kDiagTerms doubles), then their sum in block order
// on the host.
void diagnostics_launch(const double *pos, const double *vel, const double *mass,
                        const double *pot, u64 n, double *part, cudaStream_t s);
int diagnostics_blocks();
void diagnostics_finish(const double *part, double time, gtc_diagnostics *out);

}  // namespace gtc
