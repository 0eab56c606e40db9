// The per-particle tree walk: Octree::accel_pot (src/octree.cpp:275-344) for
// every body, the reference's `gravity = tree` solver (compute_gravity_tree,
// src/gravity.cpp:7-26), on the device tree.
//
// FP64 with every product and sum rounded on its own (compiled -fmad=false)
// and the reference's operand order, on nodes identical to the reference's:
// the walk visits nodes in the reference's stack order (the device numbers
// nodes that way, so the stack becomes a forward scan with skip links), the
// opening test is the Barnes (1994) offset criterion -- a cell is accepted
// when the body lies outside its slackened cube and r^2 > (2 h / theta +
// delta)^2 -- and accepted cells add monopole and quadrupole terms; opened
// leaves add their bodies, skipping the body itself. CUDA's FP64 division
// and square root round correctly, as the host's do, so the forces are the
// reference's bit for bit.
//
// One thread per body in tree order (neighbours walk alike), results to the
// caller's order. Bound: the FP64 pipe.

#include "pipeline.cuh"

namespace gtc {
namespace {

constexpr int kT = 128;

struct TreeWalkArgs {
  const double2 *geom;  // (cx, cy), (cz, half)
  const double2 *mom;   // (mx, my), (mz, mass)
  const double2 *quad;  // xx yy | zz xy | xz yz
  const double *delta;
  const u32 *nbegin, *nend, *skip;
  const u8 *isleaf;
  const double *tpos, *tmass;  // tree order
  const u32 *order;            // tree position -> caller index
  u32 n, m;
  double G, eps2, inv_theta;
  int quadrupole;
  double *acc, *pot;           // caller order
  unsigned long long *counts;  // cell, particle interactions
};

__global__ void __launch_bounds__(kT) k_tree_walk(TreeWalkArgs a) {
  const u32 t = blockIdx.x * kT + threadIdx.x;
  u64 ncell = 0, npart = 0;
  if (t < a.n) {
    const u32 self = a.order[t];
    const double x = a.tpos[3ull * t], y = a.tpos[3ull * t + 1], z = a.tpos[3ull * t + 2];
    double ax = 0, ay = 0, az = 0, phi = 0;
    u32 i = 0;
    while (i < a.m) {
      const double2 g0 = a.geom[2ull * i], g1 = a.geom[2ull * i + 1];
      const double2 c0 = a.mom[2ull * i], c1 = a.mom[2ull * i + 1];
      const double half = g1.y, mass = c1.y;
      const double dx = x - c0.x, dy = y - c0.y, dz = z - c1.x;
      const double r2 = dx * dx + dy * dy + dz * dz;
      const double crit = 2.0 * half * a.inv_theta + a.delta[i];
      const double slack = half * 1.0001;
      const bool inside = fabs(x - g0.x) <= slack && fabs(y - g0.y) <= slack &&
                          fabs(z - g1.x) <= slack;
      const u32 next = a.skip[i];
      if (!inside && r2 > crit * crit) {
        // the cell as a multipole
        const double r2s = r2 + a.eps2;
        const double inv = 1.0 / sqrt(r2s);
        const double inv3 = inv * inv * inv;
        const double gm3 = a.G * mass * inv3;
        ax -= gm3 * dx;
        ay -= gm3 * dy;
        az -= gm3 * dz;
        phi -= a.G * mass * inv;
        if (a.quadrupole) {
          const double2 qa = a.quad[3ull * i], qb = a.quad[3ull * i + 1],
                        qc = a.quad[3ull * i + 2];
          const double q[6] = {qa.x, qa.y, qb.x, qb.y, qc.x, qc.y};
          const double qx = q[0] * dx + q[3] * dy + q[4] * dz;
          const double qy = q[3] * dx + q[1] * dy + q[5] * dz;
          const double qz = q[4] * dx + q[5] * dy + q[2] * dz;
          const double rqr = dx * qx + dy * qy + dz * qz;
          const double inv5 = inv3 * inv * inv;
          const double inv7 = inv5 * inv * inv;
          ax += a.G * (qx * inv5 - 2.5 * rqr * dx * inv7);
          ay += a.G * (qy * inv5 - 2.5 * rqr * dy * inv7);
          az += a.G * (qz * inv5 - 2.5 * rqr * dz * inv7);
          phi -= 0.5 * a.G * rqr * inv5;
        }
        ++ncell;
        i = next;
      } else if (a.isleaf[i]) {
        for (u32 k = a.nbegin[i]; k < a.nend[i]; ++k) {
          if (a.order[k] == self) continue;
          const double ex = x - a.tpos[3ull * k], ey = y - a.tpos[3ull * k + 1],
                       ez = z - a.tpos[3ull * k + 2];
          const double r2s = ex * ex + ey * ey + ez * ez + a.eps2;
          const double inv = 1.0 / sqrt(r2s);
          const double gm3 = a.G * a.tmass[k] * inv * inv * inv;
          ax -= gm3 * ex;
          ay -= gm3 * ey;
          az -= gm3 * ez;
          phi -= a.G * a.tmass[k] * inv;
          ++npart;
        }
        i = next;
      } else {
        ++i;  // the children follow, in the reference's stack order
      }
    }
    a.acc[3ull * self] = ax;
    a.acc[3ull * self + 1] = ay;
    a.acc[3ull * self + 2] = az;
    a.pot[self] = phi;
  }
  // interaction counters: one atomic per warp
  ncell = __reduce_add_sync(kFullMask, static_cast<u32>(ncell));
  npart = __reduce_add_sync(kFullMask, static_cast<u32>(npart));
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&a.counts[0], static_cast<unsigned long long>(ncell));
    atomicAdd(&a.counts[1], static_cast<unsigned long long>(npart));
  }
}

}  // namespace

void tree_walk_forces(Workspace &ws, const SolverParams &sp, double *acc, double *pot,
                      unsigned long long *counts, cudaStream_t s) {
  if (ws.n == 0) return;
  TreeWalkArgs a{ws.geom.as<double2>(), ws.mom.as<double2>(), ws.quad.as<double2>(),
                 ws.delta.as<double>(), ws.nbegin.as<u32>(), ws.nend.as<u32>(),
                 ws.skip.as<u32>(), ws.isleaf.as<u8>(), ws.tpos.as<double>(),
                 ws.tmass.as<double>(), ws.idx.as<u32>(), static_cast<u32>(ws.n),
                 static_cast<u32>(ws.n_nodes), sp.G, sp.eps * sp.eps, 1.0 / sp.theta,
                 sp.quadrupole, acc, pot, counts};
  k_tree_walk<<<ceil_div(ws.n, kT), kT, 0, s>>>(a);
  GTC_LAUNCH_CHECK();
}

}  // namespace gtc
