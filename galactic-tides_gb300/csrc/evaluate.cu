// Warp-per-group evaluation of grouped interaction lists, FP32.
//
// Same arithmetic as the reference's shared kernels (gt_body / gt_cell,
// include/galactic_tides/kernels/gravity_kernels.h:71-135) and the same
// order -- all cells in list order, then all bodies in list order, skipping
// the target itself (gt_group_accel, :162-170) -- with FMA contraction and
// the SFU reciprocal square root (rsqrtf) instead of 1/sqrt.
//
// Lane l of a warp owns target begin + l of its group. The warp walks the
// list 32 entries at a time: each lane loads one entry (coalesced index
// load, then one 48-byte cell or 16-byte body), scales its mass and
// quadrupole by G once, and stages it in shared memory; then every lane
// reads the 32 staged entries back as broadcast loads (one shared-memory
// transaction serves the whole warp) and accumulates. A group of 16 or
// fewer targets splits its lists into 2-4 slices worked by separate lane
// sets (lanes that would otherwise idle), summed by shuffles at the end.
// Groups are handed out to warps by an atomic counter, so a warp that drew
// a long list does not hold back the others' next groups.

#include <algorithm>

#include "pipeline.cuh"

namespace gtc {
namespace {

constexpr int kWarpsPerBlock = 4;
constexpr int kT = 32 * kWarpsPerBlock;

struct Staged {
  float4 cm;   // com (rel. origin), G * mass
  float4 q0;   // G * (xx, yy, zz, xy)
  float4 q1;   // G * (xz, yz, -, -)
};

template <bool kQuad>
__device__ __forceinline__ void add_cell(float px, float py, float pz, const Staged &c, float eps2,
                                         float &ax, float &ay, float &az, float &pot) {
  const float dx = px - c.cm.x, dy = py - c.cm.y, dz = pz - c.cm.z;
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
  const float inv = rsqrtf(r2);
  const float inv2 = inv * inv;
  const float inv3 = inv * inv2;
  if (kQuad) {
    // a = -G m d / r^3 + G Q d / r^5 - 5/2 G (d.Q.d) d / r^7, with G folded
    // into m and Q: the monopole and quadrupole terms along d share one FMA
    // per axis.
    const float qx = fmaf(c.q0.x, dx, fmaf(c.q0.w, dy, c.q1.x * dz));
    const float qy = fmaf(c.q0.w, dx, fmaf(c.q0.y, dy, c.q1.y * dz));
    const float qz = fmaf(c.q1.x, dx, fmaf(c.q1.y, dy, c.q0.z * dz));
    const float rqr = fmaf(dx, qx, fmaf(dy, qy, dz * qz));
    const float inv5 = inv3 * inv2;
    const float inv7 = inv5 * inv2;
    const float along = fmaf(-2.5f * rqr, inv7, -c.cm.w * inv3);
    ax = fmaf(along, dx, fmaf(qx, inv5, ax));
    ay = fmaf(along, dy, fmaf(qy, inv5, ay));
    az = fmaf(along, dz, fmaf(qz, inv5, az));
    pot = fmaf(-c.cm.w, inv, fmaf(-0.5f * rqr, inv5, pot));
  } else {
    const float gm3 = c.cm.w * inv3;
    ax = fmaf(-gm3, dx, ax);
    ay = fmaf(-gm3, dy, ay);
    az = fmaf(-gm3, dz, az);
    pot = fmaf(-c.cm.w, inv, pot);
  }
}

// kSoft: eps2 > 0. Every target appears exactly once in its own group's body
// list (each body is covered once and no accepted cell holds a target), and
// with softening its self term adds exactly zero acceleration (d = 0) and a
// known -G m_i / eps to the potential, so the loop needs no self test and
// the self potential is taken back out at the end. Without softening the
// self term is singular and each entry is tested as in the reference.
template <bool kQuad, bool kSoft>
__global__ void __launch_bounds__(kT)
    k_eval(const float4 *__restrict__ bodies, const float4 *__restrict__ cells,
           const u32 *__restrict__ cell_list, const u32 *__restrict__ body_list,
           const uint4 *__restrict__ groups, u32 ngroups, float G, float eps2,
           float4 *__restrict__ out, u32 *next_group, const u32 *ng_dev = nullptr,
           const u32 *abort = nullptr) {
  // Staged entries, per warp: slice k's W entries start at float4 k (3W + 1)
  // (cells) and k (W + 1) (bodies); the 16-byte gap puts the slices on
  // different shared-memory banks, so their broadcast loads do not conflict.
  __shared__ float4 sc[kWarpsPerBlock][3 * 32 + 4];
  __shared__ float4 sb[kWarpsPerBlock][32 + 4];
  __shared__ u32 sj[kWarpsPerBlock][kSoft ? 1 : 32 + 4];  // staged body indices (self test)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // a graph replay: the group count from the device, nothing after an abort
  if (abort && *abort) return;
  if (ng_dev) ngroups = min(ngroups, *ng_dev);
  for (;;) {
    u32 g = 0;
    if (lane == 0) g = atomicAdd(next_group, 1u);
    g = __shfl_sync(kFullMask, g, 0);
    if (g >= ngroups) return;
    const uint4 ga = groups[2ull * g], gb = groups[2ull * g + 1];
    // A group of T <= 16 targets splits its lists into ns = min(4, 32 / T)
    // slices: lane l takes target l % T of slice l / T, each slice stages
    // W = 32 / ns entries per round, and the slices' sums are added up by
    // shuffles at the end (larger groups: one slice, W = 32).
    const u32 T = ga.y - ga.x;
    const u32 ns = T == 0 ? 1u : min(4u, 32u / T);
    const u32 W = 32u / ns;
    const u32 slice = T ? static_cast<u32>(lane) / T : 0u;
    const u32 t = T ? static_cast<u32>(lane) % T : 0u;
    const bool computes = slice < ns;  // lanes past ns * T only stage
    const u32 i = ga.x + t;
    const float4 bi = computes ? bodies[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const u32 stage_slice = static_cast<u32>(lane) / W, stage_pos = static_cast<u32>(lane) % W;
    float ax = 0.f, ay = 0.f, az = 0.f, pot = 0.f;

    {
      const u32 e = ga.w - ga.z;  // cells, slice k: [e k / ns, e (k + 1) / ns)
      const u32 c0 = ga.z + e * stage_slice / ns, c1 = ga.z + e * (stage_slice + 1) / ns;
      const u32 m0 = ga.z + e * slice / ns, m1 = ga.z + e * (slice + 1) / ns;
      const u32 rounds = (((e + ns - 1) / ns) + W - 1) / W;
      for (u32 r = 0; r < rounds; ++r) {
        const u32 k = c0 + r * W + stage_pos;
        if (stage_slice < ns && k < c1) {
          const u64 c = cell_list[k];
          const float4 q = __ldg(&cells[3 * c]);
          float4 *dst = &sc[warp][stage_slice * (3 * W + 1) + 3 * stage_pos];
          dst[0] = make_float4(q.x, q.y, q.z, G * q.w);
          if (kQuad) {
            const float4 c1v = __ldg(&cells[3 * c + 1]), c2v = __ldg(&cells[3 * c + 2]);
            dst[1] = make_float4(G * c1v.x, G * c1v.y, G * c1v.z, G * c1v.w);
            dst[2] = make_float4(G * c2v.x, G * c2v.y, 0.f, 0.f);
          }
        }
        __syncwarp();
        const u32 base = m0 + r * W;
        const u32 cnt = computes && base < m1 ? min(W, m1 - base) : 0u;
        const float4 *mine = &sc[warp][slice * (3 * W + 1)];
        for (u32 j = 0; j < cnt; ++j) {
          Staged st;
          st.cm = mine[3 * j];
          if (kQuad) {
            st.q0 = mine[3 * j + 1];
            st.q1 = mine[3 * j + 2];
          }
          add_cell<kQuad>(bi.x, bi.y, bi.z, st, eps2, ax, ay, az, pot);
        }
        __syncwarp();
      }
    }

    {
      const u32 e = gb.y - gb.x;
      const u32 c0 = gb.x + e * stage_slice / ns, c1 = gb.x + e * (stage_slice + 1) / ns;
      const u32 m0 = gb.x + e * slice / ns, m1 = gb.x + e * (slice + 1) / ns;
      const u32 rounds = (((e + ns - 1) / ns) + W - 1) / W;
      for (u32 r = 0; r < rounds; ++r) {
        const u32 k = c0 + r * W + stage_pos;
        if (stage_slice < ns && k < c1) {
          const u32 j = body_list[k];
          const float4 b = __ldg(&bodies[j]);
          sb[warp][stage_slice * (W + 1) + stage_pos] = make_float4(b.x, b.y, b.z, G * b.w);
          if (!kSoft) sj[warp][stage_slice * (W + 1) + stage_pos] = j;
        }
        __syncwarp();
        const u32 base = m0 + r * W;
        const u32 cnt = computes && base < m1 ? min(W, m1 - base) : 0u;
        const float4 *mine = &sb[warp][slice * (W + 1)];
        for (u32 q = 0; q < cnt; ++q) {
          const float4 b = mine[q];
          const float dx = bi.x - b.x, dy = bi.y - b.y, dz = bi.z - b.z;
          float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
          float w = b.w;
          if (!kSoft) {
            const bool self = sj[warp][kSoft ? 0 : slice * (W + 1) + q] == i;
            r2 = self ? 1.0f : r2;
            w = self ? 0.0f : w;
          }
          const float inv = rsqrtf(r2);
          const float gm = w * inv;
          const float gm3 = gm * inv * inv;
          ax = fmaf(-gm3, dx, ax);
          ay = fmaf(-gm3, dy, ay);
          az = fmaf(-gm3, dz, az);
          pot -= gm;
        }
        __syncwarp();
      }
    }
    // the slices' partial sums onto slice 0
    for (u32 k = 1; k < ns; ++k) {
      const int src = min(lane + static_cast<int>(k * T), 31);
      const float sx = __shfl_sync(kFullMask, ax, src), sy = __shfl_sync(kFullMask, ay, src),
                  sz = __shfl_sync(kFullMask, az, src), sp = __shfl_sync(kFullMask, pot, src);
      if (slice == 0) {
        ax += sx;
        ay += sy;
        az += sz;
        pot += sp;
      }
    }
    if (kSoft) pot += G * bi.w * rsqrtf(eps2);  // the self term, added once above
    if (slice == 0 && t < T) out[i] = make_float4(ax, ay, az, pot);
  }
}

// Tree order -> caller order, FP32 -> FP64 (gravity_backends.cpp:132-136).
__global__ void __launch_bounds__(256)
    k_scatter(const float4 *out, const u32 *order, u32 n, double *acc, double *pot,
              const u32 *abort = nullptr) {
  const u32 k = blockIdx.x * 256 + threadIdx.x;
  if (k >= n || (abort && *abort)) return;
  const float4 o = out[k];
  const u64 i = order[k];
  acc[3 * i] = o.x;
  acc[3 * i + 1] = o.y;
  acc[3 * i + 2] = o.z;
  pot[i] = o.w;
}

template <bool kQuad, bool kSoft>
void launch_eval(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                 const u32 *body_list, const uint4 *groups, u64 n_groups, float G, float eps2,
                 float4 *out, u32 *counter, cudaStream_t s, const Scalars *sc = nullptr) {
  int dev = 0, sms = 0, per_sm = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eval<kQuad, kSoft>, kT, 0));
  const u64 want = (n_groups + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const u32 grid = static_cast<u32>(std::min<u64>(want, static_cast<u64>(sms) * std::max(1, per_sm)));
  k_eval<kQuad, kSoft><<<grid, kT, 0, s>>>(bodies, cells, cell_list, body_list, groups,
                                           static_cast<u32>(n_groups), G, eps2, out, counter,
                                           sc ? &sc->n_groups : nullptr,
                                           sc ? &sc->abort : nullptr);
  GTC_LAUNCH_CHECK();
}

}  // namespace

void evaluate_lists(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                    const u32 *body_list, const uint4 *groups, u64 n_groups, float G, float eps2,
                    bool quadrupole, float4 *out, u32 *counter, cudaStream_t s) {
  if (n_groups == 0) return;
  GTC_CUDA(cudaMemsetAsync(counter, 0, sizeof(u32), s));
  const bool soft = eps2 > 0.0f;
  if (quadrupole && soft)
    launch_eval<true, true>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, out, counter, s);
  else if (quadrupole)
    launch_eval<true, false>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, out, counter, s);
  else if (soft)
    launch_eval<false, true>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, out, counter, s);
  else
    launch_eval<false, false>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, out, counter, s);
}

void evaluate_lists_graph(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                          const u32 *body_list, const uint4 *groups, u64 max_groups,
                          const Scalars *sc, float G, float eps2, bool quadrupole, float4 *out,
                          u32 *counter, cudaStream_t s) {
  if (max_groups == 0) return;
  GTC_CUDA(cudaMemsetAsync(counter, 0, sizeof(u32), s));
  const bool soft = eps2 > 0.0f;
  if (quadrupole && soft)
    launch_eval<true, true>(bodies, cells, cell_list, body_list, groups, max_groups, G, eps2, out, counter, s, sc);
  else if (quadrupole)
    launch_eval<true, false>(bodies, cells, cell_list, body_list, groups, max_groups, G, eps2, out, counter, s, sc);
  else if (soft)
    launch_eval<false, true>(bodies, cells, cell_list, body_list, groups, max_groups, G, eps2, out, counter, s, sc);
  else
    launch_eval<false, false>(bodies, cells, cell_list, body_list, groups, max_groups, G, eps2, out, counter, s, sc);
}

void scatter_results_graph(const float4 *out, const u32 *order, u64 n, double *acc, double *pot,
                           const Scalars *sc, cudaStream_t s) {
  if (n == 0) return;
  k_scatter<<<ceil_div(n, 256), 256, 0, s>>>(out, order, static_cast<u32>(n), acc, pot, &sc->abort);
  GTC_LAUNCH_CHECK();
}

void scatter_results(const float4 *out, const u32 *order, u64 n, double *acc, double *pot,
                     cudaStream_t s) {
  if (n == 0) return;
  k_scatter<<<ceil_div(n, 256), 256, 0, s>>>(out, order, static_cast<u32>(n), acc, pot);
  GTC_LAUNCH_CHECK();
}

}  // namespace gtc
