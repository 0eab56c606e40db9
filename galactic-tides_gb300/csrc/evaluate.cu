// Warp-per-group evaluation of grouped interaction lists, FP32.
//
// Same arithmetic as the reference's shared kernels (gt_body / gt_cell,
// include/galactic_tides/kernels/gravity_kernels.h:71-135) and the same
// order -- all cells in list order, then all bodies in list order, skipping
// the target itself (gt_group_accel, :162-170) -- with FMA contraction and
// the SFU reciprocal square root (rsqrtf; in the packed kernel the SFU
// instruction itself, rsqrt_normal, as every softened r^2 is a normal
// float) instead of 1/sqrt.
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

constexpr int kWarpsPerBlock = 8;
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

// Target i's results (tree order) into eo: the FP32 record, and the caller's
// FP64 arrays (FP32 -> FP64 exactly) and |a| when eo asks for them.
__device__ __forceinline__ void write_target(const EvalOut &eo, u32 i, float4 a) {
  eo.out[i] = a;
  if (!eo.acc) return;
  const u64 j = eo.order[i];
  eo.acc[3 * j] = a.x;
  eo.acc[3 * j + 1] = a.y;
  eo.acc[3 * j + 2] = a.z;
  eo.pot[j] = a.w;
  if (eo.amag) eo.amag[j] = sqrtf(__fmaf_rn(a.x, a.x, __fmaf_rn(a.y, a.y, __fmul_rn(a.z, a.z))));
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
           const uint4 *__restrict__ groups, u32 ngroups, float G, float eps2, EvalOut eo,
           u32 *next_group, const u32 *ng_dev = nullptr, const u32 *abort = nullptr) {
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
    const uint4 q0 = groups[4ull * g], q1 = groups[4ull * g + 1], q2 = groups[4ull * g + 2],
                q3 = groups[4ull * g + 3];
    const SegView cs = cell_segs(q1, q2), bs = body_segs(q2, q3);  // list entry -> index
    // A group of T <= 16 targets splits its lists into ns = min(4, 32 / T)
    // slices: lane l takes target l % T of slice l / T, each slice stages
    // W = 32 / ns entries per round, and the slices' sums are added up by
    // shuffles at the end (larger groups: one slice, W = 32).
    const u32 T = q0.y - q0.x;
    const u32 ns = T == 0 ? 1u : min(4u, 32u / T);
    const u32 W = 32u / ns;
    const u32 slice = T ? static_cast<u32>(lane) / T : 0u;
    const u32 t = T ? static_cast<u32>(lane) % T : 0u;
    const bool computes = slice < ns;  // lanes past ns * T only stage
    const u32 i = q0.x + t;
    const float4 bi = computes ? bodies[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const u32 stage_slice = static_cast<u32>(lane) / W, stage_pos = static_cast<u32>(lane) % W;
    float ax = 0.f, ay = 0.f, az = 0.f, pot = 0.f;

    {
      const u32 e = q0.z;  // cells, slice k: entries [e k / ns, e (k + 1) / ns)
      const u32 c0 = e * stage_slice / ns, c1 = e * (stage_slice + 1) / ns;
      const u32 m0 = e * slice / ns, m1 = e * (slice + 1) / ns;
      const u32 rounds = (((e + ns - 1) / ns) + W - 1) / W;
      for (u32 r = 0; r < rounds; ++r) {
        const u32 k = c0 + r * W + stage_pos;
        if (stage_slice < ns && k < c1) {
          const u64 c = cell_list[cs.at(k)];
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
      const u32 e = q0.w;
      const u32 c0 = e * stage_slice / ns, c1 = e * (stage_slice + 1) / ns;
      const u32 m0 = e * slice / ns, m1 = e * (slice + 1) / ns;
      const u32 rounds = (((e + ns - 1) / ns) + W - 1) / W;
      for (u32 r = 0; r < rounds; ++r) {
        const u32 k = c0 + r * W + stage_pos;
        if (stage_slice < ns && k < c1) {
          const u32 j = body_list[bs.at(k)];
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
    if (slice == 0 && t < T) write_target(eo, i, make_float4(ax, ay, az, pot));
  }
}

// The softened quadrupole evaluation (the benchmark configuration) with
// Blackwell's packed FP32 instructions: each lane works two staged entries
// at once, one in each half of a float2, so every FFMA2/FMUL2/FADD2 does two
// interactions' arithmetic and the issue count per interaction halves.
// Entries are staged as interleaved pairs (x_a, x_b, y_a, y_b, ...), with
// coordinates and G m negated so that d = p + (-c) is one FADD2; a slot
// past the list holds a dummy far away with zero mass and quadrupole, which
// adds exactly zero (its r^2 overflows to inf and rsqrt(inf) = 0).
//
// Lane fill: a group of T targets splits both lists into ns slices and
// numbers its (slice k, target t) slots v = k T + t; pass p gives slot
// 32 p + l to lane l, so ceil(ns T / 32) passes keep nearly every lane busy
// whatever T is (ns T / 32 lanes' worth of work per pass, against T of 32
// with one slice). ns is picked per group from the list lengths. A pass
// holds at most 4 slices (T >= 11: a 32-slot window spans at most
// floor(31 / T) + 2 of them; T <= 10: one pass of min(4, 32 / T) slices),
// each staged in its own shared-memory area. After a pass the lanes add
// their partial sums (even plus odd entries) onto the target's running sum
// in shared memory, slice by slice in increasing order, so the summation
// order is fixed.
constexpr float kFar = 1.0e30f;
constexpr int kPairCellF4 = 5;   // float4 per staged cell pair
constexpr int kPairBodyF4 = 2;   // float4 per staged body pair
constexpr u32 kMaxSlices = 16;   // slices per group at most
// The tile shape (EvalShape, a context option each and searched by
// gtc_autotune_eval): the staged pairs a lane works per inner-loop
// iteration (kU, 1 or 2) -- the pairs' arithmetic is independent up to the
// accumulation, which stays in list order, so results do not depend on it;
// more pairs per iteration give each warp more independent work to hide the
// rsqrt and shared-load latencies; a round's 2W staged entries (2W a
// multiple of 4) are padded with far dummies, so an iteration never reads
// past them -- and a pass's fixed cost in staged entries per lane, which
// sets how many slices a group's lists are cut into (below).

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

__device__ __forceinline__ u32 even_up(u32 x) { return (x + 1u) & ~1u; }

// Slices for a group of T targets with ec cells and eb bodies (warp-uniform):
// the ns in 1..16 that minimises passes x (pair steps per pass + pass_cost).
__device__ __forceinline__ u32 choose_slices(u32 T, u32 ec, u32 eb, int lane, u32 pass_cost) {
  if (T <= 10) return T == 0 ? 1u : min(4u, 32u / T);
  const u32 ns = static_cast<u32>(lane) % kMaxSlices + 1u;
  const u32 passes = (ns * T + 31u) / 32u;
  const u64 cost = static_cast<u64>(passes) *
                   (even_up((ec + ns - 1) / ns) + even_up((eb + ns - 1) / ns) + pass_cost);
  const u32 key = static_cast<u32>(cost < (1ull << 27) ? cost : (1ull << 27) - 1) << 4 | (ns - 1u);
  return (__reduce_min_sync(kFullMask, key) & 15u) + 1u;
}

template <int kU>
__global__ void __launch_bounds__(kT)
    k_eval_pairs(const float4 *__restrict__ bodies, const float4 *__restrict__ cells,
                 const u32 *__restrict__ cell_list, const u32 *__restrict__ body_list,
                 const uint4 *__restrict__ groups, u32 ngroups, float G, float eps2,
                 EvalOut eo, u32 *next_group, const u32 *ng_dev, const u32 *abort,
                 u32 pass_cost) {
  // per warp, staged pairs: each lane stages two entries per round, so area
  // a (2W entries) starts at float4 a * (W * per-pair + 1) (at most 4 areas:
  // 164 and 68 float4); the 16-byte gap puts the areas on different
  // shared-memory banks
  __shared__ float4 sc[kWarpsPerBlock][164];
  __shared__ float4 sb[kWarpsPerBlock][68];
  __shared__ float4 sacc[kWarpsPerBlock][32];  // per target: a and potential
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (abort && *abort) return;
  if (ng_dev) ngroups = min(ngroups, *ng_dev);
  const float2 e2 = f2(eps2, eps2), m25 = f2(-2.5f, -2.5f), mhalf = f2(-0.5f, -0.5f);
  for (;;) {
    u32 g = 0;
    if (lane == 0) g = atomicAdd(next_group, 1u);
    g = __shfl_sync(kFullMask, g, 0);
    if (g >= ngroups) return;
    const uint4 q0 = groups[4ull * g], q1 = groups[4ull * g + 1], q2 = groups[4ull * g + 2],
                q3 = groups[4ull * g + 3];
    const SegView cs = cell_segs(q1, q2), bs = body_segs(q2, q3);  // list entry -> index
    const u32 T = q0.y - q0.x;
    if (T == 0) continue;
    const u32 ec = q0.z, eb = q0.w;
    const u32 ns = choose_slices(T, ec, eb, lane, pass_cost);
    const u32 slots = ns * T;
    const u32 passes = (slots + 31u) / 32u;
    if (static_cast<u32>(lane) < T) sacc[warp][lane] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();

    for (u32 p = 0; p < passes; ++p) {
      const u32 v = 32u * p + static_cast<u32>(lane);
      const bool computes = v < slots;
      const u32 slice = v / T, t = v % T;
      const u32 k_lo = (32u * p) / T;
      const u32 nsp = min(ns - 1u, (32u * p + 31u) / T) - k_lo + 1u;  // 1..4
      const u32 W = nsp == 1u ? 32u : (nsp == 2u ? 16u : (nsp == 3u ? 10u : 8u));
      const u32 area = slice - k_lo;
      const u32 stage_area = static_cast<u32>(lane) / W, stage_pos = static_cast<u32>(lane) % W;
      const u32 stage_slice = k_lo + stage_area;
      const bool stages = stage_area < nsp;
      const u32 half = stage_pos & 1u, pair = stage_pos >> 1;
      const float4 bi = computes ? bodies[q0.x + t] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float2 px = f2(bi.x, bi.x), py = f2(bi.y, bi.y), pz = f2(bi.z, bi.z);
      float2 ax = f2(0.f, 0.f), ay = ax, az = ax, pot = ax;

      {  // cells
        const u32 cstride = W * kPairCellF4 + 1;
        const u32 c0 = ec * stage_slice / ns, c1 = ec * (stage_slice + 1) / ns;
        const u32 m0 = ec * slice / ns, m1 = ec * (slice + 1) / ns;
        const u32 rounds = ((ec + ns - 1) / ns + 2 * W - 1) / (2 * W);
        for (u32 r = 0; r < rounds; ++r) {
          if (stages) {
            // two entries per lane: positions stage_pos and stage_pos + W
            float v[2][10];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const u32 k = c0 + 2 * r * W + h * W + stage_pos;
              if (k < c1) {
                const u64 c = cell_list[cs.at(k)];
                const float4 a = __ldg(&cells[3 * c]), b = __ldg(&cells[3 * c + 1]),
                             q = __ldg(&cells[3 * c + 2]);
                v[h][0] = -a.x; v[h][1] = -a.y; v[h][2] = -a.z; v[h][3] = -G * a.w;
                v[h][4] = G * b.x; v[h][5] = G * b.y; v[h][6] = G * b.z; v[h][7] = G * b.w;
                v[h][8] = G * q.x; v[h][9] = G * q.y;
              } else {
                v[h][0] = v[h][1] = v[h][2] = -kFar;
                v[h][3] = v[h][4] = v[h][5] = v[h][6] = v[h][7] = v[h][8] = v[h][9] = 0.f;
              }
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              float *f = reinterpret_cast<float *>(
                  &sc[warp][stage_area * cstride + (pair + h * (W / 2)) * kPairCellF4]);
#pragma unroll
              for (int q = 0; q < 10; ++q) f[2 * q + half] = v[h][q];
            }
          }
          __syncwarp();
          const u32 base = m0 + 2 * r * W;
          const u32 cnt = computes && base < m1 ? min(2 * W, m1 - base) : 0u;
          const float4 *mine = &sc[warp][area * cstride];
          for (u32 j = 0; j < cnt; j += 2 * kU) {
#pragma unroll
            for (int u = 0; u < kU; ++u) {
            const float4 s0 = mine[5 * u], s1 = mine[5 * u + 1], s2 = mine[5 * u + 2],
                         s3 = mine[5 * u + 3], s4 = mine[5 * u + 4];
            // s0 = -cx, -cy  s1 = -cz, -Gm  s2 = Qxx, Qyy  s3 = Qzz, Qxy  s4 = Qxz, Qyz (pairs)
            const float2 dx = __fadd2_rn(px, f2(s0.x, s0.y)), dy = __fadd2_rn(py, f2(s0.z, s0.w)),
                         dz = __fadd2_rn(pz, f2(s1.x, s1.y));
            const float2 ngm = f2(s1.z, s1.w);
            const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
            const float2 inv = f2(rsqrt_normal(r2.x), rsqrt_normal(r2.y));
            const float2 inv2 = __fmul2_rn(inv, inv), inv3 = __fmul2_rn(inv, inv2);
            const float2 qxx = f2(s2.x, s2.y), qyy = f2(s2.z, s2.w), qzz = f2(s3.x, s3.y),
                         qxy = f2(s3.z, s3.w), qxz = f2(s4.x, s4.y), qyz = f2(s4.z, s4.w);
            const float2 qx = __ffma2_rn(qxx, dx, __ffma2_rn(qxy, dy, __fmul2_rn(qxz, dz)));
            const float2 qy = __ffma2_rn(qxy, dx, __ffma2_rn(qyy, dy, __fmul2_rn(qyz, dz)));
            const float2 qz = __ffma2_rn(qxz, dx, __ffma2_rn(qyz, dy, __fmul2_rn(qzz, dz)));
            const float2 rqr = __ffma2_rn(dx, qx, __ffma2_rn(dy, qy, __fmul2_rn(dz, qz)));
            // r.Q.r / r^5 once, for both the acceleration along d and the potential
            const float2 inv5 = __fmul2_rn(inv3, inv2), rqr5 = __fmul2_rn(rqr, inv5);
            const float2 along = __ffma2_rn(__fmul2_rn(m25, rqr5), inv2, __fmul2_rn(ngm, inv3));
            ax = __ffma2_rn(along, dx, __ffma2_rn(qx, inv5, ax));
            ay = __ffma2_rn(along, dy, __ffma2_rn(qy, inv5, ay));
            az = __ffma2_rn(along, dz, __ffma2_rn(qz, inv5, az));
            pot = __ffma2_rn(mhalf, rqr5, __ffma2_rn(ngm, inv, pot));
            }
            mine += kPairCellF4 * kU;
          }
          __syncwarp();
        }
      }

      {  // bodies
        const u32 bstride = W * kPairBodyF4 + 1;
        const u32 c0 = eb * stage_slice / ns, c1 = eb * (stage_slice + 1) / ns;
        const u32 m0 = eb * slice / ns, m1 = eb * (slice + 1) / ns;
        const u32 rounds = ((eb + ns - 1) / ns + 2 * W - 1) / (2 * W);
        for (u32 r = 0; r < rounds; ++r) {
          if (stages) {
            float v[2][4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const u32 k = c0 + 2 * r * W + h * W + stage_pos;
              if (k < c1) {
                const float4 b = __ldg(&bodies[body_list[bs.at(k)]]);
                v[h][0] = -b.x; v[h][1] = -b.y; v[h][2] = -b.z; v[h][3] = -G * b.w;
              } else {
                v[h][0] = v[h][1] = v[h][2] = -kFar;
                v[h][3] = 0.f;
              }
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              float *f = reinterpret_cast<float *>(
                  &sb[warp][stage_area * bstride + (pair + h * (W / 2)) * kPairBodyF4]);
#pragma unroll
              for (int q = 0; q < 4; ++q) f[2 * q + half] = v[h][q];
            }
          }
          __syncwarp();
          const u32 base = m0 + 2 * r * W;
          const u32 cnt = computes && base < m1 ? min(2 * W, m1 - base) : 0u;
          const float4 *mine = &sb[warp][area * bstride];
          for (u32 j = 0; j < cnt; j += 2 * kU) {
#pragma unroll
            for (int u = 0; u < kU; ++u) {
            const float4 s0 = mine[2 * u], s1 = mine[2 * u + 1];
            const float2 dx = __fadd2_rn(px, f2(s0.x, s0.y)), dy = __fadd2_rn(py, f2(s0.z, s0.w)),
                         dz = __fadd2_rn(pz, f2(s1.x, s1.y));
            const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
            const float2 inv = f2(rsqrt_normal(r2.x), rsqrt_normal(r2.y));
            const float2 gm = __fmul2_rn(f2(s1.z, s1.w), inv);       // -G m / r
            const float2 gm3 = __fmul2_rn(gm, __fmul2_rn(inv, inv));  // -G m / r^3
            ax = __ffma2_rn(gm3, dx, ax);
            ay = __ffma2_rn(gm3, dy, ay);
            az = __ffma2_rn(gm3, dz, az);
            pot = __fadd2_rn(pot, gm);
            }
            mine += kPairBodyF4 * kU;
          }
          __syncwarp();
        }
      }
      // this pass's partial sums onto the targets', slice by slice
      const float sx = ax.x + ax.y, sy = ay.x + ay.y, sz = az.x + az.y, sp = pot.x + pot.y;
      for (u32 a = 0; a < nsp; ++a) {
        if (computes && area == a) {
          float4 &acc = sacc[warp][t];
          acc.x += sx;
          acc.y += sy;
          acc.z += sz;
          acc.w += sp;
        }
        __syncwarp();
      }
    }
    if (static_cast<u32>(lane) < T) {
      const u32 i = q0.x + static_cast<u32>(lane);
      float4 acc = sacc[warp][lane];
      acc.w += G * bodies[i].w * rsqrtf(eps2);  // the self term (softened), taken back once
      write_target(eo, i, acc);
    }
  }
}

template <int kU>
void launch_pairs(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                  const u32 *body_list, const uint4 *groups, u64 n_groups, float G, float eps2,
                  const EvalOut &eo, u32 *counter, cudaStream_t s, const Scalars *sc,
                  u32 pass_cost, u64 want, int sms) {
  int per_sm = 0;
  GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eval_pairs<kU>, kT, 0));
  const u32 grid = static_cast<u32>(std::min<u64>(want, static_cast<u64>(sms) * std::max(1, per_sm)));
  k_eval_pairs<kU><<<grid, kT, 0, s>>>(bodies, cells, cell_list, body_list, groups,
                                       static_cast<u32>(n_groups), G, eps2, eo, counter,
                                       sc ? &sc->n_groups : nullptr, sc ? &sc->abort : nullptr,
                                       pass_cost);
}

template <bool kQuad, bool kSoft>
void launch_eval(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                 const u32 *body_list, const uint4 *groups, u64 n_groups, float G, float eps2,
                 const EvalOut &eo, u32 *counter, cudaStream_t s, const EvalShape &shape,
                 const Scalars *sc = nullptr) {
  int dev = 0, sms = 0, per_sm = 0;
  GTC_CUDA(cudaGetDevice(&dev));
  GTC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GTC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eval<kQuad, kSoft>, kT, 0));
  const u64 want = (n_groups + kWarpsPerBlock - 1) / kWarpsPerBlock;
  if (kQuad && kSoft) {
    if (shape.pairs == 1)
      launch_pairs<1>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, eo, counter,
                      s, sc, shape.pass_cost, want, sms);
    else
      launch_pairs<2>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, eo, counter,
                      s, sc, shape.pass_cost, want, sms);
  } else {
    const u32 grid = static_cast<u32>(std::min<u64>(want, static_cast<u64>(sms) * std::max(1, per_sm)));
    k_eval<kQuad, kSoft><<<grid, kT, 0, s>>>(bodies, cells, cell_list, body_list, groups,
                                             static_cast<u32>(n_groups), G, eps2, eo, counter,
                                             sc ? &sc->n_groups : nullptr,
                                             sc ? &sc->abort : nullptr);
  }
  GTC_LAUNCH_CHECK();
}

}  // namespace

void evaluate_lists(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                    const u32 *body_list, const uint4 *groups, u64 n_groups, float G, float eps2,
                    bool quadrupole, const EvalOut &eo, u32 *counter, cudaStream_t s,
                    const EvalShape &shape) {
  if (n_groups == 0) return;
  GTC_CUDA(cudaMemsetAsync(counter, 0, sizeof(u32), s));
  const bool soft = eps2 > 0.0f;
  if (quadrupole && soft)
    launch_eval<true, true>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, eo, counter, s, shape);
  else if (quadrupole)
    launch_eval<true, false>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, eo, counter, s, shape);
  else if (soft)
    launch_eval<false, true>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, eo, counter, s, shape);
  else
    launch_eval<false, false>(bodies, cells, cell_list, body_list, groups, n_groups, G, eps2, eo, counter, s, shape);
}

void evaluate_lists_graph(const float4 *bodies, const float4 *cells, const u32 *cell_list,
                          const u32 *body_list, const uint4 *groups, u64 max_groups,
                          const Scalars *sc, float G, float eps2, bool quadrupole,
                          const EvalOut &eo, u32 *counter, cudaStream_t s,
                          const EvalShape &shape) {
  if (max_groups == 0) return;
  GTC_CUDA(cudaMemsetAsync(counter, 0, sizeof(u32), s));
  const bool soft = eps2 > 0.0f;
  if (quadrupole && soft)
    launch_eval<true, true>(bodies, cells, cell_list, body_list, groups, max_groups, G, eps2, eo, counter, s, shape, sc);
  else if (quadrupole)
    launch_eval<true, false>(bodies, cells, cell_list, body_list, groups, max_groups, G, eps2, eo, counter, s, shape, sc);
  else if (soft)
    launch_eval<false, true>(bodies, cells, cell_list, body_list, groups, max_groups, G, eps2, eo, counter, s, shape, sc);
  else
    launch_eval<false, false>(bodies, cells, cell_list, body_list, groups, max_groups, G, eps2, eo, counter, s, shape, sc);
}

}  // namespace gtc
