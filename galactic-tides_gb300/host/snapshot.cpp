// Snapshots: a raw binary stand-in for the reference's GADGET-style HDF5
// snapshots (src/snapshot_io.cpp:113-221), which need HDF5. The content is
// the same -- per particle position, velocity, mass, ID, type and potential,
// the time, the particle count of each GADGET type and the run's metadata --
// laid out for a single sequential read:
//
//   offset  size        field
//   0       8           magic "GTSNAP01"
//   8       8           n (u64)
//   16      8           time (f64)
//   24      6 x 8       particles of each type 0..5 (u64)
//   72      8           metadata bytes m (u64)
//   80      n x 24      positions (f64 x, y, z)
//           n x 24      velocities
//           n x 8       masses (f64)
//           n x 8       IDs (u64)
//           n x 1       types (u8, 0..5)
//           n x 8       potentials (f64)
//           m           metadata: "key=value\n" lines
//
// Little-endian, as on both machines this builds for. As with the
// reference, particles are written grouped by type in ascending type order
// (stable within a type), so a read returns them that way.

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/gtc.h"

namespace gtc {
void set_contextless_error(const std::string &msg);
}

namespace {

constexpr char kMagic[8] = {'G', 'T', 'S', 'N', 'A', 'P', '0', '1'};
constexpr int kTypes = 6;

struct Header {
  char magic[8];
  uint64_t n;
  double time;
  uint64_t count[kTypes];
  uint64_t meta_bytes;
};
static_assert(sizeof(Header) == 80, "snapshot header layout");

struct FileCloser {
  void operator()(std::FILE *f) const {
    if (f) std::fclose(f);
  }
};
using File = std::unique_ptr<std::FILE, FileCloser>;

gtc_status fail(gtc_status s, const std::string &msg) {
  gtc::set_contextless_error(msg);
  return s;
}

bool put(std::FILE *f, const void *p, std::size_t bytes) {
  return bytes == 0 || std::fwrite(p, 1, bytes, f) == bytes;
}
bool get(std::FILE *f, void *p, std::size_t bytes) {
  return bytes == 0 || std::fread(p, 1, bytes, f) == bytes;
}

// Reads and checks the header; the file is left at the positions.
gtc_status read_header(const char *path, File &f, Header &h) {
  if (!path) return fail(GTC_INVALID_ARGUMENT, "snapshot: a path is required");
  f.reset(std::fopen(path, "rb"));
  if (!f) return fail(GTC_RUNTIME_ERROR, std::string("snapshot: cannot open ") + path);
  if (!get(f.get(), &h, sizeof h) || std::memcmp(h.magic, kMagic, sizeof kMagic) != 0)
    return fail(GTC_RUNTIME_ERROR, std::string("snapshot: ") + path + " is not a GTSNAP01 file");
  uint64_t total = 0;
  for (uint64_t c : h.count) total += c;
  if (total != h.n)
    return fail(GTC_RUNTIME_ERROR, std::string("snapshot: ") + path +
                                       ": per-type counts do not add up to n");
  return GTC_OK;
}

}  // namespace

extern "C" {

gtc_status gtc_write_snapshot(const char *path, uint64_t n, const double *pos, const double *vel,
                              const double *mass, const uint64_t *id, const uint8_t *type,
                              const double *pot, double time, const char *metadata) {
  if (!path) return fail(GTC_INVALID_ARGUMENT, "snapshot: a path is required");
  if (n > 0 && (!pos || !vel || !mass))
    return fail(GTC_INVALID_ARGUMENT, "snapshot: positions, velocities and masses are required");
  Header h{};
  std::memcpy(h.magic, kMagic, sizeof kMagic);
  h.n = n;
  h.time = time;
  std::vector<uint8_t> ty(n, 1);  // halo unless given (the reference's default collisionless type)
  for (uint64_t i = 0; i < n && type; ++i) {
    if (type[i] >= kTypes)
      return fail(GTC_INVALID_ARGUMENT, "snapshot: particle types are 0..5 (GADGET)");
    ty[i] = type[i];
  }
  for (uint64_t i = 0; i < n; ++i) ++h.count[ty[i]];
  const std::string meta = metadata ? metadata : "";
  h.meta_bytes = meta.size();
  // grouped by type, stable within a type
  std::vector<uint64_t> order(n);
  std::iota(order.begin(), order.end(), uint64_t{0});
  std::stable_sort(order.begin(), order.end(),
                   [&](uint64_t a, uint64_t b) { return ty[a] < ty[b]; });
  File f(std::fopen(path, "wb"));
  if (!f) return fail(GTC_RUNTIME_ERROR, std::string("snapshot: cannot create ") + path);
  bool ok = put(f.get(), &h, sizeof h);
  std::vector<double> v3(3 * n), v1(n);
  std::vector<uint64_t> u(n);
  std::vector<uint8_t> t8(n);
  auto gather3 = [&](const double *src) {
    for (uint64_t k = 0; k < n; ++k)
      for (int a = 0; a < 3; ++a) v3[3 * k + a] = src[3 * order[k] + a];
  };
  gather3(pos);
  ok = ok && put(f.get(), v3.data(), v3.size() * 8);
  gather3(vel);
  ok = ok && put(f.get(), v3.data(), v3.size() * 8);
  for (uint64_t k = 0; k < n; ++k) v1[k] = mass[order[k]];
  ok = ok && put(f.get(), v1.data(), n * 8);
  for (uint64_t k = 0; k < n; ++k) u[k] = id ? id[order[k]] : order[k];
  ok = ok && put(f.get(), u.data(), n * 8);
  for (uint64_t k = 0; k < n; ++k) t8[k] = ty[order[k]];
  ok = ok && put(f.get(), t8.data(), n);
  for (uint64_t k = 0; k < n; ++k) v1[k] = pot ? pot[order[k]] : 0.0;
  ok = ok && put(f.get(), v1.data(), n * 8);
  ok = ok && put(f.get(), meta.data(), meta.size());
  ok = std::fflush(f.get()) == 0 && ok;
  if (!ok) return fail(GTC_RUNTIME_ERROR, std::string("snapshot: writing ") + path + " failed");
  return GTC_OK;
}

gtc_status gtc_snapshot_info(const char *path, uint64_t *n, double *time,
                             uint64_t count_by_type[6], uint64_t *metadata_bytes) {
  File f;
  Header h{};
  const gtc_status s = read_header(path, f, h);
  if (s != GTC_OK) return s;
  if (n) *n = h.n;
  if (time) *time = h.time;
  if (count_by_type)
    for (int k = 0; k < kTypes; ++k) count_by_type[k] = h.count[k];
  if (metadata_bytes) *metadata_bytes = h.meta_bytes;
  return GTC_OK;
}

gtc_status gtc_read_snapshot(const char *path, uint64_t n, double *pos, double *vel, double *mass,
                             uint64_t *id, uint8_t *type, double *pot, char *metadata) {
  File f;
  Header h{};
  const gtc_status s = read_header(path, f, h);
  if (s != GTC_OK) return s;
  if (n != h.n)
    return fail(GTC_INVALID_ARGUMENT, "snapshot: the arrays hold " + std::to_string(n) +
                                          " particles, the file " + std::to_string(h.n));
  std::vector<char> skip;
  auto field = [&](void *dst, std::size_t bytes) {
    if (dst) return get(f.get(), dst, bytes);
    skip.resize(bytes);
    return get(f.get(), skip.data(), bytes);
  };
  bool ok = field(pos, 24 * n) && field(vel, 24 * n) && field(mass, 8 * n) && field(id, 8 * n) &&
            field(type, n) && field(pot, 8 * n) && field(metadata, h.meta_bytes);
  if (!ok) return fail(GTC_RUNTIME_ERROR, std::string("snapshot: ") + path + " is truncated");
  return GTC_OK;
}

}  // extern "C"
