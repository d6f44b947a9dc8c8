// Checkpoint files and run controls (no counterpart in the reference, whose
// only output is the results.<rank> text written at the end of Solve(),
// TimeSolverExplicitRK4.h:514-538).
//
// File layout (little-endian, as both supported hosts are):
//   bytes  0..7   magic "MINIAERO"
//          8..11  uint32 version (1)
//         12..15  uint32 header bytes (64)
//         16..23  int64  cells
//         24..31  int64  RK4 steps done
//         32..39  double simulated time
//         40..47  double dt
//         48..55  uint64 mesh hash (ma_mesh_hash)
//         56..63  uint64 payload hash (word-wise FNV-1a of the payload)
//   then the conserved state, component-major: 5 x cells doubles.
// A file is written to "<path>.tmp" and renamed over <path>, so a reader
// never sees a partly written checkpoint under the final name.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../../include/miniaero_gpu.h"
#include "errors.hpp"

using miniaero::set_error;

namespace {

constexpr char kMagic[8] = {'M', 'I', 'N', 'I', 'A', 'E', 'R', 'O'};
constexpr uint32_t kVersion = 1;
constexpr uint32_t kHeaderBytes = 64;
constexpr uint64_t kFnvOffset = 14695981039346656037ull;
constexpr uint64_t kFnvPrime = 1099511628211ull;

// FNV-1a applied to 64-bit words instead of bytes (one xor and one multiply
// per word).
struct WordHash {
  uint64_t h = kFnvOffset;
  void add(uint64_t w) { h = (h ^ w) * kFnvPrime; }
  void add_bytes(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
      uint64_t w;
      std::memcpy(&w, b + i, 8);
      add(w);
    }
    if (i < n) {
      uint64_t w = 0;
      std::memcpy(&w, b + i, n - i);
      add(w);
    }
  }
};

struct Header {
  char magic[8];
  uint32_t version;
  uint32_t header_bytes;
  int64_t cells;
  int64_t steps_done;
  double time;
  double dt;
  uint64_t mesh_hash;
  uint64_t payload_hash;
};
static_assert(sizeof(Header) == kHeaderBytes, "checkpoint header layout");

}  // namespace

extern "C" uint64_t ma_mesh_hash(const ma_mesh_view* v) {
  if (!v) return 0;
  WordHash h;
  h.add(static_cast<uint64_t>(v->ncells));
  if (v->ncells > 0 && v->cell_coords) h.add_bytes(v->cell_coords, sizeof(double) * 3 * static_cast<size_t>(v->ncells));
  if (v->ncells > 0 && v->cell_volumes) h.add_bytes(v->cell_volumes, sizeof(double) * static_cast<size_t>(v->ncells));
  h.add(static_cast<uint64_t>(v->internal.nfaces));
  h.add(static_cast<uint64_t>(v->nbc));
  for (int b = 0; b < v->nbc && b < MA_MAX_BC_SETS; ++b) {
    h.add(static_cast<uint64_t>(v->bc[b].type));
    h.add(static_cast<uint64_t>(v->bc[b].nfaces));
  }
  return h.h;
}

extern "C" ma_status ma_checkpoint_write(const char* path, const ma_checkpoint_info* info, const double* U,
                                         int32_t layout) {
  if (!path || !info || !U) return set_error(MA_EINVAL, "ma_checkpoint_write: null argument");
  if (info->ncells <= 0) return set_error(MA_EINVAL, "ma_checkpoint_write: no cells");
  if (layout != MA_LAYOUT_AOS && layout != MA_LAYOUT_SOA) return set_error(MA_EINVAL, "unknown state layout");
  const size_t C = static_cast<size_t>(info->ncells);
  std::vector<double> soa;
  const double* payload = U;
  if (layout == MA_LAYOUT_AOS) {
    soa.resize(5 * C);
    for (size_t c = 0; c < C; ++c)
      for (int k = 0; k < 5; ++k) soa[k * C + c] = U[5 * c + k];
    payload = soa.data();
  }
  Header hd;
  std::memcpy(hd.magic, kMagic, 8);
  hd.version = kVersion;
  hd.header_bytes = kHeaderBytes;
  hd.cells = info->ncells;
  hd.steps_done = info->steps_done;
  hd.time = info->time;
  hd.dt = info->dt;
  hd.mesh_hash = info->mesh_hash;
  WordHash ph;
  ph.add_bytes(payload, sizeof(double) * 5 * C);
  hd.payload_hash = ph.h;
  const std::string tmp = std::string(path) + ".tmp";
  {
    std::ofstream out(tmp, std::ios::binary | std::ios::trunc);
    if (!out) return set_error(MA_EIO, tmp + ": cannot open for writing");
    out.write(reinterpret_cast<const char*>(&hd), sizeof(hd));
    out.write(reinterpret_cast<const char*>(payload), static_cast<std::streamsize>(sizeof(double) * 5 * C));
    out.flush();
    if (!out) {
      std::remove(tmp.c_str());
      return set_error(MA_EIO, tmp + ": write failed");
    }
  }
  if (std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return set_error(MA_EIO, std::string(path) + ": cannot rename the written checkpoint into place");
  }
  return MA_OK;
}

extern "C" ma_status ma_checkpoint_read(const char* path, ma_checkpoint_info* info, double* U, int64_t max_cells,
                                        int32_t layout) {
  if (!path || !info) return set_error(MA_EINVAL, "ma_checkpoint_read: null argument");
  if (layout != MA_LAYOUT_AOS && layout != MA_LAYOUT_SOA) return set_error(MA_EINVAL, "unknown state layout");
  std::ifstream in(path, std::ios::binary);
  if (!in) return set_error(MA_EIO, std::string(path) + ": cannot open");
  Header hd;
  in.read(reinterpret_cast<char*>(&hd), sizeof(hd));
  if (!in) return set_error(MA_EIO, std::string(path) + ": truncated header");
  if (std::memcmp(hd.magic, kMagic, 8) != 0) return set_error(MA_EINVAL, std::string(path) + ": not a checkpoint");
  if (hd.version != kVersion || hd.header_bytes != kHeaderBytes)
    return set_error(MA_EINVAL, std::string(path) + ": unsupported checkpoint version");
  if (hd.cells <= 0) return set_error(MA_EINVAL, std::string(path) + ": bad cell count");
  info->ncells = hd.cells;
  info->steps_done = hd.steps_done;
  info->time = hd.time;
  info->dt = hd.dt;
  info->mesh_hash = hd.mesh_hash;
  if (!U) return MA_OK;  // header only
  if (hd.cells > max_cells)
    return set_error(MA_EINVAL, std::string(path) + ": holds " + std::to_string(hd.cells) +
                                    " cells, more than the buffer's " + std::to_string(max_cells));
  const size_t C = static_cast<size_t>(hd.cells);
  std::vector<double> soa(5 * C);
  in.read(reinterpret_cast<char*>(soa.data()), static_cast<std::streamsize>(sizeof(double) * 5 * C));
  if (!in) return set_error(MA_EIO, std::string(path) + ": truncated state");
  WordHash ph;
  ph.add_bytes(soa.data(), sizeof(double) * 5 * C);
  if (ph.h != hd.payload_hash) return set_error(MA_EIO, std::string(path) + ": state checksum mismatch");
  if (layout == MA_LAYOUT_SOA) {
    std::memcpy(U, soa.data(), sizeof(double) * 5 * C);
  } else {
    for (size_t c = 0; c < C; ++c)
      for (int k = 0; k < 5; ++k) U[5 * c + k] = soa[k * C + c];
  }
  return MA_OK;
}

extern "C" void ma_run_options_default(ma_run_options* r) {
  if (!r) return;
  std::memset(r, 0, sizeof(*r));
}

extern "C" ma_status ma_run_options_read(const char* path, ma_run_options* r) {
  if (!path || !r) return set_error(MA_EINVAL, "ma_run_options_read: null argument");
  ma_run_options_default(r);
  std::ifstream in(path);
  if (!in) return set_error(MA_EIO, std::string(path) + " does not exist.");
  // The 14 positional values (problem type, lx ly lz angle, nx ny nz,
  // steps, dt, output_results, output_frequency, second order, viscous) are
  // ma_options_read's; skip them. Options follow, one per line.
  std::string tok;
  for (int i = 0; i < 14; ++i)
    if (!(in >> tok)) return set_error(MA_EINVAL, std::string(path) + ": expected the positional values");
  std::string key;
  while (in >> key) {
    if (!key.empty() && key[0] == '#') { std::string rest; std::getline(in, rest); continue; }
    auto path_value = [&](char* dst) -> bool {
      std::string v;
      if (!(in >> v) || v.size() >= MA_PATH_MAX) return false;
      std::memcpy(dst, v.c_str(), v.size() + 1);
      return true;
    };
    if (key == "checkpoint") {
      if (!path_value(r->checkpoint_path)) return set_error(MA_EINVAL, std::string(path) + ": bad value for 'checkpoint'");
    } else if (key == "checkpoint_frequency") {
      if (!(in >> r->checkpoint_frequency) || r->checkpoint_frequency < 0)
        return set_error(MA_EINVAL, std::string(path) + ": bad value for 'checkpoint_frequency'");
    } else if (key == "restart") {
      if (!path_value(r->restart_path)) return set_error(MA_EINVAL, std::string(path) + ": bad value for 'restart'");
    } else {
      std::string rest;
      std::getline(in, rest);  // an option of ma_options_read: skipped here
    }
  }
  return MA_OK;
}
