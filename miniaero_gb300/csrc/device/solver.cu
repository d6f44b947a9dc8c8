// Device mesh, solver objects and the device half of the C ABI.
//
// ma_mesh_upload turns a reference-ordered mesh (MeshData, kokkos/MeshData.h)
// into the device layout:
//  * internal faces re-ordered by tile of 4096 left cells, then face class
//    (axis alignment), then (left, right) cell, for locality and uniform
//    warps; face results do not depend on the order faces are computed in;
//  * boundary faces grouped by BC type (Extrapolate, Tangent, NoSlip, Inflow);
//  * per-face Roe frame |n|, n/|n|, t/|t|, b/|b| and centroid offsets,
//    computed once with the reference's expressions;
//  * per-cell ordered contribution lists that replay the reference's serial
//    accumulation order: internal faces in permutation order, then boundary
//    sets in boundary_faces order (GreenGauss.h:300-321, StencilLimiter.h:532-616)
//    or grouped by BC type (TimeSolverExplicitRK4.h:428-475) for the residual.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../../include/miniaero_gpu.h"
#include "../host/errors.hpp"
#include "../host/parallel.hpp"
#include "../host/trace.hpp"
#include "batch_internal.hpp"
#include "kernels.cuh"

using miniaero::set_error;
namespace dev = miniaero::dev;

#define MA_CUDA_TRY(expr)                                                                   \
  do {                                                                                     \
    cudaError_t err__ = (expr);                                                            \
    if (err__ != cudaSuccess)                                                              \
      return set_error(MA_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(err__)); \
  } while (0)

namespace {

// Single device allocation carved into aligned pieces.
struct Arena {
  char* base = nullptr;
  size_t size = 0, used = 0;
  template <class T>
  T* take(size_t n) {
    const size_t off = (used + 255) & ~size_t(255);
    used = off + n * sizeof(T);
    return base ? reinterpret_cast<T*>(base + off) : nullptr;
  }
};

}  // namespace

struct ma_mesh {
  dev::TopoView topo;
  dev::TopoView topo_cf;     // topo with the CELL_FLUX lists (MA_MESH_CELL_FLUX)
  bool has_cell_flux = false;
  dev::GeomView<double> g64;
  dev::GeomView<float> g32;
  void* dmem = nullptr;
  size_t bytes = 0;
  int device = 0;
};

struct ma_solver {
  ma_mesh* mesh = nullptr;
  dev::TopoView topo;  // the mesh's lists in the gather order of the options
  ma_options opts;
  dev::PathConfig cfg;
  bool mixed = false;
  bool fma = false;  // MA_PREC_FP64_FMA: the FP64 kernels built with multiply-add contraction
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;       // graph side branch: the boundary-face flux
  cudaEvent_t fork = nullptr, join = nullptr;
  dev::StateBuffers st;
  dev::StageBuffers<double> b64;
  dev::StageBuffers<float> b32;
  void* dmem = nullptr;
  size_t bytes = 0;
  unsigned long long* dscratch = nullptr;  // 8-byte reduction slot
  cudaGraphExec_t graph = nullptr;
  bool state_set = false;
  int64_t steps_done = 0;
};

// ---------------------------------------------------------------------------
extern "C" int32_t ma_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

namespace {

ma_status validate_view(const ma_mesh_view* v) {
  if (!v) return set_error(MA_EINVAL, "mesh view is null");
  if (v->ncells <= 0) return set_error(MA_EINVAL, "mesh has no cells");
  if (!v->cell_coords || !v->cell_volumes) return set_error(MA_EINVAL, "mesh cell arrays are null");
  if (v->nbc < 0 || v->nbc > MA_MAX_BC_SETS) return set_error(MA_EINVAL, "bad boundary set count");
  auto check_set = [&](const ma_face_set& s, bool internal) -> ma_status {
    if (s.nfaces < 0) return set_error(MA_EINVAL, "negative face count");
    if (s.nfaces == 0) return MA_OK;
    if (!s.conn || !s.coords || !s.normal || !s.tangent || !s.binormal || !s.permutation)
      return set_error(MA_EINVAL, "face set has null arrays");
    if (!internal && (s.type < 0 || s.type > 3)) return set_error(MA_EINVAL, "unknown boundary condition type");
    std::vector<char> seen(static_cast<size_t>(s.nfaces), 0);
    for (int32_t i = 0; i < s.nfaces; ++i) {
      const int32_t p = s.permutation[i];
      if (p < 0 || p >= s.nfaces || seen[p]) return set_error(MA_EINVAL, "face permutation is not a permutation");
      seen[p] = 1;
      const int32_t L = s.conn[2 * i], R = s.conn[2 * i + 1];
      if (L < 0 || L >= v->ncells) return set_error(MA_EINVAL, "face left cell out of range");
      if (internal && (R < 0 || R >= v->ncells || R == L)) return set_error(MA_EINVAL, "internal face right cell out of range");
    }
    return MA_OK;
  };
  ma_status st = check_set(v->internal, true);
  if (st != MA_OK) return st;
  for (int b = 0; b < v->nbc; ++b) {
    st = check_set(v->bc[b], false);
    if (st != MA_OK) return st;
  }
  for (int32_t c = 0; c < v->ncells; ++c)
    if (!(v->cell_volumes[c] > 0.0)) return set_error(MA_EINVAL, "non-positive cell volume");
  return MA_OK;
}

constexpr int32_t kMaxMeshCells = MA_MAX_MESH_CELLS;  // floor((2^31 - 1) / 15)
static_assert(15LL * kMaxMeshCells <= 2147483647LL && 15LL * (kMaxMeshCells + 1) > 2147483647LL,
              "the largest mesh whose gradient index fits int32");

// Position of a BC type in the residual order Extrapolate, Tangent, NoSlip, Inflow.
inline int type_rank(int type) {
  switch (type) {
    case MA_BC_EXTRAPOLATE: return 0;
    case MA_BC_TANGENT: return 1;
    case MA_BC_NOSLIP: return 2;
    default: return 3;
  }
}

}  // namespace

extern "C" ma_status ma_mesh_upload(const ma_mesh_view* v, ma_mesh** out) { return ma_mesh_upload_ex(v, 0, out); }

extern "C" ma_status ma_mesh_upload_ex(const ma_mesh_view* v, int32_t flags, ma_mesh** out) {
  if (!out) return set_error(MA_EINVAL, "ma_mesh_upload: out is null");
  if (flags & ~MA_MESH_CELL_FLUX) return set_error(MA_EINVAL, "ma_mesh_upload_ex: unknown flags");
  const bool cell_flux = (flags & MA_MESH_CELL_FLUX) != 0;
  *out = nullptr;
  miniaero::TraceRange trace("ma_mesh_upload");
  // Device arrays are indexed with 32-bit arithmetic; the widest per-cell
  // array is the gradient, 15 values a cell at (3k + d) C + c.
  if (v && v->ncells > kMaxMeshCells)
    return set_error(MA_EINVAL, "mesh has " + std::to_string(v->ncells) + " cells; at most " +
                                    std::to_string(kMaxMeshCells) + " fit the device's 32-bit indexing");
  ma_status st = validate_view(v);
  if (st != MA_OK) return st;
  try {
    const int32_t C = v->ncells;
    const int32_t Fi = v->internal.nfaces;
    int64_t Fb64 = 0;
    for (int b = 0; b < v->nbc; ++b) Fb64 += v->bc[b].nfaces;
    if (static_cast<int64_t>(Fi) + Fb64 >= (1LL << 30)) return set_error(MA_EINVAL, "too many faces");
    const int32_t Fb = static_cast<int32_t>(Fb64);
    const int32_t F = Fi + Fb;

    std::vector<int32_t> order(Fi);  // device position -> internal face index
    // Face classes. A face is aligned with axis D when its area vector is
    // nonzero only along D, its tangent only along (D+2)%3 and its binormal
    // only along (D+1)%3: class D when in addition both face-to-cell offsets
    // (face centre minus cell centre, as the geometry below stores them) are
    // nonzero only along D, class D + 3 otherwise; the general faces are
    // class 6. Device order: tiles of kFaceTileCells left cells, by class
    // within a tile, (left, right) within a class. A warp then sees one class
    // (one code path), and the cells a tile's faces read are re-read by the
    // tile's other classes while they are still in L2.
    std::vector<uint8_t> fclass_dev(Fi);
    {
      auto offsets_along = [&](int32_t i, int D) {
        const double* x = &v->internal.coords[3 * static_cast<size_t>(i)];
        const double* xl = &v->cell_coords[3 * static_cast<size_t>(v->internal.conn[2 * i])];
        const double* xr = &v->cell_coords[3 * static_cast<size_t>(v->internal.conn[2 * i + 1])];
        for (int d = 0; d < 3; ++d)
          if (d != D && (x[d] - xl[d] != 0.0 || x[d] - xr[d] != 0.0)) return false;
        return true;
      };
      auto face_class = [&](int32_t i) -> int {
        const double* n = &v->internal.normal[3 * static_cast<size_t>(i)];
        const double* tt = &v->internal.tangent[3 * static_cast<size_t>(i)];
        const double* b = &v->internal.binormal[3 * static_cast<size_t>(i)];
        for (int D = 0; D < 3; ++D) {
          const int T = (D + 2) % 3, B = (D + 1) % 3;
          bool ok = n[D] != 0.0 && tt[T] != 0.0 && b[B] != 0.0;
          for (int d = 0; d < 3 && ok; ++d) {
            if (d != D && n[d] != 0.0) ok = false;
            if (d != T && tt[d] != 0.0) ok = false;
            if (d != B && b[d] != 0.0) ok = false;
          }
          if (ok) return offsets_along(i, D) ? D : D + 3;
        }
        return 6;
      };
      std::vector<uint8_t> cls(Fi);
      miniaero::parallel_for(static_cast<size_t>(Fi), [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) cls[i] = static_cast<uint8_t>(face_class(static_cast<int32_t>(i)));
      });
      // Sort by (tile of left, class, left, right, index): a stable LSD radix
      // sort (11-bit digits) of (key, index) words with key = tile | class |
      // left within the tile, then the right cell orders each run of equal
      // keys (a cell is the left cell of at most 6 faces).
      static_assert((dev::kFaceTileCells & (dev::kFaceTileCells - 1)) == 0, "tile size is a power of two");
      constexpr int kTileShift = __builtin_ctz(dev::kFaceTileCells);
      int tile_bits = 0;
      while ((static_cast<uint64_t>(C - 1) >> (kTileShift + tile_bits)) != 0) ++tile_bits;
      const int key_bits = tile_bits + 3 + kTileShift;  // < 33 for C < 2^30
      const int32_t* conn = v->internal.conn;
      std::vector<uint64_t> words(Fi), tmp(Fi);
      miniaero::parallel_for(static_cast<size_t>(Fi), [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
          const uint64_t L = static_cast<uint32_t>(conn[2 * i]);
          const uint64_t key = ((L >> kTileShift) << (3 + kTileShift)) | (static_cast<uint64_t>(cls[i]) << kTileShift) |
                               (L & (dev::kFaceTileCells - 1));
          words[i] = (key << 30) | i;  // Fi < 2^30
        }
      });
      for (int shift = 30; shift < 30 + key_bits; shift += 11) {
        size_t count[2048] = {0};
        for (const uint64_t w : words) count[(w >> shift) & 2047]++;
        size_t acc = 0;
        for (size_t& c : count) { const size_t n = c; c = acc; acc += n; }
        for (const uint64_t w : words) tmp[count[(w >> shift) & 2047]++] = w;
        words.swap(tmp);
      }
      for (int32_t g = 0; g < Fi; ++g) order[g] = static_cast<int32_t>(words[g] & ((1ull << 30) - 1));
      for (int32_t g = 0; g < Fi;) {  // runs of one left cell and class: order by right cell
        int32_t e = g + 1;
        while (e < Fi && (words[e] >> 30) == (words[g] >> 30)) ++e;
        for (int32_t a = g + 1; a < e; ++a) {
          const int32_t x = order[a];
          int32_t b = a - 1;
          while (b >= g && conn[2 * order[b] + 1] > conn[2 * x + 1]) { order[b + 1] = order[b]; --b; }
          order[b + 1] = x;
        }
        g = e;
      }
      for (int32_t g = 0; g < Fi; ++g) fclass_dev[g] = cls[order[g]];
    }
    std::vector<int32_t> gpu_of_internal(Fi);
    for (int32_t g = 0; g < Fi; ++g) gpu_of_internal[order[g]] = g;

    // Boundary faces grouped by type rank, then set order, then storage order.
    std::vector<int32_t> bc_base(v->nbc, 0);
    int32_t nbc_type[4] = {0, 0, 0, 0};
    {
      int32_t pos = Fi;
      for (int r = 0; r < 4; ++r)
        for (int b = 0; b < v->nbc; ++b)
          if (type_rank(v->bc[b].type) == r) {
            bc_base[b] = pos;
            pos += v->bc[b].nfaces;
            nbc_type[r] += v->bc[b].nfaces;
          }
    }

    // Host staging of face data in device order.
    std::vector<int32_t> fconn(2 * static_cast<size_t>(F));
    // fn3 fnu3 ftu3 fbu3 fnn1 dL3 dR3; every entry is written below (no zero fill
    // of the ~150 B per face up front: the writes spread over the threads).
    const size_t geo_size = 19 * static_cast<size_t>(F);
    std::unique_ptr<double[]> geo_buf(new double[geo_size]);
    double* const geo = geo_buf.get();
    auto put_face = [&](int32_t g, const ma_face_set& s, int32_t i, bool internal) {
      const int32_t L = s.conn[2 * i];
      const int32_t R = internal ? s.conn[2 * i + 1] : -1;
      fconn[g] = L;
      fconn[static_cast<size_t>(F) + g] = R;
      const double* n = &s.normal[3 * static_cast<size_t>(i)];
      const double* t = &s.tangent[3 * static_cast<size_t>(i)];
      const double* b = &s.binormal[3 * static_cast<size_t>(i)];
      const double* x = &s.coords[3 * static_cast<size_t>(i)];
      // Roe_Flux.h:100-118
      const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      const double tn = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
      const double bn = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
      for (int d = 0; d < 3; ++d) {
        geo[(0 + d) * static_cast<size_t>(F) + g] = n[d];
        geo[(3 + d) * static_cast<size_t>(F) + g] = n[d] / nn;
        geo[(6 + d) * static_cast<size_t>(F) + g] = t[d] / tn;
        geo[(9 + d) * static_cast<size_t>(F) + g] = b[d] / bn;
        geo[(13 + d) * static_cast<size_t>(F) + g] = x[d] - v->cell_coords[3 * static_cast<size_t>(L) + d];
        geo[(16 + d) * static_cast<size_t>(F) + g] =
            internal ? x[d] - v->cell_coords[3 * static_cast<size_t>(R) + d] : 0.0;
      }
      geo[12 * static_cast<size_t>(F) + g] = nn;
    };
    // In device order (sequential writes, gathered reads), on the host's threads.
    miniaero::parallel_for(static_cast<size_t>(Fi), [&](size_t b, size_t e) {
      for (size_t g = b; g < e; ++g) put_face(static_cast<int32_t>(g), v->internal, order[g], true);
    });
    for (int b = 0; b < v->nbc; ++b)
      for (int32_t i = 0; i < v->bc[b].nfaces; ++i) put_face(bc_base[b] + i, v->bc[b], i, false);

    // Ordered per-cell contribution lists.
    const size_t K = dev::kMaxCellFaces;
    std::vector<int32_t> csr_grad(K * C, -1), csr_nbr(K * C, -1), csr_flux(K * C, -1);
    std::vector<uint8_t> ng(C, 0), nf(C, 0);
    bool overflow = false;
    auto push = [&](std::vector<int32_t>& csr, std::vector<uint8_t>& n, int32_t cell, int32_t code, int32_t nbr,
                    bool with_nbr) {
      if (n[cell] >= K) { overflow = true; return; }
      csr[n[cell] * static_cast<size_t>(C) + cell] = code;
      if (with_nbr) csr_nbr[n[cell] * static_cast<size_t>(C) + cell] = nbr;
      n[cell]++;
    };
    for (int32_t ii = 0; ii < Fi; ++ii) {
      const int32_t i = v->internal.permutation[ii];
      const int32_t g = gpu_of_internal[i];
      const int32_t L = v->internal.conn[2 * i], R = v->internal.conn[2 * i + 1];
      push(csr_grad, ng, L, (g << 1) | 1, R, true);
      push(csr_grad, ng, R, (g << 1), L, true);
      push(csr_flux, nf, L, (g << 1) | 1, 0, false);
      push(csr_flux, nf, R, (g << 1), 0, false);
    }
    for (int b = 0; b < v->nbc; ++b)  // boundary_faces order
      for (int32_t i = 0; i < v->bc[b].nfaces; ++i)
        push(csr_grad, ng, v->bc[b].conn[2 * i], ((bc_base[b] + i) << 1) | 1, v->bc[b].conn[2 * i], true);
    for (int r = 0; r < 4; ++r)  // grouped by BC type
      for (int b = 0; b < v->nbc; ++b)
        if (type_rank(v->bc[b].type) == r)
          for (int32_t i = 0; i < v->bc[b].nfaces; ++i)
            push(csr_flux, nf, v->bc[b].conn[2 * i], ((bc_base[b] + i) << 1) | 1, 0, false);
    if (overflow) return set_error(MA_EINVAL, "a cell has more than 6 faces");

    // CELL_FLUX lists (MA_MESH_CELL_FLUX): each cell's faces in element-local
    // slot order (flux_index, Faces.h:109-110), the order in which the
    // reference's -DCELL_FLUX build sums its per-slot storage (GreenGauss.h:
    // 244-269, Flux.h:188-229); one list serves the gradient and the residual.
    std::vector<int32_t> cf_grad, cf_nbr, cf_flux;
    if (cell_flux) {
      cf_grad.assign(K * C, -1);
      cf_nbr.assign(K * C, -1);
      auto put = [&](int32_t cell, int32_t slot, int32_t code, int32_t nbr) {
        if (slot < 0 || slot >= static_cast<int32_t>(K)) return false;
        int32_t& dst = cf_grad[static_cast<size_t>(slot) * C + cell];
        if (dst != -1) return false;
        dst = code;
        cf_nbr[static_cast<size_t>(slot) * C + cell] = nbr;
        return true;
      };
      bool ok = v->internal.nfaces == 0 || v->internal.flux_index;
      for (int b = 0; b < v->nbc; ++b) ok = ok && (v->bc[b].nfaces == 0 || v->bc[b].flux_index);
      if (!ok) return set_error(MA_EINVAL, "MA_MESH_CELL_FLUX needs every face set's flux_index");
      for (int32_t i = 0; i < Fi && ok; ++i) {
        const int32_t g = gpu_of_internal[i];
        const int32_t L = v->internal.conn[2 * i], R = v->internal.conn[2 * i + 1];
        ok = put(L, v->internal.flux_index[2 * i], (g << 1) | 1, R) && put(R, v->internal.flux_index[2 * i + 1], g << 1, L);
      }
      for (int b = 0; b < v->nbc && ok; ++b)
        for (int32_t i = 0; i < v->bc[b].nfaces && ok; ++i)
          ok = put(v->bc[b].conn[2 * i], v->bc[b].flux_index[2 * i], ((bc_base[b] + i) << 1) | 1, v->bc[b].conn[2 * i]);
      if (!ok) return set_error(MA_EINVAL, "flux_index out of range or repeated within a cell");
      cf_flux = cf_grad;  // residual order: plain slot order
    }

    // Axis-aligned cells: every face area vector has exactly one nonzero
    // component and each axis owns two faces. A gradient component (k, d)
    // then receives nonzero terms only from the two d-faces; the other terms
    // are signed zeros, which cannot change an accumulator that starts at +0.
    // The gradient list of such a cell is regrouped by axis (x, x, y, y, z, z),
    // keeping the serial order within each axis, and the cell is flagged.
    std::vector<uint8_t> axis_cell(C, 0);
    {
      auto axis_of = [&](int32_t g) -> int {
        int nz = 0, ax = -1;
        for (int d = 0; d < 3; ++d)
          if (geo[d * static_cast<size_t>(F) + g] != 0.0) { ++nz; ax = d; }
        return nz == 1 ? ax : -1;
      };
      for (int32_t c = 0; c < C; ++c) {
        if (ng[c] != K) continue;
        int32_t codes[6], axes[6], count[3] = {0, 0, 0};
        bool ok = true;
        for (size_t s2 = 0; s2 < K && ok; ++s2) {
          codes[s2] = csr_grad[s2 * C + c];
          axes[s2] = axis_of(codes[s2] >> 1);
          if (axes[s2] < 0 || ++count[axes[s2]] > 2) ok = false;
        }
        if (!ok) continue;
        // Bit 1: every face-to-cell offset seen from this cell (x_f - x_c,
        // geometry rows 13..15 on the left side, 16..18 on the right) is
        // nonzero only along the face's axis.
        bool aligned = true;
        for (size_t s2 = 0; s2 < K; ++s2) {
          const size_t g = static_cast<size_t>(codes[s2] >> 1);
          const int base = (codes[s2] & 1) ? 13 : 16;
          for (int d = 0; d < 3; ++d)
            if (d != axes[s2] && geo[(base + d) * static_cast<size_t>(F) + g] != 0.0) aligned = false;
        }
        // Group a list by axis, keeping its order within each axis.
        auto regroup = [&](std::vector<int32_t>& grad, std::vector<int32_t>& nbr) {
          int32_t cs[6], ns[6], as[6];
          for (size_t s2 = 0; s2 < K; ++s2) {
            cs[s2] = grad[s2 * C + c];
            ns[s2] = nbr[s2 * C + c];
            as[s2] = axis_of(cs[s2] >> 1);
          }
          size_t out = 0;
          for (int d = 0; d < 3; ++d)
            for (size_t s2 = 0; s2 < K; ++s2)
              if (as[s2] == d) {
                grad[out * C + c] = cs[s2];
                nbr[out * C + c] = ns[s2];
                ++out;
              }
        };
        regroup(csr_grad, csr_nbr);
        if (cell_flux) regroup(cf_grad, cf_nbr);
        axis_cell[c] = aligned ? 3 : 1;
      }
    }

    // Device arena.
    Arena a;
    auto layout = [&](ma_mesh& m) {
      m.topo.vol = a.take<double>(C);
      m.topo.fconn = a.take<int32_t>(2 * static_cast<size_t>(F));
      m.topo.csr_grad = a.take<int32_t>(K * C);
      m.topo.csr_nbr = a.take<int32_t>(K * C);
      m.topo.csr_flux = a.take<int32_t>(K * C);
      m.topo.axis_cell = a.take<uint8_t>(C);
      m.topo.fclass = a.take<uint8_t>(static_cast<size_t>(Fi));
      double* g64 = a.take<double>(19 * static_cast<size_t>(F));
      float* g32 = a.take<float>(19 * static_cast<size_t>(F));
      double* vol64 = const_cast<double*>(m.topo.vol);
      float* vol32 = a.take<float>(C);
      double* vinv64 = a.take<double>(C);
      float* vinv32 = a.take<float>(C);
      if (cell_flux) {
        m.topo_cf.csr_grad = a.take<int32_t>(K * C);
        m.topo_cf.csr_nbr = a.take<int32_t>(K * C);
        m.topo_cf.csr_flux = a.take<int32_t>(K * C);
      }
      auto assign = [&](auto& gv, auto* base, auto* vol, auto* vinv) {
        gv.vol = vol;
        gv.vinv = vinv;
        gv.fn = base;
        gv.fnu = base + 3 * static_cast<size_t>(F);
        gv.ftu = base + 6 * static_cast<size_t>(F);
        gv.fbu = base + 9 * static_cast<size_t>(F);
        gv.fnn = base + 12 * static_cast<size_t>(F);
        gv.dL = base + 13 * static_cast<size_t>(F);
        gv.dR = base + 16 * static_cast<size_t>(F);
      };
      assign(m.g64, g64, vol64, vinv64);
      assign(m.g32, g32, vol32, vinv32);
    };
    ma_mesh probe;
    layout(probe);
    const size_t bytes = a.used;
    a.used = 0;
    MA_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&a.base), bytes));
    ma_mesh* m = new ma_mesh;
    layout(*m);
    m->dmem = a.base;
    m->bytes = bytes;
    cudaGetDevice(&m->device);
    m->topo.vinv = m->g64.vinv;
    m->topo.C = C;
    m->topo.Fi = Fi;
    m->topo.Fb = Fb;
    m->topo.F = F;
    for (int r = 0; r < 4; ++r) m->topo.nbc_type[r] = nbc_type[r];
    if (cell_flux) {  // same topology and flags, lists in slot order
      const dev::TopoView lists = m->topo_cf;
      m->topo_cf = m->topo;
      m->topo_cf.csr_grad = lists.csr_grad;
      m->topo_cf.csr_nbr = lists.csr_nbr;
      m->topo_cf.csr_flux = lists.csr_flux;
      m->has_cell_flux = true;
    }

    std::unique_ptr<float[]> geo32(new float[geo_size]);
    miniaero::parallel_for(geo_size, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) geo32[i] = static_cast<float>(geo[i]);
    });
    std::vector<float> vol32(C), vinv32(C);
    std::vector<double> vinv64(C);
    for (int32_t c = 0; c < C; ++c) {
      vol32[c] = static_cast<float>(v->cell_volumes[c]);
      vinv64[c] = 1.0 / v->cell_volumes[c];
      vinv32[c] = static_cast<float>(vinv64[c]);
    }
    auto copy = [&](const void* dst, const void* src, size_t n) {
      return cudaMemcpy(const_cast<void*>(dst), src, n, cudaMemcpyHostToDevice);
    };
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = copy(m->topo.vol, v->cell_volumes, sizeof(double) * C);
    if (e == cudaSuccess) e = copy(m->topo.fconn, fconn.data(), sizeof(int32_t) * fconn.size());
    if (e == cudaSuccess) e = copy(m->topo.csr_grad, csr_grad.data(), sizeof(int32_t) * csr_grad.size());
    if (e == cudaSuccess) e = copy(m->topo.csr_nbr, csr_nbr.data(), sizeof(int32_t) * csr_nbr.size());
    if (e == cudaSuccess) e = copy(m->topo.csr_flux, csr_flux.data(), sizeof(int32_t) * csr_flux.size());
    if (cell_flux) {
      if (e == cudaSuccess) e = copy(m->topo_cf.csr_grad, cf_grad.data(), sizeof(int32_t) * cf_grad.size());
      if (e == cudaSuccess) e = copy(m->topo_cf.csr_nbr, cf_nbr.data(), sizeof(int32_t) * cf_nbr.size());
      if (e == cudaSuccess) e = copy(m->topo_cf.csr_flux, cf_flux.data(), sizeof(int32_t) * cf_flux.size());
    }
    if (e == cudaSuccess) e = copy(m->topo.axis_cell, axis_cell.data(), axis_cell.size());
    if (e == cudaSuccess && Fi > 0) e = copy(m->topo.fclass, fclass_dev.data(), fclass_dev.size());
    if (e == cudaSuccess) e = copy(m->g64.fn, geo, sizeof(double) * geo_size);
    if (e == cudaSuccess) e = copy(m->g32.fn, geo32.get(), sizeof(float) * geo_size);
    if (e == cudaSuccess) e = copy(m->g32.vol, vol32.data(), sizeof(float) * vol32.size());
    if (e == cudaSuccess) e = copy(m->g64.vinv, vinv64.data(), sizeof(double) * vinv64.size());
    if (e == cudaSuccess) e = copy(m->g32.vinv, vinv32.data(), sizeof(float) * vinv32.size());
    if (e != cudaSuccess) {
      cudaFree(m->dmem);
      delete m;
      return set_error(MA_ECUDA, std::string("ma_mesh_upload: ") + cudaGetErrorString(e));
    }
    *out = m;
    return MA_OK;
  } catch (const std::bad_alloc&) {
    return set_error(MA_ENOMEM, "ma_mesh_upload: out of host memory");
  }
}

namespace miniaero {
size_t mesh_cells(const ma_mesh* m) { return static_cast<size_t>(m->topo.C); }
size_t mesh_faces(const ma_mesh* m) { return static_cast<size_t>(m->topo.F); }
dev::TopoView mesh_topo(const ma_mesh* m) { return m->topo; }
dev::TopoView mesh_topo(const ma_mesh* m, int gather) {
  return gather == MA_GATHER_CELL_FLUX ? m->topo_cf : m->topo;
}
bool mesh_has_cell_flux(const ma_mesh* m) { return m->has_cell_flux; }
int mesh_device(const ma_mesh* m) { return m->device; }
template <>
dev::GeomView<double> mesh_geom<double>(const ma_mesh* m) { return m->g64; }
template <>
dev::GeomView<float> mesh_geom<float>(const ma_mesh* m) { return m->g32; }
}  // namespace miniaero

extern "C" void ma_mesh_free(ma_mesh* m) {
  if (!m) return;
  cudaFree(m->dmem);
  delete m;
}

extern "C" size_t ma_mesh_device_bytes(const ma_mesh* m) { return m ? m->bytes : 0; }

// ---------------------------------------------------------------------------
namespace {

// One stage's kernels (those in `kernels`) in the solver's precision.
cudaError_t solver_stage(ma_solver* s, int stage, cudaStream_t stream, unsigned kernels) {
  if (s->mixed) return dev::launch_stage<float>(s->topo, s->mesh->g32, s->cfg, s->st, s->b32, stage, stream, kernels);
  if (s->fma) return dev::launch_stage_fma(s->topo, s->mesh->g64, s->cfg, s->st, s->b64, stage, stream, kernels);
  return dev::launch_stage<double>(s->topo, s->mesh->g64, s->cfg, s->st, s->b64, stage, stream, kernels);
}

ma_status capture_step_graph(ma_solver* s) {
  if (s->graph) {
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  MA_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int stage = 0; stage < 4 && e == cudaSuccess; ++stage) {
    auto launch = [&](cudaStream_t stream, unsigned kernels) { return solver_stage(s, stage, stream, kernels); };
    // The boundary-face flux reads only the stage's primitives and writes its
    // own flux slots: a side branch of the graph runs it beside the sweep and
    // the internal-face flux, and the residual waits for both branches.
    const bool fork = s->topo.Fb > 0;
    if (fork) {
      e = cudaEventRecord(s->fork, s->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s->side, s->fork, 0);
      if (e == cudaSuccess) e = launch(s->side, dev::kBcFlux);
      if (e == cudaSuccess) e = cudaEventRecord(s->join, s->side);
    }
    if (e == cudaSuccess) e = launch(s->stream, dev::kSweep1 | dev::kInternalFlux);
    if (e == cudaSuccess && fork) e = cudaStreamWaitEvent(s->stream, s->join, 0);
    if (e == cudaSuccess) e = launch(s->stream, dev::kResidual);
  }
  cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return set_error(MA_ECUDA, std::string("step capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  e = cudaGraphInstantiate(&s->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_error(MA_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return MA_OK;
}

}  // namespace

extern "C" ma_status ma_solver_create(ma_mesh* mesh, const ma_options* o, ma_solver** out) {
  if (!mesh || !o || !out) return set_error(MA_EINVAL, "ma_solver_create: null argument");
  *out = nullptr;
  if (o->precision != MA_PREC_FP64 && o->precision != MA_PREC_MIXED && o->precision != MA_PREC_FP64_FMA)
    return set_error(MA_EINVAL, "bad precision");
  if (o->limiter != MA_LIMITER_VENKAT && o->limiter != MA_LIMITER_VANALBADA) return set_error(MA_EINVAL, "bad limiter");
  if (o->viscosity_model != MA_VISC_SUTHERLAND && o->viscosity_model != MA_VISC_CONSTANT)
    return set_error(MA_EINVAL, "bad viscosity model");
  if (o->viscosity_model == MA_VISC_CONSTANT && !(o->mu >= 0.0 && o->prandtl > 0.0))
    return set_error(MA_EINVAL, "constant viscosity needs mu >= 0 and prandtl > 0");
  if (!(o->cfl > 0.0) && !(o->dt > 0.0)) return set_error(MA_EINVAL, "dt must be > 0 (or cfl > 0)");
  if (o->gather != MA_GATHER_ATOMICS && o->gather != MA_GATHER_CELL_FLUX) return set_error(MA_EINVAL, "bad gather");
  if (o->gather == MA_GATHER_CELL_FLUX && !mesh->has_cell_flux)
    return set_error(MA_EINVAL, "gather cell_flux needs a mesh uploaded with MA_MESH_CELL_FLUX");
  ma_solver* s = new (std::nothrow) ma_solver;
  if (!s) return set_error(MA_ENOMEM, "ma_solver_create: out of host memory");
  s->mesh = mesh;
  s->topo = o->gather == MA_GATHER_CELL_FLUX ? mesh->topo_cf : mesh->topo;
  s->cfg.cell_flux = o->gather == MA_GATHER_CELL_FLUX;
  s->opts = *o;
  s->mixed = o->precision == MA_PREC_MIXED;
  s->fma = o->precision == MA_PREC_FP64_FMA;
  s->cfg.second_order = o->second_order_space != 0;
  s->cfg.viscous = o->viscous != 0;
  s->cfg.limiter = o->limiter;
  s->cfg.transport = dev::make_transport(o->viscosity_model, o->mu, o->prandtl);
  for (int k = 0; k < 5; ++k) s->cfg.inflow[k] = o->inflow_state[k];
  s->cfg.dt = o->dt;
  const size_t C = mesh->topo.C, F = mesh->topo.F;
  Arena a;
  auto layout = [&]() {
    s->st.Un = a.take<double>(5 * C);
    s->st.Unp1 = a.take<double>(5 * C);
    s->st.res = o->keep_residual ? a.take<double>(5 * C) : nullptr;
    s->dscratch = a.take<unsigned long long>(1);
    if (s->mixed) {
      s->b32.W = a.take<float>(5 * C);
      s->b32.grad = a.take<float>(15 * C);
      s->b32.phi = a.take<float>(5 * C);
      s->b32.fflux = a.take<float>(5 * F);
    } else {
      s->b64.W = a.take<double>(5 * C);
      s->b64.grad = a.take<double>(15 * C);
      s->b64.phi = a.take<double>(5 * C);
      s->b64.fflux = a.take<double>(5 * F);
    }
  };
  layout();
  const size_t bytes = a.used;
  a.used = 0;
  cudaError_t e = cudaSetDevice(mesh->device);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&a.base), bytes);
  if (e != cudaSuccess) {
    delete s;
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? MA_ENOMEM : MA_ECUDA,
                     std::string("ma_solver_create: ") + cudaGetErrorString(e));
  }
  layout();
  s->dmem = a.base;
  s->bytes = bytes;
  e = cudaMemset(s->dmem, 0, bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    const std::string msg = std::string("ma_solver_create: ") + cudaGetErrorString(e);
    ma_solver_free(s);
    return set_error(MA_ECUDA, msg);
  }
  *out = s;
  return MA_OK;
}

extern "C" void ma_solver_free(ma_solver* s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->join) cudaEventDestroy(s->join);
  if (s->fork) cudaEventDestroy(s->fork);
  if (s->side) cudaStreamDestroy(s->side);
  if (s->stream) cudaStreamDestroy(s->stream);
  cudaFree(s->dmem);
  delete s;
}

namespace {

// Copies U (AOS or SOA host layout) into the device SOA array.
ma_status upload_state(ma_solver* s, const double* U, int32_t layout) {
  const size_t C = s->topo.C;
  if (layout == MA_LAYOUT_SOA) {
    MA_CUDA_TRY(cudaMemcpyAsync(s->st.Un, U, sizeof(double) * 5 * C, cudaMemcpyHostToDevice, s->stream));
  } else if (layout == MA_LAYOUT_AOS) {
    std::vector<double> soa(5 * C);
    for (size_t c = 0; c < C; ++c)
      for (int k = 0; k < 5; ++k) soa[k * C + c] = U[5 * c + k];
    MA_CUDA_TRY(cudaMemcpyAsync(s->st.Un, soa.data(), sizeof(double) * 5 * C, cudaMemcpyHostToDevice, s->stream));
    MA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  } else {
    return set_error(MA_EINVAL, "unknown state layout");
  }
  return MA_OK;
}

ma_status download(ma_solver* s, const double* src, double* U, int32_t layout) {
  const size_t C = s->topo.C;
  if (layout == MA_LAYOUT_SOA) {
    MA_CUDA_TRY(cudaMemcpyAsync(U, src, sizeof(double) * 5 * C, cudaMemcpyDeviceToHost, s->stream));
    MA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  } else if (layout == MA_LAYOUT_AOS) {
    std::vector<double> soa(5 * C);
    MA_CUDA_TRY(cudaMemcpyAsync(soa.data(), src, sizeof(double) * 5 * C, cudaMemcpyDeviceToHost, s->stream));
    MA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (size_t c = 0; c < C; ++c)
      for (int k = 0; k < 5; ++k) U[5 * c + k] = soa[k * C + c];
  } else {
    return set_error(MA_EINVAL, "unknown state layout");
  }
  return MA_OK;
}

}  // namespace

extern "C" ma_status ma_solver_set_state(ma_solver* s, const double* U, int32_t layout) {
  if (!s || !U) return set_error(MA_EINVAL, "ma_solver_set_state: null argument");
  miniaero::TraceRange trace("ma_solver_set_state");
  MA_CUDA_TRY(cudaSetDevice(s->mesh->device));
  ma_status st = upload_state(s, U, layout);
  if (st != MA_OK) return st;
  const dev::TopoView& t = s->topo;
  if (s->opts.cfl > 0.0) {
    MA_CUDA_TRY(cudaMemsetAsync(s->dscratch, 0xff, sizeof(unsigned long long), s->stream));
    // The CFL sum runs over the mesh's default lists whatever the gather
    // order, so dt does not depend on it.
    MA_CUDA_TRY(dev::launch_cfl(s->mesh->topo, s->mesh->g64, s->st.Un, s->dscratch, s->stream));
    unsigned long long bits = 0;
    MA_CUDA_TRY(cudaMemcpyAsync(&bits, s->dscratch, sizeof(bits), cudaMemcpyDeviceToHost, s->stream));
    MA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    double r;
    std::memcpy(&r, &bits, sizeof(r));
    if (!(r > 0.0) || !std::isfinite(r)) return set_error(MA_ENUMERIC, "CFL time step is not finite");
    s->cfg.dt = s->opts.cfl * r;
    if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
  }
  if (s->mixed)
    MA_CUDA_TRY(dev::launch_init_primitives<float>(t, s->st, s->b32, s->stream));
  else if (s->fma)
    MA_CUDA_TRY(dev::launch_init_primitives_fma(t, s->st, s->b64, s->stream));
  else
    MA_CUDA_TRY(dev::launch_init_primitives<double>(t, s->st, s->b64, s->stream));
  if (s->st.res) MA_CUDA_TRY(cudaMemsetAsync(s->st.res, 0, sizeof(double) * 5 * t.C, s->stream));
  MA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->state_set = true;
  s->steps_done = 0;
  return MA_OK;
}

extern "C" ma_status ma_solver_init_state(ma_solver* s, const ma_host_mesh* hm) {
  if (!s || !hm) return set_error(MA_EINVAL, "ma_solver_init_state: null argument");
  std::vector<double> U(5 * static_cast<size_t>(s->topo.C));
  ma_status st = ma_host_initial_state(hm, &s->opts, U.data());
  if (st != MA_OK) return st;
  return ma_solver_set_state(s, U.data(), MA_LAYOUT_AOS);
}

extern "C" ma_status ma_solver_get_state(ma_solver* s, double* U, int32_t layout) {
  if (!s || !U) return set_error(MA_EINVAL, "ma_solver_get_state: null argument");
  if (!s->state_set) return set_error(MA_ESTATE, "solver state has not been set");
  miniaero::TraceRange trace("ma_solver_get_state");
  MA_CUDA_TRY(cudaSetDevice(s->mesh->device));
  return download(s, s->st.Un, U, layout);
}

extern "C" ma_status ma_solver_get_residual(ma_solver* s, double* res, int32_t layout) {
  if (!s || !res) return set_error(MA_EINVAL, "ma_solver_get_residual: null argument");
  if (!s->st.res) return set_error(MA_ESTATE, "solver was created without keep_residual");
  MA_CUDA_TRY(cudaSetDevice(s->mesh->device));
  return download(s, s->st.res, res, layout);
}

extern "C" ma_status ma_solver_step(ma_solver* s, int32_t nsteps) {
  if (!s) return set_error(MA_EINVAL, "ma_solver_step: null solver");
  if (nsteps < 0) return set_error(MA_EINVAL, "ma_solver_step: negative step count");
  if (!s->state_set) return set_error(MA_ESTATE, "solver state has not been set");
  if (nsteps == 0) return MA_OK;
  miniaero::TraceRange trace("ma_solver_step");
  MA_CUDA_TRY(cudaSetDevice(s->mesh->device));
  if (!s->graph) {
    ma_status st = capture_step_graph(s);
    if (st != MA_OK) return st;
  }
  for (int32_t i = 0; i < nsteps; ++i) MA_CUDA_TRY(cudaGraphLaunch(s->graph, s->stream));
  s->steps_done += nsteps;
  return MA_OK;
}

extern "C" ma_status ma_solver_profile_steps(ma_solver* s, int32_t nsteps, double* kernel_ms, int32_t* kernel_launches) {
  if (!s || nsteps < 0 || !kernel_ms || !kernel_launches) return set_error(MA_EINVAL, "ma_solver_profile_steps: bad arguments");
  if (!s->state_set) return set_error(MA_ESTATE, "solver state has not been set");
  miniaero::TraceRange trace("ma_solver_profile_steps");
  MA_CUDA_TRY(cudaSetDevice(s->mesh->device));
  for (int k = 0; k < MA_PROFILE_KINDS; ++k) { kernel_ms[k] = 0.0; kernel_launches[k] = 0; }
  const dev::TopoView& t = s->topo;
  const unsigned bits[MA_PROFILE_KINDS] = {dev::kSweep1, dev::kInternalFlux, dev::kBcFlux, dev::kResidual};
  bool present[MA_PROFILE_KINDS] = {s->cfg.second_order || s->cfg.viscous, t.Fi > 0, t.Fb > 0, true};
  std::vector<cudaEvent_t> ev;
  std::vector<int> kind;
  auto cleanup = [&]() { for (cudaEvent_t e : ev) cudaEventDestroy(e); };
  for (int32_t step = 0; step < nsteps; ++step)
    for (int stage = 0; stage < 4; ++stage)
      for (int k = 0; k < MA_PROFILE_KINDS; ++k) {
        if (!present[k]) continue;
        cudaEvent_t a, b;
        if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
          cleanup();
          return set_error(MA_ECUDA, "ma_solver_profile_steps: cudaEventCreate failed");
        }
        ev.push_back(a);
        ev.push_back(b);
        kind.push_back(k);
        cudaEventRecord(a, s->stream);
        cudaError_t e = solver_stage(s, stage, s->stream, bits[k]);
        cudaEventRecord(b, s->stream);
        if (e != cudaSuccess) {
          cleanup();
          return set_error(MA_ECUDA, std::string("ma_solver_profile_steps: ") + cudaGetErrorString(e));
        }
      }
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    cleanup();
    return set_error(MA_ECUDA, std::string("ma_solver_profile_steps: ") + cudaGetErrorString(e));
  }
  for (size_t i = 0; i < kind.size(); ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
    kernel_ms[kind[i]] += ms;
    kernel_launches[kind[i]] += 1;
  }
  cleanup();
  s->steps_done += nsteps;
  return MA_OK;
}

extern "C" ma_status ma_solver_synchronize(ma_solver* s) {
  if (!s) return set_error(MA_EINVAL, "ma_solver_synchronize: null solver");
  MA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return MA_OK;
}

extern "C" void* ma_solver_stream(ma_solver* s) { return s ? static_cast<void*>(s->stream) : nullptr; }
extern "C" double ma_solver_dt(const ma_solver* s) { return s ? s->cfg.dt : 0.0; }
extern "C" int64_t ma_solver_steps_done(const ma_solver* s) { return s ? s->steps_done : 0; }

extern "C" int32_t ma_solver_launches_per_step(const ma_solver* s) {
  return s ? 4 * dev::launches_per_stage(s->cfg, s->topo) : 0;
}

extern "C" ma_status ma_solver_set_dt(ma_solver* s, double dt) {
  if (!s || !(dt > 0.0)) return set_error(MA_EINVAL, "ma_solver_set_dt: dt must be > 0");
  s->cfg.dt = dt;
  if (s->graph) {
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  return MA_OK;
}

extern "C" ma_status ma_solver_check_state(ma_solver* s, int64_t* bad_cell) {
  if (!s) return set_error(MA_EINVAL, "ma_solver_check_state: null solver");
  if (bad_cell) *bad_cell = -1;
  MA_CUDA_TRY(cudaSetDevice(s->mesh->device));
  MA_CUDA_TRY(cudaMemsetAsync(s->dscratch, 0xff, sizeof(unsigned long long), s->stream));
  MA_CUDA_TRY(dev::launch_check_state(s->topo.C, s->st.Un, s->dscratch, s->stream));
  unsigned long long first = 0;
  MA_CUDA_TRY(cudaMemcpyAsync(&first, s->dscratch, sizeof(first), cudaMemcpyDeviceToHost, s->stream));
  MA_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (first != ~0ULL) {
    if (bad_cell) *bad_cell = static_cast<int64_t>(first);
    return set_error(MA_ENUMERIC, "non-finite or non-positive state at cell " + std::to_string(first));
  }
  return MA_OK;
}

extern "C" ma_status ma_solver_solve(ma_solver* s, const ma_host_mesh* hm) {
  ma_status st = ma_solver_init_state(s, hm);
  if (st != MA_OK) return st;
  st = ma_solver_step(s, s->opts.ntimesteps);
  if (st != MA_OK) return st;
  return ma_solver_synchronize(s);
}

// ---------------------------------------------------------------------------
// Operator-level entry points: host arrays in, host arrays out.
namespace {

struct DevBufs {
  std::vector<void*> ptrs;
  ~DevBufs() {
    for (void* p : ptrs) cudaFree(p);
  }
  cudaError_t in(const double* h, size_t n, double** d) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(d), sizeof(double) * (n ? n : 1));
    if (e != cudaSuccess) return e;
    ptrs.push_back(*d);
    return h ? cudaMemcpy(*d, h, sizeof(double) * n, cudaMemcpyHostToDevice) : cudaSuccess;
  }
  template <class T>
  cudaError_t in(std::nullptr_t, size_t n, T** d) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(d), sizeof(T) * (n ? n : 1));
    if (e == cudaSuccess) ptrs.push_back(*d);
    return e;
  }
};

}  // namespace

extern "C" ma_status ma_op_roe_flux(int32_t n, const double* pl, const double* pr, const double* normal,
                                    const double* tangent, const double* binormal, double* flux) {
  if (n < 0 || (n > 0 && (!pl || !pr || !normal || !tangent || !binormal || !flux)))
    return set_error(MA_EINVAL, "ma_op_roe_flux: bad arguments");
  if (n == 0) return MA_OK;
  DevBufs b;
  double *dpl, *dpr, *dn, *dt, *db, *df;
  MA_CUDA_TRY(b.in(pl, 5 * (size_t)n, &dpl));
  MA_CUDA_TRY(b.in(pr, 5 * (size_t)n, &dpr));
  MA_CUDA_TRY(b.in(normal, 3 * (size_t)n, &dn));
  MA_CUDA_TRY(b.in(tangent, 3 * (size_t)n, &dt));
  MA_CUDA_TRY(b.in(binormal, 3 * (size_t)n, &db));
  MA_CUDA_TRY(b.in(nullptr, 5 * (size_t)n, &df));
  MA_CUDA_TRY(dev::launch_op_roe(n, dpl, dpr, dn, dt, db, df, 0));
  MA_CUDA_TRY(cudaMemcpy(flux, df, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost));
  return MA_OK;
}

extern "C" ma_status ma_op_viscous_flux(int32_t n, const double* grad, const double* prim, const double* area,
                                        int32_t viscosity_model, double mu, double prandtl, double* vflux) {
  if (n < 0 || (n > 0 && (!grad || !prim || !area || !vflux))) return set_error(MA_EINVAL, "ma_op_viscous_flux: bad arguments");
  if (n == 0) return MA_OK;
  DevBufs b;
  double *dg, *dp, *da, *dv;
  MA_CUDA_TRY(b.in(grad, 15 * (size_t)n, &dg));
  MA_CUDA_TRY(b.in(prim, 5 * (size_t)n, &dp));
  MA_CUDA_TRY(b.in(area, 3 * (size_t)n, &da));
  MA_CUDA_TRY(b.in(nullptr, 5 * (size_t)n, &dv));
  MA_CUDA_TRY(dev::launch_op_viscous(n, dg, dp, da, dev::make_transport(viscosity_model, mu, prandtl), dv, 0));
  MA_CUDA_TRY(cudaMemcpy(vflux, dv, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost));
  return MA_OK;
}

extern "C" ma_status ma_op_limiter(int32_t n, int32_t kind, const double* dumax, const double* dumin,
                                   const double* du, const double* d2, double* phi) {
  if (n < 0 || (n > 0 && (!dumax || !dumin || !du || !phi || (kind == 0 && !d2))) || kind < 0 || kind > 1)
    return set_error(MA_EINVAL, "ma_op_limiter: bad arguments");
  if (n == 0) return MA_OK;
  DevBufs b;
  double *a, *bb, *c, *d, *p;
  MA_CUDA_TRY(b.in(dumax, n, &a));
  MA_CUDA_TRY(b.in(dumin, n, &bb));
  MA_CUDA_TRY(b.in(du, n, &c));
  MA_CUDA_TRY(b.in(d2, d2 ? n : 0, &d));
  MA_CUDA_TRY(b.in(nullptr, n, &p));
  MA_CUDA_TRY(dev::launch_op_limiter(n, kind, a, bb, c, d, p, 0));
  MA_CUDA_TRY(cudaMemcpy(phi, p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return MA_OK;
}

extern "C" ma_status ma_debug_check_division(int32_t mode, uint64_t n, uint64_t seed, uint64_t* mismatches,
                                             double* example) {
  if (!mismatches || !example || mode < 0 || mode > 6) return set_error(MA_EINVAL, "ma_debug_check_division: bad arguments");
  DevBufs b;
  double* dex;
  MA_CUDA_TRY(b.in(nullptr, 3, &dex));
  unsigned long long* dm = reinterpret_cast<unsigned long long*>(dex + 2);
  MA_CUDA_TRY(cudaMemset(dex, 0, 3 * sizeof(double)));
  MA_CUDA_TRY(dev::launch_check_division(mode, n, seed, dm, dex, 0));
  double host[3];
  MA_CUDA_TRY(cudaMemcpy(host, dex, sizeof(host), cudaMemcpyDeviceToHost));
  std::memcpy(mismatches, &host[2], sizeof(uint64_t));
  example[0] = host[0];
  example[1] = host[1];
  return MA_OK;
}

extern "C" ma_status ma_debug_fp64_rate(int32_t op, double* inst_per_s) {
  if (!inst_per_s || op < 0 || op > 2) return set_error(MA_EINVAL, "ma_debug_fp64_rate: bad arguments");
  int dev = 0, sms = 0;
  MA_CUDA_TRY(cudaGetDevice(&dev));
  MA_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = 8 * sms, iters = 2048;
  DevBufs b;
  double* out;
  MA_CUDA_TRY(b.in(nullptr, static_cast<size_t>(blocks) * 256, &out));
  cudaEvent_t e0, e1;
  MA_CUDA_TRY(cudaEventCreate(&e0));
  cudaError_t err = cudaEventCreate(&e1);
  float best = 0.f;
  for (int r = 0; r < 4 && err == cudaSuccess; ++r) {
    err = cudaEventRecord(e0, 0);
    if (err == cudaSuccess) err = dev::launch_fp64_rate(op, blocks, iters, out, 0);
    if (err == cudaSuccess) err = cudaEventRecord(e1, 0);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && (best == 0.f || ms < best)) best = ms;  // launch 0 warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  MA_CUDA_TRY(err);
  if (!(best > 0.f)) return set_error(MA_ENUMERIC, "ma_debug_fp64_rate: no elapsed time");
  *inst_per_s = static_cast<double>(blocks) * 256.0 * iters * 4.0 / (best * 1e-3);
  return MA_OK;
}

extern "C" ma_status ma_debug_barrier_timeout(double timeout_s, int32_t* passed, int32_t* error_word,
                                              double* waited_s) {
  if (!passed || !error_word || !waited_s || !(timeout_s > 0.0) || timeout_s > 10.0)
    return set_error(MA_EINVAL, "ma_debug_barrier_timeout: bad arguments (timeout in (0, 10] s)");
  DevBufs b;
  unsigned* words;
  int* err;
  int* out;
  MA_CUDA_TRY(b.in(nullptr, 2, &words));
  MA_CUDA_TRY(b.in(nullptr, 1, &err));
  MA_CUDA_TRY(b.in(nullptr, 2, &out));
  MA_CUDA_TRY(cudaMemset(words, 0, 2 * sizeof(unsigned)));
  MA_CUDA_TRY(cudaMemset(err, 0, sizeof(int)));
  MA_CUDA_TRY(cudaMemset(out, 0xFF, 2 * sizeof(int)));
  const auto t0 = std::chrono::steady_clock::now();
  MA_CUDA_TRY(dev::launch_debug_barrier_timeout(words, err, static_cast<unsigned long long>(timeout_s * 1e9), out, 0));
  MA_CUDA_TRY(cudaDeviceSynchronize());
  *waited_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  int host[2];
  MA_CUDA_TRY(cudaMemcpy(host, out, sizeof(host), cudaMemcpyDeviceToHost));
  *passed = host[0];
  *error_word = host[1];
  return MA_OK;
}

namespace {

// One RK stage's drivers taken one at a time on a state U (the operator
// entry points below): U to the device as [5][C], W = primitives(U), and
// the work arrays of one stage.
struct FieldRun {
  DevBufs b;
  dev::StateBuffers st;
  dev::StageBuffers<double> sb;
};

ma_status field_setup(ma_mesh* m, const double* U, int32_t layout, FieldRun& r) {
  if (layout != MA_LAYOUT_AOS && layout != MA_LAYOUT_SOA) return set_error(MA_EINVAL, "bad state layout");
  const size_t C = static_cast<size_t>(m->topo.C), F = static_cast<size_t>(m->topo.F);
  std::vector<double> soa(5 * C);
  for (size_t c = 0; c < C; ++c)
    for (size_t k = 0; k < 5; ++k) soa[k * C + c] = layout == MA_LAYOUT_AOS ? U[5 * c + k] : U[k * C + c];
  MA_CUDA_TRY(cudaSetDevice(m->device));
  MA_CUDA_TRY(r.b.in(soa.data(), 5 * C, &r.st.Un));
  r.st.Unp1 = r.st.Un;
  MA_CUDA_TRY(r.b.in(nullptr, 5 * C, &r.sb.W));
  MA_CUDA_TRY(r.b.in(nullptr, 15 * C, &r.sb.grad));
  MA_CUDA_TRY(r.b.in(nullptr, 5 * C, &r.sb.phi));
  MA_CUDA_TRY(r.b.in(nullptr, 5 * F, &r.sb.fflux));
  MA_CUDA_TRY(dev::launch_field_primitives(m->topo.C, r.st.Un, r.sb.W, 0));
  return MA_OK;
}

// [n][C] device array -> host [C][n] (the reference's LayoutRight views).
ma_status download_cell_major(const double* d, size_t C, size_t n, double* out) {
  std::vector<double> h(n * C);
  MA_CUDA_TRY(cudaMemcpy(h.data(), d, sizeof(double) * n * C, cudaMemcpyDeviceToHost));
  for (size_t c = 0; c < C; ++c)
    for (size_t j = 0; j < n; ++j) out[c * n + j] = h[j * C + c];
  return MA_OK;
}

}  // namespace

extern "C" ma_status ma_op_green_gauss(ma_mesh* mesh, const double* U, int32_t layout, double* grad) {
  if (!mesh || !U || !grad) return set_error(MA_EINVAL, "ma_op_green_gauss: null argument");
  FieldRun r;
  ma_status st = field_setup(mesh, U, layout, r);
  if (st != MA_OK) return st;
  dev::PathConfig cfg;
  cfg.viscous = true;  // the sweep's gradient-only form
  MA_CUDA_TRY(dev::launch_stage<double>(mesh->topo, mesh->g64, cfg, r.st, r.sb, 0, 0, dev::kSweep1));
  return download_cell_major(r.sb.grad, mesh->topo.C, 15, grad);
}

extern "C" ma_status ma_op_stencil_limiter(ma_mesh* mesh, int32_t limiter, const double* U, int32_t layout,
                                           double* phi) {
  if (!mesh || !U || !phi) return set_error(MA_EINVAL, "ma_op_stencil_limiter: null argument");
  if (limiter != MA_LIMITER_VENKAT && limiter != MA_LIMITER_VANALBADA) return set_error(MA_EINVAL, "bad limiter");
  FieldRun r;
  ma_status st = field_setup(mesh, U, layout, r);
  if (st != MA_OK) return st;
  dev::PathConfig cfg;
  cfg.second_order = true;
  cfg.viscous = true;
  cfg.limiter = limiter;
  MA_CUDA_TRY(dev::launch_stage<double>(mesh->topo, mesh->g64, cfg, r.st, r.sb, 0, 0, dev::kSweep1));
  return download_cell_major(r.sb.phi, mesh->topo.C, 5, phi);
}

extern "C" ma_status ma_op_bc_flux(ma_mesh* mesh, const ma_options* o, const double* U, int32_t layout,
                                   double* cell_flux) {
  if (!mesh || !o || !U || !cell_flux) return set_error(MA_EINVAL, "ma_op_bc_flux: null argument");
  if (o->viscosity_model != MA_VISC_SUTHERLAND && o->viscosity_model != MA_VISC_CONSTANT)
    return set_error(MA_EINVAL, "bad viscosity model");
  FieldRun r;
  ma_status st = field_setup(mesh, U, layout, r);
  if (st != MA_OK) return st;
  dev::PathConfig cfg;
  cfg.transport = dev::make_transport(o->viscosity_model, o->mu, o->prandtl);
  for (int k = 0; k < 5; ++k) cfg.inflow[k] = o->inflow_state[k];
  MA_CUDA_TRY(dev::launch_stage<double>(mesh->topo, mesh->g64, cfg, r.st, r.sb, 0, 0, dev::kBcFlux));
  double* out;
  MA_CUDA_TRY(r.b.in(nullptr, 5 * static_cast<size_t>(mesh->topo.C), &out));
  MA_CUDA_TRY(dev::launch_bc_gather(mesh->topo, r.sb.fflux, out, 0));
  return download_cell_major(out, mesh->topo.C, 5, cell_flux);
}

extern "C" ma_status ma_op_apply_cell_flux(int32_t ncells, double dt, const double* volumes, const double* cell_flux,
                                           double* res) {
  if (ncells < 0 || (ncells > 0 && (!volumes || !cell_flux || !res)))
    return set_error(MA_EINVAL, "ma_op_apply_cell_flux: bad arguments");
  if (ncells == 0) return MA_OK;
  DevBufs b;
  double *dv, *df, *dr;
  MA_CUDA_TRY(b.in(volumes, static_cast<size_t>(ncells), &dv));
  MA_CUDA_TRY(b.in(cell_flux, 5 * static_cast<size_t>(ncells), &df));
  MA_CUDA_TRY(b.in(nullptr, 5 * static_cast<size_t>(ncells), &dr));
  MA_CUDA_TRY(dev::launch_op_apply_cell_flux(ncells, dt, dv, df, dr, 0));
  MA_CUDA_TRY(cudaMemcpy(res, dr, sizeof(double) * 5 * static_cast<size_t>(ncells), cudaMemcpyDeviceToHost));
  return MA_OK;
}

extern "C" ma_status ma_op_rk_update(int64_t n, double alpha, const double* res, const double* src, double* dst) {
  if (n < 0 || (n > 0 && (!res || !src || !dst))) return set_error(MA_EINVAL, "ma_op_rk_update: bad arguments");
  if (n == 0) return MA_OK;
  DevBufs b;
  double *dr, *ds, *dd;
  MA_CUDA_TRY(b.in(res, static_cast<size_t>(n), &dr));
  MA_CUDA_TRY(b.in(src, static_cast<size_t>(n), &ds));
  MA_CUDA_TRY(b.in(nullptr, static_cast<size_t>(n), &dd));
  MA_CUDA_TRY(dev::launch_op_rk_update(n, alpha, dr, ds, dd, 0));
  MA_CUDA_TRY(cudaMemcpy(dst, dd, sizeof(double) * static_cast<size_t>(n), cudaMemcpyDeviceToHost));
  return MA_OK;
}

extern "C" ma_status ma_op_primitives(int32_t n, const double* U, double* V) {
  if (n < 0 || (n > 0 && (!U || !V))) return set_error(MA_EINVAL, "ma_op_primitives: bad arguments");
  if (n == 0) return MA_OK;
  DevBufs b;
  double *du, *dv;
  MA_CUDA_TRY(b.in(U, 5 * (size_t)n, &du));
  MA_CUDA_TRY(b.in(nullptr, 5 * (size_t)n, &dv));
  MA_CUDA_TRY(dev::launch_op_primitives(n, du, dv, 0));
  MA_CUDA_TRY(cudaMemcpy(V, dv, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost));
  return MA_OK;
}
