// Host mesh generation for a single-rank box (or ramp) domain.
// Every floating-point expression below keeps the operand order of the
// reference so that geometry is bit-identical; build with -ffp-contract=off.
#include "mesh.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <vector>

#include "parallel.hpp"

namespace miniaero {

// ---------------------------------------------------------------------------
// glibc random(): r[0]=seed; r[i]=16807*r[i-1] mod (2^31-1) for i<31 (Schrage
// form); r[i]=r[i-31] for 31<=i<34; r[i]=r[i-31]+r[i-3] (mod 2^32) after that;
// the k-th output is r[k+344]>>1.
GlibcRand::GlibcRand(uint32_t seed) {
  int32_t r[34];
  r[0] = static_cast<int32_t>(seed == 0 ? 1 : seed);
  for (int i = 1; i < 31; ++i) {
    const int32_t hi = r[i - 1] / 127773;
    const int32_t lo = r[i - 1] % 127773;
    int32_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = word;
  }
  for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
  for (int i = 0; i < 34; ++i) buf_[i] = static_cast<uint32_t>(r[i]);
  pos_ = 34;
  for (int i = 34; i < 344; ++i) next();
}

int32_t GlibcRand::next() {
  const uint64_t i = pos_++;
  const uint32_t v = buf_[(i - 31) % 34] + buf_[(i - 3) % 34];
  buf_[i % 34] = v;
  return static_cast<int32_t>(v >> 1);
}

// ---------------------------------------------------------------------------
// Serial Kokkos BinSort with BinOp1D(n/2, min, max) and sort_within_bins:
// count per bin, exclusive scan, stable binning in index order, then a bubble
// pass per bin that swaps whenever !(key[prev] < key[next]).
std::vector<int32_t> binsort_permutation(const int32_t* keys, int32_t n, int32_t stride) {
  std::vector<int32_t> order(static_cast<size_t>(n));
  if (n <= 0) return order;
  int32_t kmin = keys[0], kmax = keys[0];
  for (int32_t i = 1; i < n; ++i) {
    const int32_t k = keys[static_cast<size_t>(i) * stride];
    if (k < kmin) kmin = k;
    if (k > kmax) kmax = k;
  }
  const int32_t max_bins_arg = n / 2;
  const int32_t nbins = max_bins_arg + 1;
  // With a single distinct key the reference divides by zero; every key then
  // lands in bin 0 here.
  const double mul = (kmax == kmin) ? 0.0 : 1.0 * max_bins_arg / (kmax - kmin);
  auto bin_of = [&](int32_t i) -> int32_t {
    return static_cast<int32_t>(mul * (keys[static_cast<size_t>(i) * stride] - kmin));
  };
  // Stable binning in index order = a stable sort of (bin, index) pairs by
  // bin, done as an LSD radix sort (11-bit digits): sequential passes instead
  // of per-bin counters hit in shuffled order.
  std::vector<uint64_t> pairs(static_cast<size_t>(n)), tmp(static_cast<size_t>(n));
  for (int32_t i = 0; i < n; ++i)
    pairs[i] = (static_cast<uint64_t>(bin_of(i)) << 32) | static_cast<uint32_t>(i);
  for (int shift = 32; (static_cast<uint64_t>(nbins - 1) >> (shift - 32)) > 0; shift += 11) {
    size_t count[2048] = {0};
    for (const uint64_t p : pairs) count[(p >> shift) & 2047]++;
    size_t acc = 0;
    for (size_t& c : count) { const size_t v = c; c = acc; acc += v; }
    for (const uint64_t p : pairs) tmp[count[(p >> shift) & 2047]++] = p;
    pairs.swap(tmp);
  }
  for (int32_t k = 0; k < n; ++k) order[k] = static_cast<int32_t>(pairs[k] & 0xFFFFFFFFu);
  auto key = [&](int32_t i) { return keys[static_cast<size_t>(i) * stride]; };
  // Bubble pass within each bin (each run of equal bins).
  for (int32_t first = 0; first < n;) {
    int32_t last = first + 1;
    while (last < n && (pairs[last] >> 32) == (pairs[first] >> 32)) ++last;
    const int32_t begin = first, count_b = last - first;
    first = last;
    if (count_b <= 1) continue;
    bool sorted = false;
    int32_t upper = begin + count_b;
    while (!sorted) {
      sorted = true;
      int32_t old_idx = order[begin];
      for (int32_t k = begin + 1; k < upper; ++k) {
        const int32_t new_idx = order[k];
        if (!(key(old_idx) < key(new_idx))) {
          order[k - 1] = new_idx;
          order[k] = old_idx;
          sorted = false;
        } else {
          old_idx = new_idx;
        }
      }
      --upper;
    }
  }
  return order;
}

// ---------------------------------------------------------------------------
namespace {

struct Box {
  int32_t nx, ny, nz;
  double lx, ly, lz, angle;
  int64_t node(int32_t i, int32_t j, int32_t k) const {
    return static_cast<int64_t>(i) * ((ny + 1) * static_cast<int64_t>(nz + 1)) +
           static_cast<int64_t>(j) * (nz + 1) + k;
  }
  // kokkos/Parallel3DMesh.h:466-487
  void coordinate(int32_t i, int32_t j, int32_t k, double* c) const {
    const double PI = 3.14159265;
    c[0] = (double)i / (nx)*lx;
    c[2] = (double)k / (nz)*lz;
    if (c[0] < lx / 2.0) {
      c[1] = (double)j / (ny)*ly;
    } else {
      const double y_ramp = (c[0] - (lx / 2.0)) * std::tan(angle * PI / 180.0);
      const double ly_scaled = ly - y_ramp;
      c[1] = y_ramp + (double)j * ly_scaled / (ny);
    }
  }
};

inline void cross3(const double a[], const double b[], double c[]) {
  c[0] = a[1] * b[2] - b[1] * a[2];
  c[1] = -a[0] * b[2] + b[0] * a[2];
  c[2] = a[0] * b[1] - b[0] * a[1];
}

// kokkos/Face.C:37-98
void face_geometry(const int32_t nodes[4], const std::vector<double>& xyz, double coords[3],
                   double a[3], double t[3], double b[3]) {
  double n[4][3];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j) n[i][j] = xyz[static_cast<size_t>(nodes[i]) * 3 + j];
  coords[0] = coords[1] = coords[2] = 0.0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j) coords[j] += n[i][j];
  const double scale = 1.0 / 4;
  for (int j = 0; j < 3; ++j) coords[j] *= scale;
  const double v1[] = {n[1][0] - n[0][0], n[1][1] - n[0][1], n[1][2] - n[0][2]};
  const double v2[] = {n[2][0] - n[0][0], n[2][1] - n[0][1], n[2][2] - n[0][2]};
  const double v3[] = {n[3][0] - n[0][0], n[3][1] - n[0][1], n[3][2] - n[0][2]};
  double c1[3], c2[3];
  cross3(v1, v2, c1);
  cross3(v2, v3, c2);
  for (int j = 0; j < 3; ++j) a[j] = 0.5 * (c1[j] + c2[j]);
  const double aa[] = {std::fabs(a[0]), std::fabs(a[1]), std::fabs(a[2])};
  int i1 = 0;
  if (aa[0] < aa[1]) i1 = 1;
  if (aa[i1] < aa[2]) i1 = 2;
  int i2 = i1 + 1, i3 = i1 + 2;
  i2 = (i2 > 2) ? i2 - 3 : i2;
  i3 = (i3 > 2) ? i3 - 3 : i3;
  const double denom = std::sqrt(a[i1] * a[i1] + a[i3] * a[i3]);
  t[i2] = 0.0;
  t[i1] = a[i3] / denom;
  t[i3] = -a[i1] / denom;
  cross3(a, t, b);
}

// kokkos/ElementTopoHexa8.C:62-148 (2x2x2 Gauss points, unit weights).
double hexa8_volume(const double ex[8], const double ey[8], const double ez[8], int* negative) {
  static const double g = 0.577350269189626;
  static const double xi_[] = {-g, g, g, -g, -g, g, g, -g};
  static const double eta_[] = {-g, -g, g, g, -g, -g, g, g};
  static const double zeta_[] = {-g, -g, -g, -g, g, g, g, g};
  double volume = 0.0;
  for (int ig = 0; ig < 8; ++ig) {
    const double xi = xi_[ig], eta = eta_[ig], zeta = zeta_[ig];
    double dx[8], de[8], dz[8];
    dx[0] = -0.125 * (1.0 - eta) * (1.0 - zeta);
    dx[1] = 0.125 * (1.0 - eta) * (1.0 - zeta);
    dx[2] = 0.125 * (1.0 + eta) * (1.0 - zeta);
    dx[3] = -0.125 * (1.0 + eta) * (1.0 - zeta);
    dx[4] = -0.125 * (1.0 - eta) * (1.0 + zeta);
    dx[5] = 0.125 * (1.0 - eta) * (1.0 + zeta);
    dx[6] = 0.125 * (1.0 + eta) * (1.0 + zeta);
    dx[7] = -0.125 * (1.0 + eta) * (1.0 + zeta);
    de[0] = -0.125 * (1.0 - xi) * (1.0 - zeta);
    de[1] = -0.125 * (1.0 + xi) * (1.0 - zeta);
    de[2] = 0.125 * (1.0 + xi) * (1.0 - zeta);
    de[3] = 0.125 * (1.0 - xi) * (1.0 - zeta);
    de[4] = -0.125 * (1.0 - xi) * (1.0 + zeta);
    de[5] = -0.125 * (1.0 + xi) * (1.0 + zeta);
    de[6] = 0.125 * (1.0 + xi) * (1.0 + zeta);
    de[7] = 0.125 * (1.0 - xi) * (1.0 + zeta);
    dz[0] = -0.125 * (1.0 - xi) * (1.0 - eta);
    dz[1] = -0.125 * (1.0 + xi) * (1.0 - eta);
    dz[2] = -0.125 * (1.0 + xi) * (1.0 + eta);
    dz[3] = -0.125 * (1.0 - xi) * (1.0 + eta);
    dz[4] = 0.125 * (1.0 - xi) * (1.0 - eta);
    dz[5] = 0.125 * (1.0 + xi) * (1.0 - eta);
    dz[6] = 0.125 * (1.0 + xi) * (1.0 + eta);
    dz[7] = 0.125 * (1.0 - xi) * (1.0 + eta);
    auto dot8 = [](const double* a, const double* b) {
      double r = 0;
      for (int i = 0; i < 8; ++i) r += a[i] * b[i];
      return r;
    };
    double J[9];
    J[0] = dot8(dx, ex); J[1] = dot8(dx, ey); J[2] = dot8(dx, ez);
    J[3] = dot8(de, ex); J[4] = dot8(de, ey); J[5] = dot8(de, ez);
    J[6] = dot8(dz, ex); J[7] = dot8(dz, ey); J[8] = dot8(dz, ez);
    const double detJ = J[0] * (J[4] * J[8] - J[5] * J[7]) +
                        J[1] * (J[5] * J[6] - J[3] * J[8]) +
                        J[2] * (J[3] * J[7] - J[4] * J[6]);
    if (detJ < 1.0e-300) ++*negative;
    volume += detJ;
  }
  return volume;
}

struct RawFace {
  int32_t cv_minus, cv_plus, flux_minus, flux_plus;
  int32_t nodes[4];  // in the creating element's face order
};

std::string fill_face_set(HostFaceSet& fs, const std::vector<RawFace>& raw, const std::vector<int64_t>& ids,
                          const std::vector<double>& xyz, GeometryEngine* engine) {
  const size_t n = ids.size();
  fs.nfaces = static_cast<int32_t>(n);
  fs.conn.resize(n * 2);
  fs.flux_index.resize(n * 2);
  fs.coords.resize(n * 3);
  fs.normal.resize(n * 3);
  fs.tangent.resize(n * 3);
  fs.binormal.resize(n * 3);
  std::vector<int32_t> nodes4(engine ? n * 4 : 0);
  // Faces come in shuffled order, so the node lookups are random: spread
  // them over the host's threads.
  parallel_for(n, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      const RawFace& f = raw[static_cast<size_t>(ids[i])];
      fs.conn[2 * i] = f.cv_minus;
      fs.conn[2 * i + 1] = f.cv_plus;
      fs.flux_index[2 * i] = f.flux_minus;
      fs.flux_index[2 * i + 1] = f.flux_plus;
      if (engine) {
        for (int q = 0; q < 4; ++q) nodes4[4 * i + q] = f.nodes[q];
      } else {
        face_geometry(f.nodes, xyz, &fs.coords[3 * i], &fs.normal[3 * i], &fs.tangent[3 * i],
                      &fs.binormal[3 * i]);
      }
    }
  });
  if (engine && n > 0) {
    const std::string err = engine->faces(n, nodes4.data(), fs.coords.data(), fs.normal.data(), fs.tangent.data(),
                                          fs.binormal.data());
    if (!err.empty()) return err;
  }
  fs.permutation = binsort_permutation(fs.conn.data(), fs.nfaces, 2);
  return std::string();
}

}  // namespace

std::string build_box_mesh(const MeshSpec& spec, HostMesh& out, GeometryEngine* engine) {
  if (spec.nx < 1 || spec.ny < 1 || spec.nz < 1) return "mesh dimensions must be >= 1";
  const int64_t ncells64 = static_cast<int64_t>(spec.nx) * spec.ny * spec.nz;
  if (ncells64 > (1LL << 30)) return "mesh too large for 32-bit cell indices";
  if (!(spec.lx > 0.0 && spec.ly > 0.0 && spec.lz > 0.0)) return "domain lengths must be > 0";
  const Box box{spec.nx, spec.ny, spec.nz, spec.lx, spec.ly, spec.lz, spec.angle};
  const int32_t nx = spec.nx, ny = spec.ny, nz = spec.nz;
  const int64_t nnodes = static_cast<int64_t>(nx + 1) * (ny + 1) * (nz + 1);
  const int32_t ncells = static_cast<int32_t>(ncells64);

  std::vector<double> xyz(static_cast<size_t>(nnodes) * 3);
  for (int32_t i = 0; i <= nx; ++i)
    for (int32_t j = 0; j <= ny; ++j)
      for (int32_t k = 0; k <= nz; ++k) box.coordinate(i, j, k, &xyz[static_cast<size_t>(box.node(i, j, k)) * 3]);

  // Element connectivity, i-major then j, k fastest (Parallel3DMesh.C:80-96).
  std::vector<int32_t> conn(static_cast<size_t>(ncells) * 8);
  {
    size_t e = 0;
    for (int32_t i = 0; i < nx; ++i)
      for (int32_t j = 0; j < ny; ++j)
        for (int32_t k = 0; k < nz; ++k) {
          int32_t* c = &conn[8 * e++];
          c[0] = (int32_t)box.node(i, j, k);         c[1] = (int32_t)box.node(i + 1, j, k);
          c[2] = (int32_t)box.node(i + 1, j + 1, k); c[3] = (int32_t)box.node(i, j + 1, k);
          c[4] = (int32_t)box.node(i, j, k + 1);     c[5] = (int32_t)box.node(i + 1, j, k + 1);
          c[6] = (int32_t)box.node(i + 1, j + 1, k + 1); c[7] = (int32_t)box.node(i, j + 1, k + 1);
        }
  }

  // Face extraction in first-visit order (MeshProcessor.C:39-128). Faces are
  // matched through a per-minimum-node list, searched in insertion order.
  static const int order[24] = {0, 1, 5, 4, 1, 2, 6, 5, 2, 3, 7, 6, 3, 0, 4, 7, 0, 3, 2, 1, 4, 5, 6, 7};
  std::vector<RawFace> raw;
  raw.reserve(static_cast<size_t>(ncells) * 3 + static_cast<size_t>(nx * ny + ny * nz + nx * nz) * 2);
  std::vector<int32_t> sorted_nodes;  // 4 per face
  sorted_nodes.reserve(raw.capacity() * 4);
  std::vector<int32_t> head(static_cast<size_t>(nnodes), -1), tail(static_cast<size_t>(nnodes), -1), next;
  next.reserve(raw.capacity());
  for (int32_t ie = 0; ie < ncells; ++ie) {
    const int32_t* en = &conn[static_cast<size_t>(ie) * 8];
    int32_t elem_face_num = 0;
    for (int ifa = 0; ifa < 6; ++ifa) {
      int32_t fn[4], sn[4];
      for (int q = 0; q < 4; ++q) fn[q] = sn[q] = en[order[4 * ifa + q]];
      std::sort(sn, sn + 4);
      const int32_t mn = sn[0];
      bool assigned = false;
      for (int32_t f = head[mn]; f >= 0; f = next[f]) {
        const int32_t* s = &sorted_nodes[static_cast<size_t>(f) * 4];
        if (s[0] == sn[0] && s[1] == sn[1] && s[2] == sn[2] && s[3] == sn[3]) {
          raw[f].cv_plus = ie;
          raw[f].flux_plus = elem_face_num++;
          assigned = true;
          break;
        }
      }
      if (assigned) continue;
      const int32_t f = static_cast<int32_t>(raw.size());
      RawFace rf;
      rf.cv_minus = ie;
      rf.cv_plus = -1;
      rf.flux_minus = elem_face_num++;
      rf.flux_plus = -1;
      for (int q = 0; q < 4; ++q) rf.nodes[q] = fn[q];
      raw.push_back(rf);
      for (int q = 0; q < 4; ++q) sorted_nodes.push_back(sn[q]);
      next.push_back(-1);
      if (head[mn] < 0) head[mn] = f; else next[tail[mn]] = f;
      tail[mn] = f;
    }
  }
  std::vector<int32_t>().swap(head);
  std::vector<int32_t>().swap(tail);
  std::vector<int32_t>().swap(next);
  std::vector<int32_t>().swap(sorted_nodes);

  // Cell volumes and centroids (MeshProcessor.C:130-171).
  out = HostMesh();
  out.nx = nx; out.ny = ny; out.nz = nz;
  out.ncells = ncells;
  out.cell_coords.resize(static_cast<size_t>(ncells) * 3);
  out.cell_volumes.resize(static_cast<size_t>(ncells));
  if (engine) {
    std::string err = engine->set_nodes(xyz.data(), static_cast<size_t>(nnodes));
    int negative = 0;
    if (err.empty())
      err = engine->cells(static_cast<size_t>(ncells), conn.data(), out.cell_volumes.data(), out.cell_coords.data(),
                          &negative);
    if (!err.empty()) return "device geometry: " + err;
    if (negative)
      std::fprintf(stderr, "miniaero: warning: %d Gauss points with Jacobian determinant < 1e-300\n", negative);
  }
  std::atomic<int> negative_total{0};
  if (!engine) parallel_for(static_cast<size_t>(ncells), [&](size_t b, size_t e) {
    int negative = 0;
    for (size_t ie = b; ie < e; ++ie) {
      const int32_t* en = &conn[ie * 8];
      double ex[8], ey[8], ez[8];
      double sx = 0, sy = 0, sz = 0;
      for (int j = 0; j < 8; ++j) {
        ex[j] = xyz[static_cast<size_t>(en[j]) * 3];
        ey[j] = xyz[static_cast<size_t>(en[j]) * 3 + 1];
        ez[j] = xyz[static_cast<size_t>(en[j]) * 3 + 2];
      }
      out.cell_volumes[ie] = hexa8_volume(ex, ey, ez, &negative);
      for (int j = 0; j < 8; ++j) { sx += ex[j]; sy += ey[j]; sz += ez[j]; }
      out.cell_coords[3 * ie] = sx / 8;
      out.cell_coords[3 * ie + 1] = sy / 8;
      out.cell_coords[3 * ie + 2] = sz / 8;
    }
    negative_total += negative;
  });
  const int negative = negative_total.load();
  if (negative) {
    std::fprintf(stderr, "miniaero: warning: %d Gauss points with Jacobian determinant < 1e-300\n", negative);
  }

  // Split internal and boundary faces, keeping order (MeshProcessor.C:189-203).
  std::vector<int64_t> internal_ids, bc_ids;
  internal_ids.reserve(raw.size());
  for (size_t f = 0; f < raw.size(); ++f) (raw[f].cv_plus == -1 ? bc_ids : internal_ids).push_back((int64_t)f);

  // Sort boundary faces onto the six sides (MeshProcessor.C:205-229).
  // A face belongs to a side when all four of its nodes lie on that side.
  auto on_side = [&](int side, int32_t node) -> bool {
    const int32_t k = node % (nz + 1);
    const int32_t j = (node / (nz + 1)) % (ny + 1);
    const int32_t i = node / ((nz + 1) * (ny + 1));
    switch (side) {
      case 0: return j == 0;   // bottom
      case 1: return j == ny;  // top
      case 2: return k == 0;   // front
      case 3: return k == nz;  // back
      case 4: return i == nx;  // right
      default: return i == 0;  // left
    }
  };
  std::vector<int64_t> side_ids[6];
  for (int side = 0; side < 6; ++side)
    for (int64_t f : bc_ids) {
      bool in = true;
      for (int q = 0; q < 4; ++q)
        if (!on_side(side, raw[static_cast<size_t>(f)].nodes[q])) { in = false; break; }
      if (in) side_ids[side].push_back(f);
    }

  // Shuffle internal faces (Parallel3DMesh.h:362): unseeded rand().
  GlibcRand rng(1);
  random_shuffle_glibc(internal_ids, rng);

  {
    const std::string err = fill_face_set(out.internal, raw, internal_ids, xyz, engine);
    if (!err.empty()) return "device geometry: " + err;
  }
  out.internal.name = "internal";
  out.internal.type = -1;

  // boundary_faces order and BC map (Parallel3DMesh.h:382-396).
  const int pt = spec.problem_type;
  const int32_t default_types[6] = {
      pt == 1 ? BC_NOSLIP : BC_TANGENT,       // bottom
      pt == 1 ? BC_EXTRAPOLATE : BC_TANGENT,  // top
      BC_TANGENT,                             // front
      BC_TANGENT,                             // back
      BC_EXTRAPOLATE,                         // right
      pt == 0 ? BC_EXTRAPOLATE : BC_INFLOW,   // left
  };
  static const char* names[4] = {"Extrapolate", "Tangent", "Inflow", "NoSlip"};
  out.bc.resize(6);
  for (int side = 0; side < 6; ++side) {
    int32_t t = spec.bc_override[side] >= 0 ? spec.bc_override[side] : default_types[side];
    if (t < 0 || t > 3) return "invalid boundary condition type";
    const std::string err = fill_face_set(out.bc[side], raw, side_ids[side], xyz, engine);
    if (!err.empty()) return "device geometry: " + err;
    out.bc[side].type = t;
    out.bc[side].name = names[t];
  }
  return std::string();
}

}  // namespace miniaero
