// Host-side structured-box Hexa8 mesh in unstructured form.
//
// Restates the single-rank path of the reference mesh setup:
//   Parallel3DMesh::fillMeshData          kokkos/Parallel3DMesh.h:173-449
//   Parallel3DMesh::getNodeCoordinate     kokkos/Parallel3DMesh.h:466-487
//   getElementNodeConnectivities          kokkos/Parallel3DMesh.C:80-96
//   create_faces / volumes / centroids    kokkos/MeshProcessor.C:39-171
//   extract_BC_faces / organize_BC_faces  kokkos/MeshProcessor.C:189-229
//   Face::Face (centroid, area, frame)    kokkos/Face.C:37-98
//   ElementTopoHexa8::ComputeVolume       kokkos/ElementTopoHexa8.C:62-148
//   copy_faces (BinSort permutation)      kokkos/Faces.h:88-145
//
// The face creation order, the internal-face shuffle and the per-set
// iteration permutation fix the serial summation order of every per-cell
// accumulator, so they are reproduced exactly; all floating-point work here
// must be compiled with -ffp-contract=off.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace miniaero {

enum BcType : int32_t { BC_EXTRAPOLATE = 0, BC_TANGENT = 1, BC_INFLOW = 2, BC_NOSLIP = 3 };

// One face list (the reference's Faces<Device>, kokkos/Faces.h:42-71), host copy.
struct HostFaceSet {
  std::string name;                 // "internal", or the BC functor name
  int32_t type = -1;                // BcType for boundary sets, -1 for internal
  int32_t nfaces = 0;
  std::vector<int32_t> conn;        // [nfaces*2] (elem1, elem2); elem2 = -1 on a boundary
  std::vector<int32_t> flux_index;  // [nfaces*2] per-cell slot of the face (CELL_FLUX layout)
  std::vector<double> coords;       // [nfaces*3] face centroid
  std::vector<double> normal;       // [nfaces*3] area vector, points out of elem1
  std::vector<double> tangent;      // [nfaces*3]
  std::vector<double> binormal;     // [nfaces*3]
  std::vector<int32_t> permutation; // [nfaces] iteration order (BinSort by elem1)
};

struct HostMesh {
  int32_t nx = 0, ny = 0, nz = 0;
  int32_t ncells = 0;
  std::vector<double> cell_coords;  // [ncells*3]
  std::vector<double> cell_volumes; // [ncells]
  HostFaceSet internal;
  // Boundary sets in the reference's boundary_faces order:
  // bottom, top, front, back, right, left (kokkos/Parallel3DMesh.h:382-396).
  std::vector<HostFaceSet> bc;
};

struct MeshSpec {
  int32_t nx = 1, ny = 1, nz = 1;
  double lx = 1.0, ly = 1.0, lz = 1.0;
  double angle = 0.0;        // ramp angle in degrees (problem_type 2)
  int32_t problem_type = 0;  // 0 Sod, 1 flat plate, 2 ramp
  // BC type override per side (bottom, top, front, back, right, left); -1 keeps
  // the reference map for problem_type.
  int32_t bc_override[6] = {-1, -1, -1, -1, -1, -1};
};

// Where the per-item geometry is computed: face centroids, area vectors and
// Roe frames (kokkos/Face.C:37-98) and cell volumes and centroids
// (kokkos/MeshProcessor.C:130-171, ElementTopoHexa8.C:62-148). The default is
// the host's threads; an engine may compute the same values elsewhere (the
// device, miniaero_gb300/csrc/device/geometry.cu) with the same operation
// order and rounding, so every result is bit-identical. Face and cell order,
// the shuffle and the BinSort stay on the host.
class GeometryEngine {
 public:
  virtual ~GeometryEngine() = default;
  // Node coordinates [nnodes*3] for the calls that follow.
  virtual std::string set_nodes(const double* xyz, size_t nnodes) = 0;
  // For n faces given by their 4 nodes in creation order ([n*4]): centroid,
  // area vector, tangent and binormal, each [n*3].
  virtual std::string faces(size_t n, const int32_t* nodes4, double* coords, double* normal, double* tangent,
                            double* binormal) = 0;
  // For ncells Hexa8 cells ([ncells*8] nodes): volume [ncells] and centroid
  // [ncells*3]; *negative += Gauss points whose Jacobian determinant is below
  // 1e-300.
  virtual std::string cells(size_t ncells, const int32_t* conn8, double* volume, double* centroid,
                            int* negative) = 0;
};

// Builds the mesh. Returns an empty string on success, else a message.
// engine: where the geometry is computed (nullptr: the host's threads).
std::string build_box_mesh(const MeshSpec& spec, HostMesh& out, GeometryEngine* engine = nullptr);

// glibc random()/rand() (TYPE_3 additive feedback generator, default seed 1).
class GlibcRand {
 public:
  explicit GlibcRand(uint32_t seed = 1);
  int32_t next();
 private:
  uint32_t buf_[34];  // r[i] for the last 34 indices i, at buf_[i % 34]
  uint64_t pos_;      // index i of the next value to generate
};

// libstdc++ std::random_shuffle(first, last) driven by GlibcRand.
template <class T>
void random_shuffle_glibc(std::vector<T>& v, GlibcRand& rng) {
  if (v.empty()) return;
  for (size_t i = 1; i < v.size(); ++i) {
    size_t j = static_cast<size_t>(rng.next()) % (i + 1);
    if (i != j) std::swap(v[i], v[j]);
  }
}

// Serial Kokkos::BinSort(keys, BinOp1D(n/2, min, max), sort_within_bins=true)
// permutation (kokkos/Faces.h:128-144).
std::vector<int32_t> binsort_permutation(const int32_t* keys, int32_t n, int32_t stride);

}  // namespace miniaero
