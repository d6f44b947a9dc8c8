// Accessors of ma_mesh (defined in solver.cu) for the batch and server code.
#pragma once
#include <cstddef>

#include "../../../include/miniaero_gpu.h"
#include "kernels.cuh"

namespace miniaero {
size_t mesh_cells(const ma_mesh* m);
size_t mesh_faces(const ma_mesh* m);
dev::TopoView mesh_topo(const ma_mesh* m);
// The mesh's lists in the given MA_GATHER_* order (the CELL_FLUX lists exist
// when the mesh was uploaded with MA_MESH_CELL_FLUX).
dev::TopoView mesh_topo(const ma_mesh* m, int gather);
bool mesh_has_cell_flux(const ma_mesh* m);
// CUDA device index the mesh was uploaded to.
int mesh_device(const ma_mesh* m);
template <class R>
dev::GeomView<R> mesh_geom(const ma_mesh* m);
template <>
dev::GeomView<double> mesh_geom<double>(const ma_mesh* m);
template <>
dev::GeomView<float> mesh_geom<float>(const ma_mesh* m);
}  // namespace miniaero
