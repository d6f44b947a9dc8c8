// Reference-build driver (test infrastructure only).
//
// Runs the reference miniAero solve from its own, unmodified sources compiled
// against the Kokkos stand-in in oracle/kokkos_shim, the way the reference's
// run() does (kokkos/Main.C:96-141): read miniaero.inp from the case
// directory (Options::read_options_file), build the mesh on the host
// (Parallel3DMesh::fillMeshData), construct TimeSolverExplicitRK4 and call
// Solve(). It then writes, bit for bit, the arrays the stand-in kept for the
// captured labels: the final conserved state ("solution_n"), the last stage's
// residual ("residual"), the cell centroids and volumes, and every face set's
// geometry, connectivity and iteration permutation, in allocation order.
//
// Usage: miniaero_ref <case dir holding miniaero.inp> <output file>
// Output: "MAREF1\n", then per array a text line
//   "<label> <i|d> <rank> <extent>..." followed by the raw little-endian
//   elements in LayoutRight order.
// The solver writes its own results.0 into the case directory when the input
// asks for output, as the reference executable does.
#include <unistd.h>

#include <cstdio>
#include <string>

#include <Kokkos_Core.hpp>

#include "MeshData.h"
#include "Options.h"
#include "Parallel3DMesh.h"
#include "TimeSolverExplicitRK4.h"

int main(int argc, char* argv[]) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <case dir> <output file>\n", argv[0]);
    return 2;
  }
  std::string out_path = argv[2];
  if (out_path[0] != '/') {
    char cwd[4096];
    if (!getcwd(cwd, sizeof(cwd))) {
      std::perror("getcwd");
      return 2;
    }
    out_path = std::string(cwd) + "/" + out_path;
  }
  if (chdir(argv[1]) != 0) {
    std::perror("chdir");
    return 2;
  }
  Options options;
  options.read_options_file();

  const char* labels[] = {"solution_n",     "residual",        "cell_coordinates",   "cell_volumes",
                          "coordinates",    "face_normal",     "face_tangent",       "face_binormal",
                          "face_cell_conn", "cell_flux_index", "cell_permute_vector"};
  for (const char* l : labels) Kokkos::shim::capture(l);

  Kokkos::initialize(argc, argv);
  {
    Parallel3DMesh mesh(options.nx, options.ny, options.nz, options.lx, options.ly, options.lz,
                        options.problem_type, options.angle);
    MeshData<Kokkos::DefaultExecutionSpace> mesh_data;
    mesh.fillMeshData<Kokkos::DefaultExecutionSpace>(mesh_data);
    TimeSolverExplicitRK4<Kokkos::DefaultExecutionSpace>* solver =
        new TimeSolverExplicitRK4<Kokkos::DefaultExecutionSpace>(mesh_data, options);
    solver->Solve();
    delete solver;
  }

  FILE* f = std::fopen(out_path.c_str(), "wb");
  if (!f) {
    std::perror("fopen");
    return 1;
  }
  std::fputs("MAREF1\n", f);
  for (const Kokkos::shim::Captured& c : Kokkos::shim::captured()) {
    size_t n = 1;
    std::fprintf(f, "%s %c %zu", c.label.c_str(), c.is_int ? 'i' : 'd', c.extents.size());
    for (size_t e : c.extents) {
      std::fprintf(f, " %zu", e);
      n *= e;
    }
    std::fputc('\n', f);
    if (n > 0 && std::fwrite(c.data, c.elem_size, n, f) != n) {
      std::perror("fwrite");
      std::fclose(f);
      return 1;
    }
  }
  std::fclose(f);
  Kokkos::finalize();
  return 0;
}
