// miniaero: drop-in command-line driver (replaces kokkos/Main.C:53-151).
//
// Reads miniaero.inp from the working directory (or the path given as the
// first argument), builds the mesh on the host, runs the RK4 solve on the GPU
// through the C ABI and, when output_results is set, writes results.0 in the
// reference's format (TimeSolverExplicitRK4.h:514-538).
#include <chrono>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "../../../include/miniaero_gpu.h"

namespace {
int fail(const char* what, ma_status s) {
  std::fprintf(stderr, "miniaero: %s failed: %s (%s)\n", what, ma_status_string(s), ma_last_error());
  return 1;
}
double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
}  // namespace

int main(int argc, char** argv) {
  const auto t_total = std::chrono::steady_clock::now();
  const char* input = argc > 1 ? argv[1] : "miniaero.inp";
  ma_options o;
  ma_status st = ma_options_read(input, &o);
  if (st != MA_OK) return fail("reading options", st);

  const auto t_setup = std::chrono::steady_clock::now();
  ma_host_mesh* hm = nullptr;
  if ((st = ma_host_mesh_build(&o, &hm)) != MA_OK) return fail("mesh setup", st);
  ma_mesh_view view;
  ma_host_mesh_view(hm, &view);
  ma_mesh* dm = nullptr;
  if ((st = ma_mesh_upload(&view, &dm)) != MA_OK) return fail("mesh upload", st);
  std::fprintf(stdout, "\n ... Setup time: %8.2f seconds ...\n", seconds_since(t_setup));

  ma_solver* s = nullptr;
  if ((st = ma_solver_create(dm, &o, &s)) != MA_OK) return fail("solver create", st);
  if ((st = ma_solver_init_state(s, hm)) != MA_OK) return fail("initial state", st);
  const double dt = ma_solver_dt(s);
  const auto t_run = std::chrono::steady_clock::now();
  // Solve loop (TimeSolverExplicitRK4.h:340-491), printing every
  // output_frequency steps as the reference does.
  int done = 0;
  const int freq = o.output_frequency > 0 ? o.output_frequency : o.ntimesteps + 1;
  while (done < o.ntimesteps) {
    int next = ((done / freq) + 1) * freq;  // next step number that prints
    if (next > o.ntimesteps) next = o.ntimesteps + 1;
    const int chunk = next - 1 - done;
    if (chunk > 0 && (st = ma_solver_step(s, chunk)) != MA_OK) return fail("step", st);
    done += chunk;
    if (done < o.ntimesteps) {
      std::fprintf(stdout, "\nTime Step #%i:  Time = %16.9e; dt = %16.9e\n", done + 1, (done + 1) * dt, dt);
      if ((st = ma_solver_step(s, 1)) != MA_OK) return fail("step", st);
      done += 1;
    }
  }
  if ((st = ma_solver_synchronize(s)) != MA_OK) return fail("solve", st);
  std::fprintf(stdout, "\n ... Device Run time: %8.2f seconds ...\n", seconds_since(t_run));
  int64_t bad = -1;
  if (ma_solver_check_state(s, &bad) != MA_OK)
    std::fprintf(stderr, "miniaero: warning: %s\n", ma_last_error());

  if (o.output_results) {
    std::vector<double> U(5 * static_cast<size_t>(view.ncells));
    if ((st = ma_solver_get_state(s, U.data(), MA_LAYOUT_AOS)) != MA_OK) return fail("state download", st);
    std::ofstream out("results.0");
    if (!out) {
      std::fprintf(stderr, "miniaero: cannot write results.0\n");
      return 1;
    }
    for (int32_t i = 0; i < view.ncells; ++i) {
      out << view.cell_coords[3 * i] << "\t";
      out << view.cell_coords[3 * i + 1] << "\t";
      out << view.cell_coords[3 * i + 2] << "\t";
      for (int k = 0; k < 5; ++k) out << U[5 * static_cast<size_t>(i) + k] << "\t";
      out << std::endl;
    }
  }
  ma_solver_free(s);
  ma_mesh_free(dm);
  ma_host_mesh_free(hm);
  std::fprintf(stdout, "\n ... Total elapsed time: %8.2f seconds ...\n", seconds_since(t_total));
  return 0;
}
