// miniaero: drop-in command-line driver (replaces kokkos/Main.C:53-151).
//
// Reads miniaero.inp from the working directory (or the path given as the
// first argument), builds the mesh on the host, runs the RK4 solve on the GPU
// through the C ABI and, when output_results is set, writes results.0 in the
// reference's format (TimeSolverExplicitRK4.h:514-538). Beyond the reference:
// "restart <file>" continues a run from a checkpoint (same mesh, same dt, up
// to ntimesteps steps in total); "checkpoint <file>" writes one at the end
// and, with "checkpoint_frequency <n>", every n steps.
#include <algorithm>
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
  ma_run_options run;
  if ((st = ma_run_options_read(input, &run)) != MA_OK) return fail("reading run controls", st);

  const auto t_setup = std::chrono::steady_clock::now();
  ma_host_mesh* hm = nullptr;
  if ((st = ma_host_mesh_build(&o, &hm)) != MA_OK) return fail("mesh setup", st);
  ma_mesh_view view;
  ma_host_mesh_view(hm, &view);
  ma_mesh* dm = nullptr;
  const int32_t upload_flags = o.gather == MA_GATHER_CELL_FLUX ? MA_MESH_CELL_FLUX : 0;
  if ((st = ma_mesh_upload_ex(&view, upload_flags, &dm)) != MA_OK) return fail("mesh upload", st);
  std::fprintf(stdout, "\n ... Setup time: %8.2f seconds ...\n", seconds_since(t_setup));

  ma_solver* s = nullptr;
  if ((st = ma_solver_create(dm, &o, &s)) != MA_OK) return fail("solver create", st);
  const uint64_t mesh_hash = ma_mesh_hash(&view);
  const size_t C = static_cast<size_t>(view.ncells);
  std::vector<double> U;
  int done = 0;
  if (run.restart_path[0]) {
    ma_checkpoint_info info;
    U.resize(5 * C);
    if ((st = ma_checkpoint_read(run.restart_path, &info, U.data(), view.ncells, MA_LAYOUT_AOS)) != MA_OK)
      return fail("reading the restart checkpoint", st);
    if (info.ncells != view.ncells || info.mesh_hash != mesh_hash) {
      std::fprintf(stderr, "miniaero: %s was written for a different mesh\n", run.restart_path);
      return 1;
    }
    if ((st = ma_solver_set_state(s, U.data(), MA_LAYOUT_AOS)) != MA_OK) return fail("restart state", st);
    if ((st = ma_solver_set_dt(s, info.dt)) != MA_OK) return fail("restart dt", st);
    done = static_cast<int>(info.steps_done);
    std::fprintf(stdout, "\n ... Restarted from %s at step %i ...\n", run.restart_path, done);
  } else if ((st = ma_solver_init_state(s, hm)) != MA_OK) {
    return fail("initial state", st);
  }
  const double dt = ma_solver_dt(s);
  auto write_checkpoint = [&](int steps) -> ma_status {
    U.resize(5 * C);
    ma_status e = ma_solver_get_state(s, U.data(), MA_LAYOUT_AOS);
    if (e != MA_OK) return e;
    ma_checkpoint_info info{view.ncells, steps, steps * dt, dt, mesh_hash};
    e = ma_checkpoint_write(run.checkpoint_path, &info, U.data(), MA_LAYOUT_AOS);
    if (e == MA_OK) std::fprintf(stdout, " ... Checkpoint %s at step %i ...\n", run.checkpoint_path, steps);
    return e;
  };
  const auto t_run = std::chrono::steady_clock::now();
  // Solve loop (TimeSolverExplicitRK4.h:340-491): "Time Step #n" is printed
  // before step n runs when n is a multiple of output_frequency, as the
  // reference does; steps run in chunks up to the next print or checkpoint.
  const int freq = o.output_frequency > 0 ? o.output_frequency : o.ntimesteps + 1;
  const int cfreq = run.checkpoint_path[0] && run.checkpoint_frequency > 0 ? run.checkpoint_frequency : 0;
  while (done < o.ntimesteps) {
    if ((done + 1) % freq == 0)
      std::fprintf(stdout, "\nTime Step #%i:  Time = %16.9e; dt = %16.9e\n", done + 1, (done + 1) * dt, dt);
    int target = std::min(o.ntimesteps, ((done + 1) / freq + 1) * freq - 1);
    if (cfreq > 0) target = std::min(target, (done / cfreq + 1) * cfreq);
    if (target <= done) target = done + 1;
    if ((st = ma_solver_step(s, target - done)) != MA_OK) return fail("step", st);
    done = target;
    if (cfreq > 0 && done % cfreq == 0 && done < o.ntimesteps && (st = write_checkpoint(done)) != MA_OK)
      return fail("writing a checkpoint", st);
  }
  if ((st = ma_solver_synchronize(s)) != MA_OK) return fail("solve", st);
  if (run.checkpoint_path[0] && (st = write_checkpoint(done)) != MA_OK) return fail("writing a checkpoint", st);
  std::fprintf(stdout, "\n ... Device Run time: %8.2f seconds ...\n", seconds_since(t_run));
  int64_t bad = -1;
  if (ma_solver_check_state(s, &bad) != MA_OK)
    std::fprintf(stderr, "miniaero: warning: %s\n", ma_last_error());

  if (o.output_results) {
    U.resize(5 * C);
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
