// Options: defaults and the miniaero.inp reader (kokkos/Options.h:47-102),
// plus "key value" extension lines after the nine positional values.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../../include/miniaero_gpu.h"
#include "errors.hpp"

using miniaero::set_error;

extern "C" void ma_options_default(ma_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  // Options::Options() (kokkos/Options.h:59-69); viscous and the lengths are
  // uninitialised there and default to 0 / 1.0 here.
  o->problem_type = 0;
  o->nx = 10; o->ny = 10; o->nz = 10;
  o->lx = 1.0; o->ly = 1.0; o->lz = 1.0; o->angle = 0.0;
  o->ntimesteps = 1;
  o->dt = 5e-8;
  o->output_results = 0;
  o->output_frequency = 10;
  o->second_order_space = 0;
  o->viscous = 0;
  o->limiter = MA_LIMITER_VENKAT;
  o->viscosity_model = MA_VISC_SUTHERLAND;
  o->mu = 1.8e-5;
  o->prandtl = 0.72;
  o->precision = MA_PREC_FP64;
  o->cfl = 0.0;
  o->ic = MA_IC_REFERENCE;
  o->sod_left[0] = 1.0; o->sod_left[1] = 1.0;
  o->sod_right[0] = 0.125; o->sod_right[1] = 0.1;
  o->sod_split = 0.0;
  o->inflow_given = 0;
  // TimeSolverExplicitRK4.h:218-223
  o->inflow_state[0] = 0.5805; o->inflow_state[1] = 503.96; o->inflow_state[2] = 0.0;
  o->inflow_state[3] = 0.0; o->inflow_state[4] = 343750.0;
  for (int i = 0; i < 6; ++i) o->bc_override[i] = -1;
  o->keep_residual = 0;
  o->gather = MA_GATHER_ATOMICS;
}

namespace {
int side_index(const std::string& s) {
  static const char* names[6] = {"bottom", "top", "front", "back", "right", "left"};
  for (int i = 0; i < 6; ++i) if (s == names[i]) return i;
  return -1;
}
int bc_index(const std::string& s) {
  static const char* names[4] = {"extrapolate", "tangent", "inflow", "noslip"};
  for (int i = 0; i < 4; ++i) if (s == names[i]) return i;
  return -1;
}
}  // namespace

extern "C" ma_status ma_options_read(const char* path, ma_options* o) {
  if (!path || !o) return set_error(MA_EINVAL, "ma_options_read: null argument");
  ma_options_default(o);
  std::ifstream in(path);
  if (!in) return set_error(MA_EIO, std::string(path) + " does not exist.");
  in >> o->problem_type;
  in >> o->lx >> o->ly >> o->lz >> o->angle;
  in >> o->nx >> o->ny >> o->nz;
  in >> o->ntimesteps;
  in >> o->dt;
  in >> o->output_results;
  in >> o->output_frequency;
  in >> o->second_order_space;
  in >> o->viscous;
  if (!in) return set_error(MA_EINVAL, std::string(path) + ": expected nine positional values");
  std::string key;
  while (in >> key) {
    if (!key.empty() && key[0] == '#') { std::string rest; std::getline(in, rest); continue; }
    bool ok = true;
    if (key == "limiter") {
      std::string v; in >> v;
      if (v == "venkat") o->limiter = MA_LIMITER_VENKAT;
      else if (v == "vanalbada") o->limiter = MA_LIMITER_VANALBADA;
      else ok = false;
    } else if (key == "viscosity") {
      std::string v; in >> v;
      if (v == "sutherland") o->viscosity_model = MA_VISC_SUTHERLAND;
      else if (v == "constant") { o->viscosity_model = MA_VISC_CONSTANT; in >> o->mu >> o->prandtl; }
      else ok = false;
    } else if (key == "precision") {
      std::string v; in >> v;
      if (v == "fp64") o->precision = MA_PREC_FP64;
      else if (v == "mixed") o->precision = MA_PREC_MIXED;
      else if (v == "fp64_fma") o->precision = MA_PREC_FP64_FMA;
      else ok = false;
    } else if (key == "cfl") {
      in >> o->cfl;
    } else if (key == "sod") {
      o->ic = MA_IC_SOD;
      in >> o->sod_left[0] >> o->sod_left[1] >> o->sod_right[0] >> o->sod_right[1];
    } else if (key == "sod_split") {
      in >> o->sod_split;
    } else if (key == "inflow") {
      o->inflow_given = 1;
      for (int k = 0; k < 5; ++k) in >> o->inflow_state[k];
    } else if (key == "ic") {
      std::string v; in >> v;
      if (v == "reference") o->ic = MA_IC_REFERENCE;
      else if (v == "sod") o->ic = MA_IC_SOD;
      else if (v == "constant") o->ic = MA_IC_CONSTANT;
      else ok = false;
    } else if (key == "bc") {
      std::string side, type; in >> side >> type;
      const int si = side_index(side), bi = bc_index(type);
      if (si < 0 || bi < 0) ok = false; else o->bc_override[si] = bi;
    } else if (key == "gather") {
      std::string v; in >> v;
      if (v == "atomics") o->gather = MA_GATHER_ATOMICS;
      else if (v == "cell_flux") o->gather = MA_GATHER_CELL_FLUX;
      else ok = false;
    } else if (key == "keep_residual") {
      in >> o->keep_residual;
    } else if (key == "checkpoint" || key == "restart") {
      std::string v; in >> v;  // run controls, read by ma_run_options_read
    } else if (key == "checkpoint_frequency") {
      int32_t v; in >> v;
    } else {
      return set_error(MA_EINVAL, std::string(path) + ": unknown option '" + key + "'");
    }
    if (!ok || !in) return set_error(MA_EINVAL, std::string(path) + ": bad value for '" + key + "'");
  }
  return MA_OK;
}
