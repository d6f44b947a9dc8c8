// Host-side C ABI: errors, host mesh, initial conditions.
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../../include/miniaero_gpu.h"
#include "trace.hpp"
#include "errors.hpp"
#include "mesh.hpp"
#include "../device/device_geometry.hpp"

namespace miniaero {
namespace {
thread_local std::string g_last_error;
}
ma_status set_error(ma_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}
const char* last_error() { return g_last_error.c_str(); }
}  // namespace miniaero

struct ma_host_mesh {
  miniaero::HostMesh mesh;
};

using miniaero::set_error;

extern "C" int32_t ma_abi_version(void) { return MA_ABI_VERSION; }
extern "C" const char* ma_last_error(void) { return miniaero::last_error(); }

extern "C" const char* ma_status_string(ma_status s) {
  switch (s) {
    case MA_OK: return "ok";
    case MA_EINVAL: return "invalid argument";
    case MA_ENOMEM: return "out of memory";
    case MA_ECUDA: return "CUDA error";
    case MA_EBUDGET: return "over device-memory budget";
    case MA_ETIMEDOUT: return "timed out";
    case MA_ENUMERIC: return "non-finite or non-physical state";
    case MA_ESTATE: return "invalid state";
    case MA_EIO: return "I/O error";
    case MA_ENOTFOUND: return "not found";
  }
  return "unknown status";
}

extern "C" ma_status ma_host_mesh_build(const ma_options* o, ma_host_mesh** out) {
  return ma_host_mesh_build_ex(o, 0, out);
}

extern "C" ma_status ma_host_mesh_build_ex(const ma_options* o, int32_t flags, ma_host_mesh** out) {
  if (!o || !out) return set_error(MA_EINVAL, "ma_host_mesh_build: null argument");
  *out = nullptr;
  if (flags & ~MA_HOST_MESH_DEVICE_GEOMETRY) return set_error(MA_EINVAL, "ma_host_mesh_build_ex: unknown flags");
  miniaero::TraceRange trace("ma_host_mesh_build");
  // The device arrays index a mesh with 32-bit arithmetic: refuse a box that
  // ma_mesh_upload would refuse before building it.
  if (o->nx > 0 && o->ny > 0 && o->nz > 0 &&
      static_cast<int64_t>(o->nx) * o->ny * o->nz > MA_MAX_MESH_CELLS)
    return set_error(MA_EINVAL, "ma_host_mesh_build: more than MA_MAX_MESH_CELLS (" +
                                    std::to_string(MA_MAX_MESH_CELLS) + ") cells");
  miniaero::MeshSpec spec;
  spec.nx = o->nx; spec.ny = o->ny; spec.nz = o->nz;
  spec.lx = o->lx; spec.ly = o->ly; spec.lz = o->lz;
  spec.angle = o->angle;
  spec.problem_type = o->problem_type;
  for (int i = 0; i < 6; ++i) spec.bc_override[i] = o->bc_override[i];
  ma_host_mesh* m = new (std::nothrow) ma_host_mesh;
  if (!m) return set_error(MA_ENOMEM, "ma_host_mesh_build: out of host memory");
  std::unique_ptr<miniaero::GeometryEngine> engine;
  if (flags & MA_HOST_MESH_DEVICE_GEOMETRY) {
    std::string why;
    engine = miniaero::make_device_geometry(&why);
    if (!engine) {
      delete m;
      return set_error(MA_ECUDA, "ma_host_mesh_build_ex: device geometry: " + why);
    }
  }
  try {
    const std::string err = miniaero::build_box_mesh(spec, m->mesh, engine.get());
    if (!err.empty() && err.compare(0, 16, "device geometry:") == 0) {
      delete m;
      return set_error(MA_ECUDA, "ma_host_mesh_build_ex: " + err);
    }
    if (!err.empty()) { delete m; return set_error(MA_EINVAL, "ma_host_mesh_build: " + err); }
  } catch (const std::bad_alloc&) {
    delete m;
    return set_error(MA_ENOMEM, "ma_host_mesh_build: out of host memory");
  }
  *out = m;
  return MA_OK;
}

static void view_set(const miniaero::HostFaceSet& s, ma_face_set& v) {
  v.nfaces = s.nfaces;
  v.type = s.type;
  v.conn = s.conn.data();
  v.flux_index = s.flux_index.data();
  v.coords = s.coords.data();
  v.normal = s.normal.data();
  v.tangent = s.tangent.data();
  v.binormal = s.binormal.data();
  v.permutation = s.permutation.data();
}

extern "C" ma_status ma_host_mesh_view(const ma_host_mesh* m, ma_mesh_view* v) {
  if (!m || !v) return set_error(MA_EINVAL, "ma_host_mesh_view: null argument");
  std::memset(v, 0, sizeof(*v));
  v->ncells = m->mesh.ncells;
  v->cell_coords = m->mesh.cell_coords.data();
  v->cell_volumes = m->mesh.cell_volumes.data();
  view_set(m->mesh.internal, v->internal);
  v->nbc = static_cast<int32_t>(m->mesh.bc.size());
  for (size_t i = 0; i < m->mesh.bc.size(); ++i) view_set(m->mesh.bc[i], v->bc[i]);
  return MA_OK;
}

extern "C" void ma_host_mesh_free(ma_host_mesh* m) { delete m; }

extern "C" ma_status ma_debug_glibc_rand(uint32_t seed, int32_t n, int32_t* out) {
  if (n < 0 || (n > 0 && !out)) return set_error(MA_EINVAL, "ma_debug_glibc_rand: bad arguments");
  miniaero::GlibcRand r(seed);
  for (int32_t i = 0; i < n; ++i) out[i] = r.next();
  return MA_OK;
}

extern "C" ma_status ma_debug_binsort(const int32_t* keys, int32_t n, int32_t* perm) {
  if (n < 0 || (n > 0 && (!keys || !perm))) return set_error(MA_EINVAL, "ma_debug_binsort: bad arguments");
  const std::vector<int32_t> p = miniaero::binsort_permutation(keys, n, 1);
  for (int32_t i = 0; i < n; ++i) perm[i] = p[i];
  return MA_OK;
}

// Initial conditions (kokkos/Initial_Conditions.h:38-133).
extern "C" ma_status ma_host_initial_state(const ma_host_mesh* hm, const ma_options* o, double* U) {
  if (!hm || !o || !U) return set_error(MA_EINVAL, "ma_host_initial_state: null argument");
  const miniaero::HostMesh& m = hm->mesh;
  const double Rgas = 287.05, gamma = 1.4;
  const double Cv = Rgas / (gamma - 1.0);
  int ic = o->ic;
  if (ic == MA_IC_REFERENCE) ic = (o->problem_type == 0) ? -1 : MA_IC_CONSTANT;
  if (ic == -1) {
    // initialize_sod3d with the reference's SI states split at lx/2.
    const double midx = o->lx / 2.0;
    const double P1 = 68947.57, T1 = 288.889, P2 = 6894.757, T2 = 231.11;
    const double d1 = P1 / (Rgas * T1), e1 = d1 * (Cv * T1);
    const double d2 = P2 / (Rgas * T2), e2 = d2 * (Cv * T2);
    for (int32_t i = 0; i < m.ncells; ++i) {
      const bool left = m.cell_coords[3 * static_cast<size_t>(i)] < midx;
      double* u = &U[5 * static_cast<size_t>(i)];
      u[0] = left ? d1 : d2; u[1] = 0.0; u[2] = 0.0; u[3] = 0.0; u[4] = left ? e1 : e2;
    }
    return MA_OK;
  }
  if (ic == MA_IC_SOD) {
    // Same construction with given (rho, p) pairs: T = p / (rho R), rhoE = rho Cv T.
    const double split = o->sod_split > 0.0 ? o->sod_split : o->lx / 2.0;
    const double dl = o->sod_left[0], dr = o->sod_right[0];
    if (!(dl > 0 && dr > 0 && o->sod_left[1] > 0 && o->sod_right[1] > 0))
      return set_error(MA_EINVAL, "Sod states need positive density and pressure");
    const double Tl = o->sod_left[1] / (dl * Rgas), Tr = o->sod_right[1] / (dr * Rgas);
    const double el = dl * (Cv * Tl), er = dr * (Cv * Tr);
    for (int32_t i = 0; i < m.ncells; ++i) {
      const bool left = m.cell_coords[3 * static_cast<size_t>(i)] < split;
      double* u = &U[5 * static_cast<size_t>(i)];
      u[0] = left ? dl : dr; u[1] = 0.0; u[2] = 0.0; u[3] = 0.0; u[4] = left ? el : er;
    }
    return MA_OK;
  }
  if (ic == MA_IC_CONSTANT) {
    for (int32_t i = 0; i < m.ncells; ++i)
      for (int k = 0; k < 5; ++k) U[5 * static_cast<size_t>(i) + k] = o->inflow_state[k];
    return MA_OK;
  }
  return set_error(MA_EINVAL, "ma_host_initial_state: unknown initial condition");
}
