// Batched multi-mesh solver (ma_batch_*): many independent meshes of uneven
// size advance together, one persistent launch per kernel kind and RK stage
// for the whole batch, the step captured once in a CUDA graph.
//
// Members own their state (U_n, U_np1, stage work arrays); meshes are shared
// ma_mesh objects. Per-member segment descriptors and per-kernel chunk tables
// (segment, first item) live in fixed device buffers whose contents change on
// add/remove; kernels read the chunk counts from device memory, so the
// captured graph stays valid while membership changes. Each cell and face is
// computed by exactly the code of the single-mesh solver, so a member's
// result is bit-identical alone or in any mix.
#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../../include/miniaero_gpu.h"
#include "../host/errors.hpp"
#include "../host/trace.hpp"
#include "batch_internal.hpp"
#include "kernels.cuh"

using miniaero::set_error;
namespace dev = miniaero::dev;

#define MB_CUDA_TRY(expr)                                                                   \
  do {                                                                                     \
    cudaError_t err__ = (expr);                                                            \
    if (err__ != cudaSuccess)                                                              \
      return set_error(MA_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(err__)); \
  } while (0)

namespace {

struct Member {
  int32_t id = -1;
  ma_mesh* mesh = nullptr;
  int gather = MA_GATHER_ATOMICS;  // list order of the batch's options
  void* dmem = nullptr;
  size_t bytes = 0;
  double dt = 0.0;
  double inflow[5] = {0, 0, 0, 0, 0};
  dev::StateBuffers st;
  dev::StageBuffers<double> b64;
  dev::StageBuffers<float> b32;
  int64_t steps = 0;
};

template <class T>
T* carve(char*& p, size_t n) {
  T* r = reinterpret_cast<T*>(p);
  p += (n * sizeof(T) + 255) & ~size_t(255);
  return r;
}

size_t padded(size_t bytes) { return (bytes + 255) & ~size_t(255); }

}  // namespace

struct ma_batch {
  ma_options opts;
  dev::PathConfig cfg;
  bool mixed = false;
  bool fma = false;  // MA_PREC_FP64_FMA
  int32_t capacity = 0;
  size_t budget = 0;
  size_t used = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // graph side branch: the boundary-face flux
  cudaEvent_t fork = nullptr, join = nullptr;
  std::map<int32_t, Member> members;
  int32_t next_id = 0;
  // device tables
  void* d_segs = nullptr;          // Segment<R>[capacity]
  int2* d_chunks[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t chunk_cap[4] = {0, 0, 0, 0};
  int* d_nchunks = nullptr;        // [4]
  dev::BatchLaunch launch;
  bool tables_dirty = true;
  cudaGraphExec_t graph = nullptr;
  int64_t cells = 0;
  unsigned long long* d_scratch = nullptr;
  int sm_count = 0;
  // Single-launch mode (ma_batch_set_single_launch): a whole ma_batch_step is
  // one cooperative launch of `single_block` x `single_grid`.
  int single_block = 0;  // 0: per-kind launches captured in a graph
  int single_grid = 0;
  unsigned* d_barrier = nullptr;  // two words: arrival count, generation
  int* d_err = nullptr;           // set by a grid barrier that gave up
};

namespace {

void drop_graph(ma_batch* b) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
}

size_t member_bytes(const ma_batch* b, const ma_mesh* m) {
  const size_t C = miniaero::mesh_cells(m), F = miniaero::mesh_faces(m);
  const size_t r = b->mixed ? sizeof(float) : sizeof(double);
  return padded(5 * C * 8) * 2 + padded(5 * C * r) + padded(15 * C * r) + padded(5 * C * r) + padded(5 * F * r);
}

template <class R>
dev::Segment<R> make_segment(const Member& m, const dev::StageBuffers<R>& sb) {
  dev::Segment<R> s;
  s.t = miniaero::mesh_topo(m.mesh, m.gather);
  s.g = miniaero::mesh_geom<R>(m.mesh);
  s.b = sb;
  s.s = m.st;
  s.dt = m.dt;
  for (int k = 0; k < 5; ++k) s.inflow.u[k] = m.inflow[k];
  return s;
}

// Rebuilds segment descriptors and chunk tables for the current members.
ma_status upload_tables(ma_batch* b) {
  std::vector<dev::Segment<double>> s64;
  std::vector<dev::Segment<float>> s32;
  std::vector<int2> chunks[4];
  int seg = 0;
  b->cells = 0;
  for (auto& kv : b->members) {
    const Member& m = kv.second;
    const dev::TopoView t = miniaero::mesh_topo(m.mesh);
    if (b->mixed) s32.push_back(make_segment<float>(m, m.b32));
    else s64.push_back(make_segment<double>(m, m.b64));
    const int32_t items[4] = {t.C, t.Fi, t.Fb, t.C};
    for (int k = 0; k < 4; ++k)
      for (int32_t start = 0; start < items[k]; start += b->launch.block[k]) chunks[k].push_back(make_int2(seg, start));
    b->cells += t.C;
    ++seg;
  }
  const size_t seg_bytes = b->mixed ? s32.size() * sizeof(dev::Segment<float>) : s64.size() * sizeof(dev::Segment<double>);
  if (seg_bytes)
    MB_CUDA_TRY(cudaMemcpyAsync(b->d_segs, b->mixed ? static_cast<const void*>(s32.data()) : static_cast<const void*>(s64.data()),
                                seg_bytes, cudaMemcpyHostToDevice, b->stream));
  int counts[4];
  for (int k = 0; k < 4; ++k) {
    counts[k] = static_cast<int>(chunks[k].size());
    if (chunks[k].size() > b->chunk_cap[k]) {
      // Grow (and drop the graph, which holds the old pointer).
      MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
      cudaFree(b->d_chunks[k]);
      b->d_chunks[k] = nullptr;
      const size_t cap = std::max<size_t>(chunks[k].size() * 3 / 2 + 64, 1024);
      MB_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&b->d_chunks[k]), cap * sizeof(int2)));
      b->chunk_cap[k] = cap;
      drop_graph(b);
    }
    if (!chunks[k].empty())
      MB_CUDA_TRY(cudaMemcpyAsync(b->d_chunks[k], chunks[k].data(), chunks[k].size() * sizeof(int2),
                                  cudaMemcpyHostToDevice, b->stream));
    b->launch.chunks[k] = b->d_chunks[k];
  }
  MB_CUDA_TRY(cudaMemcpyAsync(b->d_nchunks, counts, sizeof(counts), cudaMemcpyHostToDevice, b->stream));
  // The host vectors die here: finish the copies first.
  MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->launch.nchunks = b->d_nchunks;
  b->tables_dirty = false;
  return MA_OK;
}

ma_status launch_stage_on(ma_batch* b, int stage, unsigned kernels, cudaStream_t stream) {
  cudaError_t e = b->mixed
      ? dev::launch_batch_stage<float>(b->cfg, static_cast<const dev::Segment<float>*>(b->d_segs), b->launch, stage,
                                       stream, kernels)
      : b->fma ? dev::launch_batch_stage_fma(b->cfg, static_cast<const dev::Segment<double>*>(b->d_segs), b->launch,
                                             stage, stream, kernels)
               : dev::launch_batch_stage<double>(b->cfg, static_cast<const dev::Segment<double>*>(b->d_segs),
                                                 b->launch, stage, stream, kernels);
  if (e != cudaSuccess) return set_error(MA_ECUDA, std::string("batch stage launch: ") + cudaGetErrorString(e));
  return MA_OK;
}

ma_status launch_stage(ma_batch* b, int stage, unsigned kernels) { return launch_stage_on(b, stage, kernels, b->stream); }

// nsteps whole steps as one cooperative launch (single-launch mode).
ma_status launch_steps_single(ma_batch* b, int32_t nsteps) {
  for (int k = 0; k < 4; ++k)
    if (b->launch.block[k] != b->single_block)
      return set_error(MA_ESTATE, "ma_batch_step: launch shapes changed after ma_batch_set_single_launch; set it again");
  cudaError_t e;
  if (b->mixed)
    e = dev::launch_batch_steps_mixed(b->cfg, b->d_segs, b->launch, nsteps, b->d_barrier, b->d_err, b->single_block,
                                      b->single_grid, b->stream);
  else if (b->fma)
    e = dev::launch_batch_steps_fp64_fma(b->cfg, b->d_segs, b->launch, nsteps, b->d_barrier, b->d_err,
                                         b->single_block, b->single_grid, b->stream);
  else
    e = dev::launch_batch_steps_fp64(b->cfg, b->d_segs, b->launch, nsteps, b->d_barrier, b->d_err, b->single_block,
                                     b->single_grid, b->stream);
  if (e != cudaSuccess) return set_error(MA_ECUDA, std::string("batch single launch: ") + cudaGetErrorString(e));
  return MA_OK;
}

// After the stream has drained: MA_ETIMEDOUT if a grid barrier of the
// single-launch kernel gave up (the flag is cleared).
ma_status check_barrier_error(ma_batch* b) {
  if (!b->single_block) return MA_OK;
  int err = 0;
  MB_CUDA_TRY(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err == 0) return MA_OK;
  MB_CUDA_TRY(cudaMemset(b->d_barrier, 0, 2 * sizeof(unsigned) + sizeof(int)));
  return set_error(MA_ETIMEDOUT, "ma_batch_step: a grid barrier of the single-launch step timed out; member states "
                                 "are incomplete");
}

ma_status capture_graph(ma_batch* b) {
  drop_graph(b);
  cudaGraph_t g = nullptr;
  MB_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  ma_status st = MA_OK;
  // Per stage, the boundary-face flux (it reads only the stage's primitives)
  // runs on a side branch beside the sweep and the internal-face flux; the
  // residual waits for both branches.
  for (int stage = 0; stage < 4 && st == MA_OK; ++stage) {
    cudaError_t ef = cudaEventRecord(b->fork, b->stream);
    if (ef == cudaSuccess) ef = cudaStreamWaitEvent(b->side, b->fork, 0);
    if (ef != cudaSuccess) {
      st = set_error(MA_ECUDA, std::string("batch capture: ") + cudaGetErrorString(ef));
      break;
    }
    st = launch_stage_on(b, stage, dev::kBcFlux, b->side);
    if (st == MA_OK && cudaEventRecord(b->join, b->side) != cudaSuccess)
      st = set_error(MA_ECUDA, "batch capture: join record failed");
    if (st == MA_OK) st = launch_stage(b, stage, dev::kSweep1 | dev::kInternalFlux);
    if (st == MA_OK && cudaStreamWaitEvent(b->stream, b->join, 0) != cudaSuccess)
      st = set_error(MA_ECUDA, "batch capture: join wait failed");
    if (st == MA_OK) st = launch_stage(b, stage, dev::kResidual);
  }
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (st != MA_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return st != MA_OK ? st : set_error(MA_ECUDA, std::string("batch capture: ") + cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_error(MA_ECUDA, std::string("batch graph: ") + cudaGetErrorString(e));
  return MA_OK;
}

// Persistent grid: enough CTAs to fill every SM at the kernel's occupancy.
void default_grid(ma_batch* b) {
  for (int k = 0; k < 4; ++k) b->launch.grid[k] = b->sm_count * std::max(1, 2048 / b->launch.block[k] / 2);
}

}  // namespace

extern "C" ma_status ma_batch_create(const ma_options* o, int32_t capacity, size_t budget_bytes, ma_batch** out) {
  if (!o || !out || capacity <= 0) return set_error(MA_EINVAL, "ma_batch_create: bad arguments");
  *out = nullptr;
  if (o->precision != MA_PREC_FP64 && o->precision != MA_PREC_MIXED && o->precision != MA_PREC_FP64_FMA)
    return set_error(MA_EINVAL, "bad precision");
  if (o->gather != MA_GATHER_ATOMICS && o->gather != MA_GATHER_CELL_FLUX) return set_error(MA_EINVAL, "bad gather");
  // A failure part way releases what was created (ma_batch_free skips null handles).
  std::unique_ptr<ma_batch, void (*)(ma_batch*)> b(new (std::nothrow) ma_batch, ma_batch_free);
  if (!b) return set_error(MA_ENOMEM, "ma_batch_create: out of host memory");
  b->opts = *o;
  b->mixed = o->precision == MA_PREC_MIXED;
  b->fma = o->precision == MA_PREC_FP64_FMA;
  b->cfg.second_order = o->second_order_space != 0;
  b->cfg.viscous = o->viscous != 0;
  b->cfg.limiter = o->limiter;
  b->cfg.transport = dev::make_transport(o->viscosity_model, o->mu, o->prandtl);
  b->cfg.cell_flux = o->gather == MA_GATHER_CELL_FLUX;
  b->capacity = capacity;
  b->budget = budget_bytes;
  MB_CUDA_TRY(cudaGetDevice(&b->device));
  MB_CUDA_TRY(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device));
  const size_t seg_size = b->mixed ? sizeof(dev::Segment<float>) : sizeof(dev::Segment<double>);
  MB_CUDA_TRY(cudaMalloc(&b->d_segs, seg_size * capacity));
  // [0, 16) chunk counts, [16, 24) CFL scratch, [24, 32) grid barrier, [32, 36) barrier error.
  MB_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&b->d_nchunks), 64));
  MB_CUDA_TRY(cudaMemset(b->d_nchunks, 0, 64));
  b->d_scratch = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(b->d_nchunks) + 16);
  b->d_barrier = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(b->d_nchunks) + 24);
  b->d_err = reinterpret_cast<int*>(reinterpret_cast<char*>(b->d_nchunks) + 32);
  MB_CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  MB_CUDA_TRY(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
  MB_CUDA_TRY(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  MB_CUDA_TRY(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming));
  for (int k = 0; k < 4; ++k) b->launch.block[k] = 128;
  default_grid(b.get());
  *out = b.release();
  return MA_OK;
}

extern "C" void ma_batch_free(ma_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  for (auto& kv : b->members) cudaFree(kv.second.dmem);
  for (int k = 0; k < 4; ++k) cudaFree(b->d_chunks[k]);
  cudaFree(b->d_segs);
  cudaFree(b->d_nchunks);
  if (b->join) cudaEventDestroy(b->join);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

extern "C" size_t ma_batch_member_bytes(const ma_batch* b, const ma_mesh* m) {
  return (b && m) ? member_bytes(b, m) : 0;
}

extern "C" ma_status ma_batch_add(ma_batch* b, ma_mesh* mesh, const double* U0, int32_t layout, double dt,
                                  const double* inflow_state, int32_t* member_id) {
  if (!b || !mesh || !U0 || !member_id) return set_error(MA_EINVAL, "ma_batch_add: null argument");
  if (layout != MA_LAYOUT_AOS && layout != MA_LAYOUT_SOA) return set_error(MA_EINVAL, "ma_batch_add: bad layout");
  if (static_cast<int32_t>(b->members.size()) >= b->capacity) return set_error(MA_EBUDGET, "batch is full");
  const size_t need = member_bytes(b, mesh);
  if (b->used + need > b->budget) return set_error(MA_EBUDGET, "member does not fit the device-memory budget");
  if (!(dt > 0.0) && !(b->opts.cfl > 0.0)) return set_error(MA_EINVAL, "ma_batch_add: dt must be > 0 without cfl");
  if (b->opts.gather == MA_GATHER_CELL_FLUX && !miniaero::mesh_has_cell_flux(mesh))
    return set_error(MA_EINVAL, "gather cell_flux needs a mesh uploaded with MA_MESH_CELL_FLUX");
  Member m;
  m.mesh = mesh;
  m.gather = b->opts.gather;
  m.bytes = need;
  for (int k = 0; k < 5; ++k) m.inflow[k] = inflow_state ? inflow_state[k] : b->opts.inflow_state[k];
  cudaError_t e = cudaMalloc(&m.dmem, need);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? MA_ENOMEM : MA_ECUDA,
                     std::string("ma_batch_add: ") + cudaGetErrorString(e));
  }
  const size_t C = miniaero::mesh_cells(mesh), F = miniaero::mesh_faces(mesh);
  char* p = static_cast<char*>(m.dmem);
  m.st.Un = carve<double>(p, 5 * C);
  m.st.Unp1 = carve<double>(p, 5 * C);
  m.st.res = nullptr;
  if (b->mixed) {
    m.b32.W = carve<float>(p, 5 * C);
    m.b32.grad = carve<float>(p, 15 * C);
    m.b32.phi = carve<float>(p, 5 * C);
    m.b32.fflux = carve<float>(p, 5 * F);
  } else {
    m.b64.W = carve<double>(p, 5 * C);
    m.b64.grad = carve<double>(p, 15 * C);
    m.b64.phi = carve<double>(p, 5 * C);
    m.b64.fflux = carve<double>(p, 5 * F);
  }
  auto fail = [&](ma_status s) {
    cudaFree(m.dmem);
    return s;
  };
  // State upload (device SoA).
  std::vector<double> soa;
  const double* src = U0;
  if (layout == MA_LAYOUT_AOS) {
    soa.resize(5 * C);
    for (size_t c = 0; c < C; ++c)
      for (int k = 0; k < 5; ++k) soa[k * C + c] = U0[5 * c + k];
    src = soa.data();
  }
  e = cudaMemcpyAsync(m.st.Un, src, 5 * C * sizeof(double), cudaMemcpyHostToDevice, b->stream);
  if (e != cudaSuccess) return fail(set_error(MA_ECUDA, std::string("ma_batch_add: ") + cudaGetErrorString(e)));
  const dev::TopoView t = miniaero::mesh_topo(mesh);
  if (dt > 0.0) {
    m.dt = dt;
  } else {
    cudaMemsetAsync(b->d_scratch, 0xff, 8, b->stream);
    e = dev::launch_cfl(t, miniaero::mesh_geom<double>(mesh), m.st.Un, b->d_scratch, b->stream);
    unsigned long long bits = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, b->d_scratch, 8, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return fail(set_error(MA_ECUDA, std::string("ma_batch_add: ") + cudaGetErrorString(e)));
    double r;
    std::memcpy(&r, &bits, 8);
    if (!(r > 0.0) || bits == ~0ULL) return fail(set_error(MA_ENUMERIC, "ma_batch_add: CFL time step is not finite"));
    m.dt = b->opts.cfl * r;
  }
  e = b->mixed ? dev::launch_init_primitives<float>(t, m.st, m.b32, b->stream)
      : b->fma ? dev::launch_init_primitives_fma(t, m.st, m.b64, b->stream)
               : dev::launch_init_primitives<double>(t, m.st, m.b64, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return fail(set_error(MA_ECUDA, std::string("ma_batch_add: ") + cudaGetErrorString(e)));
  m.id = b->next_id++;
  b->used += need;
  b->members[m.id] = m;
  b->tables_dirty = true;
  *member_id = m.id;
  return MA_OK;
}

extern "C" ma_status ma_batch_remove(ma_batch* b, int32_t id) {
  if (!b) return set_error(MA_EINVAL, "ma_batch_remove: null batch");
  auto it = b->members.find(id);
  if (it == b->members.end()) return set_error(MA_ENOTFOUND, "ma_batch_remove: unknown member");
  MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  cudaFree(it->second.dmem);
  b->used -= it->second.bytes;
  b->members.erase(it);
  b->tables_dirty = true;
  return MA_OK;
}

extern "C" ma_status ma_batch_get_state(ma_batch* b, int32_t id, double* U, int32_t layout) {
  if (!b || !U) return set_error(MA_EINVAL, "ma_batch_get_state: null argument");
  auto it = b->members.find(id);
  if (it == b->members.end()) return set_error(MA_ENOTFOUND, "ma_batch_get_state: unknown member");
  const size_t C = miniaero::mesh_cells(it->second.mesh);
  MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  ma_status bst = check_barrier_error(b);
  if (bst != MA_OK) return bst;
  if (layout == MA_LAYOUT_SOA) {
    MB_CUDA_TRY(cudaMemcpyAsync(U, it->second.st.Un, 5 * C * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  } else if (layout == MA_LAYOUT_AOS) {
    std::vector<double> soa(5 * C);
    MB_CUDA_TRY(cudaMemcpyAsync(soa.data(), it->second.st.Un, 5 * C * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
    for (size_t c = 0; c < C; ++c)
      for (int k = 0; k < 5; ++k) U[5 * c + k] = soa[k * C + c];
  } else {
    return set_error(MA_EINVAL, "ma_batch_get_state: bad layout");
  }
  return MA_OK;
}

extern "C" ma_status ma_batch_step(ma_batch* b, int32_t nsteps) {
  if (!b || nsteps < 0) return set_error(MA_EINVAL, "ma_batch_step: bad arguments");
  if (nsteps == 0 || b->members.empty()) return MA_OK;
  miniaero::TraceRange trace("ma_batch_step");
  if (b->tables_dirty) {
    ma_status st = upload_tables(b);
    if (st != MA_OK) return st;
  }
  if (b->single_block) {
    ma_status st = launch_steps_single(b, nsteps);
    if (st != MA_OK) return st;
    for (auto& kv : b->members) kv.second.steps += nsteps;
    return MA_OK;
  }
  if (!b->graph) {
    ma_status st = capture_graph(b);
    if (st != MA_OK) return st;
  }
  for (int32_t i = 0; i < nsteps; ++i) MB_CUDA_TRY(cudaGraphLaunch(b->graph, b->stream));
  for (auto& kv : b->members) kv.second.steps += nsteps;
  return MA_OK;
}

extern "C" ma_status ma_batch_set_single_launch(ma_batch* b, int32_t block, int32_t* grid_out) {
  if (!b) return set_error(MA_EINVAL, "ma_batch_set_single_launch: null batch");
  if (block != 0 && (block < 64 || block > 256 || block % 32))
    return set_error(MA_EINVAL, "ma_batch_set_single_launch: block must be 0 (off) or 64..256 in steps of 32");
  MB_CUDA_TRY(cudaSetDevice(b->device));
  MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (block == 0) {
    b->single_block = 0;
    b->single_grid = 0;
    if (grid_out) *grid_out = 0;
    return MA_OK;
  }
  int per_sm = 0;
  cudaError_t e = b->mixed ? dev::batch_steps_occupancy_mixed(b->cfg, block, &per_sm)
                  : b->fma ? dev::batch_steps_occupancy_fp64_fma(b->cfg, block, &per_sm)
                           : dev::batch_steps_occupancy_fp64(b->cfg, block, &per_sm);
  if (e != cudaSuccess) return set_error(MA_ECUDA, std::string("ma_batch_set_single_launch: ") + cudaGetErrorString(e));
  if (per_sm < 1) return set_error(MA_EINVAL, "ma_batch_set_single_launch: the kernel does not fit on an SM at this block size");
  // Every kind's chunks must match the one block size of the launch.
  for (int k = 0; k < 4; ++k) b->launch.block[k] = block;
  b->single_block = block;
  b->single_grid = per_sm * b->sm_count;
  b->tables_dirty = true;
  drop_graph(b);
  MB_CUDA_TRY(cudaMemset(b->d_barrier, 0, 2 * sizeof(unsigned) + sizeof(int)));
  if (grid_out) *grid_out = b->single_grid;
  return MA_OK;
}

extern "C" ma_status ma_batch_profile_steps(ma_batch* b, int32_t nsteps, double* kernel_ms, int32_t* kernel_launches) {
  if (!b || nsteps < 0 || !kernel_ms || !kernel_launches)
    return set_error(MA_EINVAL, "ma_batch_profile_steps: bad arguments");
  for (int k = 0; k < MA_PROFILE_KINDS; ++k) {
    kernel_ms[k] = 0.0;
    kernel_launches[k] = 0;
  }
  if (nsteps == 0 || b->members.empty()) return MA_OK;
  if (b->tables_dirty) {
    ma_status st = upload_tables(b);
    if (st != MA_OK) return st;
  }
  const unsigned bits[MA_PROFILE_KINDS] = {dev::kSweep1, dev::kInternalFlux, dev::kBcFlux, dev::kResidual};
  std::vector<cudaEvent_t> ev;
  std::vector<int> kind;
  auto cleanup = [&]() { for (cudaEvent_t e : ev) cudaEventDestroy(e); };
  for (int32_t step = 0; step < nsteps; ++step)
    for (int stage = 0; stage < 4; ++stage)
      for (int k = 0; k < MA_PROFILE_KINDS; ++k) {
        cudaEvent_t a, e;
        if (cudaEventCreate(&a) != cudaSuccess) {
          cleanup();
          return set_error(MA_ECUDA, "ma_batch_profile_steps: cudaEventCreate failed");
        }
        ev.push_back(a);
        if (cudaEventCreate(&e) != cudaSuccess) {
          cleanup();
          return set_error(MA_ECUDA, "ma_batch_profile_steps: cudaEventCreate failed");
        }
        ev.push_back(e);
        kind.push_back(k);
        cudaEventRecord(a, b->stream);
        ma_status st = launch_stage(b, stage, bits[k]);
        cudaEventRecord(e, b->stream);
        if (st != MA_OK) {
          cleanup();
          return st;
        }
      }
  cudaError_t err = cudaStreamSynchronize(b->stream);
  if (err != cudaSuccess) {
    cleanup();
    return set_error(MA_ECUDA, std::string("ma_batch_profile_steps: ") + cudaGetErrorString(err));
  }
  for (size_t i = 0; i < kind.size(); ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
    kernel_ms[kind[i]] += ms;
    kernel_launches[kind[i]] += 1;
  }
  cleanup();
  for (auto& kv : b->members) kv.second.steps += nsteps;
  return MA_OK;
}

extern "C" ma_status ma_batch_synchronize(ma_batch* b) {
  if (!b) return set_error(MA_EINVAL, "ma_batch_synchronize: null batch");
  MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return check_barrier_error(b);
}

extern "C" void* ma_batch_stream(ma_batch* b) { return b ? static_cast<void*>(b->stream) : nullptr; }
extern "C" int64_t ma_batch_cells(ma_batch* b) {
  if (!b) return 0;
  int64_t n = 0;
  for (auto& kv : b->members) n += miniaero::mesh_cells(kv.second.mesh);
  return n;
}
extern "C" int32_t ma_batch_size(const ma_batch* b) { return b ? static_cast<int32_t>(b->members.size()) : 0; }
extern "C" size_t ma_batch_device_bytes(const ma_batch* b) { return b ? b->used : 0; }
extern "C" int64_t ma_batch_member_steps(const ma_batch* b, int32_t id) {
  if (!b) return -1;
  auto it = b->members.find(id);
  return it == b->members.end() ? -1 : it->second.steps;
}
extern "C" double ma_batch_member_dt(const ma_batch* b, int32_t id) {
  if (!b) return 0.0;
  auto it = b->members.find(id);
  return it == b->members.end() ? 0.0 : it->second.dt;
}

extern "C" ma_status ma_batch_get_launch(const ma_batch* b, int32_t* block, int32_t* grid) {
  if (!b || !block || !grid) return set_error(MA_EINVAL, "ma_batch_get_launch: null argument");
  for (int k = 0; k < 4; ++k) {
    block[k] = b->launch.block[k];
    grid[k] = b->launch.grid[k];
  }
  return MA_OK;
}

extern "C" ma_status ma_batch_set_launch(ma_batch* b, const int32_t* block, const int32_t* grid) {
  if (!b || !block || !grid) return set_error(MA_EINVAL, "ma_batch_set_launch: null argument");
  for (int k = 0; k < 4; ++k)
    if (block[k] < 32 || block[k] > 256 || block[k] % 32 || grid[k] < 1 || grid[k] > 65535)
      return set_error(MA_EINVAL, "ma_batch_set_launch: block must be 32..256 in steps of 32, grid 1..65535");
  MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (int k = 0; k < 4; ++k) {
    b->launch.block[k] = block[k];
    b->launch.grid[k] = grid[k];
  }
  b->tables_dirty = true;
  drop_graph(b);
  return MA_OK;
}

// Autotuner: per kernel kind, times one stage of that kernel over the current
// members for each candidate (block size x CTAs per SM) and keeps the
// fastest. Stage kernels are idempotent for a fixed input state except the
// residual update, whose timing runs operate on a scratch copy of the state.
extern "C" ma_status ma_batch_autotune(ma_batch* b, int32_t reps, double* best_ms) {
  if (!b || reps <= 0) return set_error(MA_EINVAL, "ma_batch_autotune: bad arguments");
  if (b->members.empty()) return set_error(MA_ESTATE, "ma_batch_autotune: empty batch");
  miniaero::TraceRange trace("ma_batch_autotune");
  // Save U_n, U_np1 and W of every member (the leading region of its
  // allocation); tuning runs real stages, the other arrays are recomputed by
  // the next stage before they are read.
  std::vector<std::vector<char>> saved;
  auto state_bytes = [&](const Member& m) {
    const size_t C = miniaero::mesh_cells(m.mesh);
    return padded(5 * C * 8) * 2 + padded(5 * C * (b->mixed ? sizeof(float) : sizeof(double)));
  };
  for (auto& kv : b->members) {
    saved.emplace_back(state_bytes(kv.second));
    MB_CUDA_TRY(cudaMemcpyAsync(saved.back().data(), kv.second.dmem, saved.back().size(), cudaMemcpyDeviceToHost,
                                b->stream));
  }
  MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  static const int blocks[3] = {64, 128, 256};
  static const int per_sm[5] = {1, 2, 4, 8, 16};
  const unsigned bits[4] = {dev::kSweep1, dev::kInternalFlux, dev::kBcFlux, dev::kResidual};
  cudaEvent_t e0, e1;
  MB_CUDA_TRY(cudaEventCreate(&e0));
  MB_CUDA_TRY(cudaEventCreate(&e1));
  drop_graph(b);
  ma_status st = MA_OK;
  for (int k = 0; k < 4 && st == MA_OK; ++k) {
    float best = 1e30f;
    int bb = b->launch.block[k], bg = b->launch.grid[k];
    for (int bi = 0; bi < 3 && st == MA_OK; ++bi)
      for (int pi = 0; pi < 5 && st == MA_OK; ++pi) {
        const int blk = blocks[bi];
        const int grd = b->sm_count * per_sm[pi];
        if (per_sm[pi] * blk > 2048) continue;
        b->launch.block[k] = blk;
        b->launch.grid[k] = grd;
        st = upload_tables(b);
        if (st != MA_OK) break;
        st = launch_stage(b, 1, bits[k]);  // warm-up
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < reps && st == MA_OK; ++r) st = launch_stage(b, 1, bits[k]);
        cudaEventRecord(e1, b->stream);
        if (cudaStreamSynchronize(b->stream) != cudaSuccess) {
          st = set_error(MA_ECUDA, "ma_batch_autotune: stage failed");
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          bb = blk;
          bg = grd;
        }
      }
    b->launch.block[k] = bb;
    b->launch.grid[k] = bg;
    if (best_ms) best_ms[k] = best / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  size_t i = 0;
  for (auto& kv : b->members) {
    cudaMemcpyAsync(kv.second.dmem, saved[i].data(), saved[i].size(), cudaMemcpyHostToDevice, b->stream);
    ++i;
  }
  MB_CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->tables_dirty = true;
  return st;
}
