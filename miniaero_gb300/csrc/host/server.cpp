// Serving loop (ma_server_*): continuous batching of independent solves on
// one GPU, built on the public batch API.
//
// Requests are admitted first-in first-out while their device memory fits
// the budget (member state plus the device mesh, which is cached per mesh
// specification and shared by requests of the same size). Each tick advances
// every running request by the same number of steps (the smaller of the tick
// length and the fewest steps any running request has left), so requests
// finish exactly on their step count and new arrivals join at the next tick.
// A scheduler thread drives the loop (or the caller does, through
// ma_server_poll). With the scheduler thread, a mesh shape not yet cached is
// built (host mesh and device upload) by a second thread, started when the
// request is submitted: the running requests keep stepping meanwhile, and the
// request waits at the head of the queue only if its mesh is not ready when
// its turn comes. In dry-run mode no device call is made: member and mesh
// sizes come from the mesh dimensions and ticks only advance counters, which
// is how the admission logic is tested without a GPU.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include <cuda_runtime_api.h>

#include "../../../include/miniaero_gpu.h"
#include "trace.hpp"
#include "errors.hpp"

using miniaero::set_error;

namespace {

using Clock = std::chrono::steady_clock;

struct MeshKey {
  int32_t nx, ny, nz, problem_type;
  double lx, ly, lz, angle;
  bool operator<(const MeshKey& o) const {
    return std::tie(nx, ny, nz, problem_type, lx, ly, lz, angle) <
           std::tie(o.nx, o.ny, o.nz, o.problem_type, o.lx, o.ly, o.lz, o.angle);
  }
};

struct CachedMesh {
  ma_host_mesh* host = nullptr;
  ma_mesh* dev = nullptr;
  size_t bytes = 0;
  int users = 0;
  int64_t last_used = 0;
};

struct Request {
  int64_t id = -1;
  ma_request req;
  int32_t state = MA_REQ_QUEUED;
  ma_status error = MA_OK;
  std::string message;
  int32_t member = -1;
  MeshKey key;
  size_t member_bytes = 0;
  int64_t steps_done = 0;
  int64_t t_submit = 0, t_admit = 0, t_finish = 0;
  int64_t cells = 0;
  std::vector<double> result;  // AOS, when keep_result
  double result_norm[5] = {0, 0, 0, 0, 0};
};

int64_t ns_since(Clock::time_point t0) {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
}

// Cells and faces of an nx*ny*nz box (the mesh generator's counts).
void box_counts(const ma_request& r, int64_t& cells, int64_t& faces) {
  const int64_t nx = r.nx, ny = r.ny, nz = r.nz;
  cells = nx * ny * nz;
  faces = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1);
}

}  // namespace

struct ma_server {
  ma_options physics;
  size_t budget = 0;
  int32_t tick_steps = 1;
  int32_t flags = 0;
  bool dry = false;
  ma_batch* batch = nullptr;
  Clock::time_point t0 = Clock::now();
  std::mutex mu;
  std::condition_variable cv;       // work available / state changed
  std::thread worker;
  bool stop = false;
  std::deque<int64_t> queue;
  std::map<int64_t, Request> reqs;
  std::map<MeshKey, CachedMesh> meshes;
  int64_t next_id = 1;
  size_t used = 0;                  // members + cached meshes
  int64_t max_running_cells = 0;    // 0: no cap
  int64_t running_cells = 0;
  ma_server_stats stats;
  int64_t busy_start = -1;
  // Mesh builds off the scheduler thread (thread mode, not dry-run).
  bool async_meshes = false;
  int device = 0;
  std::thread mesher;
  std::condition_variable mesh_cv;                  // a build job is waiting
  std::deque<MeshKey> mesh_jobs;
  std::map<MeshKey, std::pair<ma_options, size_t>> building;  // options, bytes reserved in `used`
  std::map<MeshKey, std::pair<ma_status, std::string>> failed_meshes;
};

namespace {

// Device bytes of a request's member state and of its mesh, from the mesh
// dimensions. They bound the allocations of ma_batch_add / ma_mesh_upload
// from above (array padding included), so admission never overshoots.
size_t dry_member_bytes(const ma_server* s, const ma_request& r) {
  int64_t C, F;
  box_counts(r, C, F);
  const size_t w = s->physics.precision == MA_PREC_MIXED ? 4 : 8;
  return static_cast<size_t>(C) * (80 + 25 * w) + static_cast<size_t>(F) * 5 * w + 6 * 256;
}

size_t dry_mesh_bytes(const ma_server* s, const ma_request& r) {
  int64_t C, F;
  box_counts(r, C, F);
  const size_t cell_flux = s->physics.gather == MA_GATHER_CELL_FLUX ? 72 : 0;  // slot-order lists
  return static_cast<size_t>(C) * (100 + cell_flux) + static_cast<size_t>(F) * 237 + 19 * 256;
}

MeshKey key_of(const ma_request& r) {
  return MeshKey{r.nx, r.ny, r.nz, r.problem_type, r.lx, r.ly, r.lz, r.angle};
}

ma_options options_of(const ma_server* s, const ma_request& r) {
  ma_options o = s->physics;
  o.nx = r.nx; o.ny = r.ny; o.nz = r.nz;
  o.lx = r.lx; o.ly = r.ly; o.lz = r.lz; o.angle = r.angle;
  o.problem_type = r.problem_type;
  o.ntimesteps = r.nsteps;
  o.ic = MA_IC_CONSTANT;
  for (int k = 0; k < 5; ++k) o.inflow_state[k] = r.inflow_state[k];
  return o;
}

// Evicts unused cached meshes (least recently used first) until `need` more
// bytes fit, without exceeding the budget. Returns whether they fit.
bool make_room(ma_server* s, size_t need) {
  while (s->used + need > s->budget) {
    auto victim = s->meshes.end();
    for (auto it = s->meshes.begin(); it != s->meshes.end(); ++it)
      if (it->second.users == 0 && (victim == s->meshes.end() || it->second.last_used < victim->second.last_used))
        victim = it;
    if (victim == s->meshes.end()) return false;
    if (!s->dry) {
      ma_mesh_free(victim->second.dev);
      ma_host_mesh_free(victim->second.host);
    }
    s->used -= victim->second.bytes;
    s->meshes.erase(victim);
  }
  return true;
}

ma_status ensure_mesh(ma_server* s, Request& q, CachedMesh** out) {
  auto it = s->meshes.find(q.key);
  if (it != s->meshes.end()) {
    *out = &it->second;
    return MA_OK;
  }
  CachedMesh cm;
  if (s->dry) {
    cm.bytes = dry_mesh_bytes(s, q.req);
  } else {
    ma_options o = options_of(s, q.req);
    ma_status st = ma_host_mesh_build_ex(&o, MA_HOST_MESH_DEVICE_GEOMETRY, &cm.host);
    if (st != MA_OK) return st;
    ma_mesh_view v;
    ma_host_mesh_view(cm.host, &v);
    st = ma_mesh_upload_ex(&v, s->physics.gather == MA_GATHER_CELL_FLUX ? MA_MESH_CELL_FLUX : 0, &cm.dev);
    if (st != MA_OK) {
      ma_host_mesh_free(cm.host);
      return st;
    }
    cm.bytes = ma_mesh_device_bytes(cm.dev);
  }
  s->used += cm.bytes;
  it = s->meshes.emplace(q.key, cm).first;
  *out = &it->second;
  return MA_OK;
}

void finish(ma_server* s, Request& q, int32_t state) {
  q.state = state;
  q.t_finish = ns_since(s->t0);
  if (state == MA_REQ_DONE) s->stats.completed++;
  else if (state == MA_REQ_FAILED) s->stats.failed++;
  else if (state == MA_REQ_CANCELLED) s->stats.cancelled++;
}

void release_member(ma_server* s, Request& q) {
  if (q.member >= 0 && !s->dry) ma_batch_remove(s->batch, q.member);
  q.member = -1;
  s->used -= q.member_bytes;
  q.member_bytes = 0;
  s->running_cells -= q.cells;
  auto it = s->meshes.find(q.key);
  if (it != s->meshes.end()) it->second.users--;
}

// Queues a build of the request's mesh on the mesh thread unless it is
// cached or already being built, reserving its device bytes (an upper bound)
// in the budget; may_evict lets unused cached meshes go to make room.
// Returns whether the mesh is cached, building or now queued. Called with mu
// held.
bool start_mesh_build(ma_server* s, const Request& q, bool may_evict) {
  if (s->meshes.count(q.key) || s->building.count(q.key)) return true;
  const size_t need = dry_mesh_bytes(s, q.req);
  if (may_evict ? !make_room(s, need) : s->used + need > s->budget) return false;
  s->used += need;
  s->building[q.key] = std::make_pair(options_of(s, q.req), need);
  s->mesh_jobs.push_back(q.key);
  s->mesh_cv.notify_one();
  return true;
}

void mesher_loop(ma_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->mesh_cv.wait(lk, [&]() { return s->stop || !s->mesh_jobs.empty(); });
    if (s->stop) return;
    const MeshKey key = s->mesh_jobs.front();
    s->mesh_jobs.pop_front();
    const ma_options o = s->building[key].first;
    lk.unlock();
    CachedMesh cm;
    ma_status st;
    std::string msg;
    {
      miniaero::TraceRange trace("ma_server_mesh_build");
      st = ma_host_mesh_build_ex(&o, MA_HOST_MESH_DEVICE_GEOMETRY, &cm.host);
      if (st == MA_OK) {
        ma_mesh_view v;
        ma_host_mesh_view(cm.host, &v);
        st = ma_mesh_upload_ex(&v, s->physics.gather == MA_GATHER_CELL_FLUX ? MA_MESH_CELL_FLUX : 0, &cm.dev);
        if (st != MA_OK) {
          msg = ma_last_error();
          ma_host_mesh_free(cm.host);
        }
      } else {
        msg = ma_last_error();
      }
    }
    lk.lock();
    s->used -= s->building[key].second;
    s->building.erase(key);
    if (st == MA_OK) {
      cm.bytes = ma_mesh_device_bytes(cm.dev);
      cm.last_used = ns_since(s->t0);
      s->used += cm.bytes;
      s->meshes.emplace(key, cm);
    } else {
      s->failed_meshes[key] = std::make_pair(st, msg);
    }
    s->cv.notify_all();
  }
}

// Admits queued requests in order while they fit. Called with mu held.
void admit(ma_server* s) {
  while (!s->queue.empty()) {
    Request& q = s->reqs[s->queue.front()];
    if (q.state != MA_REQ_QUEUED) {
      s->queue.pop_front();
      continue;
    }
    if (s->stats.running >= s->stats.capacity) return;
    {
      int64_t C, F;
      box_counts(q.req, C, F);
      // Concurrency cap: enough running cells keep the GPU busy; admitting
      // more only stretches every running request's latency.
      if (s->max_running_cells > 0 && s->running_cells > 0 && s->running_cells + C > s->max_running_cells) return;
    }
    const bool cached = s->meshes.count(q.key) != 0;
    if (!cached && s->async_meshes) {
      auto failed = s->failed_meshes.find(q.key);
      if (failed != s->failed_meshes.end()) {
        q.error = failed->second.first;
        q.message = failed->second.second;
        s->failed_meshes.erase(failed);
        s->queue.pop_front();
        finish(s, q, MA_REQ_FAILED);
        continue;
      }
      // The head of the queue waits for its mesh (the mesh thread builds it);
      // the running requests keep stepping meanwhile.
      start_mesh_build(s, q, true);
      return;
    }
    const size_t mesh_need = cached ? 0 : dry_mesh_bytes(s, q.req);
    size_t member_need = dry_member_bytes(s, q.req);
    if (!make_room(s, mesh_need + member_need)) return;  // wait for memory
    CachedMesh* cm = nullptr;
    ma_status st = ensure_mesh(s, q, &cm);
    if (st != MA_OK) {
      q.error = st;
      q.message = ma_last_error();
      s->queue.pop_front();
      finish(s, q, MA_REQ_FAILED);
      continue;
    }
    cm->users++;
    cm->last_used = ns_since(s->t0);
    if (!s->dry) {
      member_need = ma_batch_member_bytes(s->batch, cm->dev);
      const ma_options o = options_of(s, q.req);
      int64_t C, F;
      box_counts(q.req, C, F);
      std::vector<double> U(5 * static_cast<size_t>(C));
      st = ma_host_initial_state(cm->host, &o, U.data());
      int32_t mid = -1;
      if (st == MA_OK) {
        // The batch's own budget is the server's; the server checked it.
        st = ma_batch_add(s->batch, cm->dev, U.data(), MA_LAYOUT_AOS, q.req.dt, q.req.inflow_state, &mid);
      }
      if (st != MA_OK) {
        cm->users--;
        if (st == MA_EBUDGET || st == MA_ENOMEM) return;  // retry after something finishes
        q.error = st;
        q.message = ma_last_error();
        s->queue.pop_front();
        finish(s, q, MA_REQ_FAILED);
        continue;
      }
      q.member = mid;
    }
    q.member_bytes = member_need;
    s->used += member_need;
    q.state = MA_REQ_RUNNING;
    q.t_admit = ns_since(s->t0);
    int64_t C, F;
    box_counts(q.req, C, F);
    q.cells = C;
    s->running_cells += C;
    s->queue.pop_front();
    s->stats.running++;
    s->stats.admitted++;
    s->stats.peak_running = std::max(s->stats.peak_running, s->stats.running);
    s->stats.peak_bytes = std::max<int64_t>(s->stats.peak_bytes, static_cast<int64_t>(s->used));
  }
}

// One scheduling iteration. Called with mu held; releases it around GPU work.
ma_status poll_locked(ma_server* s, std::unique_lock<std::mutex>& lk, int32_t* progressed) {
  admit(s);
  std::vector<int64_t> running;
  int64_t min_left = -1;
  for (auto& kv : s->reqs)
    if (kv.second.state == MA_REQ_RUNNING) {
      running.push_back(kv.first);
      const int64_t left = kv.second.req.nsteps - kv.second.steps_done;
      if (min_left < 0 || left < min_left) min_left = left;
    }
  s->stats.queued = static_cast<int32_t>(s->queue.size());
  if (running.empty()) {
    if (progressed) *progressed = 0;
    if (s->busy_start >= 0) {
      s->stats.busy_seconds += (ns_since(s->t0) - s->busy_start) * 1e-9;
      s->busy_start = -1;
    }
    return MA_OK;
  }
  if (s->busy_start < 0) s->busy_start = ns_since(s->t0);
  const int32_t n = static_cast<int32_t>(std::min<int64_t>(s->tick_steps, std::max<int64_t>(min_left, 0)));
  int64_t cell_stages = 0;
  for (int64_t id : running) cell_stages += s->reqs[id].cells * 4 * n;
  ma_status st = MA_OK;
  if (!s->dry && n > 0) {
    lk.unlock();
    miniaero::TraceRange trace("ma_server_tick");
    st = ma_batch_step(s->batch, n);
    if (st == MA_OK) st = ma_batch_synchronize(s->batch);
    lk.lock();
  } else if (s->dry) {
    // A dry-run tick stands for device work: 1 ms, with the lock released.
    lk.unlock();
    std::this_thread::sleep_for(std::chrono::milliseconds(1));
    lk.lock();
  }
  if (st != MA_OK) return st;
  s->stats.ticks++;
  s->stats.cell_stages += cell_stages;
  for (int64_t id : running) {
    Request& q = s->reqs[id];
    if (q.state != MA_REQ_RUNNING) continue;  // cancelled meanwhile
    q.steps_done += n;
    if (q.steps_done >= q.req.nsteps) {
      if (!s->dry) {
        std::vector<double> U(5 * static_cast<size_t>(q.cells));
        ma_status gs = ma_batch_get_state(s->batch, q.member, U.data(), MA_LAYOUT_AOS);
        if (gs != MA_OK) {
          q.error = gs;
          q.message = ma_last_error();
        }
        for (int k = 0; k < 5; ++k) {
          double acc = 0.0;
          for (int64_t c = 0; c < q.cells; ++c) acc += U[5 * c + k] * U[5 * c + k];
          q.result_norm[k] = acc;
        }
        if (q.req.keep_result) q.result.swap(U);
      }
      release_member(s, q);
      s->stats.running--;
      finish(s, q, q.error == MA_OK ? MA_REQ_DONE : MA_REQ_FAILED);
    }
  }
  if (progressed) *progressed = 1;
  s->cv.notify_all();
  return MA_OK;
}

void worker_loop(ma_server* s) {
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    int32_t progressed = 0;
    ma_status st = poll_locked(s, lk, &progressed);
    if (st != MA_OK) {
      // A device failure fails every running request; the loop keeps serving.
      for (auto& kv : s->reqs)
        if (kv.second.state == MA_REQ_RUNNING) {
          kv.second.error = st;
          kv.second.message = ma_last_error();
          release_member(s, kv.second);
          s->stats.running--;
          finish(s, kv.second, MA_REQ_FAILED);
        }
      s->cv.notify_all();
    }
    if (!progressed) s->cv.wait_for(lk, std::chrono::milliseconds(50));
  }
}

}  // namespace

extern "C" ma_status ma_server_create(const ma_options* physics, size_t budget_bytes, int32_t tick_steps,
                                      int32_t capacity, int32_t flags, ma_server** out) {
  if (!physics || !out || tick_steps <= 0 || capacity <= 0 || budget_bytes == 0)
    return set_error(MA_EINVAL, "ma_server_create: bad arguments");
  *out = nullptr;
  ma_server* s = new (std::nothrow) ma_server;
  if (!s) return set_error(MA_ENOMEM, "ma_server_create: out of host memory");
  s->physics = *physics;
  s->budget = budget_bytes;
  s->tick_steps = tick_steps;
  s->flags = flags;
  s->dry = (flags & MA_SERVER_DRYRUN) != 0;
  std::memset(&s->stats, 0, sizeof(s->stats));
  s->stats.capacity = capacity;
  if (!s->dry) {
    ma_status st = ma_batch_create(physics, capacity, budget_bytes, &s->batch);
    if (st != MA_OK) {
      delete s;
      return st;
    }
  }
  if (flags & MA_SERVER_THREAD) {
    if (!s->dry) {
      cudaGetDevice(&s->device);
      s->async_meshes = true;
      s->mesher = std::thread(mesher_loop, s);
    }
    s->worker = std::thread(worker_loop, s);
  }
  *out = s;
  return MA_OK;
}

extern "C" void ma_server_free(ma_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  s->mesh_cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->mesher.joinable()) s->mesher.join();
  if (s->batch) ma_batch_free(s->batch);
  for (auto& kv : s->meshes) {
    if (kv.second.dev) ma_mesh_free(kv.second.dev);
    if (kv.second.host) ma_host_mesh_free(kv.second.host);
  }
  delete s;
}

extern "C" ma_status ma_server_set_max_running_cells(ma_server* s, int64_t cells) {
  if (!s || cells < 0) return set_error(MA_EINVAL, "ma_server_set_max_running_cells: bad arguments");
  std::lock_guard<std::mutex> g(s->mu);
  s->max_running_cells = cells;
  s->cv.notify_all();
  return MA_OK;
}

extern "C" ma_status ma_server_set_launch(ma_server* s, const int32_t* block, const int32_t* grid) {
  if (!s || !block || !grid) return set_error(MA_EINVAL, "ma_server_set_launch: null argument");
  std::lock_guard<std::mutex> g(s->mu);
  // The batch steps with the lock released: its launch shapes change only
  // while no request is queued or running.
  if (!s->queue.empty()) return set_error(MA_ESTATE, "ma_server_set_launch: requests are queued");
  for (auto& kv : s->reqs)
    if (kv.second.state == MA_REQ_RUNNING) return set_error(MA_ESTATE, "ma_server_set_launch: requests are running");
  if (s->dry) {
    for (int k = 0; k < 4; ++k)
      if (block[k] < 32 || block[k] > 256 || block[k] % 32 || grid[k] < 1 || grid[k] > 65535)
        return set_error(MA_EINVAL, "ma_server_set_launch: block must be 32..256 in steps of 32, grid 1..65535");
    return MA_OK;
  }
  return ma_batch_set_launch(s->batch, block, grid);
}

extern "C" ma_status ma_server_submit(ma_server* s, const ma_request* r, int64_t* id) {
  if (!s || !r || !id) return set_error(MA_EINVAL, "ma_server_submit: null argument");
  if (r->nx < 1 || r->ny < 1 || r->nz < 1 || r->nsteps < 0)
    return set_error(MA_EINVAL, "ma_server_submit: bad mesh size or step count");
  if (!(r->dt > 0.0) && !(s->physics.cfl > 0.0))
    return set_error(MA_EINVAL, "ma_server_submit: dt must be > 0 without cfl");
  std::lock_guard<std::mutex> g(s->mu);
  Request q;
  q.id = s->next_id++;
  q.req = *r;
  q.key = key_of(*r);
  q.t_submit = ns_since(s->t0);
  // A request that can never run is rejected now: a mesh beyond the device
  // arrays' 32-bit indexing (before any host mesh is built for it), or one
  // that cannot fit even in an empty server.
  int64_t cells, faces;
  box_counts(*r, cells, faces);
  const bool too_many = cells > MA_MAX_MESH_CELLS;
  if (too_many || dry_member_bytes(s, *r) + dry_mesh_bytes(s, *r) > s->budget) {
    q.state = MA_REQ_FAILED;
    q.error = too_many ? MA_EINVAL : MA_EBUDGET;
    q.message = too_many ? "request has more cells than MA_MAX_MESH_CELLS" : "request larger than the device-memory budget";
    q.t_finish = q.t_submit;
    s->stats.failed++;
  } else {
    s->queue.push_back(q.id);
    // Start building an uncached mesh now, while the request waits its turn
    // (only into free budget: evicting is left to admission).
    if (s->async_meshes) start_mesh_build(s, q, false);
  }
  s->stats.submitted++;
  *id = q.id;
  s->reqs[q.id] = std::move(q);
  s->cv.notify_all();
  return MA_OK;
}

extern "C" ma_status ma_server_preload_mesh(ma_server* s, const ma_request* r) {
  if (!s || !r) return set_error(MA_EINVAL, "ma_server_preload_mesh: null argument");
  std::lock_guard<std::mutex> g(s->mu);
  Request q;
  q.req = *r;
  q.key = key_of(*r);
  CachedMesh* cm = nullptr;
  const size_t need = s->meshes.count(q.key) ? 0 : dry_mesh_bytes(s, *r);
  if (need && !make_room(s, need)) return set_error(MA_EBUDGET, "mesh does not fit the budget");
  ma_status st = ensure_mesh(s, q, &cm);
  if (st == MA_OK) cm->last_used = ns_since(s->t0);
  return st;
}

extern "C" ma_status ma_server_poll(ma_server* s, int32_t* progressed) {
  if (!s) return set_error(MA_EINVAL, "ma_server_poll: null server");
  if (s->flags & MA_SERVER_THREAD) return set_error(MA_ESTATE, "ma_server_poll: the server runs its own thread");
  std::unique_lock<std::mutex> lk(s->mu);
  return poll_locked(s, lk, progressed);
}

extern "C" ma_status ma_server_cancel(ma_server* s, int64_t id) {
  if (!s) return set_error(MA_EINVAL, "ma_server_cancel: null server");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return set_error(MA_ENOTFOUND, "ma_server_cancel: unknown request");
  Request& q = it->second;
  if (q.state == MA_REQ_QUEUED) {
    finish(s, q, MA_REQ_CANCELLED);
  } else if (q.state == MA_REQ_RUNNING) {
    release_member(s, q);
    s->stats.running--;
    finish(s, q, MA_REQ_CANCELLED);
  } else {
    return set_error(MA_ESTATE, "ma_server_cancel: request already finished");
  }
  s->cv.notify_all();
  return MA_OK;
}

extern "C" ma_status ma_server_query(ma_server* s, int64_t id, ma_request_info* info) {
  if (!s || !info) return set_error(MA_EINVAL, "ma_server_query: null argument");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return set_error(MA_ENOTFOUND, "ma_server_query: unknown request");
  const Request& q = it->second;
  info->state = q.state;
  info->error = q.error;
  info->steps_done = q.steps_done;
  info->cells = q.cells;
  info->t_submit_ns = q.t_submit;
  info->t_admit_ns = q.t_admit;
  info->t_finish_ns = q.t_finish;
  for (int k = 0; k < 5; ++k) info->state_sq_norm[k] = q.result_norm[k];
  return MA_OK;
}

extern "C" ma_status ma_server_result(ma_server* s, int64_t id, double* U) {
  if (!s || !U) return set_error(MA_EINVAL, "ma_server_result: null argument");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return set_error(MA_ENOTFOUND, "ma_server_result: unknown request");
  const Request& q = it->second;
  if (q.state != MA_REQ_DONE) return set_error(MA_ESTATE, "ma_server_result: request not done");
  if (q.result.empty()) return set_error(MA_ESTATE, "ma_server_result: request did not keep its result");
  std::memcpy(U, q.result.data(), q.result.size() * sizeof(double));
  return MA_OK;
}

extern "C" ma_status ma_server_wait(ma_server* s, int64_t id, double timeout_s) {
  if (!s) return set_error(MA_EINVAL, "ma_server_wait: null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto done = [&]() {
    auto it = s->reqs.find(id);
    return it == s->reqs.end() || (it->second.state != MA_REQ_QUEUED && it->second.state != MA_REQ_RUNNING);
  };
  if (!(s->flags & MA_SERVER_THREAD)) {
    // Manual mode: drive the loop from the waiting thread.
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s);
    while (!done()) {
      if (Clock::now() > deadline) return set_error(MA_ETIMEDOUT, "ma_server_wait: timed out");
      int32_t progressed = 0;
      ma_status st = poll_locked(s, lk, &progressed);
      if (st != MA_OK) return st;
      if (!progressed && !done()) return set_error(MA_ESTATE, "ma_server_wait: request cannot make progress");
    }
  } else if (!s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return set_error(MA_ETIMEDOUT, "ma_server_wait: timed out");
  }
  if (s->reqs.find(id) == s->reqs.end()) return set_error(MA_ENOTFOUND, "ma_server_wait: unknown request");
  return MA_OK;
}

extern "C" ma_status ma_server_get_stats(ma_server* s, ma_server_stats* out) {
  if (!s || !out) return set_error(MA_EINVAL, "ma_server_get_stats: null argument");
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->stats;
  out->bytes_in_use = static_cast<int64_t>(s->used);
  out->cached_meshes = static_cast<int32_t>(s->meshes.size());
  out->queued = 0;
  for (int64_t id : s->queue)
    if (s->reqs[id].state == MA_REQ_QUEUED) out->queued++;
  if (s->busy_start >= 0) out->busy_seconds += (ns_since(s->t0) - s->busy_start) * 1e-9;
  return MA_OK;
}
