// Allocation-free CFL time step (ma_cfl_dt_noalloc).
//
// Some callers cannot allocate device memory when they need a time step: a
// host code that hands all device memory to its own pool at start-up and
// allows no driver allocation afterwards, or a time loop that must not block
// on the allocator (cudaMalloc/cudaFree synchronise the device). The solver's
// own CFL path (ma_solver_set_state) reduces into a slot of the solver's
// cudaMalloc'd arena; this variant reduces in two passes through a fixed
// scratch array that lives in the library image: the caller passes a mesh
// and a device state and receives dt, nothing is allocated or freed.
//
// Scratch: kNoallocMaxBlocks partial minima plus one result slot, 8 bytes
// each (512 KiB + 8 B, held by every GPU that loads the library until the
// process exits). Meshes of up to kNoallocMaxBlocks * kCflBlock cells
// (16,777,216) are accepted; larger ones get MA_EINVAL. Pass 1 writes the
// partial of every block that pass 2 reads and pass 2 writes the result, so no
// scratch entry has to start at zero. Every call runs on the mesh's device
// (made current for the call, the caller's current device restored after) and
// d_state must live on that device. The first call on a device looks up the
// array's device address (cudaGetSymbolAddress, which may load the module on
// that device) and keeps it for the life of the process, so a cudaDeviceReset
// of that device (which unloads the module) invalidates the entry point on
// it. The call reads dt back with a stream synchronisation: it cannot be made
// on a stream that is being captured, and its first call on a device should
// come before any capture in global mode on other streams. All calls share
// the array: calls whose kernels overlap on the GPU (different streams, or
// different host threads, without ordering between them) race on it and may
// return each other's results.
#include <cmath>
#include <mutex>
#include <string>

#include "../../../include/miniaero_gpu.h"
#include "../host/errors.hpp"
#include "batch_internal.hpp"
#include "kernels.cuh"

using miniaero::set_error;
namespace dev = miniaero::dev;

namespace {

constexpr int kCflBlock = 256;
constexpr int kNoallocMaxBlocks = 65536;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_cfl_scratch[kNoallocMaxBlocks + 1];

// Per-device address of g_cfl_scratch, looked up once with that device current.
std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Pass 1: minimum over the block's cells of V_c / sum_f(|u.n| + c|n|), the
// quantity of the solver's CFL kernel, evaluated with the same expressions.
__global__ void __launch_bounds__(kCflBlock) k_cfl_block_min(dev::TopoView t, dev::GeomView<double> g,
                                                             const double* __restrict__ Un,
                                                             double* __restrict__ partial) {
  __shared__ double smin[kCflBlock];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double r = __longlong_as_double(0x7FF0000000000000LL);  // +inf
  if (c < t.C) {
    const int C = t.C, F = t.F;
    double U[5], V[5];
    for (int k = 0; k < 5; ++k) U[k] = Un[k * C + c];
    dev::primitives(U, V);
    const double a = sqrt(1.4 * 287.05 * V[4]);
    double sum = 0.0;
    for (int s = 0; s < dev::kMaxCellFaces; ++s) {
      const int code = t.csr_grad[s * C + c];
      if (code < 0) continue;
      const int f = code >> 1;
      const double un = V[1] * g.fn[f] + V[2] * g.fn[F + f] + V[3] * g.fn[2 * F + f];
      sum += fabs(un) + a * g.fnn[f];
    }
    const double q = t.vol[c] / sum;
    if (q > 0.0) r = q;
  }
  smin[threadIdx.x] = r;
  __syncthreads();
  for (int w = kCflBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = smin[0];
}

// Pass 2: one block reduces the partials into partial[kNoallocMaxBlocks].
__global__ void __launch_bounds__(1024) k_cfl_final_min(double* __restrict__ partial, int nblocks) {
  __shared__ double smin[1024];
  double r = __longlong_as_double(0x7FF0000000000000LL);
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) r = fmin(r, partial[i]);
  smin[threadIdx.x] = r;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (threadIdx.x < w) smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[kNoallocMaxBlocks] = smin[0];
}

// Device address of the scratch array for the current device (set-up on the
// first call per device).
ma_status scratch_for_current_device(double** out) {
  int dev_id = 0;
  cudaError_t e = cudaGetDevice(&dev_id);
  if (e != cudaSuccess) return set_error(MA_ECUDA, std::string("ma_cfl_dt_noalloc: ") + cudaGetErrorString(e));
  if (dev_id < 0 || dev_id >= kMaxDevices) return set_error(MA_EINVAL, "ma_cfl_dt_noalloc: device index out of range");
  std::lock_guard<std::mutex> g(g_scratch_mu);
  if (!g_scratch_ptr[dev_id]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_cfl_scratch);
    if (e != cudaSuccess || !p)
      return set_error(MA_ECUDA, std::string("ma_cfl_dt_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_ptr[dev_id] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev_id];
  return MA_OK;
}

// Makes a device current for one call and restores the caller's afterwards.
class DeviceScope {
 public:
  explicit DeviceScope(int device) {
    ok_ = cudaGetDevice(&previous_) == cudaSuccess;
    if (ok_ && previous_ != device) {
      ok_ = cudaSetDevice(device) == cudaSuccess;
      switched_ = ok_;
    }
  }
  ~DeviceScope() {
    if (switched_) cudaSetDevice(previous_);
  }
  bool ok() const { return ok_; }

 private:
  int previous_ = 0;
  bool ok_ = false;
  bool switched_ = false;
};

}  // namespace

extern "C" ma_status ma_cfl_dt_noalloc(const ma_mesh* mesh, const double* d_state, double cfl, double* dt_out,
                                       void* stream) {
  if (!mesh || !d_state || !dt_out) return set_error(MA_EINVAL, "ma_cfl_dt_noalloc: null argument");
  if (!(cfl > 0.0)) return set_error(MA_EINVAL, "ma_cfl_dt_noalloc: cfl must be > 0");
  const dev::TopoView t = miniaero::mesh_topo(mesh);
  const long long max_cells = static_cast<long long>(kNoallocMaxBlocks) * kCflBlock;
  if (t.C <= 0) return set_error(MA_EINVAL, "ma_cfl_dt_noalloc: mesh has no cells");
  if (t.C > max_cells)
    return set_error(MA_EINVAL, "ma_cfl_dt_noalloc: mesh has " + std::to_string(t.C) +
                                    " cells; the allocation-free path accepts at most " + std::to_string(max_cells));
  DeviceScope device(miniaero::mesh_device(mesh));
  if (!device.ok()) return set_error(MA_ECUDA, "ma_cfl_dt_noalloc: cannot make the mesh's device current");
  double* scratch = nullptr;
  ma_status st = scratch_for_current_device(&scratch);
  if (st != MA_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblocks = (t.C + kCflBlock - 1) / kCflBlock;
  k_cfl_block_min<<<nblocks, kCflBlock, 0, s>>>(t, miniaero::mesh_geom<double>(mesh), d_state, scratch);
  k_cfl_final_min<<<1, 1024, 0, s>>>(scratch, nblocks);
  cudaError_t e = cudaGetLastError();
  double r = 0.0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&r, scratch + kNoallocMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(MA_ECUDA, std::string("ma_cfl_dt_noalloc: ") + cudaGetErrorString(e));
  if (!(r > 0.0) || !std::isfinite(r))
    return set_error(MA_ENUMERIC, "ma_cfl_dt_noalloc: CFL time step is not finite");
  *dt_out = cfl * r;
  return MA_OK;
}
