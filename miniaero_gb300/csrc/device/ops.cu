// Operator-level kernels (unit parity of the device physics against the
// oracle) and the state check. FP64, compiled with --fmad=false.
#include <cstdint>

#include "kernels.cuh"

namespace miniaero {
namespace dev {

namespace {

__global__ void k_check_state(int C, const double* __restrict__ Un, unsigned long long* first_bad) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 5; ++k) bad |= !isfinite(Un[k * C + c]);
  bad |= !(Un[c] > 0.0) || !(Un[4 * C + c] > 0.0);
  if (bad) atomicMin(first_bad, static_cast<unsigned long long>(c));
}

// ---- operator-level kernels ----
__global__ void k_op_roe(int n, const double* pl, const double* pr, const double* nrm, const double* tan_,
                         const double* bin, double* flux) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  FaceFrame<double> fr;
  const double* a = nrm + 3 * i;
  const double* tt = tan_ + 3 * i;
  const double* b = bin + 3 * i;
  const double nn = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double tn = sqrt(tt[0] * tt[0] + tt[1] * tt[1] + tt[2] * tt[2]);
  const double bn = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  for (int d = 0; d < 3; ++d) {
    fr.n[d] = a[d];
    fr.nu[d] = a[d] / nn;
    fr.tu[d] = tt[d] / tn;
    fr.bu[d] = b[d] / bn;
  }
  fr.nn = nn;
  roe_flux<double>(pl + 5 * i, pr + 5 * i, fr, flux + 5 * i);
}

__global__ void k_op_viscous(int n, const double* grad, const double* prim, const double* area, Transport tr,
                             double* vflux) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double g[5][3];
  for (int k = 0; k < 5; ++k)
    for (int d = 0; d < 3; ++d) g[k][d] = grad[15 * i + 3 * k + d];
  viscous_flux<double>(g, prim + 5 * i, area + 3 * i, tr, vflux + 5 * i);
}

__global__ void k_op_limiter(int n, int kind, const double* dumax, const double* dumin, const double* du,
                             const double* d2, double* phi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  phi[i] = kind == 1 ? vanalbada<double>(dumax[i], dumin[i], du[i]) : venkat<double>(dumax[i], dumin[i], du[i], d2[i]);
}

__global__ void k_op_primitives(int n, const double* U, double* V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  primitives(U + 5 * i, V + 5 * i);
}

inline unsigned blocks_for(int n, int bs) { return static_cast<unsigned>((n + bs - 1) / bs); }

}  // namespace

int launches_per_stage(const PathConfig& cfg, const TopoView& t) {
  int n = 1;  // residual
  if (cfg.second_order || cfg.viscous) ++n;
  if (t.Fi > 0) ++n;
  if (t.Fb > 0) ++n;
  return n;
}

cudaError_t launch_op_roe(int n, const double* pl, const double* pr, const double* normal, const double* tangent,
                          const double* binormal, double* flux, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_roe<<<blocks_for(n, 128), 128, 0, stream>>>(n, pl, pr, normal, tangent, binormal, flux);
  return cudaGetLastError();
}

cudaError_t launch_op_viscous(int n, const double* grad, const double* prim, const double* area, Transport tr,
                              double* vflux, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_viscous<<<blocks_for(n, 128), 128, 0, stream>>>(n, grad, prim, area, tr, vflux);
  return cudaGetLastError();
}

cudaError_t launch_op_limiter(int n, int kind, const double* dumax, const double* dumin, const double* du,
                              const double* d2, double* phi, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_limiter<<<blocks_for(n, 256), 256, 0, stream>>>(n, kind, dumax, dumin, du, d2, phi);
  return cudaGetLastError();
}

cudaError_t launch_op_primitives(int n, const double* U, double* V, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_primitives<<<blocks_for(n, 256), 256, 0, stream>>>(n, U, V);
  return cudaGetLastError();
}

cudaError_t launch_check_state(int C, const double* Un, unsigned long long* first_bad, cudaStream_t stream) {
  if (C <= 0) return cudaSuccess;
  k_check_state<<<blocks_for(C, 256), 256, 0, stream>>>(C, Un, first_bad);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace miniaero
