// Mesh geometry on the device: face centroids, area vectors and Roe frames
// (kokkos/Face.C:37-98) and Hexa8 cell volumes and centroids
// (kokkos/ElementTopoHexa8.C:62-148, MeshProcessor.C:130-171), one thread per
// face or cell. The expressions and their order are those of the host
// generator (miniaero_gb300/csrc/host/mesh.cpp), compiled with --fmad=false;
// the device's double division and square root are correctly rounded like
// the host's, so every value is bit-identical to the host path. Face order,
// the shuffle and the BinSort stay on the host (their order is defined
// sequentially); this engine takes the per-item arithmetic, which on the
// host is the largest part of building a mesh after the face extraction.
#include <cuda_runtime.h>

#include <cmath>
#include <memory>
#include <string>

#include "../host/mesh.hpp"
#include "device_geometry.hpp"

namespace miniaero {
namespace {

constexpr int kGeomBlock = 256;

__device__ __forceinline__ void cross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - b[1] * a[2];
  c[1] = -a[0] * b[2] + b[0] * a[2];
  c[2] = a[0] * b[1] - b[0] * a[1];
}

__global__ void __launch_bounds__(kGeomBlock) k_face_geometry(int64_t n, const int32_t* __restrict__ nodes4,
                                                              const double* __restrict__ xyz,
                                                              double* __restrict__ coords, double* __restrict__ a_out,
                                                              double* __restrict__ t_out, double* __restrict__ b_out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double nd[4][3];
  for (int q = 0; q < 4; ++q) {
    const int64_t node = nodes4[4 * i + q];
    for (int j = 0; j < 3; ++j) nd[q][j] = xyz[node * 3 + j];
  }
  double c[3] = {0.0, 0.0, 0.0};
  for (int q = 0; q < 4; ++q)
    for (int j = 0; j < 3; ++j) c[j] += nd[q][j];
  const double scale = 1.0 / 4;
  for (int j = 0; j < 3; ++j) c[j] *= scale;
  const double v1[3] = {nd[1][0] - nd[0][0], nd[1][1] - nd[0][1], nd[1][2] - nd[0][2]};
  const double v2[3] = {nd[2][0] - nd[0][0], nd[2][1] - nd[0][1], nd[2][2] - nd[0][2]};
  const double v3[3] = {nd[3][0] - nd[0][0], nd[3][1] - nd[0][1], nd[3][2] - nd[0][2]};
  double c1[3], c2[3], a[3], t[3], b[3];
  cross3(v1, v2, c1);
  cross3(v2, v3, c2);
  for (int j = 0; j < 3; ++j) a[j] = 0.5 * (c1[j] + c2[j]);
  const double aa[3] = {fabs(a[0]), fabs(a[1]), fabs(a[2])};
  int i1 = 0;
  if (aa[0] < aa[1]) i1 = 1;
  if (aa[i1] < aa[2]) i1 = 2;
  int i2 = i1 + 1, i3 = i1 + 2;
  i2 = (i2 > 2) ? i2 - 3 : i2;
  i3 = (i3 > 2) ? i3 - 3 : i3;
  const double denom = sqrt(a[i1] * a[i1] + a[i3] * a[i3]);
  t[i2] = 0.0;
  t[i1] = a[i3] / denom;
  t[i3] = -a[i1] / denom;
  cross3(a, t, b);
  for (int j = 0; j < 3; ++j) {
    coords[3 * i + j] = c[j];
    a_out[3 * i + j] = a[j];
    t_out[3 * i + j] = t[j];
    b_out[3 * i + j] = b[j];
  }
}

// 2x2x2 Gauss points with unit weights; the shape-function derivatives of
// ElementTopoHexa8 evaluated per point as the host generator writes them.
__global__ void __launch_bounds__(kGeomBlock) k_cell_geometry(int64_t ncells, const int32_t* __restrict__ conn8,
                                                              const double* __restrict__ xyz,
                                                              double* __restrict__ volume,
                                                              double* __restrict__ centroid, int* negative) {
  const int64_t ie = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (ie >= ncells) return;
  double ex[8], ey[8], ez[8];
  for (int j = 0; j < 8; ++j) {
    const int64_t node = conn8[8 * ie + j];
    ex[j] = xyz[node * 3];
    ey[j] = xyz[node * 3 + 1];
    ez[j] = xyz[node * 3 + 2];
  }
  const double g = 0.577350269189626;
  const double xi_[8] = {-g, g, g, -g, -g, g, g, -g};
  const double eta_[8] = {-g, -g, g, g, -g, -g, g, g};
  const double zeta_[8] = {-g, -g, -g, -g, g, g, g, g};
  double vol = 0.0;
  int neg = 0;
  for (int ig = 0; ig < 8; ++ig) {
    const double xi = xi_[ig], eta = eta_[ig], zeta = zeta_[ig];
    double dx[8], de[8], dz[8];
    dx[0] = -0.125 * (1.0 - eta) * (1.0 - zeta);
    dx[1] = 0.125 * (1.0 - eta) * (1.0 - zeta);
    dx[2] = 0.125 * (1.0 + eta) * (1.0 - zeta);
    dx[3] = -0.125 * (1.0 + eta) * (1.0 - zeta);
    dx[4] = -0.125 * (1.0 - eta) * (1.0 + zeta);
    dx[5] = 0.125 * (1.0 - eta) * (1.0 + zeta);
    dx[6] = 0.125 * (1.0 + eta) * (1.0 + zeta);
    dx[7] = -0.125 * (1.0 + eta) * (1.0 + zeta);
    de[0] = -0.125 * (1.0 - xi) * (1.0 - zeta);
    de[1] = -0.125 * (1.0 + xi) * (1.0 - zeta);
    de[2] = 0.125 * (1.0 + xi) * (1.0 - zeta);
    de[3] = 0.125 * (1.0 - xi) * (1.0 - zeta);
    de[4] = -0.125 * (1.0 - xi) * (1.0 + zeta);
    de[5] = -0.125 * (1.0 + xi) * (1.0 + zeta);
    de[6] = 0.125 * (1.0 + xi) * (1.0 + zeta);
    de[7] = 0.125 * (1.0 - xi) * (1.0 + zeta);
    dz[0] = -0.125 * (1.0 - xi) * (1.0 - eta);
    dz[1] = -0.125 * (1.0 + xi) * (1.0 - eta);
    dz[2] = -0.125 * (1.0 + xi) * (1.0 + eta);
    dz[3] = -0.125 * (1.0 - xi) * (1.0 + eta);
    dz[4] = 0.125 * (1.0 - xi) * (1.0 - eta);
    dz[5] = 0.125 * (1.0 + xi) * (1.0 - eta);
    dz[6] = 0.125 * (1.0 + xi) * (1.0 + eta);
    dz[7] = 0.125 * (1.0 - xi) * (1.0 + eta);
    double J[9];
    double r;
    r = 0; for (int k = 0; k < 8; ++k) r += dx[k] * ex[k]; J[0] = r;
    r = 0; for (int k = 0; k < 8; ++k) r += dx[k] * ey[k]; J[1] = r;
    r = 0; for (int k = 0; k < 8; ++k) r += dx[k] * ez[k]; J[2] = r;
    r = 0; for (int k = 0; k < 8; ++k) r += de[k] * ex[k]; J[3] = r;
    r = 0; for (int k = 0; k < 8; ++k) r += de[k] * ey[k]; J[4] = r;
    r = 0; for (int k = 0; k < 8; ++k) r += de[k] * ez[k]; J[5] = r;
    r = 0; for (int k = 0; k < 8; ++k) r += dz[k] * ex[k]; J[6] = r;
    r = 0; for (int k = 0; k < 8; ++k) r += dz[k] * ey[k]; J[7] = r;
    r = 0; for (int k = 0; k < 8; ++k) r += dz[k] * ez[k]; J[8] = r;
    const double detJ = J[0] * (J[4] * J[8] - J[5] * J[7]) +
                        J[1] * (J[5] * J[6] - J[3] * J[8]) +
                        J[2] * (J[3] * J[7] - J[4] * J[6]);
    if (detJ < 1.0e-300) ++neg;
    vol += detJ;
  }
  double sx = 0, sy = 0, sz = 0;
  for (int j = 0; j < 8; ++j) {
    sx += ex[j];
    sy += ey[j];
    sz += ez[j];
  }
  volume[ie] = vol;
  centroid[3 * ie] = sx / 8;
  centroid[3 * ie + 1] = sy / 8;
  centroid[3 * ie + 2] = sz / 8;
  if (neg) atomicAdd(negative, neg);
}

std::string cuda_msg(const char* what, cudaError_t e) { return std::string(what) + ": " + cudaGetErrorString(e); }

// Device buffers grown on demand and kept for the engine's lifetime; one
// stream; the caller's host arrays are copied in and out around each launch.
class DeviceGeometry final : public GeometryEngine {
 public:
  ~DeviceGeometry() override {
    if (stream_) cudaStreamSynchronize(stream_);
    cudaFree(xyz_);
    cudaFree(idx_);
    cudaFree(out_);
    cudaFree(neg_);
    if (stream_) cudaStreamDestroy(stream_);
  }

  std::string init() {
    cudaError_t e = cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_msg("cudaStreamCreate", e);
    e = cudaMalloc(reinterpret_cast<void**>(&neg_), sizeof(int));
    if (e != cudaSuccess) return cuda_msg("cudaMalloc", e);
    return std::string();
  }

  std::string set_nodes(const double* xyz, size_t nnodes) override {
    cudaFree(xyz_);
    xyz_ = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&xyz_), sizeof(double) * 3 * (nnodes ? nnodes : 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(xyz_, xyz, sizeof(double) * 3 * nnodes, cudaMemcpyHostToDevice, stream_);
    if (e != cudaSuccess) return cuda_msg("node upload", e);
    return std::string();
  }

  std::string faces(size_t n, const int32_t* nodes4, double* coords, double* normal, double* tangent,
                    double* binormal) override {
    std::string err = reserve(n * 4, n * 12);
    if (!err.empty()) return err;
    cudaError_t e = cudaMemcpyAsync(idx_, nodes4, sizeof(int32_t) * 4 * n, cudaMemcpyHostToDevice, stream_);
    const unsigned blocks = static_cast<unsigned>((n + kGeomBlock - 1) / kGeomBlock);
    if (e == cudaSuccess) {
      k_face_geometry<<<blocks, kGeomBlock, 0, stream_>>>(static_cast<int64_t>(n), idx_, xyz_, out_, out_ + 3 * n,
                                                          out_ + 6 * n, out_ + 9 * n);
      e = cudaGetLastError();
    }
    double* dst[4] = {coords, normal, tangent, binormal};
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
      e = cudaMemcpyAsync(dst[k], out_ + 3 * n * k, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, stream_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
    if (e != cudaSuccess) return cuda_msg("face geometry", e);
    return std::string();
  }

  std::string cells(size_t ncells, const int32_t* conn8, double* volume, double* centroid, int* negative) override {
    std::string err = reserve(ncells * 8, ncells * 4);
    if (!err.empty()) return err;
    cudaError_t e = cudaMemsetAsync(neg_, 0, sizeof(int), stream_);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(idx_, conn8, sizeof(int32_t) * 8 * ncells, cudaMemcpyHostToDevice, stream_);
    const unsigned blocks = static_cast<unsigned>((ncells + kGeomBlock - 1) / kGeomBlock);
    if (e == cudaSuccess && ncells > 0) {
      k_cell_geometry<<<blocks, kGeomBlock, 0, stream_>>>(static_cast<int64_t>(ncells), idx_, xyz_, out_,
                                                          out_ + ncells, neg_);
      e = cudaGetLastError();
    }
    int neg = 0;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(volume, out_, sizeof(double) * ncells, cudaMemcpyDeviceToHost, stream_);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(centroid, out_ + ncells, sizeof(double) * 3 * ncells, cudaMemcpyDeviceToHost, stream_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&neg, neg_, sizeof(int), cudaMemcpyDeviceToHost, stream_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
    if (e != cudaSuccess) return cuda_msg("cell geometry", e);
    *negative += neg;
    return std::string();
  }

 private:
  // Index buffer of at least nidx int32 and output buffer of at least nout doubles.
  std::string reserve(size_t nidx, size_t nout) {
    cudaError_t e = cudaSuccess;
    if (nidx > idx_cap_) {
      cudaStreamSynchronize(stream_);
      cudaFree(idx_);
      idx_ = nullptr;
      e = cudaMalloc(reinterpret_cast<void**>(&idx_), sizeof(int32_t) * nidx);
      idx_cap_ = e == cudaSuccess ? nidx : 0;
    }
    if (e == cudaSuccess && nout > out_cap_) {
      cudaStreamSynchronize(stream_);
      cudaFree(out_);
      out_ = nullptr;
      e = cudaMalloc(reinterpret_cast<void**>(&out_), sizeof(double) * nout);
      out_cap_ = e == cudaSuccess ? nout : 0;
    }
    if (e != cudaSuccess) return cuda_msg("cudaMalloc", e);
    return std::string();
  }

  cudaStream_t stream_ = nullptr;
  double* xyz_ = nullptr;
  int32_t* idx_ = nullptr;
  double* out_ = nullptr;
  int* neg_ = nullptr;
  size_t idx_cap_ = 0, out_cap_ = 0;
};

}  // namespace

std::unique_ptr<GeometryEngine> make_device_geometry(std::string* err) {
  std::unique_ptr<DeviceGeometry> g(new DeviceGeometry);
  const std::string e = g->init();
  if (!e.empty()) {
    if (err) *err = e;
    return nullptr;
  }
  return std::unique_ptr<GeometryEngine>(g.release());
}

}  // namespace miniaero
