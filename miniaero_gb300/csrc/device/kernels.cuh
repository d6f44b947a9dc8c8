// Kernel interface of the RK4 residual path (device views and launchers).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "physics.cuh"

namespace miniaero {
namespace dev {

constexpr int kMaxCellFaces = 6;  // Hexa8: every face is internal or boundary
constexpr int kFaceTileCells = 4096;  // internal-face order: tiles of this many left cells

// Topology shared by both precisions. Face arrays are in device order:
// internal faces [0, Fi) by tile of left cells, class, then (left, right)
// cell, then boundary faces [Fi, F) grouped by BC type (Extrapolate,
// Tangent, NoSlip, Inflow).
struct TopoView {
  int32_t C = 0, Fi = 0, Fb = 0, F = 0;
  int32_t nbc_type[4] = {0, 0, 0, 0};  // BC face counts in type order E, T, N, I
  // Class of each internal face: 0..2 frame aligned with axis D = class and
  // both face-to-cell offsets nonzero only along D; 3..5 frame aligned with
  // axis D = class - 3, general offsets; 6 general. Faces are ordered by
  // tiles of kFaceTileCells left cells, then class, so warps see one class.
  const uint8_t* fclass = nullptr;     // [Fi]
  const double* vol = nullptr;         // [C]
  const double* vinv = nullptr;        // [C] 1/V rounded to nearest
  const int32_t* fconn = nullptr;      // [2][F] (left, right); right = -1 on a boundary
  // Per-cell contribution lists, slot-major [kMaxCellFaces][C], code =
  // (face << 1) | (cell is the face's left cell), -1 for an unused slot.
  const int32_t* csr_grad = nullptr;   // Green-Gauss / min-max / limiter order
  const int32_t* csr_nbr = nullptr;    // neighbour cell of each csr_grad slot (the cell itself on a boundary face)
  const int32_t* csr_flux = nullptr;   // residual order
  // Bit 0: the cell is axis-aligned and its csr_grad list is grouped by axis
  // (two faces each for x, y, z): gradient terms along other axes are zero.
  // Bit 1 (with bit 0): the offset from the cell centre to each face centre
  // is nonzero only along that face's axis.
  const uint8_t* axis_cell = nullptr;
};

// Geometry in the arithmetic type R of the flux/gradient/limiter work.
template <class R>
struct GeomView {
  const R* vol = nullptr;  // [C]
  const R* vinv = nullptr; // [C] 1/V rounded to nearest
  const R* fn = nullptr;   // [3][F] area vector
  const R* fnu = nullptr;  // [3][F] unit normal
  const R* ftu = nullptr;  // [3][F] unit tangent
  const R* fbu = nullptr;  // [3][F] unit binormal
  const R* fnn = nullptr;  // [F] |n|
  const R* dL = nullptr;   // [3][F] face centroid - left cell centroid
  const R* dR = nullptr;   // [3][F] face centroid - right cell centroid (internal faces)
};

// Per-stage work arrays in type R (SoA, component-major).
template <class R>
struct StageBuffers {
  R* W = nullptr;      // [5][C] primitives of the stage state
  R* grad = nullptr;   // [15][C] Green-Gauss gradients, (component, direction)
  R* phi = nullptr;    // [5][C] limiter
  R* fflux = nullptr;  // [F][5] face flux (internal) or cell contribution (boundary)
};

struct StateBuffers {
  double* Un = nullptr;    // [5][C]
  double* Unp1 = nullptr;  // [5][C]
  double* res = nullptr;   // [5][C] optional
};

// Conserved inflow state passed by value to the boundary kernels.
struct InflowState {
  double u[5];
};

// One mesh instance of a batch: its mesh views, work arrays, state, time step
// and inflow state.
template <class R>
struct Segment {
  TopoView t;
  GeomView<R> g;
  StageBuffers<R> b;
  StateBuffers s;
  double dt;
  InflowState inflow;
};

struct PathConfig {
  bool second_order = false;
  bool viscous = false;
  bool cell_flux = false;  // -DCELL_FLUX residual reduction (lists in slot order)
  int limiter = 0;  // 0 Venkatakrishnan, 1 Van Albada
  Transport transport{0, 0.0, 0.0, 0.0};
  double inflow[5] = {0, 0, 0, 0, 0};
  double dt = 0.0;
};

// Launch counts per RK stage for the given configuration.
int launches_per_stage(const PathConfig& cfg, const TopoView& t);

// Kernel selection bits for launch_stage (profiling launches one at a time).
enum KernelBits : unsigned {
  kSweep1 = 1u, kInternalFlux = 2u, kBcFlux = 4u, kResidual = 8u, kAllKernels = 15u
};

template <class R>
cudaError_t launch_init_primitives(const TopoView& t, const StateBuffers& s, const StageBuffers<R>& b,
                                   cudaStream_t stream);

template <class R>
cudaError_t launch_stage(const TopoView& t, const GeomView<R>& g, const PathConfig& cfg, const StateBuffers& s,
                         const StageBuffers<R>& b, int stage, cudaStream_t stream, unsigned kernels = kAllKernels);

// Defined in kernels_fp64.cu (plain form) and kernels_mixed.cu (mixed form).
template <>
cudaError_t launch_init_primitives<double>(const TopoView&, const StateBuffers&, const StageBuffers<double>&,
                                           cudaStream_t);
template <>
cudaError_t launch_init_primitives<float>(const TopoView&, const StateBuffers&, const StageBuffers<float>&,
                                          cudaStream_t);
template <>
cudaError_t launch_stage<double>(const TopoView&, const GeomView<double>&, const PathConfig&, const StateBuffers&,
                                 const StageBuffers<double>&, int, cudaStream_t, unsigned);
template <>
cudaError_t launch_stage<float>(const TopoView&, const GeomView<float>&, const PathConfig&, const StateBuffers&,
                                const StageBuffers<float>&, int, cudaStream_t, unsigned);

// The FP64 form built with multiply-add contraction (kernels_fp64_fma.cu,
// --fmad=true): the same kernels and summation orders as launch_stage<double>,
// with a*b+c rounded once where the compiler fuses it. Not the reference's
// bits; the opt-in MA_PREC_FP64_FMA precision.
cudaError_t launch_init_primitives_fma(const TopoView& t, const StateBuffers& s, const StageBuffers<double>& b,
                                       cudaStream_t stream);
cudaError_t launch_stage_fma(const TopoView& t, const GeomView<double>& g, const PathConfig& cfg,
                             const StateBuffers& s, const StageBuffers<double>& b, int stage, cudaStream_t stream,
                             unsigned kernels = kAllKernels);

// Batched stage over segments: chunks[k] lists (segment, first item) pairs of
// kernel kind k (sweep, internal flux, boundary flux, residual), each chunk
// covering block[k] items; nchunks is a device array of 4 counts.
struct BatchLaunch {
  const int2* chunks[4] = {nullptr, nullptr, nullptr, nullptr};
  const int* nchunks = nullptr;  // device [4]
  int block[4] = {128, 128, 128, 128};
  int grid[4] = {1, 1, 1, 1};
};

template <class R>
cudaError_t launch_batch_stage(const PathConfig& cfg, const Segment<R>* segs, const BatchLaunch& bl, int stage,
                               cudaStream_t stream, unsigned kernels = kAllKernels);
template <>
cudaError_t launch_batch_stage<double>(const PathConfig&, const Segment<double>*, const BatchLaunch&, int,
                                       cudaStream_t, unsigned);
template <>
cudaError_t launch_batch_stage<float>(const PathConfig&, const Segment<float>*, const BatchLaunch&, int,
                                      cudaStream_t, unsigned);
cudaError_t launch_batch_stage_fma(const PathConfig& cfg, const Segment<double>* segs, const BatchLaunch& bl,
                                   int stage, cudaStream_t stream, unsigned kernels = kAllKernels);

// Whole batch steps as one cooperative launch (kb_steps): nsteps RK4 steps of
// every member, the phases of each stage separated by a bounded grid barrier.
// The chunk tables must use one chunk size, `block` (the launch's block
// size); grid must not exceed the resident blocks (batch_steps_occupancy
// times the SM count). barrier_words: two zeroed device words; *err is set
// when a barrier wait gave up. One function per precision (the translation
// unit that builds it).
cudaError_t launch_batch_steps_fp64(const PathConfig& cfg, const void* segs, const BatchLaunch& bl, int nsteps,
                                    unsigned* barrier_words, int* err, int block, int grid, cudaStream_t stream);
cudaError_t launch_batch_steps_mixed(const PathConfig& cfg, const void* segs, const BatchLaunch& bl, int nsteps,
                                     unsigned* barrier_words, int* err, int block, int grid, cudaStream_t stream);
cudaError_t launch_batch_steps_fp64_fma(const PathConfig& cfg, const void* segs, const BatchLaunch& bl, int nsteps,
                                        unsigned* barrier_words, int* err, int block, int grid, cudaStream_t stream);
cudaError_t batch_steps_occupancy_fp64(const PathConfig& cfg, int block, int* blocks_per_sm);
// The grid barrier's failure path: a 2-block cooperative launch in which one
// block never reaches the barrier; out[0] = passed (0), out[1] = error word (1).
cudaError_t launch_debug_barrier_timeout(unsigned* words, int* err, unsigned long long timeout_ns, int* out,
                                        cudaStream_t stream);
cudaError_t batch_steps_occupancy_mixed(const PathConfig& cfg, int block, int* blocks_per_sm);
cudaError_t batch_steps_occupancy_fp64_fma(const PathConfig& cfg, int block, int* blocks_per_sm);

// dt bound of the CFL rule: writes min_c V_c / sum_f(|u.n| + c|n|) (as the
// bits of a positive double) into *out via atomicMin; *out must start at ~0.
cudaError_t launch_cfl(const TopoView& t, const GeomView<double>& g, const double* Un, unsigned long long* out,
                       cudaStream_t stream);

// Operator-level kernels (unit parity, FP64).
cudaError_t launch_op_roe(int n, const double* pl, const double* pr, const double* normal, const double* tangent,
                          const double* binormal, double* flux, cudaStream_t stream);
cudaError_t launch_op_viscous(int n, const double* grad, const double* prim, const double* area, Transport tr,
                              double* vflux, cudaStream_t stream);
cudaError_t launch_op_limiter(int n, int kind, const double* dumax, const double* dumin, const double* du,
                              const double* d2, double* phi, cudaStream_t stream);
cudaError_t launch_op_primitives(int n, const double* U, double* V, cudaStream_t stream);

// div_by_recip against IEEE division on n generated operand pairs.
cudaError_t launch_check_division(int mode, unsigned long long n, unsigned long long seed,
                                  unsigned long long* mismatches, double* example, cudaStream_t stream);

// Each cell's boundary-face contributions (fflux slots Fi..F-1) summed in the
// cell's residual list order from +0: out [5][C].
cudaError_t launch_bc_gather(const TopoView& t, const double* fflux, double* out, cudaStream_t stream);
// W = ComputePrimitives(U) on [5][C] arrays, U taken as given.
cudaError_t launch_field_primitives(int C, const double* U, double* W, cudaStream_t stream);
// apply_cell_flux and update on host-layout arrays (n cells / n values).
cudaError_t launch_op_apply_cell_flux(int n, double dt, const double* vol, const double* flux, double* res,
                                      cudaStream_t stream);
cudaError_t launch_op_rk_update(long long n, double alpha, const double* res, const double* src, double* dst,
                                cudaStream_t stream);

// FP64 issue-rate kernel: blocks x 256 threads, 4 chains of iters operations
// each (op 0 add, 1 multiply, 2 fused multiply-add); out holds one double per thread.
cudaError_t launch_fp64_rate(int op, int blocks, int iters, double* out, cudaStream_t stream);

// State check: first cell with a non-finite value or non-positive rho / rhoE.
cudaError_t launch_check_state(int C, const double* Un, unsigned long long* first_bad, cudaStream_t stream);

}  // namespace dev
}  // namespace miniaero
