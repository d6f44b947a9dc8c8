// FP64 form with multiply-add contraction (opt-in precision
// MA_PREC_FP64_FMA). Compiled with --fmad=true: the compiler fuses a*b+c into
// one DFMA wherever the expression allows, so a face or cell takes fewer FP64
// instructions and the fused ones issue at the DFMA rate. Same kernels, data
// layout and summation orders as the plain form; each fused operation rounds
// once instead of twice, so results differ from the reference's serial bits
// at round-off level, by as much as the flow amplifies it (within 1e-12 on
// the benchmark meshes after their configured steps).
#include "kernels_impl.cuh"

namespace miniaero {
namespace dev {

cudaError_t launch_init_primitives_fma(const TopoView& t, const StateBuffers& s, const StageBuffers<double>& b,
                                       cudaStream_t stream) {
  return launch_init_primitives_impl<double>(t, s, b, stream);
}

cudaError_t launch_stage_fma(const TopoView& t, const GeomView<double>& g, const PathConfig& cfg,
                             const StateBuffers& s, const StageBuffers<double>& b, int stage, cudaStream_t stream,
                             unsigned kernels) {
  return launch_stage_impl<double>(t, g, cfg, s, b, stage, stream, kernels);
}

cudaError_t launch_batch_stage_fma(const PathConfig& cfg, const Segment<double>* segs, const BatchLaunch& bl,
                                   int stage, cudaStream_t stream, unsigned kernels) {
  return launch_batch_stage_impl<double>(cfg, segs, bl, stage, stream, kernels);
}

cudaError_t launch_batch_steps_fp64_fma(const PathConfig& cfg, const void* segs, const BatchLaunch& bl, int nsteps,
                               unsigned* barrier_words, int* err, int block, int grid, cudaStream_t stream) {
  return launch_batch_steps_impl<double>(cfg, static_cast<const Segment<double>*>(segs), bl, nsteps, barrier_words, err,
                                     block, grid, stream);
}

cudaError_t batch_steps_occupancy_fp64_fma(const PathConfig& cfg, int block, int* blocks_per_sm) {
  return batch_steps_occupancy_impl<double>(cfg, block, blocks_per_sm);
}

}  // namespace dev
}  // namespace miniaero
