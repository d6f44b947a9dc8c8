// Mixed form: FP32 face flux, gradient and limiter; FP64 residual
// accumulation and RK4 update. Built with --fmad=false like the FP64 form:
// without contraction every item's arithmetic is the same in the single-mesh
// and the batched kernels, so a solve gives identical bits alone or batched.
// FP32 division and square root are the approximate (2 ulp) forms.
#include "kernels_impl.cuh"

namespace miniaero {
namespace dev {

template <>
cudaError_t launch_init_primitives<float>(const TopoView& t, const StateBuffers& s, const StageBuffers<float>& b,
                                          cudaStream_t stream) {
  return launch_init_primitives_impl<float>(t, s, b, stream);
}

template <>
cudaError_t launch_stage<float>(const TopoView& t, const GeomView<float>& g, const PathConfig& cfg,
                                const StateBuffers& s, const StageBuffers<float>& b, int stage,
                                cudaStream_t stream, unsigned kernels) {
  return launch_stage_impl<float>(t, g, cfg, s, b, stage, stream, kernels);
}

template <>
cudaError_t launch_batch_stage<float>(const PathConfig& cfg, const Segment<float>* segs, const BatchLaunch& bl,
                                   int stage, cudaStream_t stream, unsigned kernels) {
  return launch_batch_stage_impl<float>(cfg, segs, bl, stage, stream, kernels);
}

cudaError_t launch_batch_steps_mixed(const PathConfig& cfg, const void* segs, const BatchLaunch& bl, int nsteps,
                               unsigned* barrier_words, int* err, int block, int grid, cudaStream_t stream) {
  return launch_batch_steps_impl<float>(cfg, static_cast<const Segment<float>*>(segs), bl, nsteps, barrier_words, err,
                                     block, grid, stream);
}

cudaError_t batch_steps_occupancy_mixed(const PathConfig& cfg, int block, int* blocks_per_sm) {
  return batch_steps_occupancy_impl<float>(cfg, block, blocks_per_sm);
}

}  // namespace dev
}  // namespace miniaero
