// Plain FP64 form. Compiled with --fmad=false: every multiply and add rounds
// separately, as in the reference's serial build with -ffp-contract=off.
#include "kernels_impl.cuh"

namespace miniaero {
namespace dev {

template <>
cudaError_t launch_init_primitives<double>(const TopoView& t, const StateBuffers& s, const StageBuffers<double>& b,
                                           cudaStream_t stream) {
  return launch_init_primitives_impl<double>(t, s, b, stream);
}

template <>
cudaError_t launch_stage<double>(const TopoView& t, const GeomView<double>& g, const PathConfig& cfg,
                                 const StateBuffers& s, const StageBuffers<double>& b, int stage,
                                 cudaStream_t stream, unsigned kernels) {
  return launch_stage_impl<double>(t, g, cfg, s, b, stage, stream, kernels);
}

template <>
cudaError_t launch_batch_stage<double>(const PathConfig& cfg, const Segment<double>* segs, const BatchLaunch& bl,
                                   int stage, cudaStream_t stream, unsigned kernels) {
  return launch_batch_stage_impl<double>(cfg, segs, bl, stage, stream, kernels);
}

cudaError_t launch_batch_steps_fp64(const PathConfig& cfg, const void* segs, const BatchLaunch& bl, int nsteps,
                               unsigned* barrier_words, int* err, int block, int grid, cudaStream_t stream) {
  return launch_batch_steps_impl<double>(cfg, static_cast<const Segment<double>*>(segs), bl, nsteps, barrier_words, err,
                                     block, grid, stream);
}

cudaError_t batch_steps_occupancy_fp64(const PathConfig& cfg, int block, int* blocks_per_sm) {
  return batch_steps_occupancy_impl<double>(cfg, block, blocks_per_sm);
}

cudaError_t launch_debug_barrier_timeout(unsigned* words, int* err, unsigned long long timeout_ns, int* out,
                                        cudaStream_t stream) {
  void* args[] = {(void*)&words, (void*)&err, (void*)&timeout_ns, (void*)&out};
  return cudaLaunchCooperativeKernel((const void*)k_debug_barrier_timeout, dim3(2), dim3(32), args, 0, stream);
}

}  // namespace dev
}  // namespace miniaero
