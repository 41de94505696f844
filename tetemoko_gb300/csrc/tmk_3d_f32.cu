// The mixed form of the 3-D patch step: FP32 volume arithmetic and
// intermediates, FP64 state, friction solves and boundary data (tmk_3d.cuh).
#include "tmk_3d.cuh"

namespace tmk {
namespace d3 {

cudaError_t launch_step_f32(const Step3<float>& g, const DevParams* P, DevStatus* st, cudaStream_t s,
                            const Side* side) {
  return launch_step<float>(g, P, st, s, side);
}

}  // namespace d3
}  // namespace tmk
