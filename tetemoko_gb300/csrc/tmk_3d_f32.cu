// The mixed form of the 3-D patch step: FP32 volume arithmetic and
// intermediates, FP64 state, friction solves and boundary data (tmk_3d.cuh).
#include "tmk_3d.cuh"

namespace tmk {
namespace d3 {

cudaError_t launch_one_f32(const PlanOne<float>& pl, const DevParams* P, DevStatus* st, cudaStream_t s,
                           const Side* side) {
  return launch_plan<float>(pl, P, st, s, side);
}
cudaError_t launch_many_f32(const PlanMany<float>& pl, const DevParams* P, DevStatus* st, cudaStream_t s,
                            const Side* side) {
  return launch_plan<float>(pl, P, st, s, side);
}

}  // namespace d3
}  // namespace tmk
