// FP32 instantiation (mixed form: FP32 volume stencil, FP64 friction and
// boundary data).
#include "tmk_launch_impl.cuh"
TMK_INSTANTIATE_LAUNCH(float, 32, 8, 256)
