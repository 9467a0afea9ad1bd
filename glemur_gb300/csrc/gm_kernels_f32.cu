// gm_kernels_f32.cu -- FP32-storage instantiation of the relaxation kernels.
#include "gm_kernels_impl.cuh"
#include "gm_stage_tma.cuh"

namespace gmk {
GMK_INSTANTIATE(float)
GMK_INSTANTIATE_TMA(float)
}
