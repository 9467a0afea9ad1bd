// gm_kernels_f64.cu -- FP64 instantiation of the relaxation kernels.
#include "gm_kernels_impl.cuh"
#include "gm_stage_tma.cuh"

namespace gmk {
GMK_INSTANTIATE(double)
GMK_INSTANTIATE_TMA(double)
}
