// gm_kernels_f32.cu -- FP32-storage instantiation of the relaxation kernels.
#include "gm_kernels_impl.cuh"

namespace gmk {
GMK_INSTANTIATE(float)
}
