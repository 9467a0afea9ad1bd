// gm_kernels_f64.cu -- FP64 instantiation of the relaxation kernels.
#include "gm_kernels_impl.cuh"

namespace gmk {
GMK_INSTANTIATE(double)
}
