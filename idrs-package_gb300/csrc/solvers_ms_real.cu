// solvers_ms_real.cu -- instantiates the real multishift solvers.
#include "ms_gpu_impl.cuh"

namespace idrs {
template class MsIdrsGpu<double>;
template class MsIdrsGpu<float>;
template class MsQmrGpu<double, double>;
template class MsQmrGpu<double, float>;
}  // namespace idrs
