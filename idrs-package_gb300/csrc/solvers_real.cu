// solvers_real.cu -- instantiates the real (fp64 outer, fp64/fp32 inner) solvers.
#include "idrs_gpu_impl.cuh"

namespace idrs {
template class IdrsGpu<double>;
template class IdrsGpu<float>;
template class QmrGpu<double, double>;
template class QmrGpu<double, float>;
}  // namespace idrs
