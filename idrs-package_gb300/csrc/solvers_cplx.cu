// solvers_cplx.cu -- instantiates the complex (c128 outer, c128/c64 inner) solvers.
#include "idrs_gpu_impl.cuh"

namespace idrs {
template class IdrsGpu<c128>;
template class IdrsGpu<c64>;
template class QmrGpu<c128, c128>;
template class QmrGpu<c128, c64>;
}  // namespace idrs
