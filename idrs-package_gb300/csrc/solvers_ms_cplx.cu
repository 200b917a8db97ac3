// solvers_ms_cplx.cu -- instantiates the complex multishift solvers.
#include "ms_gpu_impl.cuh"

namespace idrs {
template class MsIdrsGpu<c128>;
template class MsIdrsGpu<c64>;
template class MsQmrGpu<c128, c128>;
template class MsQmrGpu<c128, c64>;
}  // namespace idrs
