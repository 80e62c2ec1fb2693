// Extended-source kernel instantiation: triple lens, FP64, adjoint.
#include "es_kernel.cuh"

namespace cgb {
template cudaError_t launch_es_variant<3, FP64, true>(const EsParams &, const cd *, const int64_t *,
                                                          const uint8_t *, int64_t, double *, uint32_t *, int,
                                                          cudaStream_t);
}  // namespace cgb
