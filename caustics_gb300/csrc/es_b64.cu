// Extended-source kernel instantiation: binary lens, FP64.
#include "es_kernel.cuh"

namespace cgb {
template cudaError_t launch_es_variant<2, FP64, false>(const EsParams &, const cd *, const int64_t *,
                                                          const uint8_t *, int64_t, double *, uint32_t *, int,
                                                          cudaStream_t);
}  // namespace cgb
