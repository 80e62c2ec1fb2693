// Point-source kernel instantiation: FP64 Ehrlich-Aberth solver with the
// compensated Horner stopping test (the reference's `compensated=True`).
// Only the root solver and mag_point_source take this precision.
#include "point_source.cuh"

namespace cgb {
template cudaError_t launch_ea_solve_p<FP64_COMP>(const double *, const double *, double *, int64_t, int, int,
                                                  uint32_t *, cudaStream_t);
template cudaError_t launch_mag_ps_p<FP64_COMP>(const Lens &, const double *, double *, double *, uint32_t *, int64_t,
                                                int, uint32_t *, cudaStream_t);
}  // namespace cgb
