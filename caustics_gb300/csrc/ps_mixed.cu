// Point-source kernel instantiation: mixed FP32 + FP64 Ehrlich-Aberth solver.
#include "point_source.cuh"

namespace cgb {
template cudaError_t launch_ea_solve_p<MIXED>(const double *, const double *, double *, int64_t, int, int, uint32_t *,
                                              cudaStream_t);
template cudaError_t launch_mag_ps_p<MIXED>(const Lens &, const double *, double *, double *, uint32_t *, int64_t, int,
                                            uint32_t *, cudaStream_t);
template cudaError_t launch_lc_points_p<MIXED>(const Lens &, double, const double *, double, double *, uint8_t *,
                                               int64_t, int, uint32_t *, int, cudaStream_t);
template cudaError_t launch_lc_points_batched_p<MIXED>(const EsParams &, int64_t, double *, uint8_t *, uint32_t *,
                                                       unsigned long long *, int64_t *, bool, cudaStream_t);
}  // namespace cgb
