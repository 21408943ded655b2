// Warp-per-line y pass (FP32) compiled for 8 resident blocks per SM (64 registers per thread):
// the occupancy variant the setup-time autotuner can choose per grid (kernels in dstw_y.cuh).
#include "dstw_y.cuh"

namespace ib {

template cudaError_t wypass_minb<float, 8>(const Geometry&, const DstAxis<float>&, const YPassArgs<float>&,
                                           cudaStream_t);

}  // namespace ib
