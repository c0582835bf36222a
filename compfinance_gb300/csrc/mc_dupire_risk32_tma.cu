// FP32 Dupire risk kernels whose forward stages the local-vol rows into shared memory by bulk
// copies through the TMA unit, double-buffered (mc_dupire_risk32.cuh).
#include "mc_dupire_risk32.cuh"

namespace cf {

const void* dupire_risk32_ptr_tma(int prod, int rng) { return dupire_risk32_ptr_t<true>(prod, rng); }

}  // namespace cf
