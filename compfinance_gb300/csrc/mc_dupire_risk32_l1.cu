// FP32 Dupire risk kernels whose forward reads the local-vol rows through L1
// (mc_dupire_risk32.cuh), and the shared-memory size of either form.
#include "mc_dupire_risk32.cuh"

namespace cf {

const void* dupire_risk32_ptr_l1(int prod, int rng) { return dupire_risk32_ptr_t<false>(prod, rng); }

size_t dupire_risk32_smem(int rng, const McParams& p) { return r32_layout(rng, p).total; }

}  // namespace cf
