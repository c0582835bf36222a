// Instantiations of mc_kernel for one (model, precision); compiled as its own translation
// unit so the build runs the four in parallel.
#include "mc_kernel.cuh"

namespace cf {

const void* mc_kernel_ptr_dupire_f64(int prod, int rng, int risk)
{
#define CF_K(PR, RG, RK) \
    if (prod == PR && rng == RG && risk == RK) return (const void*)&mc_kernel<MODEL_DUPIRE, PR, RG, double, RK>;
#define CF_K2(PR, RG) CF_K(PR, RG, false) CF_K(PR, RG, true)
#define CF_K3(PR) CF_K2(PR, RNG_MRG) CF_K2(PR, RNG_SOBOL)
    CF_K3(PROD_EUROPEAN)
    CF_K3(PROD_UOC)
    CF_K3(PROD_EUROPEANS)
    CF_K3(PROD_CONTINGENT)
#undef CF_K3
#undef CF_K2
#undef CF_K
    return nullptr;
}

}  // namespace cf
