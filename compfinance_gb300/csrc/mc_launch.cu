// Host-side dispatch of the mc_kernel instantiations: shared-memory sizing, occupancy and
// the launch itself (cudaLaunchKernel on the caller's stream).
#include <cuda_runtime.h>

#include "mc_kernel.cuh"

namespace cf {

const void* mc_kernel_ptr_bs_f64(int prod, int rng, int risk);
const void* mc_kernel_ptr_bs_f32(int prod, int rng, int risk);
const void* mc_kernel_ptr_dupire_f64(int prod, int rng, int risk);
const void* mc_kernel_ptr_dupire_f32(int prod, int rng, int risk);

static const void* kernel_ptr(const McLaunch& l)
{
    if (l.model == MODEL_BS)
        return l.fp32 ? mc_kernel_ptr_bs_f32(l.prod, l.rng, l.risk) : mc_kernel_ptr_bs_f64(l.prod, l.rng, l.risk);
    return l.fp32 ? mc_kernel_ptr_dupire_f32(l.prod, l.rng, l.risk)
                  : mc_kernel_ptr_dupire_f64(l.prod, l.rng, l.risk);
}

int mc_smem_bytes(const McLaunch& l, const McParams& p, int stageY, size_t* bytes)
{
    *bytes = mc_layout(l.model, l.rng, l.fp32, stageY, p, MC_BLOCK).total;
    return 0;
}

int mc_occupancy(const McLaunch& l, size_t smem, int* blocksPerSM)
{
    const void* fn = kernel_ptr(l);
    if (!fn) return (int)cudaErrorInvalidDeviceFunction;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, fn, MC_BLOCK, smem);
}

int launch_mc(const McLaunch& l, const McParams& p, void* stream)
{
    const void* fn = kernel_ptr(l);
    if (!fn) return (int)cudaErrorInvalidDeviceFunction;
    McParams q = p;
    void* args[] = {&q};
    return (int)cudaLaunchKernel(fn, dim3(l.grid), dim3(MC_BLOCK), args, l.smem, (cudaStream_t)stream);
}

}  // namespace cf
