// Host-side dispatch of the mc_kernel instantiations: shared-memory sizing, occupancy and
// the launch itself (cudaLaunchKernel on the caller's stream).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "mc_kernel.cuh"

namespace cf {

const void* mc_kernel_ptr_bs_f64(int prod, int rng, int risk);
const void* mc_kernel_ptr_bs_f32(int prod, int rng, int risk);
const void* mc_kernel_ptr_dupire_f64(int prod, int rng, int risk);
const void* mc_kernel_ptr_dupire_f32(int prod, int rng, int risk);
const void* dupire_risk32_ptr_l1(int prod, int rng);
const void* dupire_risk32_ptr_tma(int prod, int rng);
size_t dupire_risk32_smem(int rng, const McParams& p);

static const void* kernel_ptr(const McLaunch& l)
{
    if (l.fast) return l.fast == 2 ? dupire_risk32_ptr_tma(l.prod, l.rng) : dupire_risk32_ptr_l1(l.prod, l.rng);
    if (l.model == MODEL_BS)
        return l.fp32 ? mc_kernel_ptr_bs_f32(l.prod, l.rng, l.risk) : mc_kernel_ptr_bs_f64(l.prod, l.rng, l.risk);
    return l.fp32 ? mc_kernel_ptr_dupire_f32(l.prod, l.rng, l.risk)
                  : mc_kernel_ptr_dupire_f64(l.prod, l.rng, l.risk);
}

int mc_smem_bytes(const McLaunch& l, const McParams& p, int stageY, size_t* bytes)
{
    *bytes = l.fast ? dupire_risk32_smem(l.rng, p) : mc_layout(l.model, l.rng, l.fp32, stageY, p, MC_BLOCK).total;
    return 0;
}

long long mc_rounds(const McLaunch& l, long long nPath, long long threads)
{
    if (threads < 32) threads = 32;
    if (l.rng == RNG_SOBOL)  // warp batches of 32 indices
    {
        const long long batches = nPath / 32 + 1, warps = threads / 32;
        return (batches + warps - 1) / warps;
    }
    const long long units = (nPath + 1) / 2;  // antithetic pairs
    return (units + threads - 1) / threads;
}

int mc_scratch_fields(const McLaunch& l, long long rounds)
{
    const int NP = l.rng == RNG_SOBOL ? 1 : 2;
    // dupire_risk32, per ring slot: Gaussian, packed step word per path, and for the barrier
    // the survival factor and spot of band dates per path; generic kernel: Gaussian, state per
    // path, and for the barrier the survival factor of band dates per path
    const int slots = int(rounds < 1 ? 1 : rounds < R32_RING ? rounds : R32_RING);
    if (l.fast) return slots * (1 + NP + (l.prod == PROD_UOC ? 2 * NP : 0));
    return 1 + NP + (l.prod == PROD_UOC ? NP : 0);
}

size_t mc_scratch_bytes(const McLaunch& l, McParams& p, long long grid)
{
    const size_t fields = size_t(p.scratchFields) * size_t(p.nSteps + 1) * size_t(grid) * 128 * (l.fp32 ? 4 : 8);
    if (!l.fast)
    {
        p.nodeSlabOffset = 0;
        return fields;
    }
    p.nodeSlabOffset = (long long)((fields + 255) & ~size_t(255));
    return size_t(p.nodeSlabOffset) + size_t(grid) * size_t(p.nS) * size_t(p.nT) * 8;
}

int mc_use_fast32(const McParams& plan, int prod, int fp32, int risk)
{
    if (!plan.fast32 || !fp32 || !risk || (prod != PROD_UOC && prod != PROD_EUROPEAN)) return 0;
    const char* env = std::getenv("CF_FAST32");
    return env && env[0] == '0' ? 0 : 1;
}

int r32_staging(McLaunch& l, McParams& p, int occ0, size_t* smem)
{
    // p.stageY: the inverse-normal table in shared memory; p.rowChunk: local-vol rows per bulk
    // copy (0: rows read through L1)
    auto occOf = [&](int stage, int chunk, size_t* b) {
        p.stageY = stage;
        p.rowChunk = chunk;
        l.fast = chunk ? 2 : 1;  // the kernel form with (2) or without (1) staged rows
        int occ = 0;
        mc_smem_bytes(l, p, 0, b);
        if (*b > 200 * 1024 || mc_occupancy(l, *b, &occ)) return 0;
        return occ;
    };
    int stage = 0, chunk = 0;
    size_t b1 = 0;
    const char* envK = std::getenv("CF_ROW_CHUNK");
    if (envK)
    {
        // a forced row chunk (tests and tuning; even, at most 16), taken at whatever occupancy
        // it leaves, with the inverse-normal table staged when that costs nothing more
        chunk = std::max(0, std::min(16, std::atoi(envK))) & ~1;
        const int o0 = occOf(0, chunk, &b1);
        stage = occOf(1, chunk, &b1) >= o0 ? 1 : 0;
    }
    else
    {
        // (inverse-normal table staged, rows per bulk copy), in order of preference; the first
        // that keeps the occupancy of the unstaged kernel is taken
        static const int opts[][2] = {{1, 8}, {0, 8}, {1, 4}, {0, 4}, {1, 2}, {0, 2}, {1, 0}};
        for (const auto& o : opts)
        {
            const int occ = occOf(o[0], o[1], &b1);
            if (occ >= 1 && occ >= occ0)
            {
                stage = o[0];
                chunk = o[1];
                break;
            }
        }
    }
    // the chosen configuration is measured last: that also leaves the kernel's dynamic
    // shared-memory limit at the size it launches with
    const int occ = occOf(stage, chunk, smem);
    if (occ >= 1) return occ;
    occOf(0, 0, smem);
    return occ0;
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
