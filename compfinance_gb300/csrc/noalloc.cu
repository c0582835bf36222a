// Allocation-free variant of the AAD-risk entry point (cf_aad_risk_aggregate_noalloc).
//
// Some callers cannot let a library allocate device memory during a call: processes whose
// device memory is already reserved by another allocator (a framework's caching allocator,
// a fixed arena sized at start-up), where a cudaMalloc would fail or fragment, and
// latency-critical callers for whom cudaMalloc / cudaFree, which can synchronise the whole
// device, is not acceptable.  This entry point runs the same risk kernel as
// cf_aad_risk_aggregate, but every byte it needs on the device (reverse-sweep scratch,
// accumulators, weights, error flag, results) lives in one file-scope device array of
// CF_NOALLOC_BYTES, which every GPU that loads the library holds until the process exits.
//
// Rules of use:
//  * The (model, product) pair must have been lowered before (any call naming it, e.g.
//    cf_shapes): lowering allocates, this entry point does not.
//  * The first call on a device looks up the array's device address (cudaGetSymbolAddress,
//    once per device, with that device current); make that first call before any stream
//    capture.  The address is kept for the life of the process, which assumes the device's
//    primary context lives as long: after a cudaDeviceReset the library must be reloaded.
//  * Black-Scholes and Dupire models only; a multi-asset plan is refused (CF_E_UNSUPPORTED)
//    before anything is launched.
//  * Every call shares the array: calls that overlap on the GPU (other threads, other
//    streams) race.  Each call clears what must start at zero (accumulators, error flag).
//  * Requests whose scratch cannot fit even one block per launch, or whose accumulators
//    exceed the array, are rejected with CF_E_SHAPE.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "cf_device.cuh"
#include "engine.h"
#include "mc_kernel.cuh"

#define CF_NOALLOC_BYTES (64u << 20)

static __device__ __align__(256) unsigned char g_noallocArena[CF_NOALLOC_BYTES];

namespace cf {

extern thread_local std::string g_lastError;

namespace {

// Error message without building a std::string: the message is copied into the thread's
// error string, whose capacity is reserved once (no heap allocation for short messages).
int fail_c(int code, const char* msg)
{
    if (g_lastError.capacity() < 512) g_lastError.reserve(512);
    g_lastError.assign(msg);
    return code;
}

constexpr int kMaxDevices = 64;
void* g_arenaPtr[kMaxDevices] = {};
std::mutex g_arenaMu;

// Device address of the arena on the current device (looked up once per device).
int arena_address(int dev, unsigned char** out)
{
    if (dev < 0 || dev >= kMaxDevices) return fail_c(CF_E_ARG, "noalloc: device index out of range");
    std::lock_guard<std::mutex> l(g_arenaMu);
    if (!g_arenaPtr[dev])
    {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocArena);
        if (e != cudaSuccess) return fail_c(CF_E_CUDA, "noalloc: cudaGetSymbolAddress failed");
        g_arenaPtr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_arenaPtr[dev]);
    return CF_OK;
}

// Accumulators -> doubles on the device: out[0..nPay) values, out[nPay] aggregate,
// out[nPay+1 ..) risks.
__global__ void noalloc_finalize(const long long* acc, int nRisk, int nPay, double invN, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nPay) out[i] = fix_value(acc[2 * (nRisk + i)], acc[2 * (nRisk + i) + 1]) * invN;
    else if (i == nPay) out[i] = fix_value(acc[2 * (nRisk + 2 * nPay)], acc[2 * (nRisk + 2 * nPay) + 1]) * invN;
    else if (i < nPay + 1 + nRisk)
    {
        const int j = i - nPay - 1;
        out[i] = fix_value(acc[2 * j], acc[2 * j + 1]) * invN;
    }
}

size_t up256(size_t n) { return (n + 255) & ~size_t(255); }

__global__ void to_float_kernel(const double* in, float* out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = float(in[i]);
}

}  // namespace
}  // namespace cf

using namespace cf;

extern "C" int cf_aad_risk_aggregate_noalloc(cf_context* ctx, const char* modelId, const char* productId,
                                             const double* notionals, const cf_num_param* num, double* payoffValues,
                                             double* aggregateValue, double* risks)
{
    if (!ctx || !modelId || !productId || !notionals || !num || !risks)
        return fail_c(CF_E_ARG, "noalloc: null argument");
    if (num->numPath <= 0) return fail_c(CF_E_ARG, "noalloc: numPath must be positive");
    std::lock_guard<std::mutex> lock(ctx->mu);
    Context& c = ctx->c;
    cudaSetDevice(c.device);
    // the pair must already be lowered (lowering allocates the device tables)
    Plan* plan = nullptr;
    for (auto& kv : c.plans)
        if (kv.first.first == modelId && kv.first.second == productId) plan = kv.second.get();
    if (!plan) return fail_c(CF_E_NOTFOUND, "noalloc: (model, product) not lowered yet; call cf_shapes first");
    // the multi-asset model runs its own kernels (md_kernel.cu) with derived-quantity
    // accumulators; only the single-asset Black-Scholes and Dupire kernels run here
    if (plan->model != MODEL_BS && plan->model != MODEL_DUPIRE)
        return fail_c(CF_E_UNSUPPORTED, "noalloc: only Black-Scholes and Dupire models are supported");
    {
        auto mi = c.models.find(modelId);
        auto pi = c.products.find(productId);
        if (mi == c.models.end() || pi == c.products.end() || mi->second.version != plan->mver ||
            pi->second.version != plan->pver)
            return fail_c(CF_E_NOTFOUND, "noalloc: model or product changed since lowering; call cf_shapes first");
    }
    const bool sobol = num->useSobol != 0, fp32 = num->precision == CF_FP32;
    if (sobol && !plan->sobolOk) return fail_c(CF_E_SHAPE, "noalloc: Sobol dimension exceeds the direction numbers");
    unsigned char* arena = nullptr;
    int rc = arena_address(c.device, &arena);
    if (rc) return rc;
    cudaStream_t st = c.stream;

    McParams p = plan->base;
    p.nPath = num->numPath;
    p.seed1 = unsigned(num->seed1);
    p.seed2 = unsigned(num->seed2);
    p.mrgJumpA = c.jumpA;
    p.mrgJumpB = c.jumpB;
    p.invnF = sobol ? c.invnSobol : c.invnMrg;
    p.nRisk = plan->nParam;
    p.nAcc = p.nRisk + 2 * plan->nPay + 2;
    // arena layout: weights | accumulators + error flag | results | scratch
    const size_t offW = 0, wBytes = up256(size_t(plan->nPay) * 12);
    const size_t offAcc = offW + wBytes, accBytes = up256(size_t(p.nAcc) * 16 + 16);
    const size_t offOut = offAcc + accBytes, outBytes = up256(size_t(plan->nPay + 1 + plan->nParam) * 8);
    const size_t offScr = offOut + outBytes;
    if (offScr >= CF_NOALLOC_BYTES) return fail_c(CF_E_SHAPE, "noalloc: accumulators exceed the 64 MiB arena");

    McLaunch l{plan->model, plan->prod, sobol ? RNG_SOBOL : RNG_MRG, fp32 ? 1 : 0, 1, 0, 128, 0, 0};
    size_t smem = 0;
    p.stageY = 0;
    int occ = 0;
    // the kernel choice of the allocating entry point (cf_aad_risk_aggregate)
    l.fast = mc_use_fast32(p, plan->prod, l.fp32, 1);
    if (l.fast)
    {
        mc_smem_bytes(l, p, 0, &smem);
        if (smem > 200 * 1024 || mc_occupancy(l, smem, &occ) || occ < 1) l.fast = 0;
    }
    if (!l.fast)
    {
        mc_smem_bytes(l, p, 0, &smem);
        if ((rc = mc_occupancy(l, smem, &occ)) || occ < 1) return fail_c(CF_E_SHAPE, "noalloc: kernel does not fit");
    }
    // scratch per block: the reverse-sweep fields of 128 threads (counted for the FP32 kernel's
    // full ring of round slots), plus its int64 node slab (and 256 bytes of alignment between
    // the two regions)
    const size_t perThread = size_t(mc_scratch_fields(l, R32_RING)) * size_t(plan->nSteps + 1) * (fp32 ? 4 : 8);
    const size_t perBlock = perThread * 128 + (l.fast ? size_t(p.nS) * size_t(p.nT) * 8 : 0);
    const long long fitBlocks = (long long)((CF_NOALLOC_BYTES - offScr - 256) / perBlock);
    if (fitBlocks < 1) return fail_c(CF_E_SHAPE, "noalloc: one block of reverse-sweep scratch exceeds the arena");
    const long long threadsNeeded = sobol ? (p.nPath / 32 + 1) * 32 : (p.nPath + 1) / 2;
    long long grid = std::min<long long>((threadsNeeded + 127) / 128, (long long)c.numSMs * occ);
    grid = std::max(1LL, std::min(grid, fitBlocks));
    const long long rounds = mc_rounds(l, p.nPath, grid * 128);
    p.scratchFields = mc_scratch_fields(l, rounds);
    p.roundCap = rounds < R32_RING ? rounds : 0;
    if (mc_scratch_bytes(l, p, grid) > CF_NOALLOC_BYTES - offScr)
        return fail_c(CF_E_SHAPE, "noalloc: reverse-sweep scratch exceeds the arena");
    l.grid = int(grid);
    l.smem = smem;
    p.scratchThreads = grid * 128;
    p.scratch = arena + offScr;
    p.w = reinterpret_cast<const double*>(arena + offW);
    p.wf = reinterpret_cast<const float*>(arena + offW + size_t(plan->nPay) * 8);
    p.acc = reinterpret_cast<long long*>(arena + offAcc);
    p.err = reinterpret_cast<int*>(arena + offAcc + size_t(p.nAcc) * 16);
    p.claim = reinterpret_cast<unsigned long long*>(arena + offAcc + size_t(p.nAcc) * 16 + 8);  // zeroed with the flag
    double* out = reinterpret_cast<double*>(arena + offOut);

    // weights: the caller's doubles are copied in; the FP32 kernel's float copy is made on
    // the device (no host staging buffer)
    cudaError_t e = cudaMemcpyAsync(arena + offW, notionals, size_t(plan->nPay) * 8, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail_c(CF_E_CUDA, "noalloc: weights upload failed");
    to_float_kernel<<<(plan->nPay + 127) / 128, 128, 0, st>>>(reinterpret_cast<const double*>(arena + offW),
                                                              reinterpret_cast<float*>(arena + offW + size_t(plan->nPay) * 8),
                                                              plan->nPay);
    if (cudaGetLastError() != cudaSuccess) return fail_c(CF_E_CUDA, "noalloc: weight conversion failed");
    if (cudaMemsetAsync(p.acc, 0, size_t(p.nAcc) * 16 + 16, st) != cudaSuccess)
        return fail_c(CF_E_CUDA, "noalloc: accumulator reset failed");
    if (launch_mc(l, p, st)) return fail_c(CF_E_CUDA, "noalloc: risk kernel launch failed");
    const int nOut = plan->nPay + 1 + plan->nParam;
    noalloc_finalize<<<(nOut + 127) / 128, 128, 0, st>>>(p.acc, p.nRisk, plan->nPay, 1.0 / double(p.nPath), out);
    if (cudaGetLastError() != cudaSuccess) return fail_c(CF_E_CUDA, "noalloc: finalize launch failed");
    int flag = 0;
    e = cudaMemcpyAsync(&flag, p.err, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && payoffValues)
        e = cudaMemcpyAsync(payoffValues, out, size_t(plan->nPay) * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && aggregateValue)
        e = cudaMemcpyAsync(aggregateValue, out + plan->nPay, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(risks, out + plan->nPay + 1, size_t(plan->nParam) * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_c(CF_E_CUDA, "noalloc: result download failed");
    if (flag) return fail_c(CF_E_DEVICE, "noalloc: kernel error flag");
    return CF_OK;
}
