// Device RNG access used by the bit-exactness checks of the C ABI (cf_sobol_points,
// cf_mrg_state, cf_gaussians): the same generators the Monte Carlo kernels use.
#include <cuda_runtime.h>

#include "cf_device.cuh"

namespace cf {

__global__ void sobol_points_kernel(const unsigned* dir, int dim, long long first, int n, unsigned* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n * dim) return;
    const long long path = i / dim;
    const int d = int(i % dim);
    out[i] = sobol_state(dir, dim, d, (unsigned long long)(first + path + 1));
}

__global__ void mrg_state_kernel(const unsigned* A, const unsigned* B, unsigned s1, unsigned s2,
                                 unsigned long long skip, unsigned* out)
{
    if (threadIdx.x || blockIdx.x) return;
    const MrgState s = mrg_jump(s1, s2, skip, A, B);
    out[0] = s.x0; out[1] = s.x1; out[2] = s.x2; out[3] = s.y0; out[4] = s.y1; out[5] = s.y2;
}

// Gaussians (or, uniform = 1, the uniforms they come from) of paths [first, first+n): Sobol
// one thread per (path, dim); mrg32k3a one thread per antithetic pair, whose second path takes
// the negated Gaussians and the uniforms 1 - u (mrg32k3a.h:117-184).
__global__ void gauss_kernel(int sobol, int uniform, const unsigned* dir, const unsigned* A,
                             const unsigned* B, unsigned s1, unsigned s2, int dim, long long first, int n,
                             double* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (sobol)
    {
        if (i >= (long long)n * dim) return;
        const long long path = i / dim;
        const int d = int(i % dim);
        const unsigned st = sobol_state(dir, dim, d, (unsigned long long)(first + path + 1));
        out[i] = uniform ? 2.3283064365387E-10 * (double)st : sobol_gauss_d(st);  // sobol.h:26, 102-116
        return;
    }
    const long long pair = first / 2 + i;
    if (2 * pair + 1 < first || 2 * pair >= first + n) return;
    MrgState s = mrg_jump(s1, s2, (unsigned long long)pair * dim, A, B);
    for (int d = 0; d < dim; ++d)
    {
        const unsigned dr = mrg_next(s);
        const double u = (double)dr / 4294967088.0;
        const double g = uniform ? u : mrg_gauss_d(dr);
        const long long pa = 2 * pair - first, pb = pa + 1;
        if (pa >= 0 && pa < n) out[pa * dim + d] = g;
        if (pb >= 0 && pb < n) out[pb * dim + d] = uniform ? 1.0 - u : -g;
    }
}

int launch_sobol_points(const unsigned* dir, int dim, long long first, int n, unsigned* out, void* stream)
{
    const long long tot = (long long)n * dim;
    sobol_points_kernel<<<unsigned((tot + 255) / 256), 256, 0, (cudaStream_t)stream>>>(dir, dim, first, n, out);
    return (int)cudaGetLastError();
}

int launch_mrg_state(const unsigned* A, const unsigned* B, unsigned s1, unsigned s2,
                     unsigned long long skip, unsigned* out, void* stream)
{
    mrg_state_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(A, B, s1, s2, skip, out);
    return (int)cudaGetLastError();
}

int launch_gauss(int sobol, int uniform, const unsigned* dir, const unsigned* A, const unsigned* B,
                 unsigned s1, unsigned s2, int dim, long long first, int n, double* out, void* stream)
{
    const long long tot = sobol ? (long long)n * dim : (long long)n / 2 + 2;
    gauss_kernel<<<unsigned((tot + 127) / 128), 128, 0, (cudaStream_t)stream>>>(sobol, uniform, dir, A, B, s1, s2, dim,
                                                                                first, n, out);
    return (int)cudaGetLastError();
}

}  // namespace cf
