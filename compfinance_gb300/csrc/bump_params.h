// Arguments and scratch layout of the pathwise bump kernel (bump_kernel.cu), shared with the
// host code that sizes and launches it (bump.cpp).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace cf {

constexpr double BUMP_SIZE = 1.0e-08;  // main.h:346

// Rows of the per-thread scratch, each row [thread] over the launched grid: doubles first
// (Gaussians per step; per path the state per point, the barrier survival factor per point
// (-1 once knocked out), the base payoffs), then ints (per path the spot interval per step),
// then the touched-node mask words.
struct BumpRows
{
    int dG, dX, dA, dP0, nDouble;
    int iK, nInt;
    int nMask;
};

__host__ __device__ inline BumpRows bump_rows(int nSteps, int nPay, int np, int maskWords)
{
    BumpRows r;
    r.dG = 0;
    r.dX = r.dG + nSteps;
    r.dA = r.dX + np * (nSteps + 1);
    r.dP0 = r.dA + np * (nSteps + 1);
    r.nDouble = r.dP0 + np * nPay;
    r.iK = 0;
    r.nInt = np * nSteps;
    r.nMask = maskWords;
    return r;
}

struct BumpArgs
{
    int nParam;          // 1 + nS nT
    int maskWords;       // ceil(nS nT / 32)
    // the spot bump: the log of the bumped spot, and the barrier's smoothing constants taken
    // from the bumped first spot of the path (mcPrd.h:247)
    double x0Bumped, barSmoothB, minusSmoothB, twoSmoothB, logBandB;
    long long* acc;      // [nParam nPay][2] payoff differences, then [nPay][2] payoff sums
    void* scratch;       // bump_rows rows of grid * 128 threads
};

}  // namespace cf
