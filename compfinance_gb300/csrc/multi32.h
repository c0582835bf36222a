// FP32 AADriskMulti of a European portfolio on the Dupire model (multi_risk32.cu): launch
// arguments shared by the host (multi.cpp) and the kernels.
#pragma once
#include <cstddef>

#include "cf_params.h"

namespace cf {

constexpr int M32_CHUNK = 256;  // list entries (paths of one bucket) per reverse chunk

struct Multi32Args
{
    McParams p;            // plan tables (the FP32 interpolation tables of dupire_risk32), RNG, sizes
    int nParam;            // 1 + nS nT
    int nBuckets;          // evOff[nEv]
    int nKs;               // sorted strikes (= payoffs)
    int pitch;             // step records per path: nSteps rounded up to even
    const int* evOff;      // [nEv+1] bucket (e, m) = evOff[e] + m, m in [0, nK_e]
    const float* ksF;      // [nKs] strikes of each maturity, sorted: maturity e at evOff[e] - e
    long long* accRisk;    // [nBuckets][nParam][2] fixed point (bucket m = 0 unused)
    long long* accVal;     // [nBuckets][5][2]: count, sum of S (the other three sums stay 0)
    unsigned* rec;         // [nPath][pitch][2]: packed step word, Gaussian bits
    unsigned short* evB;   // [nEv][nPath] in-the-money strikes m of maturity e
    float* evS;            // [nEv][nPath] spot at maturity e
    int* cnt;              // [nBuckets] entries per bucket (zeroed before the forward)
    int* cursor;           // [nBuckets] scatter cursors (zeroed)
    int* start;            // [nBuckets+1] first entry of each bucket
    int* chunkStart;       // [nBuckets+1] first chunk of each bucket; [nBuckets] = chunks
    int* work;             // reverse chunk counter (zeroed)
    int* list;             // [2 * entries]: path, spot bits; grouped by bucket
};

size_t m32_forward_smem(int rng, const Multi32Args& a);
size_t m32_reverse_smem(const Multi32Args& a);
// occupancy (blocks per SM) of the forward and reverse kernels for these shared-memory sizes
int m32_occupancy(int rng, size_t smemFwd, size_t smemRev, int* occFwd, int* occRev);
// forward, scan, scatter and reverse on one stream; returns cudaError_t
int launch_multi32(int rng, int gridFwd, size_t smemFwd, int gridRev, size_t smemRev, const Multi32Args& a,
                   void* stream);

}  // namespace cf
