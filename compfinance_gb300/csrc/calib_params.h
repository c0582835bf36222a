// Parameters of the calibration kernels (calib_kernels.cu), shared with calib.cpp.
#pragma once

namespace cf {

struct CalibParams
{
    int ivsKind;      // 0 parametric, 1 Merton
    double spot;
    double ivp[4];
    int nS, nT;
    const double* spots;
    const double* times;
    const int* il;    // [nT] first / last spot index inside +-2.5 std
    const int* ih;
    int nK, nM;       // risk view
    const double* rvK;
    const double* rvM;
    double* c;        // [nT][nS][5] calls
    double* vega;     // [nT][nS][5] d call / d vol
    double* lvT;      // [nT][nS] local vols, maturity-major
    const double* seed;   // [nS][nT] adjoint of each local vol (extrapolation folded in)
    const double* spreads;  // [nK][nM] risk-view spreads added to the implied vols, or null
    long long* acc;       // [nK*nM][2] fixed-point accumulators of d / d spread
    double* pointAdj;     // [nT][nS][5] adjoint of each call's implied vol (test hook), or null
};

int launch_calib(const CalibParams& p, int adjoint, void* stream);

}  // namespace cf
