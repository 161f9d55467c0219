// Nose-Hoover chain of the particle thermostat on the device
// (ThermostatNHC::operator(), thermostat.cpp:47-143) and its use by
// MDNVT::run (md_nvt.cpp:409-438): one half = chain(T/T0), then
// mvv *= fac^2, T *= fac^2.
#pragma once

#include "system.h"

namespace mappg {

__host__ __device__ __forceinline__ double nhc_f(double x) {
    if (fabs(x) < 0.015625) return 1.0 + x / 2.0 + x * x / 6.0 + x * x * x / 24.0;
    return (exp(x) - 1.0) / x;
}

__host__ __device__ inline double nhc_step(const NhcParams& P, double* eta, double T_r) {
    double rescale = 1.0, prev_fac, tmp;
    const int L = P.L;
    if (L == 1) {
        for (int it = 0; it < P.niters; it++) {
            eta[0] += P.ddt2 * P.freq_sq * (T_r - 1.0);
            prev_fac = exp(-P.ddt * eta[0]);
            rescale *= prev_fac;
            T_r *= prev_fac * prev_fac;
            eta[0] += P.ddt2 * P.freq_sq * (T_r - 1.0);
        }
        return rescale;
    }
    for (int it = 0; it < P.niters; it++) {
        eta[L - 1] += P.ddt2 * (eta[L - 2] * eta[L - 2] - P.freq_sq);
        prev_fac = -eta[L - 1];
        for (int ich = L - 2; ich > 0; ich--) {
            eta[ich] += P.ddt2 * nhc_f(prev_fac * P.ddt2) * (prev_fac * eta[ich] + eta[ich - 1] * eta[ich - 1] - P.freq_sq);
            prev_fac = -eta[ich];
        }
        eta[0] += P.ddt2 * nhc_f(prev_fac * P.ddt2) * (prev_fac * eta[0] + P.freq_sq * (T_r - 1.0));
        prev_fac = -eta[0];
        tmp = exp(P.ddt * prev_fac);
        rescale *= tmp;
        T_r *= tmp * tmp;
        prev_fac = (T_r - 1.0) * P.freq_sq;
        eta[0] += P.ddt2 * nhc_f(-eta[1] * P.ddt2) * (-eta[1] * eta[0] + prev_fac);
        prev_fac = P.ndof * eta[0] * eta[0] - P.freq_sq;
        for (int ich = 1; ich < L - 1; ich++) {
            eta[ich] += P.ddt2 * nhc_f(-eta[ich + 1] * P.ddt2) * (-eta[ich + 1] * eta[ich] + prev_fac);
            prev_fac = eta[ich] * eta[ich] - P.freq_sq;
        }
        eta[L - 1] += P.ddt2 * prev_fac;
    }
    return rescale;
}

template <class State>
__device__ inline double thermo_half(const NhcParams& P, State* sc) {
    double fac = nhc_step(P, sc->eta, sc->T_part / P.T);
    double f2 = fac * fac;
    for (int k = 0; k < 6; k++) sc->mvv[k] *= f2;
    sc->T_part *= f2;
    return fac;
}

// thermo row: pe, T, mvv[6], virial[6]
__device__ inline void write_thermo_row(double* thermo, const DevScalars* sc, long long row) {
    if (!thermo) return;
    double* r = thermo + 14 * row;
    r[0] = sc->energy;
    r[1] = sc->T_part;
    for (int k = 0; k < 6; k++) r[2 + k] = sc->mvv[k];
    for (int k = 0; k < 6; k++) r[8 + k] = sc->virial[k];
}

}  // namespace mappg
