// NVT molecular dynamics on the device: md.nvt(T,dt).run(atoms,nsteps).
//
// One step (MDNVT::run, md_nvt.cpp:409-438) is a fixed kernel sequence that
// is captured once into a CUDA graph and replayed:
//   k_step_open    fac_x_d *= chain(T/T0)  (first half of the thermostat)
//   k_kick_drift   v = v*fac_x_d + f*dt2/m; x += v*dt; sum of v*dt
//                  (update_x_d__x, md_nvt.cpp:70-102); the last block forms
//                  the mean displacement and clears the rebuild gate
//   k_com_skin     x -= mean displacement; skin test (DynamicMD::decide,
//                  dynamic_md.cpp:90-105) opens the rebuild gate; mixed
//                  precision also refreshes the FP32 bin-relative positions
//   rebuild chain  (system.cu) runs only when the gate is open
//   k_density, k_force (eam.cu)
//   k_kick2        v += f*dt2/m and the kinetic tensor (update_x_d,
//                  md_nvt.cpp:106-128); the last block runs the closing half
//                  of the Nose-Hoover chain (ThermostatNHC::operator(),
//                  thermostat.cpp:47-143) and writes the thermo row
// A one-thread kernel opens each step with the chain's first half.
// Velocity scaling stays lazy as in the reference: the chain's factor is
// folded into the next kick and applied once more at the end of the run
// (update_x_d_final, md_nvt.cpp:51-56).
//
// FP64 mode keeps the reference's operation order (f*dt2/m with a division,
// no fused multiply-adds) so the trajectory matches the oracle to rounding;
// mixed mode multiplies by a per-element dt2/m and lets the compiler fuse.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "system.h"

namespace mappg {

struct MdArgs {
    int n;
    double* x;
    double* v;
    const double* f;
    const double* x0;
    const uint8_t* elem;
    const int* binc;
    float4* p32;
    double masses[kMaxElem];
    double dtm[kMaxElem];  // dt2/m
    double dt, dt2, skin_sq;
    double bv[3][3];
    double* partials;
    double* thermo;  // rows of 14 or null
    int nsteps;
    int mixed;
    NhcParams nhc;
    DevScalars* sc;
};

__device__ __forceinline__ double nhc_f(double x) {
    if (fabs(x) < 0.015625) return 1.0 + x / 2.0 + x * x / 6.0 + x * x * x / 24.0;
    return (exp(x) - 1.0) / x;
}

// ThermostatNHC::operator()(T_r, ndof)  thermostat.cpp:47-143
__device__ double nhc_step(const NhcParams& P, double* eta, double T_r) {
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

// one half of the particle thermostat as MDNVT::run applies it:
// fac = chain(T/T0); mvv *= fac^2; T *= fac^2
__device__ double thermo_half(const NhcParams& P, DevScalars* sc) {
    double fac = nhc_step(P, sc->eta, sc->T_part / P.T);
    double f2 = fac * fac;
    for (int k = 0; k < 6; k++) sc->mvv[k] *= f2;
    sc->T_part *= f2;
    return fac;
}

__device__ void write_thermo(const MdArgs& a, long long row) {
    if (!a.thermo) return;
    double* r = a.thermo + 14 * row;
    DevScalars* sc = a.sc;
    r[0] = sc->energy;
    r[1] = sc->T_part;
    for (int k = 0; k < 6; k++) r[2 + k] = sc->mvv[k];
    for (int k = 0; k < 6; k++) r[8 + k] = sc->virial[k];
}

template <int K>
__device__ bool md_block_partials(double (&v)[K], double* partials, unsigned* counter) {
    __shared__ double red[32][K];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[w][k] = t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int q = 0; q < nw; q++) t += red[q][threadIdx.x];
        partials[blockIdx.x * kRedSlots + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    return last;
}

template <int K>
__device__ void md_final_sums(const double* partials, int nblk, double (&tot)[K]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double t = 0.0;
        for (int b = lane; b < nblk; b += 32) t += partials[b * kRedSlots + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        tot[k] = t;
    }
}

// pre_init (md_nvt.cpp:256-340): kinetic tensor and temperature of the
// incoming velocities
__global__ void k_mvv_init(MdArgs a) {
    double d[6] = {0, 0, 0, 0, 0, 0};
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double m = a.masses[a.elem[i]];
        double v0 = a.v[i], v1 = a.v[n + i], v2 = a.v[2 * n + i];
        d[0] += __dmul_rn(__dmul_rn(v0, v0), m);
        d[1] += __dmul_rn(__dmul_rn(v0, v1), m);
        d[2] += __dmul_rn(__dmul_rn(v0, v2), m);
        d[3] += __dmul_rn(__dmul_rn(v1, v1), m);
        d[4] += __dmul_rn(__dmul_rn(v1, v2), m);
        d[5] += __dmul_rn(__dmul_rn(v2, v2), m);
    }
    if (md_block_partials<6>(d, a.partials, &a.sc->counter[3]) && threadIdx.x < 32) {
        double t[6];
        md_final_sums<6>(a.partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            for (int k = 0; k < 6; k++) a.sc->mvv[k] = t[k];
            a.sc->T_part = (t[0] + (t[3] + t[5])) / a.nhc.ndof_kB;
            a.sc->counter[3] = 0;
            a.sc->step = 0;
        }
    }
}

// run start: thermo row 0, no pending velocity scale
__global__ void k_run_begin(MdArgs a) {
    write_thermo(a, 0);
    a.sc->fac_x_d = 1.0;
}

// opening thermostat half of a step: fac_x_d *= chain(T/T0)
__global__ void k_step_open(MdArgs a) { a.sc->fac_x_d *= thermo_half(a.nhc, a.sc); }

template <bool MIX>
__global__ void __launch_bounds__(256) k_kick_drift(MdArgs a) {
    const int n = a.n;
    const double fac = a.sc->fac_x_d;
    double dsum[3] = {0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int e = a.elem[i];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double vv = a.v[c * n + i], ff = a.f[c * n + i], xx = a.x[c * n + i];
            if (MIX) {
                vv = vv * fac + ff * a.dtm[e];
                double dx = vv * a.dt;
                dsum[c] += dx;
                xx += dx;
            } else {
                vv = __dadd_rn(__dmul_rn(vv, fac), __ddiv_rn(__dmul_rn(ff, a.dt2), a.masses[e]));
                double dx = __dmul_rn(vv, a.dt);
                dsum[c] = __dadd_rn(dsum[c], dx);
                xx = __dadd_rn(xx, dx);
            }
            a.v[c * n + i] = vv;
            a.x[c * n + i] = xx;
        }
    }
    if (md_block_partials<3>(dsum, a.partials, &a.sc->counter[4]) && threadIdx.x < 32) {
        double t[3];
        md_final_sums<3>(a.partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            double natms = (double)n;
            for (int c = 0; c < 3; c++) a.sc->com[c] = t[c] / natms;
            a.sc->rebuild = 0;
            a.sc->counter[4] = 0;
        }
    }
}

template <bool MIX>
__global__ void __launch_bounds__(256) k_com_skin(MdArgs a) {
    const int n = a.n;
    const double c0 = a.sc->com[0], c1 = a.sc->com[1], c2 = a.sc->com[2];
    int moved = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double x0 = __dsub_rn(a.x[i], c0), x1 = __dsub_rn(a.x[n + i], c1), x2 = __dsub_rn(a.x[2 * n + i], c2);
        a.x[i] = x0;
        a.x[n + i] = x1;
        a.x[2 * n + i] = x2;
        double d0 = __dsub_rn(a.x0[i], x0), d1 = __dsub_rn(a.x0[n + i], x1), d2 = __dsub_rn(a.x0[2 * n + i], x2);
        double r = __dadd_rn(__dmul_rn(d0, d0), __dadd_rn(__dmul_rn(d1, d1), __dmul_rn(d2, d2)));
        moved |= r > a.skin_sq;
        if (MIX) {
            int bc = a.binc[i];
            double b0 = bc & 1023, b1 = (bc >> 10) & 1023, b2 = (bc >> 20) & 1023;
            double o0 = b0 * a.bv[0][0] + b1 * a.bv[1][0] + b2 * a.bv[2][0];
            double o1 = b1 * a.bv[1][1] + b2 * a.bv[2][1];
            double o2 = b2 * a.bv[2][2];
            float4 p = a.p32[i];
            p.x = (float)(x0 - o0);
            p.y = (float)(x1 - o1);
            p.z = (float)(x2 - o2);
            a.p32[i] = p;
        }
    }
    if (__syncthreads_or(moved) && threadIdx.x == 0) a.sc->rebuild = 1;
}

template <bool MIX>
__global__ void __launch_bounds__(256) k_kick2(MdArgs a) {
    const int n = a.n;
    double d[6] = {0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int e = a.elem[i];
        const double m = a.masses[e];
        double vv[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double v0 = a.v[c * n + i], ff = a.f[c * n + i];
            if (MIX)
                v0 += ff * a.dtm[e];
            else
                v0 = __dadd_rn(v0, __ddiv_rn(__dmul_rn(ff, a.dt2), m));
            a.v[c * n + i] = v0;
            vv[c] = v0;
        }
        d[0] += __dmul_rn(__dmul_rn(vv[0], vv[0]), m);
        d[1] += __dmul_rn(__dmul_rn(vv[0], vv[1]), m);
        d[2] += __dmul_rn(__dmul_rn(vv[0], vv[2]), m);
        d[3] += __dmul_rn(__dmul_rn(vv[1], vv[1]), m);
        d[4] += __dmul_rn(__dmul_rn(vv[1], vv[2]), m);
        d[5] += __dmul_rn(__dmul_rn(vv[2], vv[2]), m);
    }
    if (md_block_partials<6>(d, a.partials, &a.sc->counter[5]) && threadIdx.x < 32) {
        double t[6];
        md_final_sums<6>(a.partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            DevScalars* sc = a.sc;
            for (int k = 0; k < 6; k++) sc->mvv[k] = t[k];
            sc->T_part = (t[0] + (t[3] + t[5])) / a.nhc.ndof_kB;
            // closing half of this step
            sc->fac_x_d = thermo_half(a.nhc, sc);
            long long st = ++sc->step;
            if (st <= a.nsteps) write_thermo(a, st);
            if (!(isfinite(sc->energy) && isfinite(sc->T_part))) sc->bad = 1;
            sc->counter[5] = 0;
        }
    }
}

__global__ void k_run_end(MdArgs a) {
    const int n = a.n;
    const double fac = a.sc->fac_x_d;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += gridDim.x * blockDim.x)
        a.v[i] = __dmul_rn(a.v[i], fac);
}

}  // namespace mappg

using namespace mappg;

namespace mappg {
void sys_build(mappg_sys* s);

static MdArgs md_args(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, int nsteps,
                      double* thermo_dev) {
    MdArgs a;
    memset(&a, 0, sizeof(a));
    a.n = s->n;
    a.x = s->x;
    a.v = s->v;
    a.f = s->f;
    a.x0 = s->x0;
    a.elem = s->elem;
    a.binc = s->binc;
    a.p32 = s->p32;
    a.dt = dt;
    a.dt2 = dt / 2.0;
    for (int e = 0; e < s->ne; e++) {
        a.masses[e] = s->masses[e];
        a.dtm[e] = a.dt2 / s->masses[e];
    }
    a.skin_sq = 0.25 * s->skin * s->skin;
    for (int d = 0; d < 3; d++)
        for (int k = 0; k < 3; k++) a.bv[d][k] = s->box.H[d][k] / s->nb[d];
    a.partials = s->partials;
    a.thermo = thermo_dev;
    a.nsteps = nsteps;
    a.mixed = s->precision == MAPPG_MIXED;
    // ThermostatNHC(dt/2, t_relax, L, niters)  md_nvt.cpp:19, thermostat.cpp:20-36
    const double tdt = dt / 2.0;
    a.nhc.T = T;
    a.nhc.ddt = tdt / (double)niters;
    a.nhc.ddt2 = 0.5 * tdt / (double)niters;
    a.nhc.freq_sq = 1.0 / (t_relax * t_relax);
    a.nhc.kB = kB;
    a.nhc.ndof = 3 * s->n;
    a.nhc.ndof_kB = a.nhc.ndof * kB;
    a.nhc.L = L;
    a.nhc.niters = niters;
    a.sc = s->sc;
    return a;
}

template <bool MIX>
static void launch_step(mappg_sys* s, const MdArgs& a) {
    int g = grid_for(s, s->n, 256);
    k_step_open<<<1, 1, 0, s->stream>>>(a);
    k_kick_drift<MIX><<<g, 256, 0, s->stream>>>(a);
    k_com_skin<MIX><<<g, 256, 0, s->stream>>>(a);
    launch_rebuild_chain(s);
    launch_force(s);
    k_kick2<MIX><<<g, 256, 0, s->stream>>>(a);
}

struct NvtRun {
    MdArgs a;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    int L = 3;
    long long planned = 0;
    long long done = 0;
    bool thermo = false;
};

static void run_clear(mappg_sys* s) {
    NvtRun* r = (NvtRun*)s->run;
    if (!r) return;
    if (r->exec) cudaGraphExecDestroy(r->exec);
    if (r->graph) cudaGraphDestroy(r->graph);
    delete r;
    s->run = nullptr;
}

void nvt_free(mappg_sys* s) { run_clear(s); }

// MDNVT::init + the opening force call of MDNVT::run, then the step graph
void nvt_begin(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, long long nsteps,
               const double* eta, bool thermo) {
    if (!(kB == kB)) throw Error{MAPPG_ERR_ARG, "boltzmann constant should be set prior to MD"};
    if (L < 1 || L > kMaxChain) throw Error{MAPPG_ERR_ARG, "L must be in 1..16"};
    if (niters < 1) throw Error{MAPPG_ERR_ARG, "niters must be positive"};
    if (!(dt > 0.0)) throw Error{MAPPG_ERR_ARG, "dt must be positive"};
    if (!(T > 0.0)) throw Error{MAPPG_ERR_ARG, "T must be positive"};
    if (!(t_relax > 0.0)) throw Error{MAPPG_ERR_ARG, "t_relax must be positive"};
    if (nsteps < 0) throw Error{MAPPG_ERR_ARG, "nsteps must be >= 0"};
    if (!s->have_v) throw Error{MAPPG_ERR_ARG, "velocities must be set before MD"};
    run_clear(s);
    double* tdev = nullptr;
    if (thermo) {
        long long need = 14LL * (nsteps + 1);
        if (need > s->thermo_cap) {
            if (s->thermo_dev) cudaFree(s->thermo_dev);
            s->thermo_dev = nullptr;
            s->thermo_cap = 0;
            MAPPG_CUDA(cudaMalloc(&s->thermo_dev, sizeof(double) * need));
            s->thermo_cap = need;
        }
        tdev = s->thermo_dev;
    }
    NvtRun* r = new NvtRun();
    s->run = r;
    r->a = md_args(s, T, dt, kB, t_relax, L, niters, (int)std::min<long long>(nsteps, 1LL << 30), tdev);
    r->L = L;
    r->planned = nsteps;
    r->thermo = thermo;
    MdArgs& a = r->a;
    double eta_h[kMaxChain] = {0};
    if (eta)
        for (int k = 0; k < L; k++) eta_h[k] = eta[k];
    MAPPG_CUDA(cudaMemcpyAsync(s->sc->eta, eta_h, sizeof(double) * kMaxChain, cudaMemcpyHostToDevice, s->stream));
    int g = grid_for(s, s->n, 256);
    k_mvv_init<<<g, 256, 0, s->stream>>>(a);
    sys_build(s);
    launch_force(s);
    k_run_begin<<<1, 1, 0, s->stream>>>(a);
    MAPPG_CUDA(cudaGetLastError());
    MAPPG_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    try {
        if (s->precision == MAPPG_MIXED)
            launch_step<true>(s, a);
        else
            launch_step<false>(s, a);
    } catch (...) {
        cudaGraph_t g2;
        cudaStreamEndCapture(s->stream, &g2);
        if (g2) cudaGraphDestroy(g2);
        throw;
    }
    MAPPG_CUDA(cudaStreamEndCapture(s->stream, &r->graph));
    MAPPG_CUDA(cudaGraphInstantiate(&r->exec, r->graph, 0));
}

// enqueue steps (no host synchronisation)
void nvt_steps(mappg_sys* s, long long nsteps) {
    NvtRun* r = (NvtRun*)s->run;
    if (!r) throw Error{MAPPG_ERR_ARG, "no NVT run has begun on this system"};
    if (r->done + nsteps > r->planned) throw Error{MAPPG_ERR_ARG, "more steps than the run was begun with"};
    for (long long st = 0; st < nsteps; st++) MAPPG_CUDA(cudaGraphLaunch(r->exec, s->stream));
    r->done += nsteps;
}

// update_x_d_final, chain state out, thermo rows, checks
void nvt_end(mappg_sys* s, double* eta, double* thermo) {
    NvtRun* r = (NvtRun*)s->run;
    if (!r) throw Error{MAPPG_ERR_ARG, "no NVT run has begun on this system"};
    int g = grid_for(s, s->n, 256);
    k_run_end<<<g, 256, 0, s->stream>>>(r->a);
    MAPPG_CUDA(cudaGetLastError());
    DevScalars h;
    MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s->stream));
    if (thermo && r->thermo)
        MAPPG_CUDA(cudaMemcpyAsync(thermo, r->a.thermo, sizeof(double) * 14 * (r->done + 1), cudaMemcpyDeviceToHost,
                                   s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    if (eta)
        for (int k = 0; k < r->L; k++) eta[k] = h.eta[k];
    run_clear(s);
    s->forces_valid = true;
    if (h.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during the run"};
    if (h.bad) throw Error{MAPPG_ERR_NAN, "non-finite position, energy or temperature during the run"};
}

void nvt_run(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, int nsteps, double* eta,
             double* thermo) {
    nvt_begin(s, T, dt, kB, t_relax, L, niters, nsteps, eta, thermo != nullptr);
    nvt_steps(s, nsteps);
    nvt_end(s, eta, thermo);
}

}  // namespace mappg
