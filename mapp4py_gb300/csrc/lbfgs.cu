// L-BFGS minimization with back-tracking line search on the device:
// md.min_lbfgs(m,e_tol,max_dx,ls=ls_bt(c,rho,min_alpha)).run(atoms,nsteps).
//
// The iteration is MinLBFGS::__run (min_l-bfgs.h:113-219) over the line-
// search object MinMDHandler<false,true> (min_cg.h:215-309) and
// LineSearchBackTrack::min (ls.h:711-769):
//   x0 = x; h = f0 = f; two-loop recursion over the m most recent (s, y);
//   f.h < 0 -> h = f, history dropped; Armijo back-tracking from
//   alpha = min(max_dx/max|h|, 1); force call; stop on the energy tolerance,
//   on max|F| < f_tol (added), or on the iteration limit; history update
//   s0 = alpha*h, y0 = f0 - f, rho0 = 1/(s0.y0), gamma = s0.y0/(y0.y0).
// All vectors live on the device in the system's SoA layout.  The recursion
// keeps its scalars on the device: each kernel reads the coefficient it
// needs, applies its update and reduces the next dot product in the same
// pass, so the host only reads the line-search energies and f.h.  Dot
// products are FP64 with a fixed reduction order.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "linesearch.h"
#include "system.h"

namespace mappg {

void sys_build(mappg_sys* s);
void lb_update(mappg_sys* s);

// device scalars of the recursion (one block of doubles)
struct LbScal {
    double dot[2 * 64 + 8];  // dot products, one slot per use
    double rho[64];
    double alpha[64];
    double gamma;
    double fh, hh, hmax, fmax;
    double tau;    // scale of the learned diagonal, (s.y)/(y.P.y)
    double dxmax;  // max |x - x_build| component (list validity of line-search trials)
    unsigned long long dxbits;  // the same by k_lb_dxmax (bits of a non-negative double)
};

__device__ __forceinline__ void warp_sum(double& t) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
}

template <int K>
__device__ bool lb_block(double (&v)[K], double* partials, unsigned* counter, bool is_max = false) {
    __shared__ double red[32][K];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double u = __shfl_xor_sync(0xffffffffu, t, o);
            t = is_max ? fmax(t, u) : t + u;
        }
        if (lane == 0) red[w][k] = t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = is_max ? 0.0 : 0.0;
        for (int q = 0; q < nw; q++) t = is_max ? fmax(t, red[q][threadIdx.x]) : t + red[q][threadIdx.x];
        partials[blockIdx.x * kRedSlots + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    return last;
}

template <int K>
__device__ void lb_final(const double* partials, int nblk, double (&tot)[K], bool is_max = false) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double t = 0.0;
        for (int b = lane; b < nblk; b += 32) t = is_max ? fmax(t, partials[b * kRedSlots + k]) : t + partials[b * kRedSlots + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double u = __shfl_xor_sync(0xffffffffu, t, o);
            t = is_max ? fmax(t, u) : t + u;
        }
        tot[k] = t;
    }
}

// h <- h + coef*y, then dot = s.h (s may be null: no dot).  coef is read
// from the device: mode 0: coef = 0 (plain dot); mode 1: alpha_i =
// -rho_i*dot_in, stored; mode 2: beta = -alpha_i - rho_i*dot_in; mode 3:
// coef applies as a scale: h <- gamma*h; mode 4: h <- tau*P*h elementwise
// with P (passed as y) the learned diagonal initial inverse Hessian and tau
// its scale from the newest pair
__global__ void __launch_bounds__(256) k_lb_axpy_dot(int N, double* __restrict__ h, const double* __restrict__ y,
                                                     const double* __restrict__ s, LbScal* L, int mode, int idx,
                                                     int dot_in, int dot_out, double* partials, unsigned* counter) {
    double coef = 0.0;
    if (mode == 1) {
        coef = -L->rho[idx] * L->dot[dot_in];
        if (blockIdx.x == 0 && threadIdx.x == 0) L->alpha[idx] = coef;
    } else if (mode == 2) {
        coef = -L->alpha[idx] - L->rho[idx] * L->dot[dot_in];
    } else if (mode == 3) {
        coef = L->gamma;
    }
    double acc = 0.0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) {
        double hv = h[q];
        if (mode == 1 || mode == 2)
            hv = hv + coef * y[q];
        else if (mode == 3)
            hv = hv * coef;
        else if (mode == 4)
            hv = hv * (L->tau * y[q]);
        if (mode) h[q] = hv;
        if (s) acc += s[q] * hv;
    }
    if (!s) return;
    double v[1] = {acc};
    if (lb_block<1>(v, partials, counter) && threadIdx.x < 32) {
        double t[1];
        lb_final<1>(partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            L->dot[dot_out] = t[0];
            *counter = 0;
        }
    }
}

// dots f.h, h.h and max|h| (line-search preparation) and max|f|; with x
// and xb (the neighbour list's build positions) also max|x - xb| over
// components
__global__ void __launch_bounds__(256) k_lb_prep(int N, const double* __restrict__ f, const double* __restrict__ h,
                                                 const double* __restrict__ x, const double* __restrict__ xb,
                                                 LbScal* L, double* partials, unsigned* counter) {
    double v[2] = {0.0, 0.0};
    double mx[3] = {0.0, 0.0, 0.0};
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) {
        double hv = h[q], fv = f[q];
        v[0] += fv * hv;
        v[1] += hv * hv;
        mx[0] = fmax(mx[0], fabs(hv));
        mx[1] = fmax(mx[1], fabs(fv));
        if (x) mx[2] = fmax(mx[2], fabs(x[q] - xb[q]));
    }
    // sums into slots 0,1 and maxima into slots 2,3,4 of the same partial row
    __shared__ double red[32][5];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double t[5] = {v[0], v[1], mx[0], mx[1], mx[2]};
#pragma unroll
    for (int k = 0; k < 5; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double u = __shfl_xor_sync(0xffffffffu, t[k], o);
            t[k] = k < 2 ? t[k] + u : fmax(t[k], u);
        }
        if (lane == 0) red[w][k] = t[k];
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double r = 0.0;
        for (int q = 0; q < nw; q++) r = threadIdx.x < 2 ? r + red[q][threadIdx.x] : fmax(r, red[q][threadIdx.x]);
        partials[blockIdx.x * kRedSlots + threadIdx.x] = r;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last && threadIdx.x < 32) {
        double s2[2], m3[3];
        for (int k = 0; k < 2; k++) {
            double a = 0.0;
            for (int bb = lane; bb < (int)gridDim.x; bb += 32) a += partials[bb * kRedSlots + k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
            s2[k] = a;
        }
        for (int k = 0; k < 3; k++) {
            double b = 0.0;
            for (int bb = lane; bb < (int)gridDim.x; bb += 32) b = fmax(b, partials[bb * kRedSlots + 2 + k]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
            m3[k] = b;
        }
        if (threadIdx.x == 0) {
            L->fh = s2[0];
            L->hh = s2[1];
            L->hmax = m3[0];
            L->fmax = m3[1];
            L->dxmax = m3[2];
            *counter = 0;
        }
    }
}

// max |x - xb| over components into *out (the bits of a non-negative double
// order as the values do, so an integer maximum of the bits is the maximum)
__global__ void k_lb_dxmax(int N, const double* __restrict__ x, const double* __restrict__ xb,
                           unsigned long long* out) {
    double m = 0.0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x)
        m = fmax(m, fabs(x[q] - xb[q]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// the search direction as one float4 per atom (Cartesian) for k_de32
__global__ void k_lb_h32(int n, const double* __restrict__ h, float4* __restrict__ h32) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        h32[i] = make_float4((float)h[i], (float)h[n + i], (float)h[2 * n + i], 0.f);
}

// x = x0 + alpha*h  (MinMDHandler::F, min_cg.h:260-267)
__global__ void k_lb_trial(int N, double* __restrict__ x, const double* __restrict__ x0, const double* __restrict__ h,
                           double alpha) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x)
        x[q] = x0[q] + alpha * h[q];
}

// s0 = alpha*h, y0 = f0 - f; dots s0.y0, y0.y0 -> rho0, gamma (and y0.P.y0
// -> tau with a learned diagonal).  A pair without positive curvature
// (s0.y0 <= 0, e.g. a step that underflowed to zero) gets rho0 = 0, so it
// takes no part in the recursion, and leaves gamma as it was; the
// reference would divide by it.
__global__ void __launch_bounds__(256) k_lb_hist(int N, double* __restrict__ s0, double* __restrict__ y0,
                                                 const double* __restrict__ h, const double* __restrict__ f0,
                                                 const double* __restrict__ f, const double* __restrict__ P,
                                                 double alpha, LbScal* L, double* partials, unsigned* counter) {
    double v[3] = {0.0, 0.0, 0.0};
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) {
        double sv = alpha * h[q];
        double yv = f0[q] - f[q];
        s0[q] = sv;
        y0[q] = yv;
        v[0] += sv * yv;
        v[1] += yv * yv;
        if (P) v[2] += yv * yv * P[q];
    }
    if (lb_block<3>(v, partials, counter) && threadIdx.x < 32) {
        double t[3];
        lb_final<3>(partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            if (t[0] > 0.0 && t[1] > 0.0) {
                L->gamma = t[0] / t[1];
                L->rho[0] = 1.0 / t[0];
                if (t[2] > 0.0) L->tau = t[0] / t[2];
            } else {
                L->rho[0] = 0.0;
            }
            *counter = 0;
        }
    }
}

__global__ void k_lb_shift_rho(LbScal* L, int m) {
    for (int i = m - 1; i > 0; i--) L->rho[i] = L->rho[i - 1];
}

struct LbState {
    mappg_sys* s;
    int N, grid;
    double *f0, *h, *xs;  // xs: the minimizer's x0
    std::vector<double*> sv, yv;
    LbScal* L;
    unsigned* counter;
};

void launch_energy64(mappg_sys* s);  // eam.cu
void launch_de32(mappg_sys* s, double alpha);  // eam32.cu

static double lb_energy(mappg_sys* s) {
    // skin test and (gated) rebuild, then the energy kernel; mixed systems
    // compare FP64 line-search energies, so FP32 rounding of the pair terms
    // does not decide the Armijo test near convergence
    lb_update(s);
    if (s->precision == MAPPG_MIXED)
        launch_energy64(s);
    else
        launch_energy(s);
    double e;
    MAPPG_CUDA(cudaMemcpyAsync(&e, &s->sc->energy, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    return e;
}

__global__ void k_clear_rebuild(DevScalars* sc) { sc->rebuild = 0; }

void lb_update(mappg_sys* s) {
    k_clear_rebuild<<<1, 1, 0, s->stream>>>(s->sc);
    launch_skin_test(s);
    launch_rebuild_chain(s);
    // positions moved without a rebuild: refresh the mixed kernels' frame
    if (s->precision == MAPPG_MIXED) launch_shadow(s, false);
    MAPPG_CUDA(cudaGetLastError());
    // a relaxation can crowd atoms beyond the rows' capacity: a rebuild that
    // ran out of room is redone with wider rows
    int ov = 0;
    MAPPG_CUDA(cudaMemcpyAsync(&ov, &s->sc->overflow, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    if (ov) sys_build(s);
}

static void lb_force(mappg_sys* s, double* pe) {
    launch_force(s);
    sync_forces64(s);
    MAPPG_CUDA(cudaMemcpyAsync(pe, &s->sc->energy, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
}

// The caller's function after an iteration's force call, where the
// reference writes its periodic export (ExportHandler::print, min.h:216-220)
void iteration_hook(mappg_sys* s, int istep) {
    if (!s->hook || s->hook_every <= 0 || (istep + 1) % s->hook_every != 0) return;
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    if (s->hook(s->hook_user, (long long)istep + 1) != 0)
        throw Error{MAPPG_ERR_ARG, "the iteration hook stopped the run"};
}

// The minimizers' line-search function (MinMDHandler::F and F_reset,
// min_cg.h:260-276): a trial moves x to x0 + alpha h and evaluates the
// energy; reset restores x0.  Trial energies by mode:
//   E64      the FP64 energy (FP64 systems; mixed systems on FP64 forces)
//   DELTA    e0 + dE, dE from the energy-difference pass (launch_de32) on
//            x0's rows and frame positions; no skin test or rebuild (the
//            caller has checked that every trial stays within the skin)
//   E32DIFF  e0 + (E32(trial) - E32(x0)) with the skin test and rebuilds:
//            searches whose first step is too long for DELTA, where the
//            energy changes are large next to the FP32 rounding
struct TrialLine {
    enum Mode { E64, DELTA, E32DIFF };
    mappg_sys* s;
    int N, grid;
    const double* xs;  // x0
    const double* h;
    long long* n_en;
    LbScal* L;
    Mode mode = E64;
    double e0 = 0.0;     // energy of x0 (DELTA, E32DIFF)
    double e0_32 = 0.0;  // FP32 energy of x0 (E32DIFF)
    double hmax = 0.0;   // max |h_c| of the direction
    double F(double a) {
        // an E32DIFF search whose trials have become short goes over to
        // energy differences (FP32 differences would drown in rounding)
        if (mode == E32DIFF && 1.7320508075688772 * a * hmax < 0.25 * s->skin) to_delta(a);
        k_lb_trial<<<grid, 256, 0, s->stream>>>(N, s->x, xs, h, a);
        (*n_en)++;
        if (mode == E64) return lb_energy(s);
        double e;
        if (mode == DELTA) {
            launch_de32(s, a);
            MAPPG_CUDA(cudaMemcpyAsync(&e, &s->sc->de, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
            MAPPG_CUDA(cudaStreamSynchronize(s->stream));
            return e0 + e;
        }
        return e0 + (energy32(s) - e0_32);
    }
    void reset() {
        MAPPG_CUDA(cudaMemcpyAsync(s->x, xs, sizeof(double) * N, cudaMemcpyDeviceToDevice, s->stream));
        if (mode != DELTA) lb_update(s);
    }
    // back at x0 with a list around it; DELTA when the trial of step a then
    // stays within half the skin
    void to_delta(double a) {
        MAPPG_CUDA(cudaMemcpyAsync(s->x, xs, sizeof(double) * N, cudaMemcpyDeviceToDevice, s->stream));
        lb_update(s);
        MAPPG_CUDA(cudaMemsetAsync(&L->dxbits, 0, sizeof(unsigned long long), s->stream));
        k_lb_dxmax<<<grid, 256, 0, s->stream>>>(N, s->x, s->x0, &L->dxbits);
        unsigned long long bits = 0;
        MAPPG_CUDA(cudaMemcpyAsync(&bits, &L->dxbits, sizeof(bits), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        double dx;
        memcpy(&dx, &bits, sizeof(dx));
        if (1.7320508075688772 * (a * hmax + dx) < 0.5 * s->skin) mode = DELTA;
    }
    // skin test, gated rebuild, then the FP32 energy
    static double energy32(mappg_sys* s) {
        lb_update(s);
        launch_energy(s);
        double e;
        MAPPG_CUDA(cudaMemcpyAsync(&e, &s->sc->energy, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        return e;
    }
};

// grid of the FP64 vector kernels with grid-wide sums: two blocks per SM, so
// that each thread adds up N / (2 x SMs x 256) components (~10 for 250,000
// atoms) before the block and last-block reductions, whose FP64 shuffle
// trees would otherwise cost more than the components themselves (the order
// stays fixed for a given N)
static int lb_grid(mappg_sys* s, int N) { return std::max(1, std::min((N + 255) / 256, 2 * s->sm_count)); }

// a mixed-precision search that fails may be FP32 force noise, not a minimum
static bool ls_failed(int err) { return err == LS_MIN_ALPHA || err == B_F_DOWNHILL; }

void lbfgs_run(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, const LsParams& ls, int nsteps,
               double* stats, const double* P, long long* n_fallback) {
    if (m < 0 || m > 64) throw Error{MAPPG_ERR_ARG, "m must be in 0..64"};
    if (!(max_dx > 0.0)) throw Error{MAPPG_ERR_ARG, "max_dx must be positive"};
    if (!(e_tol >= 0.0)) throw Error{MAPPG_ERR_ARG, "e_tol must be >= 0"};
    if (nsteps < 0) throw Error{MAPPG_ERR_ARG, "nsteps must be >= 0"};
    const int N = 3 * s->n;
    const int grid = lb_grid(s, N);
    std::vector<void*> owned;
    auto dalloc = [&](size_t bytes) {
        void* p = nullptr;
        MAPPG_CUDA(cudaMalloc(&p, bytes));
        owned.push_back(p);
        return p;
    };
    struct Guard {
        std::vector<void*>& o;
        ~Guard() {
            for (void* p : o) cudaFree(p);
        }
    } guard{owned};
    double* f0 = (double*)dalloc(sizeof(double) * N);
    double* h = (double*)dalloc(sizeof(double) * N);
    double* xs = (double*)dalloc(sizeof(double) * N);
    std::vector<double*> sv(m), yv(m);
    for (int i = 0; i < m; i++) {
        sv[i] = (double*)dalloc(sizeof(double) * N);
        yv[i] = (double*)dalloc(sizeof(double) * N);
    }
    LbScal* L = (LbScal*)dalloc(sizeof(LbScal));
    unsigned* counter = (unsigned*)dalloc(sizeof(unsigned) * 4);
    MAPPG_CUDA(cudaMemsetAsync(L, 0, sizeof(LbScal), s->stream));
    MAPPG_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned) * 4, s->stream));
    const double one = 1.0;  // gamma starts at 1 (min_l-bfgs.h:140), as does tau
    MAPPG_CUDA(cudaMemcpyAsync(&L->gamma, &one, sizeof(double), cudaMemcpyHostToDevice, s->stream));
    MAPPG_CUDA(cudaMemcpyAsync(&L->tau, &one, sizeof(double), cudaMemcpyHostToDevice, s->stream));
    // a mixed relaxation that stalls above f_tol (its FP32 forces no longer
    // point downhill on the FP64 energy) goes on with FP64 forces
    struct Promote {
        mappg_sys* s;
        ~Promote() { s->force64 = false; }
    } promote{s};
    cudaStream_t st = s->stream;
    double* part = s->partials;
    // mixed systems: line-search trials inside the skin take energy
    // differences (TrialLine delta mode), which need x0's FP64 density and
    // the direction as float4
    const bool mixed = s->precision == MAPPG_MIXED;
    struct KeepRho {
        mappg_sys* s;
        ~KeepRho() {
            s->keep_rho64 = false;
            s->h32 = nullptr;
        }
    } keep_rho{s};
    if (mixed) {
        s->keep_rho64 = true;
        s->h32 = (float4*)dalloc(sizeof(float4) * (size_t)s->n);
    }

    // NewDynamicMD::init then the opening force call
    sys_build(s);
    long long n_en = 0, n_fc = 1;
    double e_curr, pe_force;
    lb_force(s, &pe_force);
    // the line search's reference energy is an FP64 energy in both modes
    e_curr = s->precision == MAPPG_MIXED ? lb_energy(s) : pe_force;
    double e_prev, alpha_m = 0.0;
    int k = 0;
    int err = nsteps == 0 ? MIN_F_MAX_ITER : LS_S;
    double dxmax = 0.0;
    auto read_prep = [&](double* fh, double* hh, double* hmax, double* fmax_) {
        k_lb_prep<<<grid, 256, 0, st>>>(N, s->f, h, s->x, s->x0, L, part, counter);
        MAPPG_CUDA(cudaGetLastError());
        double buf[6];
        MAPPG_CUDA(cudaMemcpyAsync(buf, &L->fh, sizeof(buf), cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        *fh = buf[0];
        *hh = buf[1];
        *hmax = buf[2];
        *fmax_ = buf[3];
        dxmax = buf[5];
    };
    double fh, hh, hmax, fmaxv;
    if (err == LS_S && f_tol > 0.0) {
        MAPPG_CUDA(cudaMemcpyAsync(h, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        read_prep(&fh, &hh, &hmax, &fmaxv);
        if (fmaxv < f_tol) err = MIN_S_FTOL;
    }
    // the two-loop recursion (min_l-bfgs.h:148-170) with the initial inverse
    // Hessian gamma*I, or diag(P) when a learned preconditioner is given
    auto two_loop = [&](bool diag) {
        MAPPG_CUDA(cudaMemcpyAsync(h, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        // first loop: alpha_i = -rho_i (s_i.h); h += alpha_i y_i
        if (k > 0) k_lb_axpy_dot<<<grid, 256, 0, st>>>(N, h, nullptr, sv[0], L, 0, 0, 0, 0, part, counter);
        for (int i = 0; i < k; i++) {
            const double* nxt = (i + 1 < k) ? sv[i + 1] : nullptr;
            k_lb_axpy_dot<<<grid, 256, 0, st>>>(N, h, yv[i], nxt, L, 1, i, i, i + 1, part, counter);
        }
        // h *= H0, and the first dot of the second loop y_{k-1}.h
        k_lb_axpy_dot<<<grid, 256, 0, st>>>(N, h, diag ? P : nullptr, k > 0 ? yv[k - 1] : nullptr, L, diag ? 4 : 3,
                                            0, 0, 64, part, counter);
        for (int i = k - 1; i > -1; i--) {
            const double* nxt = i > 0 ? yv[i - 1] : nullptr;
            k_lb_axpy_dot<<<grid, 256, 0, st>>>(N, h, sv[i], nxt, L, 2, i, 64 + (k - 1 - i), 64 + (k - i), part,
                                                counter);
        }
        MAPPG_CUDA(cudaGetLastError());
    };
    TrialLine line{s, N, grid, xs, h, &n_en, L};
    LineSearch<TrialLine> search(ls, line);
    int istep = 0;
    for (; err == LS_S; istep++) {
        if (P && s->precond_every > 0 && istep > 0 && istep % s->precond_every == 0) s->precond_refresh();
        MAPPG_CUDA(cudaMemcpyAsync(xs, s->x, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        MAPPG_CUDA(cudaMemcpyAsync(f0, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        two_loop(P != nullptr);
        e_prev = e_curr;
        read_prep(&fh, &hh, &hmax, &fmaxv);
        if (P && fh < 0.0) {
            // a non-descent preconditioned direction: plain L-BFGS instead
            if (n_fallback) (*n_fallback)++;
            two_loop(false);
            read_prep(&fh, &hh, &hmax, &fmaxv);
        }
        if (fh < 0.0) {
            MAPPG_CUDA(cudaMemcpyAsync(h, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            k = 0;
            read_prep(&fh, &hh, &hmax, &fmaxv);
        }
        // ls->min(&handler, e_curr, alpha_m, 0) (min_l-bfgs.h:173)
        double dfa = -fh, max_a;
        int lerr = LS_S;
        if (hh == 0.0) {
            max_a = 0.0;
            dfa = 0.0;
        } else if (dfa >= 0.0) {
            max_a = 0.0;
            dfa = 1.0;
        } else {
            max_a = fabs(max_dx / hmax);
        }
        // mixed: trials that keep every atom within half the skin of the
        // list's build positions (the first, largest trial moves an atom by
        // at most sqrt(3) alpha max|h_c|) take energy differences on x0's
        // list; longer searches take differences of FP32 energies
        line.mode = TrialLine::E64;
        if (mixed && !s->force64 && dfa < 0.0 && max_a > 0.0) {
            line.e0 = e_curr;
            line.hmax = hmax;
            k_lb_h32<<<grid_for(s, s->n, 256), 256, 0, st>>>(s->n, h, s->h32);
            MAPPG_CUDA(cudaGetLastError());
            const double a1 = std::min(max_a, 1.0);
            if (1.7320508075688772 * (a1 * hmax + dxmax) < 0.5 * s->skin) {
                line.mode = TrialLine::DELTA;
            } else {
                // the FP32 energy of x0 is the last force call's: the same
                // pair terms and compensated sums as the trials' energy pass
                line.mode = TrialLine::E32DIFF;
                line.e0_32 = pe_force;
            }
        }
        if (dfa == 0.0)
            lerr = LS_F_GRAD0;
        else if (max_a == 0.0)
            lerr = LS_MIN_ALPHA;
        else if (dfa >= 0.0)
            lerr = LS_F_DOWNHILL;
        else
            lerr = search.min(dfa, max_a, e_curr, alpha_m, 0);
        err = lerr;
        if (line.mode == TrialLine::DELTA) {
            // the accepted (or restored) positions: skin test, and the FP32
            // frame positions the force call reads
            lb_update(s);
        }
        if (ls_failed(err) && s->precision == MAPPG_MIXED && !s->force64 && f_tol > 0.0) {
            s->force64 = true;
            lb_force(s, &pe_force);
            n_fc++;
            e_curr = lb_energy(s);
            k = 0;
            MAPPG_CUDA(cudaMemcpyAsync(&L->gamma, &one, sizeof(double), cudaMemcpyHostToDevice, st));
            MAPPG_CUDA(cudaMemcpyAsync(&L->tau, &one, sizeof(double), cudaMemcpyHostToDevice, st));
            err = LS_S;
            istep--;
            continue;
        }
        if (err != LS_S) {
            istep--;
            continue;
        }
        // handler.force_calc(): forces and atoms->pe; e_curr stays the line
        // search's energy, as in min_l-bfgs.h:181-188
        lb_force(s, &pe_force);
        n_fc++;
        iteration_hook(s, istep);
        if (e_prev - e_curr < e_tol) err = MIN_S_TOLERANCE;
        if (f_tol > 0.0) {
            read_prep(&fh, &hh, &hmax, &fmaxv);
            if (fmaxv < f_tol) err = MIN_S_FTOL;
        }
        if (istep + 1 == nsteps) err = MIN_F_MAX_ITER;
        if (err) continue;
        if (m) {
            if (k != m) k++;
            double* ts = sv[k - 1];
            double* ty = yv[k - 1];
            for (int i = k - 1; i > 0; i--) {
                sv[i] = sv[i - 1];
                yv[i] = yv[i - 1];
            }
            sv[0] = ts;
            yv[0] = ty;
            k_lb_shift_rho<<<1, 1, 0, st>>>(L, m);
            k_lb_hist<<<grid, 256, 0, st>>>(N, sv[0], yv[0], h, f0, s->f, P, alpha_m, L, part, counter);
            MAPPG_CUDA(cudaGetLastError());
        } else {
            // gamma = alpha_m (h.f0 - h.f)/(f.f + f0.f0 - 2 f.f0) on the host
            std::vector<double> hv(N), fv(N), f0v(N);
            MAPPG_CUDA(cudaMemcpyAsync(hv.data(), h, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
            MAPPG_CUDA(cudaMemcpyAsync(fv.data(), s->f, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
            MAPPG_CUDA(cudaMemcpyAsync(f0v.data(), f0, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
            MAPPG_CUDA(cudaStreamSynchronize(st));
            double hf0 = 0, hf = 0, ff = 0, f0f0 = 0, ff0 = 0;
            for (int q = 0; q < N; q++) {
                hf0 += hv[q] * f0v[q];
                hf += hv[q] * fv[q];
                ff += fv[q] * fv[q];
                f0f0 += f0v[q] * f0v[q];
                ff0 += fv[q] * f0v[q];
            }
            double g = alpha_m * (hf0 - hf) / (ff + f0f0 - 2.0 * ff0);
            MAPPG_CUDA(cudaMemcpyAsync(&L->gamma, &g, sizeof(double), cudaMemcpyHostToDevice, st));
        }
    }
    if (f_tol <= 0.0 || err != MIN_S_FTOL) {
        MAPPG_CUDA(cudaMemcpyAsync(h, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        read_prep(&fh, &hh, &hmax, &fmaxv);
    }
    DevScalars hs;
    MAPPG_CUDA(cudaMemcpyAsync(&hs, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
    MAPPG_CUDA(cudaStreamSynchronize(st));
    if (hs.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during minimization"};
    if (hs.bad) throw Error{MAPPG_ERR_NAN, "non-finite value during minimization"};
    if (stats) {
        stats[0] = istep;
        stats[1] = pe_force;
        stats[2] = fmaxv;
        stats[3] = err;
        stats[4] = (double)n_en;
        stats[5] = (double)n_fc;
    }
}

}  // namespace mappg

// ------------------------------------------------------------------ MinCG
// md.min_cg(e_tol,max_dx,ls=ls_bt(...)).run(atoms,nsteps): MinCG::__run
// (min_cg.h:454-536), Polak-Ribiere directions h = ratio h + f with ratio =
// (f.f - f.f0)/(f0.f0), over LineSearchBackTrack::min with init_flag 1
// (ls.h:711-769: the first trial step is capped by -prev/dfa, prev being
// the previous step's decrease -dfa*alpha; LineSearch::reset, ls.h:42,
// starts prev at -1).  Same vectors and kernels as the L-BFGS driver.
namespace mappg {

// f.f and f.f0 into L->dot[0], L->dot[1]
__global__ void __launch_bounds__(256) k_cg_dots(int N, const double* __restrict__ f, const double* __restrict__ f0,
                                                 LbScal* L, double* partials, unsigned* counter) {
    double v[2] = {0.0, 0.0};
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) {
        v[0] += f[q] * f[q];
        v[1] += f[q] * f0[q];
    }
    if (lb_block<2>(v, partials, counter) && threadIdx.x < 32) {
        double t[2];
        lb_final<2>(partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            L->dot[0] = t[0];
            L->dot[1] = t[1];
            *counter = 0;
        }
    }
}

__global__ void k_cg_dir(int N, double* __restrict__ h, const double* __restrict__ f, double ratio) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) h[q] = ratio * h[q] + f[q];
}

void cg_run(mappg_sys* s, double e_tol, double max_dx, double f_tol, const LsParams& ls, int nsteps, double* stats) {
    if (!(max_dx > 0.0)) throw Error{MAPPG_ERR_ARG, "max_dx must be positive"};
    if (!(e_tol >= 0.0)) throw Error{MAPPG_ERR_ARG, "e_tol must be >= 0"};
    if (nsteps < 0) throw Error{MAPPG_ERR_ARG, "nsteps must be >= 0"};
    const int N = 3 * s->n;
    const int grid = lb_grid(s, N);
    std::vector<void*> owned;
    auto dalloc = [&](size_t bytes) {
        void* p = nullptr;
        MAPPG_CUDA(cudaMalloc(&p, bytes));
        owned.push_back(p);
        return p;
    };
    struct Guard {
        std::vector<void*>& o;
        ~Guard() {
            for (void* p : o) cudaFree(p);
        }
    } guard{owned};
    double* f0 = (double*)dalloc(sizeof(double) * N);
    double* h = (double*)dalloc(sizeof(double) * N);
    double* xs = (double*)dalloc(sizeof(double) * N);
    LbScal* L = (LbScal*)dalloc(sizeof(LbScal));
    unsigned* counter = (unsigned*)dalloc(sizeof(unsigned) * 4);
    cudaStream_t st = s->stream;
    MAPPG_CUDA(cudaMemsetAsync(L, 0, sizeof(LbScal), st));
    MAPPG_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned) * 4, st));
    double* part = s->partials;
    double dxmax = 0.0;
    auto read_prep = [&](double* fh, double* hh, double* hmax, double* fmax_) {
        k_lb_prep<<<grid, 256, 0, st>>>(N, s->f, h, s->x, s->x0, L, part, counter);
        MAPPG_CUDA(cudaGetLastError());
        double buf[6];
        MAPPG_CUDA(cudaMemcpyAsync(buf, &L->fh, sizeof(buf), cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        *fh = buf[0];
        *hh = buf[1];
        *hmax = buf[2];
        *fmax_ = buf[3];
        dxmax = buf[5];
    };
    sys_build(s);
    long long n_en = 0, n_fc = 1;
    double pe_force;
    lb_force(s, &pe_force);
    double e_curr = s->precision == MAPPG_MIXED ? lb_energy(s) : pe_force, e_prev;
    int err = nsteps == 0 ? MIN_F_MAX_ITER : LS_S;
    double fh, hh, hmax, fmaxv;
    MAPPG_CUDA(cudaMemcpyAsync(h, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    read_prep(&fh, &hh, &hmax, &fmaxv);
    if (err == LS_S && f_tol > 0.0 && fmaxv < f_tol) err = MIN_S_FTOL;
    double f0_f0 = fh;  // f.f with h = f
    TrialLine line{s, N, grid, xs, h, &n_en, L};
    LineSearch<TrialLine> search(ls, line);  // prev_val starts at -1 (LineSearch::reset)
    double alpha = 0.0;
    struct Promote {
        mappg_sys* s;
        ~Promote() { s->force64 = false; }
    } promote{s};
    int istep = 0;
    for (; err == LS_S; istep++) {
        if (f0_f0 == 0.0) {
            err = LS_F_GRAD0;
            continue;
        }
        MAPPG_CUDA(cudaMemcpyAsync(xs, s->x, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        MAPPG_CUDA(cudaMemcpyAsync(f0, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        e_prev = e_curr;
        read_prep(&fh, &hh, &hmax, &fmaxv);
        if (fh < 0.0) {
            MAPPG_CUDA(cudaMemcpyAsync(h, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            read_prep(&fh, &hh, &hmax, &fmaxv);
            fh = f0_f0;
        }
        double dfa = -fh, max_a;
        int lerr = LS_S;
        if (hh == 0.0) {
            max_a = 0.0;
            dfa = 0.0;
        } else if (dfa >= 0.0) {
            max_a = 0.0;
            dfa = 1.0;
        } else {
            max_a = fabs(max_dx / hmax);
        }
        if (dfa == 0.0)
            lerr = LS_F_GRAD0;
        else if (max_a == 0.0)
            lerr = LS_MIN_ALPHA;
        else if (dfa >= 0.0)
            lerr = LS_F_DOWNHILL;
        else
            lerr = search.min(dfa, max_a, e_curr, alpha, 1);  // init_flag 1 (min_cg.h:504)
        err = lerr;
        if (ls_failed(err) && s->precision == MAPPG_MIXED && !s->force64 && f_tol > 0.0) {
            // stalled on FP32 forces above f_tol: restart from x0 with FP64 forces
            s->force64 = true;
            lb_force(s, &pe_force);
            n_fc++;
            e_curr = lb_energy(s);
            MAPPG_CUDA(cudaMemcpyAsync(h, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            read_prep(&fh, &hh, &hmax, &fmaxv);
            f0_f0 = fh;
            search.prev_val = -1.0;
            err = LS_S;
            istep--;
            continue;
        }
        if (err != LS_S) {
            istep--;
            continue;
        }
        lb_force(s, &pe_force);
        n_fc++;
        iteration_hook(s, istep);
        if (e_prev - e_curr < e_tol) err = MIN_S_TOLERANCE;
        if (f_tol > 0.0) {
            read_prep(&fh, &hh, &hmax, &fmaxv);
            if (fmaxv < f_tol) err = MIN_S_FTOL;
        }
        if (istep + 1 == nsteps) err = MIN_F_MAX_ITER;
        if (err) continue;
        k_cg_dots<<<grid, 256, 0, st>>>(N, s->f, f0, L, part, counter);
        MAPPG_CUDA(cudaGetLastError());
        double dd[2];
        MAPPG_CUDA(cudaMemcpyAsync(dd, &L->dot[0], sizeof(dd), cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        const double ratio = (dd[0] - dd[1]) / f0_f0;
        k_cg_dir<<<grid, 256, 0, st>>>(N, h, s->f, ratio);
        MAPPG_CUDA(cudaGetLastError());
        f0_f0 = dd[0];
    }
    MAPPG_CUDA(cudaMemcpyAsync(h, s->f, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    read_prep(&fh, &hh, &hmax, &fmaxv);
    DevScalars hs;
    MAPPG_CUDA(cudaMemcpyAsync(&hs, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
    MAPPG_CUDA(cudaStreamSynchronize(st));
    if (hs.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during minimization"};
    if (hs.bad) throw Error{MAPPG_ERR_NAN, "non-finite value during minimization"};
    if (stats) {
        stats[0] = istep;
        stats[1] = pe_force;
        stats[2] = fmaxv;
        stats[3] = err;
        stats[4] = (double)n_en;
        stats[5] = (double)n_fc;
    }
}

}  // namespace mappg

// ------------------------------------------------------------------ C entry
namespace mappg {
void sys_upload(mappg_sys* s, const double* host, double* dev);  // system.cu
}

// The energy change E(x + alpha h) - E(x) of a mixed-precision system as its
// minimizers' line searches take it (k_de32), without moving the atoms.
extern "C" int mappg_sys_energy_delta(mappg_sys* s, const double* h, double alpha, double* de) {
    using namespace mappg;
    try {
        if (!s || !h || !de) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->precision != MAPPG_MIXED) throw Error{MAPPG_ERR_ARG, "energy differences are for mixed-precision systems"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "energy differences run per single cell"};
        if (!s->built) sys_build(s);
        const int n = s->n;
        double* hd = nullptr;
        float4* h32 = nullptr;
        LbScal* L = nullptr;
        unsigned* counter = nullptr;
        // released on every return, including a failed allocation or launch
        struct Free {
            double*& a;
            float4*& b;
            LbScal*& l;
            unsigned*& c;
            mappg_sys* s;
            ~Free() {
                if (a) cudaFree(a);
                if (b) cudaFree(b);
                if (l) cudaFree(l);
                if (c) cudaFree(c);
                s->h32 = nullptr;
                s->keep_rho64 = false;
            }
        } fr{hd, h32, L, counter, s};
        MAPPG_CUDA(cudaMalloc(&hd, sizeof(double) * 3 * (size_t)n));
        MAPPG_CUDA(cudaMalloc(&h32, sizeof(float4) * (size_t)n));
        // the list must hold every pair inside the cutoff at x and at x + alpha h
        double hmax = 0.0;
        for (size_t q = 0; q < 3 * (size_t)n; q++) hmax = std::max(hmax, std::fabs(h[q]));
        lb_update(s);
        sys_upload(s, h, hd);
        const int N = 3 * n, grid = grid_for(s, N, 256);
        MAPPG_CUDA(cudaMalloc(&L, sizeof(LbScal)));
        MAPPG_CUDA(cudaMalloc(&counter, sizeof(unsigned)));
        MAPPG_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), s->stream));
        k_lb_prep<<<grid, 256, 0, s->stream>>>(N, hd, hd, s->x, s->x0, L, s->partials, counter);
        MAPPG_CUDA(cudaGetLastError());
        double dxmax = 0.0;
        MAPPG_CUDA(cudaMemcpyAsync(&dxmax, &L->dxmax, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        if (!(1.7320508075688772 * (std::fabs(alpha) * hmax + dxmax) < 0.5 * s->skin))
            throw Error{MAPPG_ERR_ARG, "alpha*h moves atoms beyond the neighbour list's skin"};
        s->keep_rho64 = true;
        s->h32 = h32;
        launch_force(s);  // density of x kept in FP64, F'(rho) and forces of x
        k_lb_h32<<<grid_for(s, n, 256), 256, 0, s->stream>>>(n, hd, h32);
        launch_de32(s, alpha);
        MAPPG_CUDA(cudaMemcpyAsync(de, &s->sc->de, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        return MAPPG_OK;
    } catch (const Error& e) {
        set_error(e.msg);
        return e.code;
    } catch (const std::exception& e) {
        set_error(e.what());
        return MAPPG_ERR_ARG;
    }
}
