// NST molecular dynamics: md.nst(S,T,dt).run(atoms,nsteps) (MDNST::run,
// md_nst.cpp:374-450).  The box moves every step, driven by the box velocity
// V_H (lower triangular) that the applied stress S, the virial and the
// kinetic tensor accelerate (update_V_H, md_nst.cpp:315-341); the atoms and
// the box advance with the matrix propagators of MDMath::calc
// (md_nst.cpp:887-1000) and two Nose-Hoover chains, one for the particles and
// one for the box (thermo_baro).
//
// A step is host-driven: the 3x3 algebra and both chains run on the host in
// FP64, the per-atom updates and the force in device kernels; one host read
// per step brings back the kinetic tensor, the energy and the virial.  As the
// box changes each step, the neighbour list is rebuilt for the new box at
// every step (the reference rebuilds only past the skin; the forces are the
// same while no pair crosses the cutoff unseen).  In mixed precision the
// density and force passes are the FP32 kernels, whose forces are converted
// into the FP64 array that the per-atom updates read; the state, the box
// algebra and the chains stay FP64.
#include <math.h>
#include <string.h>

#include <limits>
#include <vector>

#include "eam_common.cuh"
#include "nhc.cuh"

namespace mappg {

void sys_alloc_bins(mappg_sys* s);
void sys_build(mappg_sys* s);

namespace {

struct M3 {
    double m[3][3];
};

struct NstAtoms {
    int n;
    double* x;
    double* v;
    const double* f;
    const uint8_t* elem;
    const uint8_t* dof;  // x_dof bits, read by the opening kinetic tensor only (null: all free)
    double masses[kMaxElem];
    M3 M0, M1, M2, VH;
    double xi;
    double* part;       // [grid][6]
    unsigned* counter;
    double* out;        // [6]
};

// row vector times lower-triangular M (V_mul_MLT order)
__host__ __device__ __forceinline__ void vmlt(const double* v, const double (&M)[3][3], double* o) {
    const double o0 = M[0][0] * v[0] + (M[1][0] * v[1] + M[2][0] * v[2]);
    const double o1 = M[1][1] * v[1] + M[2][1] * v[2];
    const double o2 = M[2][2] * v[2];
    o[0] = o0;
    o[1] = o1;
    o[2] = o2;
}

template <int K>
__device__ void nst_reduce(const NstAtoms& a, double (&v)[K]) {
    if (block_partials<K>(v, a.part, 0, a.counter)) {
        if (threadIdx.x < 32) {
            double tot[K];
            final_sums<K>(a.part, gridDim.x, tot);
            if (threadIdx.x == 0) {
                for (int k = 0; k < K; k++) a.out[k] = tot[k];
                *a.counter = 0;
            }
        }
    }
}

// first half of update_x_d__x__x_d (md_nst.cpp:70-118): v = v M0 (xi on
// the z component) + f M1 / m, w = (x V_H + v) M2, x += w; the sum of w for
// the mean shift
__global__ void __launch_bounds__(256) k_nst_x(NstAtoms a) {
    double d[3] = {0.0, 0.0, 0.0};
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double m_inv = 1.0 / a.masses[a.elem[i]];
        double v[3] = {a.v[i], a.v[n + i], a.v[2 * n + i]};
        double f[3] = {a.f[i], a.f[n + i], a.f[2 * n + i]};
        double x[3] = {a.x[i], a.x[n + i], a.x[2 * n + i]};
        double p[3], q[3], v0[3], w[3];
        // the reference scales the velocity by xi in SCL_V_mul_MLT's in-place
        // form, which applies xi to the last component only
        vmlt(v, a.M0.m, p);
        p[2] = __dmul_rn(__dmul_rn(a.xi, v[2]), a.M0.m[2][2]);
        vmlt(f, a.M1.m, q);
        for (int k = 0; k < 3; k++) v[k] = __dadd_rn(p[k], __dmul_rn(m_inv, q[k]));
        vmlt(x, a.VH.m, v0);
        for (int k = 0; k < 3; k++) v0[k] = __dadd_rn(v0[k], v[k]);
        vmlt(v0, a.M2.m, w);
        for (int k = 0; k < 3; k++) {
            a.v[k * n + i] = v[k];
            a.x[k * n + i] = __dadd_rn(x[k], w[k]);
            d[k] += w[k];
        }
    }
    nst_reduce<3>(a, d);
}

__global__ void k_nst_shift(int n, double* x, const double* dsum) {
    const double d0 = dsum[0] / (double)n, d1 = dsum[1] / (double)n, d2 = dsum[2] / (double)n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] -= d0;
        x[n + i] -= d1;
        x[2 * n + i] -= d2;
    }
}

// second half (md_nst.cpp:123-143): v = v M0 + f M1 / m, kinetic tensor
__global__ void __launch_bounds__(256) k_nst_v(NstAtoms a) {
    double t[6] = {0, 0, 0, 0, 0, 0};
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double m = a.masses[a.elem[i]], m_inv = 1.0 / m;
        double v[3] = {a.v[i], a.v[n + i], a.v[2 * n + i]};
        double f[3] = {a.f[i], a.f[n + i], a.f[2 * n + i]};
        double p[3], q[3];
        vmlt(v, a.M0.m, p);
        vmlt(f, a.M1.m, q);
        for (int k = 0; k < 3; k++) {
            v[k] = __dadd_rn(p[k], __dmul_rn(m_inv, q[k]));
            a.v[k * n + i] = v[k];
        }
        t[0] += m * v[0] * v[0];
        t[1] += m * v[0] * v[1];
        t[2] += m * v[0] * v[2];
        t[3] += m * v[1] * v[1];
        t[4] += m * v[1] * v[2];
        t[5] += m * v[2] * v[2];
    }
    nst_reduce<6>(a, t);
}

__global__ void k_nst_kinetic(NstAtoms a) {
    double t[6] = {0, 0, 0, 0, 0, 0};
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double m = a.masses[a.elem[i]];
        double v0 = a.v[i], v1 = a.v[n + i], v2 = a.v[2 * n + i];
        if (a.dof) {  // MDNVT::pre_init leaves frozen components out (md_nvt.cpp:318-330)
            const unsigned b = a.dof[i];
            if (!(b & 1u)) v0 = 0.0;
            if (!(b & 2u)) v1 = 0.0;
            if (!(b & 4u)) v2 = 0.0;
        }
        t[0] += m * v0 * v0;
        t[1] += m * v0 * v1;
        t[2] += m * v0 * v2;
        t[3] += m * v1 * v1;
        t[4] += m * v1 * v2;
        t[5] += m * v2 * v2;
    }
    nst_reduce<6>(a, t);
}

__global__ void k_scale(int N, double* v, double c) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) v[q] *= c;
}

// ------------------------------------------------------------------ MDMath
// phi(x) = (e^x - 1)/x and its derivatives, by series near 0
double phi0(double x) {
    if (fabs(x) < 0.015625) return 1.0 + x / 2.0 + x * x / 6.0 + x * x * x / 24.0;
    return (exp(x) - 1.0) / x;
}
double phi1(double x) {
    if (fabs(x) < 0.015625) return 0.5 + x / 3.0 + x * x / 8.0 + x * x * x / 30.0;
    const double e = exp(x);
    return (e - (e - 1.0) / x) / x;
}
double phi2(double x) {
    if (fabs(x) < 0.015625) return 1.0 / 3.0 + x / 4.0 + x * x / 10.0 + x * x * x / 36.0;
    const double e = exp(x);
    return (e - 2.0 * ((e - (e - 1.0) / x) / x)) / x;
}
const double kSqrtEps = sqrt(std::numeric_limits<double>::epsilon());

// first divided differences of exp and phi, second ones at three points
double dd_exp(double x, double y, double fx, double fy) {
    if (fabs(x - y) < kSqrtEps) return exp(0.5 * (x + y));
    return (fx - fy) / (x - y);
}
double dd_phi(double x, double y, double fx, double fy) {
    const double mid = 0.5 * (x + y);
    if (fabs(x - y) < sqrt(std::numeric_limits<double>::epsilon() * phi0(mid) / phi2(mid))) return phi1(mid);
    return (fx - fy) / (x - y);
}
double dd_phi3(double x, double y, double z, double f_yz, double f_zx, double f_xy) {
    const double c = phi2((x + y + z) / 3.0);
    const double lim = sqrt(std::numeric_limits<double>::epsilon() * phi0((x + y + z) / 3.0) / c);
    if (fabs(x - z) > lim) return (f_xy - f_yz) / (x - z);
    if (fabs(y - x) > lim) return (f_yz - f_zx) / (y - x);
    if (fabs(z - y) > lim) return (f_zx - f_xy) / (z - y);
    return c;
}
double dd_exp3(double x, double y, double z, double g_yz, double g_zx, double g_xy) {
    if (fabs(x - z) > kSqrtEps) return (g_xy - g_yz) / (x - z);
    if (fabs(y - x) > kSqrtEps) return (g_yz - g_zx) / (y - x);
    if (fabs(z - y) > kSqrtEps) return (g_zx - g_xy) / (z - y);
    return exp((x + y + z) / 3.0);
}

// propagators of a lower-triangular A (MDMath::calc): E = exp(-dt2 (A + a)),
// F0 = dt2 phi(-dt2 (A + a)), F1 = dt phi(dt A), the off-diagonal entries by
// divided differences of the diagonal ones
void propagators(double a, double dt, double dt2, const double (&A)[3][3], M3& E, M3& F0, M3& F1) {
    const double x = -dt2 * (A[0][0] + a), y = -dt2 * (A[1][1] + a), z = -dt2 * (A[2][2] + a);
    const double X = dt * A[0][0], Y = dt * A[1][1], Z = dt * A[2][2];
    memset(&E, 0, sizeof(E));
    memset(&F0, 0, sizeof(F0));
    memset(&F1, 0, sizeof(F1));
    F0.m[0][0] = phi0(x);
    F0.m[1][1] = phi0(y);
    F0.m[2][2] = phi0(z);
    F1.m[0][0] = phi0(X);
    F1.m[1][1] = phi0(Y);
    F1.m[2][2] = phi0(Z);
    E.m[0][0] = exp(x);
    E.m[1][1] = exp(y);
    E.m[2][2] = exp(z);
    double f_yz = 0, f_zx = 0, f_xy = 0, F_yz = 0, F_zx = 0, F_xy = 0, g_yz = 0, g_zx = 0, g_xy = 0;
    if (A[2][1] != 0.0) {
        f_yz = dd_phi(y, z, F0.m[1][1], F0.m[2][2]);
        F_yz = dd_phi(Y, Z, F1.m[1][1], F1.m[2][2]);
        g_yz = dd_exp(y, z, E.m[1][1], E.m[2][2]);
    }
    if (A[2][0] != 0.0) {
        f_zx = dd_phi(z, x, F0.m[2][2], F0.m[0][0]);
        F_zx = dd_phi(Z, X, F1.m[2][2], F1.m[0][0]);
        g_zx = dd_exp(z, x, E.m[2][2], E.m[0][0]);
    }
    if (A[1][0] != 0.0) {
        f_xy = dd_phi(x, y, F0.m[0][0], F0.m[1][1]);
        F_xy = dd_phi(X, Y, F1.m[0][0], F1.m[1][1]);
        g_xy = dd_exp(x, y, E.m[0][0], E.m[1][1]);
    }
    for (int k = 0; k < 3; k++) {
        F0.m[k][k] *= dt2;
        F1.m[k][k] *= dt;
    }
    F0.m[2][1] = -A[2][1] * dt2 * dt2 * f_yz;
    F0.m[2][0] = -A[2][0] * dt2 * dt2 * f_zx;
    F0.m[1][0] = -A[1][0] * dt2 * dt2 * f_xy;
    F1.m[2][1] = A[2][1] * dt * dt * F_yz;
    F1.m[2][0] = A[2][0] * dt * dt * F_zx;
    F1.m[1][0] = A[1][0] * dt * dt * F_xy;
    E.m[2][1] = -A[2][1] * dt2 * g_yz;
    E.m[2][0] = -A[2][0] * dt2 * g_zx;
    E.m[1][0] = -A[1][0] * dt2 * g_xy;
    if (A[1][0] == 0.0 || A[2][1] == 0.0) return;
    F0.m[2][0] += dt2 * dt2 * dt2 * A[2][1] * A[1][0] * dd_phi3(x, y, z, f_yz, f_zx, f_xy);
    F1.m[2][0] += dt * dt * dt * A[2][1] * A[1][0] * dd_phi3(X, Y, Z, F_yz, F_zx, F_xy);
    E.m[2][0] += dt2 * dt2 * A[2][1] * A[1][0] * dd_exp3(x, y, z, g_yz, g_zx, g_xy);
}

// C = L R, both lower triangular (MLT_mul_MLT order); C may alias L
void lt_mul(const double (&L)[3][3], const double (&R)[3][3], double (&C)[3][3]) {
    double T[3][3] = {};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j <= i; j++) {
            double t = R[i][j] * L[i][i];
            for (int k = i - 1; k >= j; k--) t = R[k][j] * L[i][k] + t;
            T[i][j] = t;
        }
    memcpy(C, T, sizeof(T));
}

constexpr int kVoigt[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};

struct Nst {
    mappg_sys* s;
    double T, dt, dt2, kB;
    int ndof_part, ndof_baro = 0;
    bool S_dof[3][3];
    double S[3][3], S_dev[3][3] = {}, s_hyd, tau[3][3], VH[3][3] = {}, prefac[3][3] = {};
    double B_ref[3][3], vol_ref, T_baro = 0.0, T_part, mvv[6];
    double pe, FH[6];

    // MDNST::update_V_H
    void update_V_H() {
        double M0[3][3], M1[3][3], M2[3][3];
        lt_mul(B_ref, s->box.H, M0);
        // the stress product M0^T S_dev M0 with S_dev as stored (its lower
        // triangle; the reference leaves the upper part zero)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double t = 0.0;
                for (int k = j; k < 3; k++) t += S_dev[i][k] * M0[k][j];
                M1[i][j] = t;
            }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double t = 0.0;
                for (int k = i; k < 3; k++) t += M0[k][i] * M1[k][j];
                M2[i][j] = t;
            }
        const double vol = s->box.vol;
        for (int i = 0; i < 3; i++)
            if (S_dof[i][i]) VH[i][i] += (kB * T_part + vol * s_hyd) * prefac[i][i] * dt2;
        T_baro = 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j <= i; j++)
                if (S_dof[i][j]) {
                    const double S_pe = -FH[kVoigt[i][j]] / vol;
                    VH[i][j] += (vol_ref * M2[i][j] - vol * S_pe + mvv[kVoigt[i][j]]) * prefac[i][j] * dt2;
                    T_baro += VH[i][j] * VH[i][j] * tau[i][j] * tau[i][j];
                }
        T_baro *= ndof_part * T / ndof_baro;
    }
};

}  // namespace

// S, tau: 9 doubles (row-major, lower triangle read; S NaN = no degree of
// freedom); state: V_H[9], eta[L], eta_S[L_S] in/out; thermo (nsteps+1)x23
void nst_run(mappg_sys* s, const double* S, const double* tau, double T, double dt, double kB, double t_relax, int L,
             int niters, double t_relax_S, int L_S, int niters_S, int nreset, int nsteps, double* V_H, double* eta,
             double* eta_S, double* thermo) {
    if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "NST runs on a single cell"};
    if (!(kB == kB)) throw Error{MAPPG_ERR_ARG, "boltzmann constant should be set prior to MD"};
    if (!(T > 0.0) || !(dt > 0.0)) throw Error{MAPPG_ERR_ARG, "T and dt must be positive"};
    if (L < 1 || L > kMaxChain || L_S < 1 || L_S > kMaxChain) throw Error{MAPPG_ERR_ARG, "L must be in 1..16"};
    if (niters < 1 || niters_S < 1) throw Error{MAPPG_ERR_ARG, "niters must be positive"};
    if (!(t_relax > 0.0) || !(t_relax_S > 0.0)) throw Error{MAPPG_ERR_ARG, "t_relax must be positive"};
    if (nsteps < 0) throw Error{MAPPG_ERR_ARG, "nsteps must be >= 0"};
    if (!s->have_v) throw Error{MAPPG_ERR_ARG, "velocities must be set before MD"};
    Nst q;
    q.s = s;
    q.T = T;
    q.dt = dt;
    q.dt2 = dt / 2.0;
    q.kB = kB;
    const int n = s->n;
    // x_dof: frozen components leave the degrees of freedom (MDNVT::pre_init,
    // md_nvt.cpp:265-291); their forces are zero, and otherwise the steps
    // treat them as MDNST::run does (update_x_d__x__x_d, update_x_d_final)
    q.ndof_part = 3 * n - (s->dof_frozen[0] + s->dof_frozen[1] + s->dof_frozen[2]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            const int lo = j <= i ? 3 * i + j : 3 * j + i;
            q.S_dof[i][j] = !std::isnan(S[lo]);
            q.S[i][j] = q.S_dof[i][j] ? S[lo] : 0.0;
            q.tau[i][j] = tau[lo];
            if (j <= i) q.VH[i][j] = V_H[3 * i + j];
        }
    // MDNST::pre_run_chk (md_nst.cpp:259-279): no stress along a direction in
    // which an atom is frozen
    std::string chk;
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++)
            if (q.S_dof[i][j] && s->dof_frozen[i]) {
                if (!chk.empty()) chk += "\n";
                chk += "cannot impose stress component [" + std::to_string(i) + "][" + std::to_string(j) +
                       "] while any of the atoms do not have degree freedom in " + std::to_string(i) + " direction";
            }
    if (!chk.empty()) throw Error{MAPPG_ERR_ARG, chk};
    // MDNST::pre_init (md_nst.cpp:281-311)
    for (int i = 0; i < 3; i++)
        for (int j = 0; j <= i; j++) {
            if (q.S_dof[i][j]) {
                if (!(q.tau[i][j] > 0.0)) throw Error{MAPPG_ERR_ARG, "tau must be positive"};
                q.prefac[i][j] = 1.0 / (q.tau[i][j] * q.tau[i][j] * q.ndof_part * kB * T);
                q.ndof_baro++;
                q.T_baro += q.VH[i][j] * q.VH[i][j] * q.tau[i][j] * q.tau[i][j];
            } else {
                q.S[i][j] = 0.0;
                q.VH[i][j] = 0.0;
            }
            q.S_dev[i][j] = q.S[i][j];
        }
    if (q.ndof_baro == 0) throw Error{MAPPG_ERR_ARG, "no stress component has a degree of freedom"};
    q.T_baro *= T * q.ndof_part * kB / q.ndof_baro;
    q.s_hyd = (q.S[0][0] + q.S[1][1] + q.S[2][2]) / 3.0;
    for (int i = 0; i < 3; i++) q.S_dev[i][i] = q.S[i][i] - q.s_hyd;

    NhcParams pp, pb;
    auto chain = [&](NhcParams& P, double tr, int LL, int ni, int ndof) {
        P.T = T;
        P.ddt = 0.5 * dt / (double)ni;
        P.ddt2 = 0.25 * dt / (double)ni;
        P.freq_sq = 1.0 / (tr * tr);
        P.kB = kB;
        P.ndof = ndof;
        P.ndof_kB = ndof * kB;
        P.L = LL;
        P.niters = ni;
    };
    chain(pp, t_relax, L, niters, q.ndof_part);
    chain(pb, t_relax_S, L_S, niters_S, q.ndof_baro);
    double eta_p[kMaxChain] = {0}, eta_b[kMaxChain] = {0};
    for (int k = 0; k < L; k++) eta_p[k] = eta[k];
    for (int k = 0; k < L_S; k++) eta_b[k] = eta_S[k];

    // device scratch
    const int grid = std::min(grid_for(s, n, 256), 4 * s->sm_count);
    std::vector<void*> owned;
    struct Free {
        std::vector<void*>& o;
        ~Free() {
            for (void* p : o) cudaFree(p);
        }
    } guard{owned};
    auto dalloc = [&](size_t bytes) {
        void* p = nullptr;
        MAPPG_CUDA(cudaMalloc(&p, bytes));
        owned.push_back(p);
        return p;
    };
    NstAtoms a;
    a.n = n;
    a.x = s->x;
    a.v = s->v;
    a.f = s->f;
    a.elem = s->elem;
    a.dof = s->dof;
    for (int e = 0; e < kMaxElem; e++) a.masses[e] = s->masses[e];
    a.part = (double*)dalloc(sizeof(double) * kRedSlots * grid);
    a.counter = (unsigned*)dalloc(sizeof(unsigned));
    a.out = (double*)dalloc(sizeof(double) * 8);
    a.xi = 1.0;
    cudaStream_t st = s->stream;
    MAPPG_CUDA(cudaMemsetAsync(a.counter, 0, sizeof(unsigned), st));

    auto read_force = [&](bool with_mvv) {
        DevScalars h;
        MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
        double m6[8];
        if (with_mvv) MAPPG_CUDA(cudaMemcpyAsync(m6, a.out, sizeof(double) * 6, cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        if (!std::isfinite(h.energy)) throw Error{MAPPG_ERR_NAN, "non-finite energy during the run"};
        q.pe = h.energy;
        for (int k = 0; k < 6; k++) q.FH[k] = h.virial[k];
        if (with_mvv)
            for (int k = 0; k < 6; k++) q.mvv[k] = m6[k];
    };
    int row = 0;
    auto thermo_row = [&]() {
        if (!thermo) return;
        double* r = thermo + (size_t)23 * row;
        r[0] = q.pe;
        r[1] = q.T_part;
        for (int k = 0; k < 6; k++) r[2 + k] = q.mvv[k];
        for (int k = 0; k < 6; k++) r[8 + k] = q.FH[k];
        for (int k = 0; k < 9; k++) r[14 + k] = s->box.H[k / 3][k % 3];
        row++;
    };
    auto set_box = [&](const double (&H)[3][3]) {
        double h9[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) h9[3 * i + j] = H[i][j];
        const int nb_old = s->nbins;
        sys_set_box(s, h9);
        if (s->nbins != nb_old) sys_alloc_bins(s);
        s->built = false;
    };

    // MDNVT::pre_init: kinetic tensor of the incoming velocities
    k_nst_kinetic<<<grid, 256, 0, st>>>(a);
    MAPPG_CUDA(cudaGetLastError());
    sys_build(s);
    launch_force(s);
    sync_forces64(s);  // mixed precision: the FP32 forces as the FP64 array the updates read
    read_force(true);
    q.T_part = (q.mvv[0] + (q.mvv[3] + q.mvv[5])) / (q.ndof_part * kB);
    thermo_row();
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) q.B_ref[i][j] = j <= i ? s->box.B[i][j] : 0.0;
    q.vol_ref = s->box.vol;

    double fac, fac_x_d = 1.0;
    auto baro_half = [&]() {
        fac = nhc_step(pb, eta_b, q.T_baro / T);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j <= i; j++) q.VH[i][j] *= fac;
        q.T_baro *= fac * fac;
    };
    auto part_half = [&]() {
        fac = nhc_step(pp, eta_p, q.T_part / T);
        const double f2 = fac * fac;
        for (int k = 0; k < 6; k++) q.mvv[k] *= f2;
        q.T_part *= f2;
    };
    for (int istep = 0; istep < nsteps; istep++) {
        baro_half();
        part_half();
        fac_x_d *= fac;
        q.update_V_H();
        // update_x_d__x__x_d
        M3 M0, M1, M2;
        const double tr = q.VH[0][0] + q.VH[1][1] + q.VH[2][2];
        propagators(tr / q.ndof_part, dt, q.dt2, q.VH, M0, M1, M2);
        a.M0 = M0;
        a.M1 = M1;
        a.M2 = M2;
        memcpy(a.VH.m, q.VH, sizeof(q.VH));
        a.xi = fac_x_d;
        k_nst_x<<<grid, 256, 0, st>>>(a);
        k_nst_shift<<<grid, 256, 0, st>>>(n, s->x, a.out);
        MAPPG_CUDA(cudaGetLastError());
        // H <- H (I + M2 V_H)
        double G[3][3], Hn[3][3];
        lt_mul(M2.m, q.VH, G);
        for (int k = 0; k < 3; k++) G[k][k] += 1.0;
        lt_mul(s->box.H, G, Hn);
        set_box(Hn);
        sys_build(s);
        launch_force(s);
        sync_forces64(s);
        k_nst_v<<<grid, 256, 0, st>>>(a);
        MAPPG_CUDA(cudaGetLastError());
        read_force(true);
        q.T_part = (q.mvv[0] + (q.mvv[3] + q.mvv[5])) / (q.ndof_part * kB);
        q.update_V_H();
        part_half();
        fac_x_d = fac;
        baro_half();
        if (nreset && (istep + 1) % nreset == 0) {
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) q.B_ref[i][j] = j <= i ? s->box.B[i][j] : 0.0;
            q.vol_ref = s->box.vol;
        }
        thermo_row();
        // MDNST::run's exports (md_nst.cpp:374-450): the host hook after every
        // hook_every-th step and after the last one, before the final
        // velocity scale, as md.nvt's snapshots
        if (s->hook && s->hook_every > 0 && ((istep + 1) % s->hook_every == 0 || istep + 1 == nsteps)) {
            MAPPG_CUDA(cudaStreamSynchronize(st));
            if (s->hook(s->hook_user, (long long)istep + 1) != 0)
                throw Error{MAPPG_ERR_ARG, "the iteration hook stopped the run"};
        }
    }
    // update_x_d_final
    k_scale<<<grid, 256, 0, st>>>(3 * n, s->v, fac_x_d);
    MAPPG_CUDA(cudaGetLastError());
    DevScalars h;
    MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
    MAPPG_CUDA(cudaStreamSynchronize(st));
    if (h.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during the run"};
    if (h.bad) throw Error{MAPPG_ERR_NAN, "non-finite position during the run"};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) V_H[3 * i + j] = j <= i ? q.VH[i][j] : 0.0;
    for (int k = 0; k < L; k++) eta[k] = eta_p[k];
    for (int k = 0; k < L_S; k++) eta_S[k] = eta_b[k];
}

}  // namespace mappg
