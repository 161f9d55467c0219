// Minimization with box degrees of freedom: md.min_lbfgs / md.min_cg with
// H_dof set, or with affine atoms (MinLBFGS::__run min_l-bfgs.h:113-219 and
// MinCG::__run min_cg.h:454-536 instantiated with BC = true or X = false;
// MinMDHandler min_cg.h:89-331).
//
// Every minimizer vector carries, besides the atoms' 3n components (none when
// the atoms move affinely), a box part A: the lower triangle of a 3x3 tensor
// (the vector-tensor type of new_min_vec.h).  Dot products add the box part
// after the atoms' sum, in the order (0,0) (1,0) (1,1) (2,0) (2,1) (2,2)
// (TOP, new_min_vec.h:224-322).  The force's box part is F_H masked by H_dof
// (post_force_calc_box, min_cg.h:324-329).  A search direction h moves the
// atoms along x_d = h + x0 h.A (affine: x0 h.A only) and the box along
// H0 h.A (prep_x_d / prep_x_d_affine, min_cg.h:298-321); a line-search trial
// at alpha sets x = x0 + alpha x_d, H = H0 + alpha H0 h.A, rebuilds the
// neighbour list for the new box and evaluates the energy.
//
// The atoms' vectors stay on the device (the system's layout); the box parts
// and the L-BFGS scalars are host doubles.  Dot products are deterministic
// device reductions read by the host, one per product.
#include <math.h>
#include <string.h>

#include <vector>

#include "eam_common.cuh"
#include "linesearch.h"

namespace mappg {

void sys_alloc_bins(mappg_sys* s);
void sys_build(mappg_sys* s);
void launch_energy64(mappg_sys* s);
void iteration_hook(mappg_sys* s, int istep);  // lbfgs.cu

namespace {

constexpr int kLt[6][2] = {{0, 0}, {1, 0}, {1, 1}, {2, 0}, {2, 1}, {2, 2}};
constexpr int kBlk = 256;

// sum of a[q]*b[q] and max |a[q]|, one partial pair per block, the last block
// adds them in a fixed order
__global__ void __launch_bounds__(kBlk) k_bx_dot(int N, const double* __restrict__ a, const double* __restrict__ b,
                                                 double* part, unsigned* counter, double* out) {
    double sum = 0.0, mx = 0.0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) {
        sum += a[q] * b[q];
        mx = fmax(mx, fabs(a[q]));
    }
    __shared__ double red[kBlk / 32][2];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) {
        red[w][0] = sum;
        red[w][1] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, m = 0.0;
        for (int k = 0; k < kBlk / 32; k++) {
            t += red[k][0];
            m = fmax(m, red[k][1]);
        }
        part[2 * blockIdx.x] = t;
        part[2 * blockIdx.x + 1] = m;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && w == 0) {
        __threadfence();
        double t = 0.0, m = 0.0;
        for (int k = lane; k < (int)gridDim.x; k += 32) {
            t += part[2 * k];
            m = fmax(m, part[2 * k + 1]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            t += __shfl_xor_sync(0xffffffffu, t, o);
            m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        }
        if (lane == 0) {
            out[0] = t;
            out[1] = m;
            *counter = 0;
        }
    }
}

__global__ void k_bx_scale(int N, double* __restrict__ y, double c) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) y[q] *= c;
}

// y = cy*y + cx*x
__global__ void k_bx_lin(int N, double* __restrict__ y, double cy, const double* __restrict__ x, double cx) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x)
        y[q] = cy * y[q] + cx * x[q];
}

struct Lt {
    double a[6];  // (0,0) (1,0) (1,1) (2,0) (2,1) (2,2)
};

// x_d = h + x0 h.A per atom (h null: x0 h.A), as V_mul_MLT(_add_in): component
// c is A[c][c] x0[c] + (A[c+1][c] x0[c+1] + A[c+2][c] x0[c+2])
__global__ void k_bx_dir(int n, const double* __restrict__ x0, const double* __restrict__ h, Lt A,
                         double* __restrict__ xd) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double p0 = x0[i], p1 = x0[n + i], p2 = x0[2 * n + i];
        const double d0 = A.a[0] * p0 + (A.a[1] * p1 + A.a[3] * p2);
        const double d1 = A.a[2] * p1 + A.a[4] * p2;
        const double d2 = A.a[5] * p2;
        if (h) {
            xd[i] = h[i] + d0;
            xd[n + i] = h[n + i] + d1;
            xd[2 * n + i] = h[2 * n + i] + d2;
        } else {
            xd[i] = d0;
            xd[n + i] = d1;
            xd[2 * n + i] = d2;
        }
    }
}

__global__ void k_bx_trial(int N, double* __restrict__ x, const double* __restrict__ x0, const double* __restrict__ xd,
                           double a) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < N; q += gridDim.x * blockDim.x) x[q] = x0[q] + a * xd[q];
}

// A vector of the minimizer: atoms part v on the device (null when the atoms
// are not degrees of freedom) and the box part
struct Vt {
    double* v = nullptr;
    double A[3][3] = {};
};

struct BoxMin {
    mappg_sys* s;
    int n, N, grid;
    bool X;
    bool hdof[3][3];
    double max_dx;
    cudaStream_t st;
    std::vector<void*> owned;
    double* part = nullptr;
    unsigned* counter = nullptr;
    double* res = nullptr;
    long long n_en = 0, n_fc = 0;
    double H0[3][3];   // the box at the start of the iteration
    double xdA[3][3];  // the box direction H0 h.A
    double *x0 = nullptr, *xd = nullptr;
    double pe_force = 0.0;

    BoxMin(mappg_sys* s_, bool X_, const int* H_dof, double max_dx_) : s(s_), X(X_), max_dx(max_dx_) {
        n = s->n;
        N = 3 * n;
        grid = std::min(grid_for(s, N, kBlk), 4 * 152);
        st = s->stream;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) hdof[i][j] = j <= i && H_dof[3 * i + j] != 0;
        part = (double*)alloc(sizeof(double) * 2 * grid);
        counter = (unsigned*)alloc(sizeof(unsigned));
        res = (double*)alloc(sizeof(double) * 2);
        MAPPG_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
        x0 = (double*)alloc(sizeof(double) * N);
        xd = (double*)alloc(sizeof(double) * N);
    }
    ~BoxMin() {
        for (void* p : owned) cudaFree(p);
    }
    void* alloc(size_t bytes) {
        void* p = nullptr;
        MAPPG_CUDA(cudaMalloc(&p, bytes));
        owned.push_back(p);
        return p;
    }
    Vt vec() {
        Vt v;
        if (X) v.v = (double*)alloc(sizeof(double) * N);
        return v;
    }

    // device sum a.b and max|a| of the atoms' parts
    void dev_dot(const double* a, const double* b, double* sum, double* mx) {
        k_bx_dot<<<grid, kBlk, 0, st>>>(N, a, b, part, counter, res);
        MAPPG_CUDA(cudaGetLastError());
        double r[2];
        MAPPG_CUDA(cudaMemcpyAsync(r, res, sizeof(r), cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        if (sum) *sum = r[0];
        if (mx) *mx = r[1];
    }
    // VT::operator* (new_min_vec.h:596-606): atoms' sum, then the box part
    double dot(const Vt& a, const Vt& b) {
        double r = 0.0;
        if (X) dev_dot(a.v, b.v, &r, nullptr);
        for (auto& e : kLt) r += a.A[e[0]][e[1]] * b.A[e[0]][e[1]];
        return r;
    }
    // y = cy*y + cx*x
    void lin(Vt& y, double cy, const Vt& x, double cx) {
        if (X) {
            k_bx_lin<<<grid, kBlk, 0, st>>>(N, y.v, cy, x.v, cx);
            MAPPG_CUDA(cudaGetLastError());
        }
        for (auto& e : kLt) y.A[e[0]][e[1]] = cy * y.A[e[0]][e[1]] + cx * x.A[e[0]][e[1]];
    }
    void scale(Vt& y, double c) {
        if (X) {
            k_bx_scale<<<grid, kBlk, 0, st>>>(N, y.v, c);
            MAPPG_CUDA(cudaGetLastError());
        }
        for (auto& e : kLt) y.A[e[0]][e[1]] *= c;
    }
    void copy(Vt& y, const Vt& x) {
        if (X) MAPPG_CUDA(cudaMemcpyAsync(y.v, x.v, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        memcpy(y.A, x.A, sizeof(y.A));
    }
    // y = a*x (VTMulScl assignment)
    void scaled(Vt& y, double a, const Vt& x) { lin(y, 0.0, x, a); }

    // ForceFieldMD::derivative + post_force_calc_box: atoms' forces (in s->f)
    // and F_H masked by H_dof into f's box part
    void force(Vt& f) {
        launch_force(s);
        sync_forces64(s);
        DevScalars h;
        MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        if (!std::isfinite(h.energy)) throw Error{MAPPG_ERR_NAN, "non-finite energy during minimization"};
        pe_force = h.energy;
        static const int vi[6] = {0, 0, 0, 1, 1, 2}, vj[6] = {0, 1, 2, 1, 2, 2};
        double FH[3][3];
        for (int k = 0; k < 6; k++) FH[vi[k]][vj[k]] = FH[vj[k]][vi[k]] = h.virial[k];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) f.A[i][j] = (j <= i && hdof[i][j]) ? FH[i][j] : 0.0;
        if (X) f.v = s->f;
        n_fc++;
    }

    double energy() {
        if (s->precision == MAPPG_MIXED)
            launch_energy64(s);
        else
            launch_energy(s);
        double e;
        MAPPG_CUDA(cudaMemcpyAsync(&e, &s->sc->energy, sizeof(double), cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        return e;
    }

    void set_box(const double (&H)[3][3]) {
        double h9[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) h9[3 * i + j] = H[i][j];
        const int nb_old = s->nbins;
        sys_set_box(s, h9);
        if (s->nbins != nb_old) sys_alloc_bins(s);
        s->built = false;
    }

    // x0 = x (atoms and box)
    void save_x0() {
        MAPPG_CUDA(cudaMemcpyAsync(x0, s->x, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        memcpy(H0, s->box.H, sizeof(H0));
    }

    // MinMDHandler::prep: x_d for the atoms, H0 h.A for the box, and
    // max|x_d| (GetMaxAlphaX)
    double prep(const Vt& h) {
        Lt A;
        for (int k = 0; k < 6; k++) A.a[k] = h.A[kLt[k][0]][kLt[k][1]];
        k_bx_dir<<<std::min(grid_for(s, n, kBlk), 4 * 152), kBlk, 0, st>>>(n, x0, X ? h.v : nullptr, A, xd);
        MAPPG_CUDA(cudaGetLastError());
        // MLT_mul_MLT(H0, h.A): entry (i,j) sums H0[i][k] hA[k][j] for k = j..i
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double t = 0.0;
                if (j <= i) {
                    t = H0[i][i] * h.A[i][j];
                    for (int k = i - 1; k >= j; k--) t = H0[i][k] * h.A[k][j] + t;
                }
                xdA[i][j] = t;
            }
        double mx;
        dev_dot(xd, xd, nullptr, &mx);
        return mx;
    }

    // MinMDHandler::F: x = x0 + a x_d, H = H0 + a H0 h.A, list for the new
    // box, energy
    double F(double a) {
        double H[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) H[i][j] = H0[i][j] + a * xdA[i][j];
        set_box(H);
        k_bx_trial<<<grid, kBlk, 0, st>>>(N, s->x, x0, xd, a);
        MAPPG_CUDA(cudaGetLastError());
        sys_build(s);
        n_en++;
        return energy();
    }
    void reset() {
        set_box(H0);
        MAPPG_CUDA(cudaMemcpyAsync(s->x, x0, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        sys_build(s);
    }
};

}  // namespace

// method 0: L-BFGS (m history pairs), 1: conjugate gradients.
// stats: iterations, pe, max|F| of the atoms, stop code, energy calls, force calls
void box_min_run(mappg_sys* s, int method, int m, double e_tol, double max_dx, const int* H_dof, bool affine,
                 const LsParams& ls, int nsteps, double* stats) {
    if (method != 0 && method != 1) throw Error{MAPPG_ERR_ARG, "method must be 0 (L-BFGS) or 1 (CG)"};
    if (m < 0 || m > 64) throw Error{MAPPG_ERR_ARG, "m must be in 0..64"};
    if (!(max_dx > 0.0)) throw Error{MAPPG_ERR_ARG, "max_dx must be positive"};
    if (!(e_tol >= 0.0)) throw Error{MAPPG_ERR_ARG, "e_tol must be >= 0"};
    if (nsteps < 0) throw Error{MAPPG_ERR_ARG, "nsteps must be >= 0"};
    BoxMin B(s, !affine, H_dof, max_dx);
    const bool X = B.X;
    Vt f, f0 = B.vec(), h = B.vec();
    std::vector<Vt> sv, yv;
    std::vector<double> rho(m ? m : 1), alph(m ? m : 1);
    if (method == 0)
        for (int i = 0; i < m; i++) {
            sv.push_back(B.vec());
            yv.push_back(B.vec());
        }
    struct Line {
        BoxMin& b;
        double F(double a) { return b.F(a); }
        void reset() { b.reset(); }
    } line{B};
    LineSearch<Line> search(ls, line);

    // NewDynamicMD::init, then handler.force_calc()
    sys_build(s);
    B.force(f);
    double e_curr = s->precision == MAPPG_MIXED ? B.energy() : B.pe_force, e_prev;
    int err = nsteps == 0 ? MIN_F_MAX_ITER : LS_S;
    double f_h, alpha_m = 0.0, gamma = 1.0, f0_f0 = 0.0;
    int k = 0;
    if (method == 1) {
        B.copy(h, f);
        f0_f0 = B.dot(f, f);
    }
    int istep = 0;
    for (; err == LS_S; istep++) {
        if (method == 1 && f0_f0 == 0.0) {
            err = LS_F_GRAD0;
            continue;
        }
        B.save_x0();
        B.copy(f0, f);
        if (method == 0) {
            // two-loop recursion over the vector-tensor history (min_l-bfgs.h:148-170)
            B.copy(h, f);
            for (int i = 0; i < k; i++) {
                alph[i] = -rho[i] * B.dot(sv[i], h);
                B.lin(h, 1.0, yv[i], alph[i]);
            }
            B.scale(h, gamma);
            for (int i = k - 1; i > -1; i--) {
                double scl0 = -alph[i] - rho[i] * B.dot(yv[i], h);
                B.lin(h, 1.0, sv[i], scl0);
            }
        }
        e_prev = e_curr;
        f_h = B.dot(f, h);
        if (f_h < 0.0) {
            B.copy(h, f);
            if (method == 0) {
                k = 0;
                f_h = B.dot(f, f);
            } else {
                f_h = f0_f0;
            }
        }
        const double max_xd = B.prep(h);
        // MinMDHandler::ls_prep
        double h_norm = B.dot(h, h), dfa = -f_h, max_a;
        int lerr;
        if (h_norm == 0.0) {
            max_a = 0.0;
            dfa = 0.0;
        } else if (dfa >= 0.0) {
            max_a = 0.0;
            dfa = 1.0;
        } else {
            max_a = fabs(max_dx / max_xd);
        }
        if (dfa == 0.0)
            lerr = LS_F_GRAD0;
        else if (max_a == 0.0)
            lerr = LS_MIN_ALPHA;
        else if (dfa >= 0.0)
            lerr = LS_F_DOWNHILL;
        else
            lerr = search.min(dfa, max_a, e_curr, alpha_m, method == 0 ? 0 : 1);
        err = lerr;
        if (err != LS_S) {
            istep--;
            continue;
        }
        B.force(f);
        iteration_hook(s, istep);
        if (e_prev - e_curr < e_tol) err = MIN_S_TOLERANCE;
        if (istep + 1 == nsteps) err = MIN_F_MAX_ITER;
        if (err) continue;
        if (method == 1) {
            double f_f = B.dot(f, f), f_f0 = B.dot(f, f0);
            double ratio = (f_f - f_f0) / f0_f0;
            B.lin(h, ratio, f, 1.0);
            f0_f0 = f_f;
        } else if (m) {
            if (k != m) k++;
            // cyclic_shift of the history (new_min_vec.h:902-935)
            Vt ts = sv[k - 1], ty = yv[k - 1];
            for (int i = k - 1; i > 0; i--) {
                sv[i] = sv[i - 1];
                yv[i] = yv[i - 1];
            }
            sv[0] = ts;
            yv[0] = ty;
            for (int i = m - 1; i > 0; i--) rho[i] = rho[i - 1];
            B.scaled(sv[0], alpha_m, h);
            B.copy(yv[0], f0);
            B.lin(yv[0], 1.0, f, -1.0);
            double inner0 = B.dot(sv[0], yv[0]);
            double inner1 = B.dot(yv[0], yv[0]);
            gamma = inner0 / inner1;
            rho[0] = 1.0 / inner0;
        } else {
            gamma = alpha_m * (B.dot(h, f0) - B.dot(h, f)) / (B.dot(f, f) + B.dot(f0, f0) - 2.0 * B.dot(f, f0));
        }
    }
    double fmaxv = 0.0;
    if (X) B.dev_dot(s->f, s->f, nullptr, &fmaxv);
    DevScalars hs;
    MAPPG_CUDA(cudaMemcpyAsync(&hs, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    if (hs.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during minimization"};
    if (hs.bad) throw Error{MAPPG_ERR_NAN, "non-finite value during minimization"};
    if (stats) {
        stats[0] = istep;
        stats[1] = B.pe_force;
        stats[2] = fmaxv;
        stats[3] = err;
        stats[4] = (double)B.n_en;
        stats[5] = (double)B.n_fc;
    }
}

}  // namespace mappg
