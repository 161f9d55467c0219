// L-BFGS over a batch of independent cells: every cell runs its own
// MinLBFGS::__run (min_l-bfgs.h:113-219) with back-tracking line search
// (ls.h:711-769), with its own history, gamma, step length and stopping
// state, while the kernels of one phase cover all cells at once.
//
// Phases of an iteration (cells that have stopped sit out):
//   direction   x0 = x, f0 = f, h = f; two-loop recursion over the cell's
//               history (per-cell dot products), initial inverse Hessian
//               gamma*I or the learned diag(P); non-descent -> plain, then
//               h = f with the history dropped (as the reference)
//   line search x = x0 + a h for the cells still searching; one energy pass
//               over the batch gives every cell its trial energy; Armijo
//               test per cell; a *= rho until accepted or below min_alpha
//   force       one force pass; per-cell max|F|, tolerances, history update
// History slots form a ring per cell: the i-th newest pair (s, y) of cell c
// is slot (head_c - i) mod m.  Per-cell sums come from per-chunk partials
// (chunks never cross cells) added by one warp per cell in a fixed order.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "system.h"

namespace mappg {

void sys_build(mappg_sys* s);
void lb_update(mappg_sys* s);
void launch_force(mappg_sys* s);
void launch_energy(mappg_sys* s);
void sync_forces64(mappg_sys* s);
void launch_energy64(mappg_sys* s);
void launch_energy32(mappg_sys* s, const EamArgs& a);  // eam32.cu
void launch_de32b(mappg_sys* s, const double* cell_alpha);

constexpr int kBlMaxHist = 32;
enum BlState { BL_RUN = 0, BL_PLAIN = 1, BL_LS = 2, BL_ACCEPT = 3, BL_DONE = 4 };
enum BlErr { BL_S = 0, BL_DOWNHILL = 1, BL_GRAD0 = 2, BL_MIN_ALPHA = 3, BL_ETOL = 4, BL_MAXITER = 5, BL_FTOL = 100 };

struct BlCell {
    double gamma, tau, rho[kBlMaxHist], alpha[kBlMaxHist];
    double dot;
    double fh, hh, hmax, fmax;
    double e_curr, e_prev, e0, a, dfa, pe;
    double dxmax;  // max |x - x_build| component over the cell's atoms
    double e0_32;  // FP32 energy of x0 (searches of FP32 energy differences)
    int k, head, state, err, niter, n_en, n_fc, nfb;
};

// how a line search of mixed-precision cells takes trial energies
enum BlEnergy { BL_E64 = 0, BL_EDELTA = 1, BL_E32DIFF = 2 };

struct BlArgs {
    int n, ncell, nchunk, m;
    const int* chunk_begin;
    const int* chunk_cell;
    const int* cell_chunk;
    const int* cell_of;
    BlCell* cs;
    const CellMd* cmd;
    double *x, *x0, *f, *f0, *h;
    const double* P;
    double *S, *Y;   // [m][3n]
    double* part;    // [nchunk][4]
    int* count;      // cells still searching
    double c_ls, rho_ls, min_alpha, max_dx, e_tol, f_tol;
    int nsteps;
    int emode;              // BlEnergy of the current search
    const double* xb;       // neighbour list build positions
    double skin_half;
    uint8_t* active;        // per cell: the chunk kernels work on it
    double* alpha_cell;     // per cell trial step (energy differences)
    uint8_t* cell_reb;      // per cell: rebuild its list at the next list check
    DevScalars* sc;
};

__device__ __forceinline__ int slot_of(const BlCell& c, int i, int m) { return (c.head - i + m) % m; }

// block sums (K <= 4) of one chunk into part[ch][0..K-1]; op 1 = max
template <int K>
__device__ __forceinline__ void bl_store(const double (&v)[K], const int (&op)[K], double* out) {
    __shared__ double red[8][4];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_xor_sync(0xffffffffu, t, o);
            t = op[k] ? fmax(t, u) : t + u;
        }
        if (lane == 0) red[w][k] = t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int q = 0; q < nw; q++) t = op[threadIdx.x] ? fmax(t, red[q][threadIdx.x]) : t + red[q][threadIdx.x];
        out[threadIdx.x] = t;
    }
    __syncthreads();
}

// per-cell totals of part[.][k] over the cell's chunks (warp per cell)
__device__ __forceinline__ double bl_cell_total(const BlArgs& a, int c, int k, bool is_max) {
    const int lane = threadIdx.x & 31;
    double t = 0.0;
    for (int ch = a.cell_chunk[c] + lane; ch < a.cell_chunk[c + 1]; ch += 32) {
        const double v = a.part[(size_t)ch * 4 + k];
        t = is_max ? fmax(t, v) : t + v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, t, o);
        t = is_max ? fmax(t, u) : t + u;
    }
    return t;
}

// x0 = x, f0 = f, h = f for the cells in `st`
__global__ void k_bl_start(BlArgs a, int st) {
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int s = a.cs[a.cell_of[i]].state;
        if (s != st) continue;
        for (int q = 0; q < 3; q++) {
            const size_t j = (size_t)q * n + i;
            if (st == BL_RUN) {
                a.x0[j] = a.x[j];
                a.f0[j] = a.f[j];
            }
            a.h[j] = a.f[j];
        }
    }
}

// one step of the recursion for the cells in `st`, chunk by chunk:
//   mode 0: dot = V[slot(i)].h only
//   mode 1: h += alpha_i Y[slot(i)] with alpha_i = -rho dot (first loop)
//   mode 2: h += (-alpha_i - rho dot) S[slot(i)]      (second loop)
//   mode 3: h *= gamma, mode 4: h *= tau P (the learned diagonal, scaled
//   by (s.y)/(y.P.y) of the newest pair)
// then the partial of the next dot, Vn[slot(i_next)].h (none if Vn null)
__global__ void __launch_bounds__(256) k_bl_step(BlArgs a, int st, int mode, int i, const double* __restrict__ Vu,
                                                 const double* __restrict__ Vn, int i_next) {
    const int n = a.n;
    const size_t N3 = 3 * (size_t)n;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const BlCell& c = a.cs[a.chunk_cell[ch]];
        const bool on = c.state == st;
        if (!on) continue;  // uniform per block: the chunk's partial is not read
        double coef = 0.0;
        int su = 0, sn = 0;
        if (on) {
            if (mode == 1 && i < c.k) coef = c.alpha[i];
            if (mode == 2 && i < c.k) coef = -c.alpha[i] - c.rho[slot_of(c, i, a.m)] * c.dot;
            if (mode == 3) coef = c.gamma;
            su = slot_of(c, i, a.m);
            sn = slot_of(c, i_next, a.m);
        }
        double acc = 0.0;
        const bool dot_on = on && Vn && i_next >= 0 && i_next < c.k;
        for (int ii = a.chunk_begin[ch] + threadIdx.x; ii < a.chunk_begin[ch + 1]; ii += blockDim.x) {
            if (!on) break;
            for (int q = 0; q < 3; q++) {
                const size_t j = (size_t)q * n + ii;
                double hv = a.h[j];
                if ((mode == 1 || mode == 2) && coef != 0.0) hv += coef * Vu[(size_t)su * N3 + j];
                if (mode == 3) hv *= coef;
                if (mode == 4) hv *= c.tau * a.P[j];
                if (mode) a.h[j] = hv;
                if (dot_on) acc += Vn[(size_t)sn * N3 + j] * hv;
            }
        }
        const double v[1] = {acc};
        const int op[1] = {0};
        bl_store<1>(v, op, a.part + (size_t)ch * 4);
    }
}

// per-cell dot from the chunk partials; mode 1 also forms alpha_i
__global__ void k_bl_cells_dot(BlArgs a, int st, int set_alpha, int i) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    const double t = bl_cell_total(a, c, 0, false);
    if ((threadIdx.x & 31) != 0) return;
    BlCell& cs = a.cs[c];
    if (cs.state != st) return;
    cs.dot = t;
    if (set_alpha) cs.alpha[i] = i < cs.k ? -cs.rho[slot_of(cs, i, a.m)] * t : 0.0;
}

// f.h, h.h, max|h|, max|f| per chunk (cells in `st`, or all with st < 0)
__global__ void __launch_bounds__(256) k_bl_prep(BlArgs a, int st) {
    const int n = a.n;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const bool on = st < 0 || a.cs[a.chunk_cell[ch]].state == st;
        if (!on) continue;
        double v[4] = {0.0, 0.0, 0.0, 0.0};
        for (int ii = a.chunk_begin[ch] + threadIdx.x; on && ii < a.chunk_begin[ch + 1]; ii += blockDim.x)
            for (int q = 0; q < 3; q++) {
                const size_t j = (size_t)q * n + ii;
                const double hv = a.h[j], fv = a.f[j];
                v[0] += fv * hv;
                v[1] += hv * hv;
                v[2] = fmax(v[2], fabs(hv));
                v[3] = fmax(v[3], fabs(fv));
            }
        const int op[4] = {0, 0, 1, 1};
        bl_store<4>(v, op, a.part + (size_t)ch * 4);
    }
}

// after the direction: learned cells with a non-descent direction go to
// BL_PLAIN (recomputed with gamma*I); plain ones fall back to h = f
__global__ void k_bl_cells_dir(BlArgs a, int st, int learned) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    double t[4];
    for (int k = 0; k < 4; k++) t[k] = bl_cell_total(a, c, k, k >= 2);
    if ((threadIdx.x & 31) != 0) return;
    BlCell& cs = a.cs[c];
    if (cs.state != st) return;
    cs.fh = t[0];
    cs.hh = t[1];
    cs.hmax = t[2];
    cs.fmax = t[3];
    if (cs.fh < 0.0) cs.state = learned ? BL_PLAIN : BL_LS;  // BL_LS marks "reset to h = f" here
    else cs.state = BL_ACCEPT;                               // direction final
    if (learned && cs.fh < 0.0) cs.nfb++;
}

// h = f and the history dropped for the cells marked by k_bl_cells_dir
__global__ void k_bl_reset_dir(BlArgs a) {
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const BlCell& c = a.cs[a.cell_of[i]];
        if (c.state != BL_LS) continue;
        for (int q = 0; q < 3; q++) a.h[(size_t)q * n + i] = a.f[(size_t)q * n + i];
    }
}

// line-search set-up per cell (LineSearchBackTrack::min, ls.h:711-740)
__global__ void k_bl_cells_ls_init(BlArgs a) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    double t[4];
    for (int k = 0; k < 4; k++) t[k] = bl_cell_total(a, c, k, k >= 2);
    if ((threadIdx.x & 31) != 0) return;
    BlCell& cs = a.cs[c];
    if (cs.state == BL_DONE) return;
    if (cs.state == BL_LS) cs.k = 0;  // direction reset to f: history dropped
    cs.fh = t[0];
    cs.hh = t[1];
    cs.hmax = t[2];
    cs.e_prev = cs.e_curr;
    double dfa = -cs.fh, max_a;
    if (cs.hh == 0.0) {
        max_a = 0.0;
        dfa = 0.0;
    } else if (dfa >= 0.0) {
        max_a = 0.0;
        dfa = 1.0;
    } else {
        max_a = fabs(a.max_dx / cs.hmax);
    }
    int err = BL_S;
    if (dfa == 0.0) err = BL_GRAD0;
    else if (max_a == 0.0) err = BL_MIN_ALPHA;
    else if (dfa >= 0.0) err = BL_DOWNHILL;
    else {
        max_a = fmin(max_a, 1.0);
        if (max_a <= a.min_alpha) err = BL_MIN_ALPHA;
    }
    if (err != BL_S) {
        cs.err = err;
        cs.state = BL_DONE;
        return;
    }
    cs.dfa = dfa;
    cs.a = max_a;
    cs.e0 = cs.e_curr;
    cs.state = BL_LS;
}

// x = x0 + a h for the cells searching (MinMDHandler::F, min_cg.h:260-267)
__global__ void k_bl_trial(BlArgs a) {
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const BlCell& c = a.cs[a.cell_of[i]];
        if (c.state != BL_LS) continue;
        for (int q = 0; q < 3; q++) {
            const size_t j = (size_t)q * n + i;
            a.x[j] = a.x0[j] + c.a * a.h[j];
        }
    }
}

// Armijo test of every searching cell on its trial energy: the FP64
// energy, x0's energy plus the energy difference of the trial, or plus the
// difference of two FP32 energies
__global__ void k_bl_cells_ls(BlArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncell) return;
    BlCell& cs = a.cs[c];
    if (cs.state != BL_LS) return;
    const double e = a.cmd[c].energy;
    const double cur = a.emode == BL_EDELTA ? cs.e0 + e : a.emode == BL_E32DIFF ? cs.e0 + (e - cs.e0_32) : e;
    cs.n_en++;
    if (cur <= cs.e0 + cs.a * a.c_ls * cs.dfa) {
        cs.e_curr = cur;
        cs.state = BL_ACCEPT;
        return;
    }
    cs.a *= a.rho_ls;
    if (cs.a <= a.min_alpha) {
        cs.e_curr = cs.e0;
        cs.err = BL_MIN_ALPHA;
        cs.state = BL_DONE;
        cs.a = -1.0;  // marks "restore x0"
        return;
    }
    atomicAdd(a.count, 1);
}

// failed searches go back to x0
__global__ void k_bl_restore(BlArgs a) {
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const BlCell& c = a.cs[a.cell_of[i]];
        if (!(c.state == BL_DONE && c.a == -1.0)) continue;
        for (int q = 0; q < 3; q++) a.x[(size_t)q * n + i] = a.x0[(size_t)q * n + i];
    }
}

// after the force pass: tolerances and, for cells going on, the history
// pair of this step: S[head] = a h, Y[head] = f0 - f, with s.y and y.y
__global__ void __launch_bounds__(256) k_bl_hist(BlArgs a) {
    const int n = a.n;
    const size_t N3 = 3 * (size_t)n;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const BlCell& c = a.cs[a.chunk_cell[ch]];
        const bool on = c.state == BL_ACCEPT;
        if (!on) continue;
        const int hd = (c.head + 1) % a.m;
        double v[4] = {0.0, 0.0, 0.0, 0.0};
        for (int ii = a.chunk_begin[ch] + threadIdx.x; on && ii < a.chunk_begin[ch + 1]; ii += blockDim.x)
            for (int q = 0; q < 3; q++) {
                const size_t j = (size_t)q * n + ii;
                const double sv = c.a * a.h[j], yv = a.f0[j] - a.f[j];
                if (a.m > 0) {
                    a.S[(size_t)hd * N3 + j] = sv;
                    a.Y[(size_t)hd * N3 + j] = yv;
                }
                v[0] += sv * yv;
                v[1] += yv * yv;
                v[2] = fmax(v[2], fabs(a.f[j]));
                if (a.P) v[3] += yv * yv * a.P[j];
            }
        const int op[4] = {0, 0, 1, 0};
        bl_store<4>(v, op, a.part + (size_t)ch * 4);
    }
}

__global__ void k_bl_cells_step(BlArgs a) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    const double sy = bl_cell_total(a, c, 0, false);
    const double yy = bl_cell_total(a, c, 1, false);
    const double fm = bl_cell_total(a, c, 2, true);
    const double ypy = bl_cell_total(a, c, 3, false);
    if ((threadIdx.x & 31) != 0) return;
    BlCell& cs = a.cs[c];
    if (cs.state != BL_ACCEPT) return;
    cs.n_fc++;
    cs.niter++;
    cs.pe = a.cmd[c].energy;
    cs.fmax = fm;
    int err = BL_S;
    if (cs.e_prev - cs.e_curr < a.e_tol) err = BL_ETOL;
    if (a.f_tol > 0.0 && fm < a.f_tol) err = BL_FTOL;
    if (cs.niter == a.nsteps) err = BL_MAXITER;
    if (err != BL_S) {
        cs.err = err;
        cs.state = BL_DONE;
        return;
    }
    if (a.m > 0) {
        cs.head = (cs.head + 1) % a.m;
        if (cs.k != a.m) cs.k++;
        // a pair without positive curvature takes no part (rho = 0)
        if (sy > 0.0 && yy > 0.0) {
            cs.rho[cs.head] = 1.0 / sy;
            cs.gamma = sy / yy;
            if (ypy > 0.0) cs.tau = sy / ypy;
        } else {
            cs.rho[cs.head] = 0.0;
        }
    }
    cs.state = BL_RUN;
}

// start: per-cell energy from the opening force call, max|F|, f_tol check
__global__ void k_bl_cells_open(BlArgs a) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    const double fm = bl_cell_total(a, c, 3, true);
    if ((threadIdx.x & 31) != 0) return;
    BlCell& cs = a.cs[c];
    memset(&cs, 0, sizeof(BlCell));
    cs.gamma = 1.0;  // min_l-bfgs.h:140
    cs.tau = 1.0;
    cs.e_curr = a.cmd[c].energy;
    cs.pe = cs.e_curr;
    cs.fmax = fm;
    cs.n_fc = 1;
    cs.head = a.m > 0 ? a.m - 1 : 0;
    cs.state = BL_RUN;
    if (a.nsteps == 0) {
        cs.err = BL_MAXITER;
        cs.state = BL_DONE;
    } else if (a.f_tol > 0.0 && fm < a.f_tol) {
        cs.err = BL_FTOL;
        cs.state = BL_DONE;
    }
}

// cells whose mixed-precision search stalled above f_tol go on with FP64
// forces from where they stopped (history dropped)
__global__ void k_bl_revive(BlArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncell) return;
    BlCell& cs = a.cs[c];
    if (!(cs.state == BL_DONE && cs.err == BL_MIN_ALPHA)) return;
    cs.state = BL_RUN;
    cs.err = BL_S;
    cs.k = 0;
    cs.gamma = 1.0;
    cs.tau = 1.0;
    cs.head = a.m - 1;
    cs.a = 0.0;
    cs.e_curr = a.cmd[c].energy;
    cs.n_fc++;
    atomicAdd(a.count, 1);
}

// the chunk kernels' cell mask: cells in state st
__global__ void k_bl_active(BlArgs a, int st) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.ncell) a.active[c] = a.cs[c].state == st ? 1 : 0;
}

// per-chunk max |x - x_build| of the searching cells into part[ch][0]
__global__ void __launch_bounds__(256) k_bl_dx(BlArgs a) {
    const int n = a.n;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const bool on = a.cs[a.chunk_cell[ch]].state == BL_LS;
        if (!on) continue;
        double v[1] = {0.0};
        for (int ii = a.chunk_begin[ch] + threadIdx.x; on && ii < a.chunk_begin[ch + 1]; ii += blockDim.x)
            for (int q = 0; q < 3; q++) {
                const size_t j = (size_t)q * n + ii;
                v[0] = fmax(v[0], fabs(a.x[j] - a.xb[j]));
            }
        const int op[1] = {1};
        bl_store<1>(v, op, a.part + (size_t)ch * 4);
    }
}

// counts the searching cells whose first (largest) trial could take an atom
// beyond half the skin of the list's build positions
__global__ void k_bl_cells_bound(BlArgs a) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    const double dx = bl_cell_total(a, c, 0, true);
    if ((threadIdx.x & 31) != 0) return;
    BlCell& cs = a.cs[c];
    if (cs.state != BL_LS) return;
    cs.dxmax = dx;
    if (!(1.7320508075688772 * (cs.a * cs.hmax + dx) < a.skin_half)) atomicAdd(a.count, 1);
}

// the searching cells that fail that bound only through the distance their
// atoms moved since their list was built: their lists are rebuilt at the
// search start (the batch rebuilds cells one by one, so a cell's list can be
// older than its neighbours' in the batch); counts them
__global__ void k_bl_refresh(BlArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncell) return;
    const BlCell& cs = a.cs[c];
    if (cs.state != BL_LS) return;
    const double step = 1.7320508075688772 * cs.a * cs.hmax;
    if (step < a.skin_half && !(step + 1.7320508075688772 * cs.dxmax < a.skin_half)) {
        a.cell_reb[c] = 1;
        a.sc->rebuild = 1;
        atomicAdd(a.count, 1);
    }
}

// the search start of the searching cells after a rebuild wrapped x
__global__ void k_bl_restart(BlArgs a) {
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (a.cs[a.cell_of[i]].state != BL_LS) continue;
        for (int q = 0; q < 3; q++) a.x0[(size_t)q * n + i] = a.x[(size_t)q * n + i];
    }
}

// counts the searching cells whose next trial moves an atom by a quarter of
// the skin or more (a search of FP32 energy differences goes over to energy
// differences once none does)
__global__ void k_bl_count_long(BlArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncell) return;
    const BlCell& cs = a.cs[c];
    if (cs.state == BL_LS && !(1.7320508075688772 * cs.a * cs.hmax < 0.5 * a.skin_half)) atomicAdd(a.count, 1);
}

// the searching cells back at x0
__global__ void k_bl_restore_ls(BlArgs a) {
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (a.cs[a.cell_of[i]].state != BL_LS) continue;
        for (int q = 0; q < 3; q++) a.x[(size_t)q * n + i] = a.x0[(size_t)q * n + i];
    }
}

// per-cell trial steps for the energy-difference pass; FP32 energies of x0
__global__ void k_bl_alpha(BlArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.ncell) a.alpha_cell[c] = a.cs[c].state == BL_LS ? a.cs[c].a : 0.0;
}

__global__ void k_bl_e0_32(BlArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.ncell && a.cs[c].state == BL_LS) a.cs[c].e0_32 = a.cmd[c].energy;
}

__global__ void k_lb_h32b(int n, const double* __restrict__ h, float4* __restrict__ h32) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        h32[i] = make_float4((float)h[i], (float)h[n + i], (float)h[2 * n + i], 0.f);
}

__global__ void k_bl_count(BlArgs a, int st) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.ncell && a.cs[c].state == st) atomicAdd(a.count, 1);
}

// ------------------------------------------------------------------ host
// the rebuild chain for the cells flagged in s->cell_reb (the gate set by
// k_bl_refresh), the frame positions, and the capacity check of lb_update
static void bl_rebuild_flagged(mappg_sys* s) {
    launch_rebuild_chain(s);
    launch_shadow(s, false);
    int ov = 0;
    MAPPG_CUDA(cudaMemcpyAsync(&ov, &s->sc->overflow, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    if (ov) sys_build(s);
}

void batch_lbfgs_run(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, double c_ls, double rho_ls,
                     double min_alpha, int nsteps, const double* P, double* stats) {
    if (m < 1 || m > kBlMaxHist) throw Error{MAPPG_ERR_ARG, "m must be in 1..32 for a batch"};
    if (!(max_dx > 0.0)) throw Error{MAPPG_ERR_ARG, "max_dx must be positive"};
    if (!(e_tol >= 0.0)) throw Error{MAPPG_ERR_ARG, "e_tol must be >= 0"};
    if (nsteps < 0) throw Error{MAPPG_ERR_ARG, "nsteps must be >= 0"};
    const int n = s->n, nc = s->ncell;
    const size_t N3 = 3 * (size_t)n;
    std::vector<void*> owned;
    auto dalloc = [&](size_t bytes) {
        void* p = nullptr;
        MAPPG_CUDA(cudaMalloc(&p, bytes > 0 ? bytes : 16));
        owned.push_back(p);
        return p;
    };
    struct Guard {
        std::vector<void*>& o;
        ~Guard() {
            for (void* p : o) cudaFree(p);
        }
    } guard{owned};
    BlArgs a;
    memset(&a, 0, sizeof(a));
    a.n = n;
    a.ncell = nc;
    a.nchunk = s->nchunk;
    a.m = m;
    a.chunk_begin = s->chunk_begin;
    a.chunk_cell = s->chunk_cell;
    a.cell_chunk = s->cell_chunk;
    a.cell_of = s->cell_of;
    a.cs = (BlCell*)dalloc(sizeof(BlCell) * nc);
    a.cmd = s->cmd;
    a.x = s->x;
    a.f = s->f;
    a.x0 = (double*)dalloc(sizeof(double) * N3);
    a.f0 = (double*)dalloc(sizeof(double) * N3);
    a.h = (double*)dalloc(sizeof(double) * N3);
    a.S = (double*)dalloc(sizeof(double) * N3 * std::max(m, 1));
    a.Y = (double*)dalloc(sizeof(double) * N3 * std::max(m, 1));
    a.part = (double*)dalloc(sizeof(double) * 4 * s->nchunk);
    a.count = (int*)dalloc(sizeof(int));
    a.P = P;
    a.c_ls = c_ls;
    a.rho_ls = rho_ls;
    a.min_alpha = min_alpha;
    a.max_dx = max_dx;
    a.e_tol = e_tol;
    a.f_tol = f_tol;
    a.nsteps = nsteps;
    a.xb = s->x0;
    a.skin_half = 0.5 * s->skin;
    a.active = (uint8_t*)dalloc(nc);
    a.alpha_cell = (double*)dalloc(sizeof(double) * nc);
    a.cell_reb = s->cell_reb;
    a.sc = s->sc;
    const bool mixed = s->precision == MAPPG_MIXED;
    float4* h32 = mixed ? (float4*)dalloc(sizeof(float4) * (size_t)n) : nullptr;
    // the masks and the kept density belong to this run only
    struct Masks {
        mappg_sys* s;
        ~Masks() {
            s->cell_active = nullptr;
            s->keep_rho64 = false;
            s->h32 = nullptr;
        }
    } masks{s};
    s->keep_rho64 = mixed;
    s->h32 = h32;
    cudaStream_t st = s->stream;
    const int gc = std::min(s->nchunk, s->sm_count * 8);
    const int ga = grid_for(s, n, 256);
    const int gw = (nc * 32 + 255) / 256, g1 = (nc + 255) / 256;
    auto count = [&](int state) {
        MAPPG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
        k_bl_count<<<g1, 256, 0, st>>>(a, state);
        int h = 0;
        MAPPG_CUDA(cudaMemcpyAsync(&h, a.count, sizeof(int), cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        return h;
    };
    // the recursion for the cells in state `cst`
    auto two_loop = [&](int cst, bool diag) {
        k_bl_start<<<ga, 256, 0, st>>>(a, cst);
        if (m > 0) k_bl_step<<<gc, 256, 0, st>>>(a, cst, 0, 0, nullptr, a.S, 0);
        for (int i = 0; i < m; i++) {
            k_bl_cells_dot<<<gw, 256, 0, st>>>(a, cst, 1, i);
            k_bl_step<<<gc, 256, 0, st>>>(a, cst, 1, i, a.Y, i + 1 < m ? a.S : nullptr, i + 1);
        }
        k_bl_step<<<gc, 256, 0, st>>>(a, cst, diag ? 4 : 3, 0, nullptr, m > 0 ? a.Y : nullptr, m - 1);
        for (int i = m - 1; i >= 0; i--) {
            k_bl_cells_dot<<<gw, 256, 0, st>>>(a, cst, 0, i);
            k_bl_step<<<gc, 256, 0, st>>>(a, cst, 2, i, a.S, i > 0 ? a.Y : nullptr, i - 1);
        }
        MAPPG_CUDA(cudaGetLastError());
    };

    // NewDynamicMD::init then the opening force call
    sys_build(s);
    launch_force(s);
    sync_forces64(s);
    launch_energy64(s);  // FP64 reference energies of the line searches
    MAPPG_CUDA(cudaMemcpyAsync(a.h, a.f, sizeof(double) * N3, cudaMemcpyDeviceToDevice, st));
    k_bl_prep<<<gc, 256, 0, st>>>(a, -1);
    k_bl_cells_open<<<gw, 256, 0, st>>>(a);
    MAPPG_CUDA(cudaGetLastError());
    struct Promote {
        mappg_sys* s;
        ~Promote() { s->force64 = false; }
    } promote{s};
    for (int phase = 0; phase < 2; phase++) {
    if (phase == 1) {
        // mixed cells that stalled above f_tol: FP64 forces from here on
        if (!(s->precision == MAPPG_MIXED && f_tol > 0.0)) break;
        s->force64 = true;
        lb_update(s);
        launch_force(s);
        sync_forces64(s);
        launch_energy64(s);
        MAPPG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
        k_bl_revive<<<g1, 256, 0, st>>>(a);
        int nrev = 0;
        MAPPG_CUDA(cudaMemcpyAsync(&nrev, a.count, sizeof(int), cudaMemcpyDeviceToHost, st));
        MAPPG_CUDA(cudaStreamSynchronize(st));
        if (nrev == 0) break;
    }
    long long bit = 0;
    while (count(BL_RUN) > 0) {
        if (P && s->precond_every > 0 && bit > 0 && bit % s->precond_every == 0) s->precond_refresh();
        bit++;
        // direction: learned (or plain) two-loop for the running cells
        two_loop(BL_RUN, P != nullptr);
        k_bl_prep<<<gc, 256, 0, st>>>(a, BL_RUN);
        k_bl_cells_dir<<<gw, 256, 0, st>>>(a, BL_RUN, P != nullptr);
        if (P) {
            two_loop(BL_PLAIN, false);
            k_bl_prep<<<gc, 256, 0, st>>>(a, BL_PLAIN);
            k_bl_cells_dir<<<gw, 256, 0, st>>>(a, BL_PLAIN, 0);
        }
        k_bl_reset_dir<<<ga, 256, 0, st>>>(a);
        k_bl_prep<<<gc, 256, 0, st>>>(a, -1);
        k_bl_cells_ls_init<<<gw, 256, 0, st>>>(a);
        MAPPG_CUDA(cudaGetLastError());
        // line search over all searching cells.  Mixed cells take energy
        // differences on x0's lists when every searching cell's trials stay
        // within half the skin (BL_EDELTA), else differences of FP32
        // energies with rebuilds (large steps, where the differences are
        // large); FP64 systems and FP64-force cells compare FP64 energies.
        const int gb = (nc + 255) / 256;
        a.emode = BL_E64;
        if (mixed && !s->force64) {
            MAPPG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
            k_bl_dx<<<gc, 256, 0, st>>>(a);
            k_bl_cells_bound<<<gw, 256, 0, st>>>(a);
            int wide = 0;
            MAPPG_CUDA(cudaMemcpyAsync(&wide, a.count, sizeof(int), cudaMemcpyDeviceToHost, st));
            MAPPG_CUDA(cudaStreamSynchronize(st));
            if (wide > 0) {
                // cells held back only by an old list: rebuild those at the
                // search start (x does not move; the rebuild may wrap it,
                // so the start is taken again) and test the bound again
                MAPPG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
                k_bl_refresh<<<g1, 256, 0, st>>>(a);
                int nref = 0;
                MAPPG_CUDA(cudaMemcpyAsync(&nref, a.count, sizeof(int), cudaMemcpyDeviceToHost, st));
                MAPPG_CUDA(cudaStreamSynchronize(st));
                if (nref > 0) {
                    bl_rebuild_flagged(s);
                    k_bl_restart<<<ga, 256, 0, st>>>(a);
                    MAPPG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
                    k_bl_dx<<<gc, 256, 0, st>>>(a);
                    k_bl_cells_bound<<<gw, 256, 0, st>>>(a);
                    MAPPG_CUDA(cudaMemcpyAsync(&wide, a.count, sizeof(int), cudaMemcpyDeviceToHost, st));
                    MAPPG_CUDA(cudaStreamSynchronize(st));
                }
            }
            a.emode = wide == 0 ? BL_EDELTA : BL_E32DIFF;
            k_bl_active<<<gb, 256, 0, st>>>(a, BL_LS);
            s->cell_active = a.active;
            if (a.emode == BL_EDELTA) {
                k_lb_h32b<<<ga, 256, 0, st>>>(n, a.h, h32);
            } else {
                // each searching cell's FP32 energy of x0 is its last force
                // call's (CellMd::energy): every searching cell took a step
                // and a force call in the previous iteration (or is at the
                // opening force call)
                k_bl_e0_32<<<gb, 256, 0, st>>>(a);
            }
            MAPPG_CUDA(cudaGetLastError());
        }
        while (true) {
            k_bl_trial<<<ga, 256, 0, st>>>(a);
            if (a.emode == BL_EDELTA) {
                k_bl_active<<<gb, 256, 0, st>>>(a, BL_LS);
                k_bl_alpha<<<gb, 256, 0, st>>>(a);
                launch_de32b(s, a.alpha_cell);
            } else {
                lb_update(s);
                if (a.emode == BL_E32DIFF) {
                    k_bl_active<<<gb, 256, 0, st>>>(a, BL_LS);
                    launch_energy32(s, eam_args(s));
                } else {
                    k_bl_active<<<gb, 256, 0, st>>>(a, BL_LS);
                    s->cell_active = a.active;
                    launch_energy64(s);
                    s->cell_active = nullptr;
                }
            }
            MAPPG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
            k_bl_cells_ls<<<g1, 256, 0, st>>>(a);
            int left = 0;
            MAPPG_CUDA(cudaMemcpyAsync(&left, a.count, sizeof(int), cudaMemcpyDeviceToHost, st));
            MAPPG_CUDA(cudaStreamSynchronize(st));
            if (left == 0) break;
            if (a.emode == BL_E32DIFF) {
                // once every remaining trial is short, differences of FP32
                // energies would drown in their rounding: back to x0 (and a
                // list around it) and on with energy differences
                MAPPG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
                k_bl_count_long<<<gb, 256, 0, st>>>(a);
                int longer = 0;
                MAPPG_CUDA(cudaMemcpyAsync(&longer, a.count, sizeof(int), cudaMemcpyDeviceToHost, st));
                MAPPG_CUDA(cudaStreamSynchronize(st));
                if (longer == 0) {
                    k_bl_restore_ls<<<ga, 256, 0, st>>>(a);
                    lb_update(s);
                    MAPPG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
                    k_bl_dx<<<gc, 256, 0, st>>>(a);
                    k_bl_cells_bound<<<gw, 256, 0, st>>>(a);
                    int wide = 0;
                    MAPPG_CUDA(cudaMemcpyAsync(&wide, a.count, sizeof(int), cudaMemcpyDeviceToHost, st));
                    MAPPG_CUDA(cudaStreamSynchronize(st));
                    if (wide == 0) {
                        a.emode = BL_EDELTA;
                        k_lb_h32b<<<ga, 256, 0, st>>>(n, a.h, h32);
                        MAPPG_CUDA(cudaGetLastError());
                    }
                }
            }
        }
        k_bl_restore<<<ga, 256, 0, st>>>(a);
        lb_update(s);
        // force pass of the cells that took a step, tolerances and history
        k_bl_active<<<gb, 256, 0, st>>>(a, BL_ACCEPT);
        s->cell_active = a.active;
        launch_force(s);
        sync_forces64(s);
        s->cell_active = nullptr;
        k_bl_hist<<<gc, 256, 0, st>>>(a);
        k_bl_cells_step<<<gw, 256, 0, st>>>(a);
        MAPPG_CUDA(cudaGetLastError());
    }
    }
    DevScalars hs;
    std::vector<BlCell> cs(nc);
    MAPPG_CUDA(cudaMemcpyAsync(&hs, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, st));
    MAPPG_CUDA(cudaMemcpyAsync(cs.data(), a.cs, sizeof(BlCell) * nc, cudaMemcpyDeviceToHost, st));
    MAPPG_CUDA(cudaStreamSynchronize(st));
    if (hs.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during minimization"};
    if (hs.bad) throw Error{MAPPG_ERR_NAN, "non-finite value during minimization"};
    if (stats)
        for (int c = 0; c < nc; c++) {
            double* o = stats + 7 * (size_t)c;
            o[0] = cs[c].niter;
            o[1] = cs[c].pe;
            o[2] = cs[c].fmax;
            o[3] = cs[c].err;
            o[4] = cs[c].n_en;
            o[5] = cs[c].n_fc;
            o[6] = cs[c].nfb;
        }
}

}  // namespace mappg
