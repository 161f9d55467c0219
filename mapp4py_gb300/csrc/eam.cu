// FP64 EAM kernels over the full neighbour list (the plain path), and the
// launch dispatch for both precisions (the mixed kernels are in eam32.cu).
//
// The reference (ForceFieldEAM::__force_calc, ff_eam.cpp:65-240) walks a half
// list twice and scatters to both atoms of a pair.  Here every atom owns a
// full row, so each atom's sums are private and no atomics are needed:
//   k_density64  rho_i = sum_j rho_{e_j->e_i}(r_ij), then F(rho_i) and
//                F'(rho_i) in the same kernel (the row is complete when the
//                sum ends), with the linear extrapolation above rho_max
//                (ff_eam.cpp:180-191)
//   k_force64    f_i = sum_j -(phi'(r) + F'_i rho'_{j->i}(r) + F'_j rho'_{i->j}(r))
//                * (x_i - x_j)/r, pair energy phi/2 and virial fpair*dx(x)dx/2
//                per entry (each pair appears in both rows)
//   k_energy64   energy only (ff_eam.cpp:244-318): density and pair energy in
//                one pass, then F(rho_i)
// A group of TPA lanes serves one atom; lanes stride over the row, reduce
// with shuffles, and one lane writes the atom's results.  Per-lane energy
// and virial accumulators are reduced per block and then over blocks in a
// fixed order by the last block to finish (deterministic).
//
// Spline evaluation (value ((c3 p + c2) p + c1) p + c0, derivative
// ((3 c3 p + 2 c2) p + c1)/dr) and the index rule m = min(int(r/dr), nr-2),
// p = min(r/dr - m, 1) follow ff_eam.cpp:122-140.  Neighbour images are read
// as x_j + n*H with n from the entry's bin step and atom i's bin.
#include <math.h>

#include <algorithm>

#include "eam_common.cuh"

namespace mappg {

__device__ __forceinline__ double spl_val(const Dbl4& c, double p) { return ((c.w * p + c.z) * p + c.y) * p + c.x; }
__device__ __forceinline__ double spl_der(const Dbl4& c, double p) { return (3.0 * c.w * p + 2.0 * c.z) * p + c.y; }

// atom i's position and the bin-edge flags that turn a bin step into an image
struct Pos64 {
    double x, y, z;
    int lo[3], hi[3];
    __device__ __forceinline__ void load(const EamArgs& a, int i) {
        x = a.x[i];
        y = a.x[a.n + i];
        z = a.x[2 * a.n + i];
        int bc = a.binc[i];
        int b[3] = {bc & 1023, (bc >> 10) & 1023, (bc >> 20) & 1023};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            lo[d] = b[d] == 0;
            hi[d] = b[d] == a.nb[d] - 1;
        }
    }
    // dx = x_i - (x_j + n*H)
    __device__ __forceinline__ void delta(const EamArgs& a, const double (*sh)[3], int e, double& dx, double& dy,
                                          double& dz) const {
        const int j = entry_j(e);
        const int d0 = entry_step(e, 0), d1 = entry_step(e, 1), d2 = entry_step(e, 2);
        int n0 = (d0 < 0 && lo[0]) ? -1 : ((d0 > 0 && hi[0]) ? 1 : 0);
        int n1 = (d1 < 0 && lo[1]) ? -1 : ((d1 > 0 && hi[1]) ? 1 : 0);
        int n2 = (d2 < 0 && lo[2]) ? -1 : ((d2 > 0 && hi[2]) ? 1 : 0);
        const double* s = sh[(n0 + 1) + 3 * (n1 + 1) + 9 * (n2 + 1)];
        dx = x - (__ldg(a.x + j) + s[0]);
        dy = y - (__ldg(a.x + a.n + j) + s[1]);
        dz = z - (__ldg(a.x + 2 * a.n + j) + s[2]);
    }
};

// batch: atom i's position and image flags from its cell's bins; image
// shifts n*H from the cell's box
struct PosCell {
    double x, y, z;
    int lo[3], hi[3];
    double h6[6];
    __device__ __forceinline__ void load(const EamArgs& a, const int* cell_of, int i) {
        const CellGeo& g = a.cells[cell_of[i]];
        x = a.x[i];
        y = a.x[a.n + i];
        z = a.x[2 * a.n + i];
        const int bc = a.binc[i];
        const int b[3] = {bc & 1023, (bc >> 10) & 1023, (bc >> 20) & 1023};
        for (int d = 0; d < 3; d++) {
            lo[d] = b[d] == 0;
            hi[d] = b[d] == g.nb[d] - 1;
        }
        for (int k = 0; k < 6; k++) h6[k] = g.h6[k];
    }
    __device__ __forceinline__ void delta(const EamArgs& a, const double (*)[3], int e, double& dx, double& dy,
                                          double& dz) const {
        const int j = entry_j(e);
        const int d0 = entry_step(e, 0), d1 = entry_step(e, 1), d2 = entry_step(e, 2);
        const int n0 = (d0 < 0 && lo[0]) ? -1 : ((d0 > 0 && hi[0]) ? 1 : 0);
        const int n1 = (d1 < 0 && lo[1]) ? -1 : ((d1 > 0 && hi[1]) ? 1 : 0);
        const int n2 = (d2 < 0 && lo[2]) ? -1 : ((d2 > 0 && hi[2]) ? 1 : 0);
        // rows of H: (h0,0,0), (h1,h3,0), (h2,h4,h5)
        const double s0 = n0 * h6[0] + n1 * h6[1] + n2 * h6[2];
        const double s1 = n1 * h6[3] + n2 * h6[4];
        const double s2 = n2 * h6[5];
        dx = x - (__ldg(a.x + j) + s0);
        dy = y - (__ldg(a.x + a.n + j) + s1);
        dz = z - (__ldg(a.x + 2 * a.n + j) + s2);
    }
};

struct Smem64 {
    double sh[27][3];
    double cut_sq[kMaxElem * kMaxElem];
    __device__ void fill(const EamArgs& a) {
        for (int t = threadIdx.x; t < 27; t += blockDim.x) {
            sh[t][0] = a.shift[t][0];
            sh[t][1] = a.shift[t][1];
            sh[t][2] = a.shift[t][2];
        }
        for (int t = threadIdx.x; t < a.ne * a.ne; t += blockDim.x) cut_sq[t] = a.cut_sq[t];
        __syncthreads();
    }
};

// F(rho), F'(rho) with the reference's extrapolation above rho_max
__device__ __forceinline__ void embed64(const EamArgs& a, int ei, double rho, double& Fv, double& dFv) {
    double p = rho * a.drho_inv;
    int m = p < (double)(a.nrho - 2) ? (int)p : a.nrho - 2;
    if (m < 0) m = 0;
    p -= (double)m;
    p = fmin(p, 1.0);
    Dbl4 c = ldg4(a.F64 + (size_t)ei * a.nrho + m);
    dFv = ((3.0 * c.w * p + 2.0 * c.z) * p + c.y) * a.drho_inv;
    Fv = ((c.w * p + c.z) * p + c.y) * p + c.x;
    if (rho > a.rho_max) Fv += dFv * (rho - a.rho_max);
}

__device__ __forceinline__ int knot64(double r, const EamArgs& a, double& p) {
    p = r * a.dr_inv;
    int m = min((int)p, a.nr - 2);
    p -= (double)m;
    p = fmin(p, 1.0);
    return m;
}

// one lane's share of atom i's density (FP64)
template <int TPA, class POS>
__device__ __forceinline__ double density64_lane(const EamArgs& a, const Smem64& S, const POS& P, int ei, int i,
                                                 int lane) {
    double acc = 0.0;
    const int nn = __ldg(a.nnbr + i);
    const int* row = a.nbr + (size_t)i * a.maxnbr;
    for (int k = lane; k < nn; k += TPA) {
        const int e = __ldg(row + k);
        const int ej = entry_elem(e);
        double dx, dy, dz;
        P.delta(a, S.sh, e, dx, dy, dz);
        double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < S.cut_sq[ei * a.ne + ej]) {
            double p;
            int m = knot64(sqrt(rsq), a, p);
            acc += spl_val(ldg4(a.rho64 + (size_t)(ej * a.ne + ei * a.rho_ei) * a.nr + m), p);
        }
    }
    return acc;
}

// one lane's share of atom i's force, pair energy and virial (FP64)
template <int TPA, class POS>
__device__ __forceinline__ void force64_lane(const EamArgs& a, const Smem64& S, const POS& P, int ei, double dFi,
                                             int i, int lane, double& fx, double& fy, double& fz, double& ep,
                                             double (&w)[6]) {
    const double dri = a.dr_inv;
    const int nn = __ldg(a.nnbr + i);
    const int* row = a.nbr + (size_t)i * a.maxnbr;
    for (int k = lane; k < nn; k += TPA) {
        const int e = __ldg(row + k);
        const int ej = entry_elem(e);
        double dx, dy, dz;
        P.delta(a, S.sh, e, dx, dy, dz);
        double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < S.cut_sq[ei * a.ne + ej]) {
            const int j = entry_j(e);
            // 1/r from the FP64 reciprocal square root and r = rsq/r: one
            // root instead of a root and a division, within an ulp or two of
            // sqrt and 1/sqrt (GB300's FP64 pipe bounds this kernel)
            const double rinv = rsqrt(rsq);
            const double r = rsq * rinv;
            double p;
            const int m = knot64(r, a, p);
            const double der_i = spl_der(ldg4(a.rho64 + (size_t)(ej * a.ne + ei * a.rho_ei) * a.nr + m), p) * dri;
            double der_j = der_i;
            if (ej != ei) der_j = spl_der(ldg4(a.rho64 + (size_t)(ei * a.ne + ej * a.rho_ei) * a.nr + m), p) * dri;
            const Dbl4 cz = ldg4(a.rphi64 + (size_t)(ei * a.ne + ej) * a.nr + m);
            const double z = spl_val(cz, p);
            const double zp = spl_der(cz, p) * dri;
            const double phi = z * rinv;
            const double dphi = (zp - phi) * rinv;
            const double fp = -(dphi + dFi * der_i + __ldg(a.dF + j) * der_j) * rinv;
            const double fdx = fp * dx, fdy = fp * dy, fdz = fp * dz;
            fx += fdx;
            fy += fdy;
            fz += fdz;
            ep += phi;
            w[0] += fdx * dx;
            w[1] += fdx * dy;
            w[2] += fdx * dz;
            w[3] += fdy * dy;
            w[4] += fdy * dz;
            w[5] += fdz * dz;
        }
    }
}

template <int TPA>
__global__ void __launch_bounds__(256) k_density64(EamArgs a) {
    __shared__ Smem64 S;
    S.fill(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    double eacc = 0.0;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        double acc = 0.0;
        int ei = 0;
        if (active) {
            Pos64 P;
            P.load(a, i);
            ei = a.elem[i];
            acc = density64_lane<TPA>(a, S, P, ei, i, lane);
        }
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPA);
        if (active && lane == 0) {
            double Fv, dFv;
            embed64(a, ei, acc, Fv, dFv);
            a.rho[i] = acc;
            a.dF[i] = dFv;
            eacc += Fv;
        }
    }
    double v[1] = {eacc};
    if (block_partials<1>(v, a.partials, 15, &a.sc->counter[1]) && threadIdx.x == 0) a.sc->counter[1] = 0;
}

// batch: FP64 density per chunk, embedding energy into chunk slot 13
template <int TPA>
__global__ void __launch_bounds__(256) k_density64b(EamArgs a, const int* __restrict__ cell_of) {
    __shared__ Smem64 S;
    S.fill(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        if (a.cell_active && !a.cell_active[a.chunk_cell[ch]]) continue;
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        double eacc = 0.0;
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            const bool active = i < hi;
            double acc = 0.0;
            int ei = 0;
            if (active) {
                PosCell P;
                P.load(a, cell_of, i);
                ei = a.elem[i];
                acc = density64_lane<TPA>(a, S, P, ei, i, lane);
            }
#pragma unroll
            for (int o = TPA / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPA);
            if (active && lane == 0) {
                double Fv, dFv;
                embed64(a, ei, acc, Fv, dFv);
                a.rho[i] = acc;
                a.dF[i] = dFv;
                eacc += Fv;
            }
        }
        chunk_store<1>([&](int) { return eacc; }, a.chunk_part + (size_t)ch * kChunkSlots + 13);
    }
}

template <int TPA>
__global__ void __launch_bounds__(256) k_force64(EamArgs a) {
    __shared__ Smem64 S;
    S.fill(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    double ep = 0;
    double w[6] = {0, 0, 0, 0, 0, 0};
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        double fx = 0, fy = 0, fz = 0;
        if (active) {
            Pos64 P;
            P.load(a, i);
            const int ei = a.elem[i];
            force64_lane<TPA>(a, S, P, ei, __ldg(a.dF + i), i, lane, fx, fy, fz, ep, w);
        }
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, o, TPA);
            fy += __shfl_xor_sync(0xffffffffu, fy, o, TPA);
            fz += __shfl_xor_sync(0xffffffffu, fz, o, TPA);
        }
        if (active && lane == 0) {
            a.f[i] = fx;
            a.f[a.n + i] = fy;
            a.f[2 * a.n + i] = fz;
        }
    }
    double v[7] = {0.5 * ep, 0.5 * w[0], 0.5 * w[1], 0.5 * w[2], 0.5 * w[3], 0.5 * w[4], 0.5 * w[5]};
    if (block_partials<7>(v, a.partials, 0, &a.sc->counter[0]) && threadIdx.x < 32) {
        // totals over blocks in a fixed order; slot 15 holds the embedding
        // energy written by the density kernel on the same grid
        double tot[16];
        final_sums<16>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            a.sc->energy = tot[0] + tot[15];
            for (int k = 0; k < 6; k++) a.sc->virial[k] = tot[k + 1];
            a.sc->counter[0] = 0;
        }
    }
}

// batch: FP64 forces per chunk, pair energy and virial into slots 0-6
template <int TPA>
__global__ void __launch_bounds__(256) k_force64b(EamArgs a, const int* __restrict__ cell_of) {
    __shared__ Smem64 S;
    S.fill(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        if (a.cell_active && !a.cell_active[a.chunk_cell[ch]]) continue;
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        double ep = 0;
        double w[6] = {0, 0, 0, 0, 0, 0};
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            const bool active = i < hi;
            double fx = 0, fy = 0, fz = 0;
            if (active) {
                PosCell P;
                P.load(a, cell_of, i);
                const int ei = a.elem[i];
                force64_lane<TPA>(a, S, P, ei, __ldg(a.dF + i), i, lane, fx, fy, fz, ep, w);
            }
#pragma unroll
            for (int o = TPA / 2; o > 0; o >>= 1) {
                fx += __shfl_xor_sync(0xffffffffu, fx, o, TPA);
                fy += __shfl_xor_sync(0xffffffffu, fy, o, TPA);
                fz += __shfl_xor_sync(0xffffffffu, fz, o, TPA);
            }
            if (active && lane == 0) {
                a.f[i] = fx;
                a.f[a.n + i] = fy;
                a.f[2 * a.n + i] = fz;
            }
        }
        chunk_store<7>([&](int k) { return 0.5 * (k == 0 ? ep : w[k - 1]); }, a.chunk_part + (size_t)ch * kChunkSlots);
    }
}

// input features of the learned preconditioner, per atom: 16 Gaussian radial
// functions exp(-(r - mu_k)^2 / (2 w^2)) fc(r), mu_k = 2.0 + 3.5 k/15 A,
// w = 0.3 A, fc(r) = (1 + cos(pi r / 5.5))/2 for r < 5.5 A, summed over the
// neighbours of each species (A in 0..15, B in 16..31), and the host
// density rho_i (32); FP64 positions, FP32 sums
constexpr int kDescR = 16;
constexpr float kDescRc = 5.5f, kDescW = 0.3f;

template <int TPA, bool BATCH>
__global__ void __launch_bounds__(256) k_descriptors(EamArgs a, const int* __restrict__ cell_of,
                                                     float* __restrict__ out) {
    __shared__ Smem64 S;
    S.fill(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    const float inv2w2 = 1.f / (2.f * kDescW * kDescW);
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        float g[2 * kDescR];
#pragma unroll
        for (int q = 0; q < 2 * kDescR; q++) g[q] = 0.f;
        double rho = 0.0;
        if (active) {
            Pos64 P;
            PosCell PC;
            if (BATCH)
                PC.load(a, cell_of, i);
            else
                P.load(a, i);
            const int ei = a.elem[i];
            const int nn = __ldg(a.nnbr + i);
            const int* row = a.nbr + (size_t)i * a.maxnbr;
            for (int k = lane; k < nn; k += TPA) {
                const int e = __ldg(row + k);
                const int ej = entry_elem(e);
                double dx, dy, dz;
                if (BATCH)
                    PC.delta(a, nullptr, e, dx, dy, dz);
                else
                    P.delta(a, S.sh, e, dx, dy, dz);
                const double rsq = dx * dx + dy * dy + dz * dz;
                if (rsq < S.cut_sq[ei * a.ne + ej]) {
                    double p;
                    const int m = knot64(sqrt(rsq), a, p);
                    rho += spl_val(ldg4(a.rho64 + (size_t)(ej * a.ne + ei * a.rho_ei) * a.nr + m), p);
                }
                const float r = (float)sqrt(rsq);
                if (r < kDescRc && ej < 2) {
                    const float fc = 0.5f * (1.f + cosf(3.14159265f * r / kDescRc));
#pragma unroll
                    for (int q = 0; q < kDescR; q++) {
                        const float d = r - (2.0f + 3.5f * (float)q / 15.f);
                        const float v = expf(-d * d * inv2w2) * fc;
                        if (ej == 0)
                            g[q] += v;
                        else
                            g[kDescR + q] += v;
                    }
                }
            }
        }
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) {
#pragma unroll
            for (int q = 0; q < 2 * kDescR; q++) g[q] += __shfl_xor_sync(0xffffffffu, g[q], o, TPA);
            rho += __shfl_xor_sync(0xffffffffu, rho, o, TPA);
        }
        if (active && lane == 0) {
            float* o = out + (size_t)i * (2 * kDescR + 1);
#pragma unroll
            for (int q = 0; q < 2 * kDescR; q++) o[q] = g[q];
            o[2 * kDescR] = (float)rho;
        }
    }
}

template <int TPA>
__global__ void __launch_bounds__(256) k_energy64(EamArgs a) {
    __shared__ Smem64 S;
    S.fill(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    double ep = 0.0, eacc = 0.0;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        double acc = 0.0;
        int ei = 0;
        if (active) {
            Pos64 P;
            P.load(a, i);
            ei = a.elem[i];
            const int nn = __ldg(a.nnbr + i);
            const int* row = a.nbr + (size_t)i * a.maxnbr;
            for (int k = lane; k < nn; k += TPA) {
                const int e = __ldg(row + k);
                const int ej = entry_elem(e);
                double dx, dy, dz;
                P.delta(a, S.sh, e, dx, dy, dz);
                double rsq = dx * dx + dy * dy + dz * dz;
                if (rsq < S.cut_sq[ei * a.ne + ej]) {
                    const double rinv = rsqrt(rsq);  // as in force64_lane
                    double p;
                    const int m = knot64(rsq * rinv, a, p);
                    acc += spl_val(ldg4(a.rho64 + (size_t)(ej * a.ne + ei * a.rho_ei) * a.nr + m), p);
                    ep += spl_val(ldg4(a.rphi64 + (size_t)(ei * a.ne + ej) * a.nr + m), p) * rinv;
                }
            }
        }
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPA);
        if (active && lane == 0) {
            double Fv, dFv;
            embed64(a, ei, acc, Fv, dFv);
            eacc += Fv;
        }
    }
    double v[1] = {eacc + 0.5 * ep};
    if (block_partials<1>(v, a.partials, 0, &a.sc->counter[2]) && threadIdx.x < 32) {
        double tot[1];
        final_sums<1>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            a.sc->energy = tot[0];
            a.sc->counter[2] = 0;
        }
    }
}

// batch: FP64 energy of every cell (the line-search energies of mixed
// batches), chunk sums into slot 0 of the chunk partials
template <int TPA>
__global__ void __launch_bounds__(256) k_energy64b(EamArgs a, const int* __restrict__ cell_of) {
    __shared__ Smem64 S;
    S.fill(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        if (a.cell_active && !a.cell_active[a.chunk_cell[ch]]) continue;
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        double ep = 0.0, eacc = 0.0;
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            const bool active = i < hi;
            double acc = 0.0;
            int ei = 0;
            if (active) {
                PosCell P;
                P.load(a, cell_of, i);
                ei = a.elem[i];
                const int nn = __ldg(a.nnbr + i);
                const int* row = a.nbr + (size_t)i * a.maxnbr;
                for (int k = lane; k < nn; k += TPA) {
                    const int e = __ldg(row + k);
                    const int ej = entry_elem(e);
                    double dx, dy, dz;
                    P.delta(a, nullptr, e, dx, dy, dz);
                    const double rsq = dx * dx + dy * dy + dz * dz;
                    if (rsq < S.cut_sq[ei * a.ne + ej]) {
                        const double rinv = rsqrt(rsq);  // as in force64_lane
                        double p;
                        const int m = knot64(rsq * rinv, a, p);
                        acc += spl_val(ldg4(a.rho64 + (size_t)(ej * a.ne + ei * a.rho_ei) * a.nr + m), p);
                        ep += spl_val(ldg4(a.rphi64 + (size_t)(ei * a.ne + ej) * a.nr + m), p) * rinv;
                    }
                }
            }
#pragma unroll
            for (int o = TPA / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPA);
            if (active && lane == 0) {
                double Fv, dFv;
                embed64(a, ei, acc, Fv, dFv);
                eacc += Fv;
            }
        }
        chunk_store<1>([&](int) { return eacc + 0.5 * ep; }, a.chunk_part + (size_t)ch * kChunkSlots);
    }
}

template <int TPA>
static int grid64(mappg_sys* s) {
    return grid_for(s, (long long)s->n * TPA, 256);
}

#define MAPPG_TPA64(KERNEL)                                                                    \
    switch (s->tpa) {                                                                          \
        case 4: KERNEL<4><<<grid64<4>(s), 256, 0, s->stream>>>(a); break;                     \
        case 16: KERNEL<16><<<grid64<16>(s), 256, 0, s->stream>>>(a); break;                  \
        case 32: KERNEL<32><<<grid64<32>(s), 256, 0, s->stream>>>(a); break;                  \
        default: KERNEL<8><<<grid64<8>(s), 256, 0, s->stream>>>(a); break;                    \
    }

void launch_cells_done(mappg_sys* s, const EamArgs& a, int what);  // eam32.cu

void launch_density_only(mappg_sys* s) {
    EamArgs a = eam_args(s);
    if (s->precision == MAPPG_MIXED && !s->force64) {
        launch_density32(s, a);
        return;
    }
    if (s->ncell > 1) {
        k_density64b<8><<<std::min(s->nchunk, s->sm_count * 8), 256, 0, s->stream>>>(a, s->cell_of);
    } else {
        MAPPG_TPA64(k_density64)
    }
    MAPPG_CUDA(cudaGetLastError());
}

// ForceFieldMD::force_calc (ff_md.cpp:138-144): components without a
// degree of freedom carry no force
template <class T>
__global__ void k_dof_mask(int n, const uint8_t* __restrict__ dof, T* __restrict__ f) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned d = dof[i];
        if (d == 7u) continue;
        for (int c = 0; c < 3; c++)
            if (!((d >> c) & 1u)) f[(size_t)c * n + i] = T(0);
    }
}

void launch_dof_mask(mappg_sys* s, bool f32) {
    if (!s->dof) return;
    if (f32)
        k_dof_mask<float><<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->dof, s->f32);
    else
        k_dof_mask<double><<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->dof, s->f);
    MAPPG_CUDA(cudaGetLastError());
}

void launch_force_only(mappg_sys* s) {
    EamArgs a = eam_args(s);
    if (s->precision == MAPPG_MIXED && !s->force64) {
        launch_force32(s, a);
        launch_dof_mask(s, true);
        s->f_is_f32 = true;
        return;
    }
    if (s->ncell > 1) {
        k_force64b<8><<<std::min(s->nchunk, s->sm_count * 8), 256, 0, s->stream>>>(a, s->cell_of);
        MAPPG_CUDA(cudaGetLastError());
        launch_cells_done(s, a, 0);
    } else {
        MAPPG_TPA64(k_force64)
        MAPPG_CUDA(cudaGetLastError());
    }
    launch_dof_mask(s, false);
    s->f_is_f32 = false;
}

void launch_force(mappg_sys* s) {
    launch_density_only(s);
    launch_force_only(s);
}

// preconditioner features of every atom (bin order), n x 33 floats
void launch_descriptors(mappg_sys* s, float* out) {
    EamArgs a = eam_args(s);
    if (s->ncell > 1)
        k_descriptors<8, true><<<grid64<8>(s), 256, 0, s->stream>>>(a, s->cell_of, out);
    else
        k_descriptors<8, false><<<grid64<8>(s), 256, 0, s->stream>>>(a, nullptr, out);
    MAPPG_CUDA(cudaGetLastError());
}

// FP64 density and force passes whose outputs, partial sums and device
// scalars are the ones in `a` (mappg_sys_force_noalloc points them at its
// scratch); launches only, no allocation
void launch_force64_args(mappg_sys* s, const EamArgs& a) {
    MAPPG_TPA64(k_density64)
    MAPPG_TPA64(k_force64)
    MAPPG_CUDA(cudaGetLastError());
}

// loads every instantiation launch_force64_args can pick onto the current
// device, so that later launches do no module loading of their own
void preload_force64() {
    cudaFuncAttributes fa;
    MAPPG_CUDA(cudaFuncGetAttributes(&fa, k_density64<4>));
    MAPPG_CUDA(cudaFuncGetAttributes(&fa, k_density64<8>));
    MAPPG_CUDA(cudaFuncGetAttributes(&fa, k_density64<16>));
    MAPPG_CUDA(cudaFuncGetAttributes(&fa, k_density64<32>));
    MAPPG_CUDA(cudaFuncGetAttributes(&fa, k_force64<4>));
    MAPPG_CUDA(cudaFuncGetAttributes(&fa, k_force64<8>));
    MAPPG_CUDA(cudaFuncGetAttributes(&fa, k_force64<16>));
    MAPPG_CUDA(cudaFuncGetAttributes(&fa, k_force64<32>));
}

// FP64 energy in either precision (line searches of mixed systems compare
// FP64 energies): sc->energy for one cell, CellMd::energy per cell of a batch
void launch_energy64(mappg_sys* s) {
    EamArgs a = eam_args(s);
    if (s->ncell > 1) {
        k_energy64b<8><<<std::min(s->nchunk, s->sm_count * 8), 256, 0, s->stream>>>(a, s->cell_of);
        MAPPG_CUDA(cudaGetLastError());
        launch_cells_done(s, a, 1);
        return;
    }
    MAPPG_TPA64(k_energy64)
    MAPPG_CUDA(cudaGetLastError());
}

void launch_energy(mappg_sys* s) {
    EamArgs a = eam_args(s);
    if (s->precision == MAPPG_MIXED) {
        launch_energy32(s, a);
        return;
    }
    MAPPG_TPA64(k_energy64)
    MAPPG_CUDA(cudaGetLastError());
}

}  // namespace mappg
