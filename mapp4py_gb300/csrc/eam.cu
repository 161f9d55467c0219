// EAM kernels over the full neighbour list.
//
// The reference (ForceFieldEAM::__force_calc, ff_eam.cpp:65-240) walks a half
// list twice and scatters to both atoms of a pair.  Here every atom owns a
// full row, so each atom's sums are private and no atomics are needed:
//   k_density  rho_i = sum_j rho_{e_j->e_i}(r_ij), then F(rho_i) and F'(rho_i)
//              in the same kernel (the row is complete when the sum ends),
//              with the linear extrapolation above rho_max (ff_eam.cpp:180-191)
//   k_force    f_i = sum_j -(phi'(r) + F'_i rho'_{j->i}(r) + F'_j rho'_{i->j}(r))
//              * (x_i - x_j)/r, pair energy phi/2 and virial fpair*dx(x)dx/2
//              per entry (each pair appears in both rows)
//   k_energy   energy only (ff_eam.cpp:244-318): density and pair energy in
//              one pass, then F(rho_i)
// A group of TPA lanes serves one atom; lanes stride over the row, reduce
// with shuffles, and one lane writes the atom's results.  Per-lane energy
// and virial accumulators are reduced per block and then over blocks in a
// fixed order by the last block to finish (deterministic, FP64).
//
// Spline evaluation (value ((c3 p + c2) p + c1) p + c0, derivative
// ((3 c3 p + 2 c2) p + c1)/dr) and the index rule m = min(int(r/dr), nr-2),
// p = min(r/dr - m, 1) follow ff_eam.cpp:122-140.
//
// MIX = false: FP64 everywhere, positions read as x_j + n*H.
// MIX = true : FP32 pair math on bin-relative float4 positions with a per-code
//              bin offset; FP32 tables; atom results stored as FP64; energy
//              and virial reduced in FP64 across lanes and blocks.
#include <math.h>

#include "system.h"

namespace mappg {

template <bool MIX>
struct Prec;
template <>
struct Prec<false> {
    using R = double;
    using R4 = double4;
};
template <>
struct Prec<true> {
    using R = float;
    using R4 = float4;
};

// r/dr with 1/dr split as hi + lo so the FP32 index carries no systematic
// scale error (a plain FP32 1/dr is off by up to 3e-8 relative, which biases
// every pair the same way)
__device__ __forceinline__ float r_over_dr(float r, float hi, float lo) { return fmaf(r, hi, r * lo); }
__device__ __forceinline__ double r_over_dr(double r, double hi, double) { return r * hi; }

template <typename R, typename R4>
__device__ __forceinline__ R spl_val(const R4& c, R p) {
    return ((c.w * p + c.z) * p + c.y) * p + c.x;
}
// r*phi value with the FP32 table's constant term carried as head + tail:
// the head's rounding is shared by every pair that lands on the knot and
// would otherwise bias the pair energy
template <bool MIX>
__device__ __forceinline__ typename Prec<MIX>::R z_val(const EamArgs& a, size_t k, const typename Prec<MIX>::R4& c,
                                                       typename Prec<MIX>::R p) {
    if constexpr (MIX)
        return c.x + (__ldg(a.rphi32_lo + k) + ((c.w * p + c.z) * p + c.y) * p);
    else
        return ((c.w * p + c.z) * p + c.y) * p + c.x;
}

template <typename R, typename R4>
__device__ __forceinline__ R spl_der(const R4& c, R p) {
    return (R(3) * c.w * p + R(2) * c.z) * p + c.y;
}

// read-only path loads of one spline interval (4 coefficients)
__device__ __forceinline__ double4 ldg4(const double4* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldg(q), b = __ldg(q + 1);
    return make_double4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

__device__ __forceinline__ float my_sqrt(float v) { return sqrtf(v); }
__device__ __forceinline__ double my_sqrt(double v) { return sqrt(v); }

// block-wide sum of K doubles into partials[blockIdx.x*kRedSlots + slot0 + k];
// returns true in the block that finished last (its threads then see all
// partials)
template <int K>
__device__ bool block_partials(double (&v)[K], double* partials, int slot0, unsigned* counter) {
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
        partials[blockIdx.x * kRedSlots + slot0 + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

// sums of the first K partial slots over nblk blocks by one warp, in a fixed
// order (lane-strided, then a shuffle tree): every lane gets the totals
template <int K>
__device__ void final_sums(const double* partials, int nblk, double (&tot)[K]) {
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

// one pass over an atom's row: the geometry of entry e
template <bool MIX>
struct Pos;

template <>
struct Pos<false> {
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
    __device__ __forceinline__ void delta(const EamArgs& a, const double (*sh)[3], int j, int c, double& dx,
                                          double& dy, double& dz, int& ej) const {
        int d0 = c % 3 - 1, d1 = (c / 3) % 3 - 1, d2 = c / 9 - 1;
        int n0 = (d0 < 0 && lo[0]) ? -1 : ((d0 > 0 && hi[0]) ? 1 : 0);
        int n1 = (d1 < 0 && lo[1]) ? -1 : ((d1 > 0 && hi[1]) ? 1 : 0);
        int n2 = (d2 < 0 && lo[2]) ? -1 : ((d2 > 0 && hi[2]) ? 1 : 0);
        const double* s = sh[(n0 + 1) + 3 * (n1 + 1) + 9 * (n2 + 1)];
        dx = x - (__ldg(a.x + j) + s[0]);
        dy = y - (__ldg(a.x + a.n + j) + s[1]);
        dz = z - (__ldg(a.x + 2 * a.n + j) + s[2]);
        ej = __ldg(a.elem + j);
    }
};

template <>
struct Pos<true> {
    float4 p;
    __device__ __forceinline__ void load(const EamArgs& a, int i) { p = a.p32[i]; }
    // dx = ((p_i - p_j) + offset head) + offset tail: the tail removes the
    // rounding of the per-code offset, which is shared by every pair that
    // crosses that bin face and would otherwise bias those distances alike
    __device__ __forceinline__ void delta(const EamArgs& a, const float4* off, const float4* offlo, int j, int c,
                                          float& dx, float& dy, float& dz, int& ej) const {
        float4 q = __ldg(a.p32 + j);
        float4 o = off[c], l = offlo[c];
        dx = ((p.x - q.x) + o.x) + l.x;
        dy = ((p.y - q.y) + o.y) + l.y;
        dz = ((p.z - q.z) + o.z) + l.z;
        ej = __float_as_int(q.w);
    }
};

template <bool MIX>
__device__ __forceinline__ const typename Prec<MIX>::R4* rho_tab(const EamArgs& a);
template <>
__device__ __forceinline__ const double4* rho_tab<false>(const EamArgs& a) { return a.rho64; }
template <>
__device__ __forceinline__ const float4* rho_tab<true>(const EamArgs& a) { return a.rho32; }
template <bool MIX>
__device__ __forceinline__ const typename Prec<MIX>::R4* rphi_tab(const EamArgs& a);
template <>
__device__ __forceinline__ const double4* rphi_tab<false>(const EamArgs& a) { return a.rphi64; }
template <>
__device__ __forceinline__ const float4* rphi_tab<true>(const EamArgs& a) { return a.rphi32; }

// shared copies of the small per-kernel tables
template <bool MIX>
struct Smem {
    double sh[27][3];
    float4 off[27];
    float4 offlo[27];
    typename Prec<MIX>::R cut_sq[kMaxElem * kMaxElem];
    __device__ void fill(const EamArgs& a) {
        for (int t = threadIdx.x; t < 27; t += blockDim.x) {
            sh[t][0] = a.shift[t][0];
            sh[t][1] = a.shift[t][1];
            sh[t][2] = a.shift[t][2];
            off[t] = make_float4(a.off32[t][0], a.off32[t][1], a.off32[t][2], 0.f);
            offlo[t] = make_float4(a.off32lo[t][0], a.off32lo[t][1], a.off32lo[t][2], 0.f);
        }
        for (int t = threadIdx.x; t < a.ne * a.ne; t += blockDim.x) cut_sq[t] = (typename Prec<MIX>::R)a.cut_sq[t];
        __syncthreads();
    }
};

template <bool MIX, typename R>
__device__ __forceinline__ void geom(const Pos<MIX>& P, const EamArgs& a, const Smem<MIX>& S, int e, R& dx, R& dy,
                                     R& dz, int& ej) {
    int j = e >> kCodeBits, c = e & 31;
    if constexpr (MIX)
        P.delta(a, S.off, S.offlo, j, c, dx, dy, dz, ej);
    else
        P.delta(a, S.sh, j, c, dx, dy, dz, ej);
}

// F(rho), F'(rho) with the reference's extrapolation above rho_max (FP64)
__device__ __forceinline__ void embed64(const EamArgs& a, int ei, double rho, double& Fv, double& dFv) {
    double p = rho * a.drho_inv;
    int m = p < (double)(a.nrho - 2) ? (int)p : a.nrho - 2;
    if (m < 0) m = 0;
    p -= (double)m;
    p = fmin(p, 1.0);
    double4 c = ldg4(a.F64 + (size_t)ei * a.nrho + m);
    dFv = ((3.0 * c.w * p + 2.0 * c.z) * p + c.y) * a.drho_inv;
    Fv = ((c.w * p + c.z) * p + c.y) * p + c.x;
    if (rho > a.rho_max) Fv += dFv * (rho - a.rho_max);
}

__device__ __forceinline__ void embed32(const EamArgs& a, int ei, float rho, float& Fv, float& dFv) {
    const float drho_inv = (float)a.drho_inv, rho_max = (float)a.rho_max;
    float p = rho * drho_inv;
    int m = p < (float)(a.nrho - 2) ? (int)p : a.nrho - 2;
    if (m < 0) m = 0;
    p -= (float)m;
    p = fminf(p, 1.f);
    float4 c = ldg4(a.F32 + (size_t)ei * a.nrho + m);
    dFv = ((3.f * c.w * p + 2.f * c.z) * p + c.y) * drho_inv;
    Fv = ((c.w * p + c.z) * p + c.y) * p + c.x;
    if (rho > rho_max) Fv += dFv * (rho - rho_max);
}

template <int TPA, bool MIX>
__global__ void __launch_bounds__(256) k_density(EamArgs a) {
    using R = typename Prec<MIX>::R;
    using R4 = typename Prec<MIX>::R4;
    __shared__ Smem<MIX> S;
    S.fill(a);
    const R dr_inv = (R)a.dr_inv;
    const R dr_lo = (R)(a.dr_inv - (double)dr_inv);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    const R4* rt = rho_tab<MIX>(a);
    double eacc = 0.0;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        R acc = 0;
        int ei = 0;
        if (active) {
            Pos<MIX> P;
            P.load(a, i);
            ei = __ldg(a.elem + i);
            const int nn = __ldg(a.nnbr + i);
            const int* row = a.nbr + (size_t)i * a.maxnbr;
            for (int k = lane; k < nn; k += TPA) {
                R dx, dy, dz;
                int ej;
                geom<MIX, R>(P, a, S, __ldg(row + k), dx, dy, dz, ej);
                R rsq = dx * dx + dy * dy + dz * dz;
                if (rsq < S.cut_sq[ei * a.ne + ej]) {
                    R r = my_sqrt(rsq);
                    R p = r_over_dr(r, dr_inv, dr_lo);
                    int m = min((int)p, a.nr - 2);
                    p -= (R)m;
                    p = p < R(1) ? p : R(1);
                    acc += spl_val<R, R4>(ldg4(rt + (size_t)(ej * a.ne + ei) * a.nr + m), p);
                }
            }
        }
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPA);
        if (active && lane == 0) {
            double Fv, dFv;
            if constexpr (MIX) {
                // F' in FP32 feeds the FP32 force pass; the energy value is
                // taken in FP64 (one spline per atom) so that rounding of the
                // FP32 table does not bias the total
                float F32v, dF32v;
                embed32(a, ei, acc, F32v, dF32v);
                double dF64;
                embed64(a, ei, (double)acc, Fv, dF64);
                dFv = dF32v;
                a.dF32[i] = dF32v;
            } else {
                embed64(a, ei, acc, Fv, dFv);
            }
            a.rho[i] = (double)acc;
            a.dF[i] = dFv;
            eacc += Fv;
        }
    }
    double v[1] = {eacc};
    if (block_partials<1>(v, a.partials, 7, &a.sc->counter[1])) {
        if (threadIdx.x == 0) a.sc->counter[1] = 0;
    }
}

template <int TPA, bool MIX>
__global__ void __launch_bounds__(256) k_force(EamArgs a) {
    using R = typename Prec<MIX>::R;
    using R4 = typename Prec<MIX>::R4;
    __shared__ Smem<MIX> S;
    S.fill(a);
    const R dr_inv = (R)a.dr_inv;
    const R dr_lo = (R)(a.dr_inv - (double)dr_inv);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    const R4* rt = rho_tab<MIX>(a);
    const R4* zt = rphi_tab<MIX>(a);
    R ep = 0, w0 = 0, w1 = 0, w2 = 0, w3 = 0, w4 = 0, w5 = 0;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        R fx = 0, fy = 0, fz = 0;
        if (active) {
            Pos<MIX> P;
            P.load(a, i);
            const int ei = __ldg(a.elem + i);
            R dFi;
            if constexpr (MIX)
                dFi = __ldg(a.dF32 + i);
            else
                dFi = __ldg(a.dF + i);
            const int nn = __ldg(a.nnbr + i);
            const int* row = a.nbr + (size_t)i * a.maxnbr;
            for (int k = lane; k < nn; k += TPA) {
                const int e = __ldg(row + k);
                R dx, dy, dz;
                int ej;
                geom<MIX, R>(P, a, S, e, dx, dy, dz, ej);
                R rsq = dx * dx + dy * dy + dz * dz;
                if (rsq < S.cut_sq[ei * a.ne + ej]) {
                    const int j = e >> kCodeBits;
                    R r = my_sqrt(rsq);
                    R rinv = R(1) / r;
                    R p = r_over_dr(r, dr_inv, dr_lo);
                    int m = min((int)p, a.nr - 2);
                    p -= (R)m;
                    p = p < R(1) ? p : R(1);
                    const R4 ci = ldg4(rt + (size_t)(ej * a.ne + ei) * a.nr + m);
                    const R der_i = spl_der<R, R4>(ci, p) * dr_inv;
                    R der_j = der_i;
                    if (ej != ei) der_j = spl_der<R, R4>(ldg4(rt + (size_t)(ei * a.ne + ej) * a.nr + m), p) * dr_inv;
                    const size_t kz = (size_t)(ei * a.ne + ej) * a.nr + m;
                    const R4 cz = ldg4(zt + kz);
                    const R z = z_val<MIX>(a, kz, cz, p);
                    const R zp = spl_der<R, R4>(cz, p) * dr_inv;
                    const R phi = z * rinv;
                    const R dphi = zp * rinv - phi * rinv;
                    R dFj;
                    if constexpr (MIX)
                        dFj = __ldg(a.dF32 + j);
                    else
                        dFj = __ldg(a.dF + j);
                    const R fp = -(dphi + dFi * der_i + dFj * der_j) * rinv;
                    fx += fp * dx;
                    fy += fp * dy;
                    fz += fp * dz;
                    ep += phi;
                    w0 += fp * dx * dx;
                    w1 += fp * dx * dy;
                    w2 += fp * dx * dz;
                    w3 += fp * dy * dy;
                    w4 += fp * dy * dz;
                    w5 += fp * dz * dz;
                }
            }
        }
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, o, TPA);
            fy += __shfl_xor_sync(0xffffffffu, fy, o, TPA);
            fz += __shfl_xor_sync(0xffffffffu, fz, o, TPA);
        }
        if (active && lane == 0) {
            a.f[i] = (double)fx;
            a.f[a.n + i] = (double)fy;
            a.f[2 * a.n + i] = (double)fz;
        }
    }
    double v[7] = {0.5 * (double)ep, 0.5 * (double)w0, 0.5 * (double)w1, 0.5 * (double)w2,
                   0.5 * (double)w3, 0.5 * (double)w4, 0.5 * (double)w5};
    if (block_partials<7>(v, a.partials, 0, &a.sc->counter[0])) {
        // last block: totals over blocks in a fixed order; slot 7 holds the
        // embedding energy written by k_density on the same grid
        if (threadIdx.x < 32) {
            double tot[8];
            final_sums<8>(a.partials, gridDim.x, tot);
            if (threadIdx.x == 0) {
                a.sc->energy = tot[0] + tot[7];
                for (int k = 0; k < 6; k++) a.sc->virial[k] = tot[k + 1];
                a.sc->counter[0] = 0;
            }
        }
    }
}

template <int TPA, bool MIX>
__global__ void __launch_bounds__(256) k_energy(EamArgs a) {
    using R = typename Prec<MIX>::R;
    using R4 = typename Prec<MIX>::R4;
    __shared__ Smem<MIX> S;
    S.fill(a);
    const R dr_inv = (R)a.dr_inv;
    const R dr_lo = (R)(a.dr_inv - (double)dr_inv);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    const R4* rt = rho_tab<MIX>(a);
    const R4* zt = rphi_tab<MIX>(a);
    R ep = 0;
    double eacc = 0.0;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        R acc = 0;
        int ei = 0;
        if (active) {
            Pos<MIX> P;
            P.load(a, i);
            ei = __ldg(a.elem + i);
            const int nn = __ldg(a.nnbr + i);
            const int* row = a.nbr + (size_t)i * a.maxnbr;
            for (int k = lane; k < nn; k += TPA) {
                R dx, dy, dz;
                int ej;
                geom<MIX, R>(P, a, S, __ldg(row + k), dx, dy, dz, ej);
                R rsq = dx * dx + dy * dy + dz * dz;
                if (rsq < S.cut_sq[ei * a.ne + ej]) {
                    R r = my_sqrt(rsq);
                    R p = r_over_dr(r, dr_inv, dr_lo);
                    int m = min((int)p, a.nr - 2);
                    p -= (R)m;
                    p = p < R(1) ? p : R(1);
                    acc += spl_val<R, R4>(ldg4(rt + (size_t)(ej * a.ne + ei) * a.nr + m), p);
                    const size_t kz = (size_t)(ei * a.ne + ej) * a.nr + m;
                    ep += z_val<MIX>(a, kz, ldg4(zt + kz), p) / r;
                }
            }
        }
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPA);
        if (active && lane == 0) {
            double Fv, dFv;
            embed64(a, ei, (double)acc, Fv, dFv);
            eacc += Fv;
        }
    }
    double v[1] = {eacc + 0.5 * (double)ep};
    if (block_partials<1>(v, a.partials, 0, &a.sc->counter[2])) {
        if (threadIdx.x < 32) {
            double tot[1];
            final_sums<1>(a.partials, gridDim.x, tot);
            if (threadIdx.x == 0) {
                a.sc->energy = tot[0];
                a.sc->counter[2] = 0;
            }
        }
    }
}

template <int TPA, bool MIX>
static void launch_force_t(mappg_sys* s) {
    EamArgs a = eam_args(s);
    int g = grid_for(s, (long long)s->n * TPA, 256);
    k_density<TPA, MIX><<<g, 256, 0, s->stream>>>(a);
    k_force<TPA, MIX><<<g, 256, 0, s->stream>>>(a);
    MAPPG_CUDA(cudaGetLastError());
}

template <int TPA, bool MIX>
static void launch_density_t(mappg_sys* s) {
    EamArgs a = eam_args(s);
    k_density<TPA, MIX><<<grid_for(s, (long long)s->n * TPA, 256), 256, 0, s->stream>>>(a);
    MAPPG_CUDA(cudaGetLastError());
}

template <int TPA, bool MIX>
static void launch_force_only_t(mappg_sys* s) {
    EamArgs a = eam_args(s);
    k_force<TPA, MIX><<<grid_for(s, (long long)s->n * TPA, 256), 256, 0, s->stream>>>(a);
    MAPPG_CUDA(cudaGetLastError());
}

template <int TPA, bool MIX>
static void launch_energy_t(mappg_sys* s) {
    EamArgs a = eam_args(s);
    int g = grid_for(s, (long long)s->n * TPA, 256);
    k_energy<TPA, MIX><<<g, 256, 0, s->stream>>>(a);
    MAPPG_CUDA(cudaGetLastError());
}

#define MAPPG_TPA_DISPATCH(FN, MIX)            \
    switch (s->tpa) {                          \
        case 4: FN<4, MIX>(s); break;          \
        case 16: FN<16, MIX>(s); break;        \
        case 32: FN<32, MIX>(s); break;        \
        default: FN<8, MIX>(s); break;         \
    }

void launch_force(mappg_sys* s) {
    if (s->precision == MAPPG_MIXED) {
        MAPPG_TPA_DISPATCH(launch_force_t, true)
    } else {
        MAPPG_TPA_DISPATCH(launch_force_t, false)
    }
}

void launch_density_only(mappg_sys* s) {
    if (s->precision == MAPPG_MIXED) {
        MAPPG_TPA_DISPATCH(launch_density_t, true)
    } else {
        MAPPG_TPA_DISPATCH(launch_density_t, false)
    }
}

void launch_force_only(mappg_sys* s) {
    if (s->precision == MAPPG_MIXED) {
        MAPPG_TPA_DISPATCH(launch_force_only_t, true)
    } else {
        MAPPG_TPA_DISPATCH(launch_force_only_t, false)
    }
}

void launch_energy(mappg_sys* s) {
    if (s->precision == MAPPG_MIXED) {
        MAPPG_TPA_DISPATCH(launch_energy_t, true)
    } else {
        MAPPG_TPA_DISPATCH(launch_energy_t, false)
    }
}

}  // namespace mappg
