// Mixed-precision EAM kernels: FP32 pair geometry and spline arithmetic in
// the scaled bin frame (system.h), FP64 state, FP64 totals.
//
//   k_density32  rho_i in FP32, then F'(rho_i) and F(rho_i) from the FP32
//                embedding table with its constant term carried as head +
//                tail; writes q32[i] = (p'_i, F'_i) for the force pass
//   k_force32    forces, pair energy and virial from one 32-byte record per
//                (pair type, knot) (plus a 16-byte one for unlike pairs);
//                F'_j rides in q32[j].w, so a neighbour costs one 16-byte
//                gather plus the record
//   k_force32s   k_force32 with one element group's records in shared
//                memory at a time (an autotuner candidate)
//   k_energy32   energy only (line-search trials)
//   k_de32       energy differences E(x0 + alpha h) - E(x0) pair by pair
//                (line-search trials within half the skin)
//
// Precision: every per-pair term is computed in FP32; the sums of them are
// accumulated with compensation (Kahan: an FP32 sum and an FP32 correction
// holding its lost low part), which carries the sum of FP32 terms as an FP64
// accumulator would: per-atom density, force and pair energy within a lane,
// and the energy across all atoms a thread visits.  The virial is summed in
// plain FP32 per thread (a few hundred pair terms: six more compensated sums
// per pair cost 6 % of the force pass) and in FP64 across threads, which
// keeps the stress within ~1e-7 of its scale.  Lane partials are combined
// with exact two-sums (the correction keeps every rounding error), block and
// grid totals are FP64 in a fixed order.  The embedding's knot index and
// fraction come from the density's sum and correction without rounding them
// to one FP32 value (embed32f).  Constants shared by many
// pairs (1/dr, the frame-to-Cartesian scale, the spline constant terms) are
// carried as head + tail so their rounding does not bias the totals.
//
// Table index: p = r/dr, m = floor(p) via an add with round-toward-zero
// against 2^23, then the reference's clamps m <= nr-2, p - m <= 1
// (ff_eam.cpp:122-128).
#include <math.h>

#include <algorithm>
#include <type_traits>

#include "eam_common.cuh"
#include "nhc.cuh"

namespace mappg {

struct Smem32 {
    float4 off[27];
    float cut_sq[kMaxElem * kMaxElem];
    __device__ void fill(const EamArgs& a) {
        for (int t = threadIdx.x; t < 27; t += blockDim.x)
            off[t] = make_float4(a.fr.off[t][0], a.fr.off[t][1], a.fr.off[t][2], 0.f);
        for (int t = threadIdx.x; t < a.ne * a.ne; t += blockDim.x) cut_sq[t] = (float)a.cut_sq[t];
        __syncthreads();
    }
};

// frame offset -8 d of a neighbour image from its entry's bin steps: with
// k_q = d_q + 1 in bits 2q..2q+1, the float whose bits are 0x4B000000 | (e &
// (3 << 2q)) is 2^23 + 4^q k_q, and one FMA takes it to 8 - 8 k_q:
// (2^23 + 4^q k) (-8 / 4^q) + (2^26 / 4^q + 8).  Every value involved is a
// multiple of 8 / 4^q below 2^27 / 4^q, so the product and the sum are exact.
// Two instructions per axis (a LOP3 and an FFMA): the density pass is bound
// by instruction issue
__device__ __forceinline__ void image_offset(int e, float4& o) {
    o.x = fmaf(__int_as_float(0x4B000000 | (e & 3)), -8.0f, 67108872.0f);
    o.y = fmaf(__int_as_float(0x4B000000 | (e & 12)), -2.0f, 16777224.0f);
    o.z = fmaf(__int_as_float(0x4B000000 | (e & 48)), -0.5f, 4194312.0f);
    o.w = 0.f;
}

// frame displacement (a,b,c) to Cartesian with the head + tail scale
template <bool ORTHO, class FR>
__device__ __forceinline__ void cart(const FR& fr, float a, float b, float c, float& x, float& y, float& z) {
    if (ORTHO) {
        x = fmaf(a, fr.G[0][0], a * fr.Glo[0][0]);
        y = fmaf(b, fr.G[1][1], b * fr.Glo[1][1]);
        z = fmaf(c, fr.G[2][2], c * fr.Glo[2][2]);
    } else {
        x = fmaf(a, fr.G[0][0], fmaf(b, fr.G[1][0], fmaf(c, fr.G[2][0], a * fr.Glo[0][0] + b * fr.Glo[1][0] +
                                                                        c * fr.Glo[2][0])));
        y = fmaf(b, fr.G[1][1], fmaf(c, fr.G[2][1], b * fr.Glo[1][1] + c * fr.Glo[2][1]));
        z = fmaf(c, fr.G[2][2], c * fr.Glo[2][2]);
    }
}

// 1/r from the hardware reciprocal square root and one Newton step
__device__ __forceinline__ float inv_sqrt(float x) {
    // one Newton step written as y + y * (1/2 - x y^2 / 2): the correction is
    // small and added with a single rounding, so the result carries no
    // systematic bias (the form y * (3/2 - x y^2 / 2) rounds a factor next to
    // 1.0, where the spacing of floats changes, and comes out low by ~1e-8)
    const float y = rsqrtf(x);
    return fmaf(y, fmaf(-0.5f * x * y, y, 0.5f), y);
}

// knot index and fraction: m = min(floor(p), nmax), p - m clamped to 1
__device__ __forceinline__ int knot32(float p, int nmax, float& fr) {
    const float t = __fadd_rz(p, 8388608.0f);
    int m = __float_as_int(t) - 0x4B000000;
    fr = p - (t - 8388608.0f);
    if (m > nmax) {
        m = nmax;
        fr = 1.0f;
    }
    return m;
}

// compensated FP32 accumulation (s, c) += v
__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

struct Consts32 {
    float dri, dri_lo;
    __device__ Consts32(const EamArgs& a) {
        dri = (float)a.dr_inv;
        dri_lo = (float)(a.dr_inv - (double)dri);
    }
};

// s + e == a + b exactly (Knuth's two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// a lane's compensated partial (s, c), whose value is s - c, summed over the
// TPA lanes of one atom: the rounding error of every addition goes into the
// correction, so lane 0 ends with (s, c) of the whole sum; FP32 instructions
// only (GB300's FP64 pipe is narrow, and per-lane FP64 shuffles and
// conversions took a quarter of it)
template <int TPA>
__device__ __forceinline__ void lane_sum_comp(float& s, float& c) {
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o, TPA);
        const float c2 = __shfl_xor_sync(0xffffffffu, c, o, TPA);
        float t, e;
        two_sum(s, s2, t, e);
        s = t;
        c = (c + c2) - e;
    }
}

// embedding F and F' of the FP64 density: knot and fraction from rho/drho
// in FP64, then the FP32 table with its constant term as head + tail
// (ff_eam.cpp:180-187).  Above rho_max every atom uses the last knot's
// record at p = 1 and extrapolates linearly (ff_eam.cpp:188-189); one FP32
// copy of that single record would bias all such atoms alike, so this rare
// branch reads the FP64 record.
__device__ __forceinline__ void embed32(const EamArgs& a, int ei, double rho, float& Fv, float& dFv) {
    if (rho > a.rho_max) {
        const Dbl4 c = ldg4(a.F64 + (size_t)ei * a.nrho + (a.nrho - 2));
        const double d1 = ((3.0 * c.w + 2.0 * c.z) + c.y) * a.drho_inv;
        const double f0 = ((c.w + c.z) + c.y) + c.x;
        dFv = (float)d1;
        Fv = (float)(f0 + d1 * (rho - a.rho_max));
        return;
    }
    const double p = rho * a.drho_inv;
    int m = (int)p;
    float fr = (float)(p - (double)m);
    if (m > a.nrho - 2) {
        m = a.nrho - 2;
        fr = 1.0f;
    }
    const size_t k = (size_t)ei * a.nrho + m;
    const float4 c = __ldg(a.F32 + k);
    dFv = fmaf(fmaf(3.0f * c.w, fr, 2.0f * c.z), fr, c.y) * (float)a.drho_inv;
    Fv = c.x + (__ldg(a.F32lo + k) + fr * fmaf(fmaf(c.w, fr, c.z), fr, c.y));
}

// F and F' of the density s - c (a compensated FP32 pair) without FP64
// arithmetic: p = rho/drho as head ph + tail pl (the exact error of the head
// product by an FMA, plus the tails of s*(1/drho) and of c), m = floor(ph)
// corrected by the tail, fr = (ph - m) + pl (ph - m is exact).  The last
// knot interval and the extrapolation above rho_max take embed32's FP64
// route.  The density pass's lane 0 per atom runs this; on GB300's narrow
// FP64 pipe the FP64 form cost 1 % of the pass
__device__ __forceinline__ void embed32f(const EamArgs& a, int ei, float s, float c, float& Fv, float& dFv) {
    const float dhi = (float)a.drho_inv;
    const float dlo = (float)(a.drho_inv - (double)dhi);
    const float ph = s * dhi;
    const float pl = fmaf(s, dlo, fmaf(-c, dhi, fmaf(s, dhi, -ph)));
    if (!(ph < (float)(a.nrho - 2))) {
        embed32(a, ei, (double)s - (double)c, Fv, dFv);
        return;
    }
    int m = (int)ph;
    float fr = (ph - (float)m) + pl;
    if (fr < 0.f) {
        m -= 1;
        fr += 1.f;
    } else if (fr >= 1.f) {
        m += 1;
        fr -= 1.f;
    }
    if (m < 0) {
        m = 0;
        fr = 0.f;
    }
    const size_t k = (size_t)ei * a.nrho + m;
    const float4 cc = __ldg(a.F32 + k);
    dFv = fmaf(fmaf(3.0f * cc.w, fr, 2.0f * cc.z), fr, cc.y) * dhi;
    Fv = cc.x + (__ldg(a.F32lo + k) + fr * fmaf(fmaf(cc.w, fr, cc.z), fr, cc.y));
}

// per-kernel persistent grid: as many blocks as fit on the GPU at once
template <class Kern>
static int occupancy_grid(mappg_sys* s, Kern k, int block) {
    int per_sm = 0;
    MAPPG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, 0));
    if (per_sm < 1) per_sm = 1;
    long long g = (long long)per_sm * s->sm_count;
    if (g > kMaxBlocks) g = kMaxBlocks;
    return (int)g;
}

// frame of a batch cell (the G head/tail of CellGeo), read once per chunk
struct CellFrame {
    float G[3][3], Glo[3][3];
};

template <bool ORTHO>
__device__ __forceinline__ CellFrame cell_frame(const CellGeo* g) {
    CellFrame f;
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const bool used = ORTHO ? d == k : k <= d;
            f.G[d][k] = used ? g->G[d][k] : 0.f;
            f.Glo[d][k] = used ? g->Glo[d][k] : 0.f;
        }
    return f;
}

// one atom's density row (TPA lanes), its embedding terms and q32 record;
// SM: the density records of knots from a.rho_mlo on come from the
// shared-memory copy stab (k_density32s), lower knots from global memory
template <int TPA, bool ORTHO, int U, class FR, bool SM = false>
__device__ __forceinline__ void density_atom(const EamArgs& a, const Smem32& S, const Consts32& K, const FR& fr,
                                             int i, int lane, bool active, float& es, float& ec,
                                             const float4* stab = nullptr) {
    float acc = 0.f, acc_c = 0.f;
    int ei = 0;
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
        pi = __ldg(a.p32 + i);
        ei = a.elem[i];
        const int nn = __ldg(a.nnbr + i);
        const int* row = a.nbr + (size_t)i * a.maxnbr;
        const float cut0 = S.cut_sq[0];
        auto pair = [&](int e, const float4& q) -> bool {
            const int ej = entry_elem(e);
            float4 o;
            image_offset(e, o);
            float dx, dy, dz;
            cart<ORTHO>(fr, (pi.x - q.x) + o.x, (pi.y - q.y) + o.y, (pi.z - q.z) + o.z, dx, dy, dz);
            const float rsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (rsq < (a.cut_uniform ? cut0 : S.cut_sq[ei * a.ne + ej])) {
                const float r = rsq * inv_sqrt(rsq);
                float fr;
                const int m = knot32(fmaf(r, K.dri, r * K.dri_lo), a.nr - 2, fr);
                float4 c;
                const int ms = m - a.rho_mlo;
                if (SM && ms >= 0)
                    c = stab[(a.rho_ei ? ej * a.ne + ei : ej) * a.rho_w + ms];
                else
                    c = __ldg(a.rho32 + (size_t)(ej * a.ne + ei * a.rho_ei) * a.nr + m);
                kahan_add(acc, acc_c, fmaf(fmaf(fmaf(c.w, fr, c.z), fr, c.y), fr, c.x));
                return true;
            }
            return false;
        };
        // bit t of `bits`: this lane's t-th entry (row slot lane + t TPA) is
        // inside the cutoff
        unsigned bits = 0u;
        if (U == 1) {
            int t = 0;
            for (int k = lane; k < nn; k += TPA, t++) {
                const int e = __ldg(row + k);
                if (pair(e, __ldg(a.p32 + entry_j(e))) && t < 32) bits |= 1u << t;
            }
        } else {
            // two entries per step: both gathers are in flight together;
            // the additions keep the order of the one-entry loop
            int t = 0;
            for (int k = lane; k < nn; k += 2 * TPA, t += 2) {
                const bool v1 = k + TPA < nn;
                const int e0 = __ldg(row + k);
                const int e1 = v1 ? __ldg(row + k + TPA) : e0;
                const float4 q0 = __ldg(a.p32 + entry_j(e0));
                const float4 q1 = __ldg(a.p32 + entry_j(e1));
                if (pair(e0, q0) && t < 32) bits |= 1u << t;
                if (v1 && pair(e1, q1) && t + 1 < 32) bits |= 1u << (t + 1);
            }
        }
        if (a.cutmask && nn <= 32 * TPA) a.cutmask[(size_t)i * TPA + lane] = bits;
    }
    lane_sum_comp<TPA>(acc, acc_c);
    if (active && lane == 0) {
        float Fv, dFv;
        embed32f(a, ei, acc, acc_c, Fv, dFv);
        a.q32[i] = make_float4(pi.x, pi.y, pi.z, dFv);
        a.rho32out[i] = acc - acc_c;
        if (a.rho_keep) a.rho_keep[i] = (double)acc - (double)acc_c;
        kahan_add(es, ec, Fv);
    }
}

template <int TPA, bool ORTHO, int U>
__global__ void __launch_bounds__(256) k_density32(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    float es = 0.f, ec = 0.f;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        density_atom<TPA, ORTHO, U>(a, S, K, a.fr, i, lane, active, es, ec);
    }
    double v[1] = {(double)es - (double)ec};
    if (block_partials<1>(v, a.partials, 0, &a.sc->counter[1]) && threadIdx.x < 32) {
        double tot[1];
        final_sums<1>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            a.sc->e_embed = tot[0];
            a.sc->counter[1] = 0;
        }
    }
}

// k_density32 with the density tables in shared memory: one 1024-thread
// block per SM copies the knots rho_mlo.. of every density table (94 KB)
// and reads its spline records there instead of through L1; pairs closer
// than the first copied knot read global memory
template <int TPA, bool ORTHO, int U>
__global__ void __launch_bounds__(1024, 1) k_density32s(EamArgs a) {
    extern __shared__ float4 stab[];
    const int W = a.rho_w, ntab = a.rho_ntab;
    for (int k = threadIdx.x; k < ntab * W; k += blockDim.x) {
        const int ts = k / W, w = k - ts * W;
        const int gt = a.rho_ei ? ts : ts * a.ne;
        stab[k] = __ldg(a.rho32 + (size_t)gt * a.nr + a.rho_mlo + w);
    }
    __shared__ Smem32 S;
    S.fill(a);  // ends with __syncthreads
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    float es = 0.f, ec = 0.f;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        density_atom<TPA, ORTHO, U, Frame, true>(a, S, K, a.fr, i, lane, active, es, ec, stab);
    }
    double v[1] = {(double)es - (double)ec};
    if (block_partials<1>(v, a.partials, 0, &a.sc->counter[1]) && threadIdx.x < 32) {
        double tot[1];
        final_sums<1>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            a.sc->e_embed = tot[0];
            a.sc->counter[1] = 0;
        }
    }
}

// batch: blocks walk chunks; the chunk's embedding energy goes to slot 13
template <int TPA, bool ORTHO, int U>
__global__ void __launch_bounds__(256) k_density32b(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        if (a.cell_active && !a.cell_active[a.chunk_cell[ch]]) continue;
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        const CellFrame fr = cell_frame<ORTHO>(a.cells + a.chunk_cell[ch]);
        float es = 0.f, ec = 0.f;
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            density_atom<TPA, ORTHO, U>(a, S, K, fr, i, lane, i < hi, es, ec);
        }
        chunk_store<1>([&](int) { return (double)es - (double)ec; }, a.chunk_part + (size_t)ch * kChunkSlots + 13);
    }
}

// one atom's force row (TPA lanes): force, pair energy and virial;
// SM: the records of knots from a.fs_mlo on come from the shared-memory copy
// stab of atom i's element group (k_force32s), lower knots from global
// memory; both hold the same values, so the forces are the same
template <int TPA, bool ORTHO, int U, class FR, bool SM = false>
__device__ __forceinline__ void force_atom(const EamArgs& a, const Smem32& S, const Consts32& K, const FR& fr,
                                           int i, int lane, bool active, float& es, float& ec, float (&w)[6],
                                           const float4* stab = nullptr) {
    float fx = 0.f, fy = 0.f, fz = 0.f, ep = 0.f;
    float fxc = 0.f, fyc = 0.f, fzc = 0.f, epc = 0.f;
    int ei = 0;
    if (active) {
        const float4 pi = __ldg(a.q32 + i);
        const float dFi = pi.w;
        ei = a.elem[i];
        const int nn = __ldg(a.nnbr + i);
        const int* row = a.nbr + (size_t)i * a.maxnbr;
        const float cut0 = S.cut_sq[0];
        // inside: the entry is known to lie inside the cutoff (a set bit of the
        // density pass's mask: the same positions and arithmetic give the same
        // test), so the test is left out
        auto pair = [&](int e, const float4& q, bool inside) {
            const int ej = entry_elem(e);
            const int t = ei * a.ne + ej;
            float4 o;
            image_offset(e, o);
            float dx, dy, dz;
            cart<ORTHO>(fr, (pi.x - q.x) + o.x, (pi.y - q.y) + o.y, (pi.z - q.z) + o.z, dx, dy, dz);
            const float rsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (inside || rsq < (a.cut_uniform ? cut0 : S.cut_sq[t])) {
                const float rinv = inv_sqrt(rsq);
                const float r = rsq * rinv;
                float fr;
                const int m = knot32(fmaf(r, K.dri, r * K.dri_lo), a.nr - 2, fr);
                const size_t kt = (size_t)t * a.nr + m;
                const int ms = m - a.fs_mlo;
                const bool in_smem = SM && ms >= 0 && ms < a.fs_w;
                float4 r0, r1;
                if (in_smem) {
                    const float4 z = stab[ej * a.fs_w + ms];
                    const float4 d = stab[(a.ne + ej) * a.fs_w + ms];
                    r0 = make_float4(d.x, d.y, d.z, z.w);
                    r1 = make_float4(z.x, z.y, z.z, d.w);
                } else {
                    ldg8(a.ftab + 2 * kt, r0, r1);
                }
                const float der_i = fmaf(fmaf(r0.z, fr, r0.y), fr, r0.x);
                float der_j = der_i;
                if (ej != ei) {
                    float4 r2;
                    if (in_smem) {
                        // rho'_{g->ej}: with one density function per source
                        // element it is the group's own rho'_{g->g} record
                        const int rj = a.rho_ei ? 2 * a.ne + (ej < ei ? ej : ej - 1) : a.ne + ei;
                        r2 = stab[rj * a.fs_w + ms];
                    } else {
                        r2 = __ldg(a.fjtab + kt);
                    }
                    der_j = fmaf(fmaf(r2.z, fr, r2.y), fr, r2.x);
                }
                const float zpoly = fmaf(fmaf(r1.z, fr, r1.y), fr, r1.x);
                const float z = r0.w + fmaf(fr, zpoly, r1.w);
                const float zp = fmaf(fmaf(3.0f * r1.z, fr, 2.0f * r1.y), fr, r1.x) * K.dri;
                const float phi = z * rinv;
                const float dphi = (zp - phi) * rinv;
                const float fp = -fmaf(dFi, der_i, fmaf(q.w, der_j, dphi)) * rinv;
                const float fdx = fp * dx, fdy = fp * dy, fdz = fp * dz;
                kahan_add(fx, fxc, fdx);
                kahan_add(fy, fyc, fdy);
                kahan_add(fz, fzc, fdz);
                kahan_add(ep, epc, phi);
                w[0] = fmaf(fdx, dx, w[0]);
                w[1] = fmaf(fdx, dy, w[1]);
                w[2] = fmaf(fdx, dz, w[2]);
                w[3] = fmaf(fdy, dy, w[3]);
                w[4] = fmaf(fdy, dz, w[4]);
                w[5] = fmaf(fdz, dz, w[5]);
            }
        };
        if (a.cutmask && nn <= 32 * TPA) {
            // only the entries the density pass found inside the cutoff (the
            // same positions), in the same order: the skin shell's entries
            // cost no gather and no geometry here
            unsigned bits = __ldg(a.cutmask + (size_t)i * TPA + lane);
            if (U == 1) {
                while (bits) {
                    const int t = __ffs(bits) - 1;
                    bits &= bits - 1u;
                    const int e = __ldg(row + lane + t * TPA);
                    pair(e, __ldg(a.q32 + entry_j(e)), true);
                }
            } else {
                while (bits) {
                    const int t0 = __ffs(bits) - 1;
                    bits &= bits - 1u;
                    const bool v1 = bits != 0u;
                    const int t1 = v1 ? __ffs(bits) - 1 : t0;
                    if (v1) bits &= bits - 1u;
                    const int e0 = __ldg(row + lane + t0 * TPA);
                    const int e1 = v1 ? __ldg(row + lane + t1 * TPA) : e0;
                    const float4 q0 = __ldg(a.q32 + entry_j(e0));
                    const float4 q1 = __ldg(a.q32 + entry_j(e1));
                    pair(e0, q0, true);
                    if (v1) pair(e1, q1, true);
                }
            }
        } else if (U == 1) {
            for (int k = lane; k < nn; k += TPA) {
                const int e = __ldg(row + k);
                pair(e, __ldg(a.q32 + entry_j(e)), false);
            }
        } else {
            // two entries per step, sums in the order of the one-entry loop
            for (int k = lane; k < nn; k += 2 * TPA) {
                const bool v1 = k + TPA < nn;
                const int e0 = __ldg(row + k);
                const int e1 = v1 ? __ldg(row + k + TPA) : e0;
                const float4 q0 = __ldg(a.q32 + entry_j(e0));
                const float4 q1 = __ldg(a.q32 + entry_j(e1));
                pair(e0, q0, false);
                if (v1) pair(e1, q1, false);
            }
        }
        kahan_add(es, ec, ep);
        ec += epc;  // the atom's own correction (small): the thread total is es - ec
    }
    lane_sum_comp<TPA>(fx, fxc);
    lane_sum_comp<TPA>(fy, fyc);
    lane_sum_comp<TPA>(fz, fzc);
    if (active && lane == 0) {
        a.f32[i] = fx - fxc;
        a.f32[a.n + i] = fy - fyc;
        a.f32[2 * a.n + i] = fz - fzc;
    }
}

template <int TPA, bool ORTHO, int U>
__global__ void __launch_bounds__(256, 4) k_force32(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    float es = 0.f, ec = 0.f;  // pair energy, compensated
    float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // virial: plain FP32 per thread
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        force_atom<TPA, ORTHO, U>(a, S, K, a.fr, i, lane, active, es, ec, w);
    }
    auto sum_k = [&](int k) -> double {
        return k == 0 ? 0.5 * ((double)es - (double)ec) : 0.5 * (double)w[k - 1];
    };
    __shared__ double tot[7];
    if (block_partials_fn<7>(sum_k, a.partials, 0, &a.sc->counter[0]) && threadIdx.x < 32) {
        final_sums_smem<7>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            DevScalars* sc = a.sc;
            sc->energy = tot[0] + sc->e_embed;
            for (int k = 0; k < 6; k++) sc->virial[k] = tot[k + 1];
            sc->counter[0] = 0;
        }
    }
}

// k_force32 with the force records in shared memory: one 1024-thread block
// per SM works through the atoms one element group at a time, each group
// with its own records (r*phi of the group's pair types and the density
// derivatives they need) copied into shared memory first, so that a pair's
// records cost shared-memory reads instead of L1/L2 traffic
template <int TPA, bool ORTHO, int U>
__global__ void __launch_bounds__(1024, 1) k_force32s(EamArgs a) {
    extern __shared__ float4 ftab_s[];
    __shared__ Smem32 S;
    S.fill(a);  // ends with __syncthreads
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    const int nrec = a.fs_rec * a.fs_w;
    float es = 0.f, ec = 0.f;
    float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int g = 0; g < a.ne; g++) {
        const int lo = a.grp_begin[g], hi = a.grp_begin[g + 1];
        if (lo == hi) continue;
        __syncthreads();  // every thread is done with the previous group's records
        const float4* src = a.fs_tab + (size_t)g * a.fs_rec * a.fs_stride + a.fs_off;
        for (int k = threadIdx.x; k < nrec; k += blockDim.x) {
            const int r = k / a.fs_w;
            ftab_s[k] = __ldg(src + (size_t)r * a.fs_stride + (k - r * a.fs_w));
        }
        __syncthreads();
        for (int base = lo;; base += stride) {
            const int q = base + gid;
            const bool active = q < hi;
            if (!__any_sync(0xffffffffu, active)) break;
            const int i = !active ? 0 : (a.grp_atoms ? a.grp_atoms[q] : q);
            force_atom<TPA, ORTHO, U, Frame, true>(a, S, K, a.fr, i, lane, active, es, ec, w, ftab_s);
        }
    }
    auto sum_k = [&](int k) -> double {
        return k == 0 ? 0.5 * ((double)es - (double)ec) : 0.5 * (double)w[k - 1];
    };
    __shared__ double tot[7];
    if (block_partials_fn<7>(sum_k, a.partials, 0, &a.sc->counter[0]) && threadIdx.x < 32) {
        final_sums_smem<7>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            DevScalars* sc = a.sc;
            sc->energy = tot[0] + sc->e_embed;
            for (int k = 0; k < 6; k++) sc->virial[k] = tot[k + 1];
            sc->counter[0] = 0;
        }
    }
}

// the group records of k_force32s from the global force records (same
// values): out[(g * R + r) * W + w] for knot mlo + w
__global__ void k_fs_fill(EamArgs a, float4* __restrict__ out, int R, int W, int mlo) {
    const long long total = (long long)a.ne * R * W;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int w = (int)(idx % W);
        const int r = (int)((idx / W) % R);
        const int g = (int)(idx / ((long long)W * R));
        const int m = mlo + w;
        float4 v;
        if (r < a.ne) {
            const size_t kt = (size_t)(g * a.ne + r) * a.nr + m;
            const float4 r0 = a.ftab[2 * kt], r1 = a.ftab[2 * kt + 1];
            v = make_float4(r1.x, r1.y, r1.z, r0.w);
        } else if (r < 2 * a.ne) {
            const size_t kt = (size_t)(g * a.ne + (r - a.ne)) * a.nr + m;
            const float4 r0 = a.ftab[2 * kt], r1 = a.ftab[2 * kt + 1];
            v = make_float4(r0.x, r0.y, r0.z, r1.w);
        } else {
            const int k = r - 2 * a.ne;
            const int ej = k < g ? k : k + 1;
            v = a.fjtab[(size_t)(g * a.ne + ej) * a.nr + m];
        }
        out[idx] = v;
    }
}

// batch: chunk slots 0 pair energy, 1-6 virial
template <int TPA, bool ORTHO, int U>
__global__ void __launch_bounds__(256, 4) k_force32b(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        if (a.cell_active && !a.cell_active[a.chunk_cell[ch]]) continue;
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        const CellFrame fr = cell_frame<ORTHO>(a.cells + a.chunk_cell[ch]);
        float es = 0.f, ec = 0.f;
        float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            force_atom<TPA, ORTHO, U>(a, S, K, fr, i, lane, i < hi, es, ec, w);
        }
        chunk_store<7>(
            [&](int k) -> double {
                return k == 0 ? 0.5 * ((double)es - (double)ec) : 0.5 * (double)w[k - 1];
            },
            a.chunk_part + (size_t)ch * kChunkSlots);
    }
}

// one atom's energy: density and pair terms in one pass, then F(rho_i)
template <int TPA, bool ORTHO, class FR>
__device__ __forceinline__ void energy_atom(const EamArgs& a, const Smem32& S, const Consts32& K, const FR& fr,
                                            int i, int lane, bool active, float& es, float& ec) {
    float acc = 0.f, acc_c = 0.f, ep = 0.f, epc = 0.f;
    int ei = 0;
    if (active) {
        const float4 pi = __ldg(a.p32 + i);
        ei = a.elem[i];
        const int nn = __ldg(a.nnbr + i);
        const int* row = a.nbr + (size_t)i * a.maxnbr;
        for (int k = lane; k < nn; k += TPA) {
            const int e = __ldg(row + k);
            const int ej = entry_elem(e);
            const int t = ei * a.ne + ej;
            const float4 q = __ldg(a.p32 + entry_j(e));
            float4 o;
            image_offset(e, o);
            float dx, dy, dz;
            cart<ORTHO>(fr, (pi.x - q.x) + o.x, (pi.y - q.y) + o.y, (pi.z - q.z) + o.z, dx, dy, dz);
            const float rsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (rsq < S.cut_sq[t]) {
                const float rinv = inv_sqrt(rsq);
                const float r = rsq * rinv;
                float fr;
                const int m = knot32(fmaf(r, K.dri, r * K.dri_lo), a.nr - 2, fr);
                const float4 c = __ldg(a.rho32 + (size_t)(ej * a.ne + ei * a.rho_ei) * a.nr + m);
                kahan_add(acc, acc_c, fmaf(fmaf(fmaf(c.w, fr, c.z), fr, c.y), fr, c.x));
                const float4* rec = a.ftab + 2 * ((size_t)t * a.nr + m);
                float4 r0, r1;
                ldg8(rec, r0, r1);
                const float z = r0.w + fmaf(fr, fmaf(fmaf(r1.z, fr, r1.y), fr, r1.x), r1.w);
                kahan_add(ep, epc, 0.5f * z * rinv);
            }
        }
    }
    lane_sum_comp<TPA>(acc, acc_c);
    if (active) {
        kahan_add(es, ec, ep);
        ec += epc;
    }
    if (active && lane == 0) {
        float Fv, dFv;
        embed32f(a, ei, acc, acc_c, Fv, dFv);  // as the density pass (line searches compare the two)
        kahan_add(es, ec, Fv);
    }
}

template <int TPA, bool ORTHO>
__global__ void __launch_bounds__(256) k_energy32(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    float es = 0.f, ec = 0.f;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        energy_atom<TPA, ORTHO>(a, S, K, a.fr, i, lane, active, es, ec);
    }
    double v[1] = {(double)es - (double)ec};
    if (block_partials<1>(v, a.partials, 0, &a.sc->counter[2]) && threadIdx.x < 32) {
        double tot[1];
        final_sums<1>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            a.sc->energy = tot[0];
            a.sc->counter[2] = 0;
        }
    }
}

// batch: the chunk's energy goes to slot 0
template <int TPA, bool ORTHO>
__global__ void __launch_bounds__(256) k_energy32b(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        if (a.cell_active && !a.cell_active[a.chunk_cell[ch]]) continue;
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        const CellFrame fr = cell_frame<ORTHO>(a.cells + a.chunk_cell[ch]);
        float es = 0.f, ec = 0.f;
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            energy_atom<TPA, ORTHO>(a, S, K, fr, i, lane, i < hi, es, ec);
        }
        chunk_store<1>([&](int) { return (double)es - (double)ec; }, a.chunk_part + (size_t)ch * kChunkSlots);
    }
}

// ------------------------------------------------------------------ energy differences
// dE = E(x0 + alpha h) - E(x0) for the line-search trials of a mixed-
// precision minimizer.  FP32 energies of the two configurations each carry
// ~1e-4 eV of rounding at 10^5 atoms (mostly from r, whose relative error is
// ~1e-7, through rho'(r) and phi'(r)), as much as the energy decrease the
// Armijo test has to resolve near max|F| = 1e-4.  Differences are therefore
// formed pair by pair, where they are small, instead of between totals:
//   d' = d + alpha (h_i - h_j)                       (displacement, Cartesian)
//   r'^2 - r^2 = dd . (2 d + dd),  r' - r = (r'^2 - r^2) / (r + r')
//   g(r') - g(r) of a cubic spline from the knot fraction p and its change
//   dp = (r' - r)/dr: dp (c1 + c2 (p + p') + c3 (p^2 + p p' + p'^2)) inside
//   an interval, split at the knot when the step crosses one
//   phi' - phi = (dz r - z dr) / (r r'),  z = r phi
// so each term, and the total, is accurate relative to the difference itself.
// The embedding change F(rho0 + drho) - F(rho0) is taken per atom in FP64
// from the FP64 density of x0 (kept by the density pass) and the FP64 table.
// The neighbour rows and the FP32 frame positions are those of x0; the
// caller guarantees that x0 and the trial stay within half the skin of the
// list's build positions, so every pair inside the cutoff at either end is
// in the rows.

// change of one cubic c0 + c1 p + c2 p^2 + c3 p^3 from p to p + dp
__device__ __forceinline__ float cubic_step(float c1, float c2, float c3, float p, float dp) {
    const float q = p + dp;
    return dp * fmaf(c3, fmaf(p, p + q, q * q), fmaf(c2, p + q, c1));
}

// g(knot m1, p1) - g(knot m, p) of one spline whose knot-m coefficients are
// returned by coef(m) as (c0, c1, c2, c3): within one interval or across one
// knot by the step formula, otherwise (steps of more than one interval,
// where the difference is large) as the difference of the two values
template <class Coef>
__device__ __forceinline__ float spline_step(Coef coef, int m, float p, float dp, int mmax, int m1, float p1) {
    const float t = p + dp;
    const float4 c = coef(m);
    if (t >= 0.f && t < 1.f) return cubic_step(c.y, c.z, c.w, p, dp);
    if (t >= 1.f && t < 2.f && m + 1 <= mmax) {
        const float4 d = coef(m + 1);
        return cubic_step(c.y, c.z, c.w, p, 1.f - p) + cubic_step(d.y, d.z, d.w, 0.f, t - 1.f);
    }
    if (t < 0.f && t >= -1.f && m >= 1) {
        const float4 d = coef(m - 1);
        return cubic_step(c.y, c.z, c.w, p, -p) + cubic_step(d.y, d.z, d.w, 1.f, t);
    }
    const float4 d = coef(m1);
    const float g1 = fmaf(fmaf(fmaf(d.w, p1, d.z), p1, d.y), p1, d.x);
    const float g0 = fmaf(fmaf(fmaf(c.w, p, c.z), p, c.y), p, c.x);
    return g1 - g0;
}

// F(rho) in FP64 with the reference's clamps and linear extrapolation
// (ff_eam.cpp:180-189)
__device__ __forceinline__ double embed64(const EamArgs& a, int ei, double rho) {
    const double p = rho * a.drho_inv;
    int m = (int)p;
    if (m > a.nrho - 2) m = a.nrho - 2;
    double q = p - (double)m;
    if (q > 1.0) q = 1.0;
    const Dbl4 c = ldg4(a.F64 + (size_t)ei * a.nrho + m);
    double F = ((c.w * q + c.z) * q + c.y) * q + c.x;
    if (rho > a.rho_max) F += ((3.0 * c.w * q + 2.0 * c.z) * q + c.y) * a.drho_inv * (rho - a.rho_max);
    return F;
}

template <int TPA, bool ORTHO, class FR>
__device__ __forceinline__ void de_atom(const EamArgs& a, const Smem32& S, const Consts32& K, const FR& fr, int i,
                                        int lane, bool active, float alpha, float& es, float& ec) {
    float dr = 0.f, drc = 0.f, dp = 0.f, dpc = 0.f;  // density change, pair-energy change (compensated)
    int ei = 0;
    if (active) {
        const float4 pi = __ldg(a.p32 + i);
        const float4 hi = __ldg(a.h32 + i);
        ei = a.elem[i];
        const int nn = __ldg(a.nnbr + i);
        const int* row = a.nbr + (size_t)i * a.maxnbr;
        const int mmax = a.nr - 2;
        for (int k = lane; k < nn; k += TPA) {
            const int e = __ldg(row + k);
            const int j = entry_j(e), ej = entry_elem(e);
            const int t = ei * a.ne + ej;
            const float4 q = __ldg(a.p32 + j);
            const float4 hj = __ldg(a.h32 + j);
            float4 o;
            image_offset(e, o);
            float dx, dy, dz;
            cart<ORTHO>(fr, (pi.x - q.x) + o.x, (pi.y - q.y) + o.y, (pi.z - q.z) + o.z, dx, dy, dz);
            const float ux = alpha * (hi.x - hj.x), uy = alpha * (hi.y - hj.y), uz = alpha * (hi.z - hj.z);
            const float rsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float drsq = fmaf(ux, fmaf(2.f, dx, ux), fmaf(uy, fmaf(2.f, dy, uy), uz * fmaf(2.f, dz, uz)));
            const float rsq1 = rsq + drsq;
            const float cut = S.cut_sq[t];
            const bool in0 = rsq < cut, in1 = rsq1 < cut;
            if (!(in0 || in1)) continue;
            const float rinv = inv_sqrt(rsq), rinv1 = inv_sqrt(rsq1);
            const float r = rsq * rinv, r1 = rsq1 * rinv1;
            float p0, p1;
            const int m = knot32(fmaf(r, K.dri, r * K.dri_lo), mmax, p0);
            const int m1 = knot32(fmaf(r1, K.dri, r1 * K.dri_lo), mmax, p1);
            const float4* rt = a.rho32 + (size_t)(ej * a.ne + ei * a.rho_ei) * a.nr;
            const float4* ft = a.ftab + 2 * (size_t)t * a.nr;
            // the rphi record: (c0 head in .w of the first half, c1 c2 c3 and
            // the c0 tail in the second half)
            auto zc = [&](int mm) {
                float4 r0, r1r;
                ldg8(ft + 2 * (size_t)mm, r0, r1r);
                return make_float4(r0.w + r1r.w, r1r.x, r1r.y, r1r.z);
            };
            auto rc = [&](int mm) { return __ldg(rt + mm); };
            float drho, dphi;
            if (in0 && in1) {
                const float ddr = drsq / (r + r1);
                const float dpk = fmaf(ddr, K.dri, ddr * K.dri_lo);
                drho = spline_step(rc, m, p0, dpk, mmax, m1, p1);
                float4 r0, r1r;
                ldg8(ft + 2 * (size_t)m, r0, r1r);
                const float z = r0.w + fmaf(p0, fmaf(fmaf(r1r.z, p0, r1r.y), p0, r1r.x), r1r.w);
                const float dz = spline_step(zc, m, p0, dpk, mmax, m1, p1);
                dphi = fmaf(dz, r, -z * ddr) * (rinv * rinv1);
            } else {
                // the pair enters or leaves the cutoff: the change is the
                // (small, near-cutoff) value at the end inside
                const int mm = in1 ? m1 : m;
                const float pp = in1 ? p1 : p0, ri = in1 ? rinv1 : rinv, sg = in1 ? 1.f : -1.f;
                const float4 c = rc(mm);
                drho = sg * fmaf(fmaf(fmaf(c.w, pp, c.z), pp, c.y), pp, c.x);
                float4 r0, r1r;
                ldg8(ft + 2 * (size_t)mm, r0, r1r);
                const float z = r0.w + fmaf(pp, fmaf(fmaf(r1r.z, pp, r1r.y), pp, r1r.x), r1r.w);
                dphi = sg * z * ri;
            }
            kahan_add(dr, drc, drho);
            kahan_add(dp, dpc, dphi);
        }
    }
    lane_sum_comp<TPA>(dr, drc);
    if (active) {
        kahan_add(es, ec, 0.5f * dp);
        ec += 0.5f * dpc;
    }
    if (active && lane == 0) {
        const double drho_i = (double)dr - (double)drc;
        const double r0 = a.rho0[i];
        const double dF = embed64(a, ei, r0 + drho_i) - embed64(a, ei, r0);
        // dF carries FP64 precision; added as head and tail
        const float h = (float)dF;
        kahan_add(es, ec, h);
        kahan_add(es, ec, (float)(dF - (double)h));
    }
}

template <int TPA, bool ORTHO>
__global__ void __launch_bounds__(256) k_de32(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const float alpha = (float)a.alpha;
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    float es = 0.f, ec = 0.f;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        de_atom<TPA, ORTHO>(a, S, K, a.fr, i, lane, active, alpha, es, ec);
    }
    double v[1] = {(double)es - (double)ec};
    if (block_partials<1>(v, a.partials, 0, &a.sc->counter[6]) && threadIdx.x < 32) {
        double tot[1];
        final_sums<1>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            a.sc->de = tot[0];
            a.sc->counter[6] = 0;
        }
    }
}

// batch: the chunk's energy difference goes to slot 0 (cells in
// cell_active only)
template <int TPA, bool ORTHO>
__global__ void __launch_bounds__(256) k_de32b(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const int cell = a.chunk_cell[ch];
        if (a.cell_active && !a.cell_active[cell]) continue;
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        const CellFrame fr = cell_frame<ORTHO>(a.cells + cell);
        const float alpha = (float)a.cell_alpha[cell];
        float es = 0.f, ec = 0.f;
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            de_atom<TPA, ORTHO>(a, S, K, fr, i, lane, i < hi, alpha, es, ec);
        }
        chunk_store<1>([&](int) { return (double)es - (double)ec; }, a.chunk_part + (size_t)ch * kChunkSlots);
    }
}

// per-cell totals of a batch from the chunk slots, one warp per cell in a
// fixed order: what = 0 after a force pass (energy = pair + embedding,
// virial), 1 after an energy pass, 2 after a force pass with the MD tail
// (kinetic tensor and the closing half of each cell's chain, thermo rows of
// pe and T per cell)
__global__ void k_cells_done(EamArgs a, const int* __restrict__ cell_chunk, CellMd* __restrict__ cmd, int what) {
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    const int lo = cell_chunk[c], hi = cell_chunk[c + 1];
    double t[14];
#pragma unroll 1
    for (int k = 0; k < 14; k++) {
        double v = 0.0;
        const bool need = what == 1 ? k == 0 : (what == 0 ? (k <= 6 || k == 13) : true);
        if (need)
            for (int ch = lo + lane; ch < hi; ch += 32) v += a.chunk_part[(size_t)ch * kChunkSlots + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        t[k] = v;
    }
    if (lane != 0) return;
    CellMd* m = cmd + c;
    if (what == 1) {
        m->energy = t[0];
        return;
    }
    m->e_embed = t[13];
    m->energy = t[0] + t[13];
    for (int k = 0; k < 6; k++) m->virial[k] = t[1 + k];
    if (what == 2) {
        NhcParams P = a.nhc;
        P.T = m->T;
        P.ndof = (int)m->ndof;
        P.ndof_kB = m->ndof_kB;
        for (int k = 0; k < 6; k++) m->mvv[k] = t[7 + k];
        m->T_part = (t[7] + (t[10] + t[12])) / m->ndof_kB;
        m->fac_close = thermo_half(P, m);
        m->pending_kick = 1;
        const long long st = ++m->step;
        if (a.thermo && st <= a.nsteps) {
            double* r = a.thermo + 2 * ((size_t)st * a.ncell + c);
            r[0] = m->energy;
            r[1] = m->T_part;
        }
        if (!(isfinite(m->energy) && isfinite(m->T_part))) a.sc->bad = 1;
    }
}

// ------------------------------------------------------------------ launchers
// kernels take (lanes per atom TPA, orthorhombic frame, neighbour entries per
// loop step U); TPA and U come from the system (mappg_sys_autotune)
template <int TPA, bool ORTHO, int U>
static void density_t(mappg_sys* s, const EamArgs& a) {
    static bool attr = false;
    if (!attr) {
        MAPPG_CUDA(cudaFuncSetAttribute(k_density32s<TPA, ORTHO, U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)kDensSmemBytes));
        attr = true;
    }
    const size_t bytes = sizeof(float4) * (size_t)a.rho_ntab * a.rho_w;
    k_density32s<TPA, ORTHO, U><<<s->sm_count, 1024, bytes, s->stream>>>(a);
}

template <int TPA, bool ORTHO, int U>
static void force_t(mappg_sys* s, const EamArgs& a) {
    if (s->force_smem > 0 && a.fs_tab) {
        static bool attr = false;
        if (!attr) {
            MAPPG_CUDA(cudaFuncSetAttribute(k_force32s<TPA, ORTHO, U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            s->smem_optin - (int)kForceSmemReserve));
            attr = true;
        }
        const size_t bytes = sizeof(float4) * (size_t)a.fs_rec * a.fs_w;
        k_force32s<TPA, ORTHO, U><<<s->sm_count, 1024, bytes, s->stream>>>(a);
        return;
    }
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_force32<TPA, ORTHO, U>, 256);
    k_force32<TPA, ORTHO, U><<<grid, 256, 0, s->stream>>>(a);
}

template <int TPA, bool ORTHO, int U>
static void energy_t(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_energy32<TPA, ORTHO>, 256);
    k_energy32<TPA, ORTHO><<<grid, 256, 0, s->stream>>>(a);
}

template <int TPA, bool ORTHO, int U>
static void de_t(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_de32<TPA, ORTHO>, 256);
    k_de32<TPA, ORTHO><<<grid, 256, 0, s->stream>>>(a);
}

template <int TPA, bool ORTHO, int U>
static void de_b(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_de32b<TPA, ORTHO>, 256);
    k_de32b<TPA, ORTHO><<<std::min(grid, a.nchunk), 256, 0, s->stream>>>(a);
}

template <int TPA, bool ORTHO, int U>
static void density_b(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_density32b<TPA, ORTHO, U>, 256);
    k_density32b<TPA, ORTHO, U><<<std::min(grid, a.nchunk), 256, 0, s->stream>>>(a);
}

template <int TPA, bool ORTHO, int U>
static void force_b(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_force32b<TPA, ORTHO, U>, 256);
    k_force32b<TPA, ORTHO, U><<<std::min(grid, a.nchunk), 256, 0, s->stream>>>(a);
}

template <int TPA, bool ORTHO, int U>
static void energy_b(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_energy32b<TPA, ORTHO>, 256);
    k_energy32b<TPA, ORTHO><<<std::min(grid, a.nchunk), 256, 0, s->stream>>>(a);
}

// a batch takes the orthorhombic kernels only when every cell is orthorhombic
static bool all_ortho(const mappg_sys* s) {
    for (const CellGeo& g : s->cells)
        if (!g.ortho) return false;
    return true;
}

template <int TPA, int U, class F>
static void pick_ortho(bool o, F&& fn) {
    if (o)
        fn(std::integral_constant<int, TPA>(), std::true_type(), std::integral_constant<int, U>());
    else
        fn(std::integral_constant<int, TPA>(), std::false_type(), std::integral_constant<int, U>());
}

// dispatch on the system's lanes per atom, unroll and frame shape
#define MAPPG_DISPATCH32U(FN, ORTHO_EXPR, UNROLL)                                                     \
    do {                                                                                              \
        const bool o = (ORTHO_EXPR);                                                                  \
        auto call = [&](auto T, auto O, auto U) { FN<decltype(T)::value, decltype(O)::value, decltype(U)::value>(s, a); }; \
        const bool u2 = (UNROLL) == 2;                                                                \
        switch (s->tpa) {                                                                             \
            case 4: u2 ? pick_ortho<4, 2>(o, call) : pick_ortho<4, 1>(o, call); break;                \
            case 16: u2 ? pick_ortho<16, 2>(o, call) : pick_ortho<16, 1>(o, call); break;            \
            case 32: pick_ortho<32, 1>(o, call); break;                                               \
            default: u2 ? pick_ortho<8, 2>(o, call) : pick_ortho<8, 1>(o, call); break;               \
        }                                                                                             \
        MAPPG_CUDA(cudaGetLastError());                                                               \
    } while (0)

#define MAPPG_DISPATCH32(FN, ORTHO_EXPR) MAPPG_DISPATCH32U(FN, ORTHO_EXPR, s->unroll)
#define MAPPG_TPA32(FN) MAPPG_DISPATCH32(FN, a.fr.ortho != 0)
#define MAPPG_TPA32B(FN) MAPPG_DISPATCH32(FN, all_ortho(s))
// the force pass's entries per loop step (it may differ from the density pass's)
#define MAPPG_FORCE_U (s->unroll_force ? s->unroll_force : s->unroll)

static void cells_done(mappg_sys* s, const EamArgs& a, int what) {
    k_cells_done<<<(s->ncell * 32 + 255) / 256, 256, 0, s->stream>>>(a, s->cell_chunk, s->cmd, what);
    MAPPG_CUDA(cudaGetLastError());
}

void launch_cells_done(mappg_sys* s, const EamArgs& a, int what) { cells_done(s, a, what); }

void launch_density32(mappg_sys* s, const EamArgs& a) {
    if (s->ncell > 1)
        MAPPG_TPA32B(density_b);
    else
        MAPPG_TPA32(density_t);
}
// the group records of k_force32s for as many knots as fit in the shared
// memory a block may opt in to, from the knot of the cutoff down (a table
// may reach beyond the cutoff; knots there are never read)
bool force_smem_available(mappg_sys* s) {
    if (s->ncell > 1 || s->precision != MAPPG_MIXED || s->ne > kMaxElem) return false;
    if (s->fs_tab) return true;
    const int nr = s->ff->dev.nr;
    const int R = s->ff->dev.rho_ei ? 3 * s->ne - 1 : 2 * s->ne;
    const long long budget = (long long)s->smem_optin - (long long)kForceSmemReserve;
    const int mhi = std::min(nr - 2, (int)((s->max_cut - s->skin) * s->ff->dev.dr_inv) + 1);
    const int W = (int)std::min<long long>(mhi + 1, budget / ((long long)sizeof(float4) * R));
    if (W < 16) return false;
    MAPPG_CUDA(cudaMalloc(&s->fs_tab, sizeof(float4) * (size_t)s->ne * R * W));
    EamArgs a = eam_args(s);
    k_fs_fill<<<256, 256, 0, s->stream>>>(a, s->fs_tab, R, W, mhi + 1 - W);
    MAPPG_CUDA(cudaGetLastError());
    s->fs_rec = R;
    s->fs_w = W;
    s->fs_mlo = mhi + 1 - W;
    return true;
}

int force_smem_max_kb(const mappg_sys* s) {
    return s->fs_rec > 0 ? (int)(((long long)sizeof(float4) * s->fs_rec * s->fs_w + 1023) / 1024) : 0;
}

void launch_force32(mappg_sys* s, const EamArgs& a) {
    if (s->ncell > 1) {
        MAPPG_DISPATCH32U(force_b, all_ortho(s), MAPPG_FORCE_U);
        cells_done(s, a, 0);
    } else {
        MAPPG_DISPATCH32U(force_t, a.fr.ortho != 0, MAPPG_FORCE_U);
    }
}
// E(x0 + alpha h) - E(x0) into sc->de (one cell; p32, rows and rho of x0,
// h32 set by the caller)
void launch_de32(mappg_sys* s, double alpha) {
    EamArgs a = eam_args(s);
    a.alpha = alpha;
    MAPPG_TPA32(de_t);
}

// batch: per-cell energy differences with each cell's trial step
// cell_alpha[c], for the cells in cell_active, into CellMd::energy
void launch_de32b(mappg_sys* s, const double* cell_alpha) {
    EamArgs a = eam_args(s);
    a.cell_alpha = cell_alpha;
    MAPPG_TPA32B(de_b);
    cells_done(s, a, 1);
}

void launch_energy32(mappg_sys* s, const EamArgs& a) {
    if (s->ncell > 1) {
        MAPPG_TPA32B(energy_b);
        cells_done(s, a, 1);
    } else {
        MAPPG_TPA32(energy_t);
    }
}

}  // namespace mappg
