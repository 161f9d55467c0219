// Mixed-precision EAM kernels: FP32 pair geometry and spline arithmetic in
// the scaled bin frame (system.h), FP64 state, FP64 totals.
//
//   k_density32  rho_i in FP32, then F'(rho_i) and F(rho_i) from the FP32
//                embedding table with its constant term carried as head +
//                tail; writes q32[i] = (p'_i, F'_i) for the force pass
//   k_force32    forces, pair energy and virial from one 48-byte record per
//                (pair type, knot); F'_j rides in q32[j].w, so a neighbour
//                costs one 16-byte gather plus the record; optional MD tail:
//                kinetic tensor of v + f dt/2m and the closing half of the
//                Nose-Hoover chain in the last block
//   k_energy32   energy only (line-search trials)
//
// Precision: every per-pair term is FP32; per-atom sums are FP32 within a
// lane group; energies are accumulated per lane with compensated FP32 sums
// and reduced in FP64 across lanes and blocks.  Constants shared by many
// pairs (1/dr, the frame-to-Cartesian scale, the spline constant terms) are
// carried as head + tail so their rounding does not bias the totals.
//
// Table index: p = r/dr, m = floor(p) via an add with round-toward-zero
// against 2^23, then the reference's clamps m <= nr-2, p - m <= 1
// (ff_eam.cpp:122-128).
#include <math.h>

#include <algorithm>

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

// frame offset of a neighbour image from its entry's bin-step code
// c = (d0+1) + 3(d1+1) + 9(d2+1): -8 d, computed instead of read from a
// table (the pair loops are bound by the L1 data pipe, which a shared-
// memory table would share)
__device__ __forceinline__ void code_offset(int e, float& ox, float& oy, float& oz) {
    const int c = entry_code(e);
    const int t9 = (c >= 9) + (c >= 18);
    const int r9 = c - 9 * t9;
    const int t3 = (r9 >= 3) + (r9 >= 6);
    const int t1 = r9 - 3 * t3;
    ox = (float)(8 - 8 * t1);
    oy = (float)(8 - 8 * t3);
    oz = (float)(8 - 8 * t9);
}

// squared cutoffs of up to four pair types held in registers
struct Cut4 {
    float c0, c1, c2, c3;
    __device__ Cut4(const Smem32& S, int ne) {
        c0 = S.cut_sq[0];
        c1 = ne * ne > 1 ? S.cut_sq[1] : c0;
        c2 = ne * ne > 2 ? S.cut_sq[2] : c0;
        c3 = ne * ne > 3 ? S.cut_sq[3] : c0;
    }
    __device__ __forceinline__ float operator()(const Smem32& S, int t) const {
        if (t > 3) return S.cut_sq[t];  // more than two elements
        return (t & 2) ? ((t & 1) ? c3 : c2) : ((t & 1) ? c1 : c0);
    }
};

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
    float dri, dri_lo, drhoi, drhoi_lo, rho_max;
    __device__ Consts32(const EamArgs& a) {
        dri = (float)a.dr_inv;
        dri_lo = (float)(a.dr_inv - (double)dri);
        drhoi = (float)a.drho_inv;
        drhoi_lo = (float)(a.drho_inv - (double)drhoi);
        rho_max = (float)a.rho_max;
    }
};

// embedding F and F' from the FP32 table, constant term as head + tail;
// linear extrapolation above rho_max as ff_eam.cpp:180-191
__device__ __forceinline__ void embed32(const EamArgs& a, const Consts32& K, int ei, float rho, float& Fv,
                                        float& dFv) {
    float fr;
    const int m = knot32(fmaf(rho, K.drhoi, rho * K.drhoi_lo), a.nrho - 2, fr);
    const size_t k = (size_t)ei * a.nrho + m;
    const float4 c = __ldg(a.F32 + k);
    dFv = fmaf(fmaf(3.0f * c.w, fr, 2.0f * c.z), fr, c.y) * K.drhoi;
    Fv = c.x + (__ldg(a.F32lo + k) + fr * fmaf(fmaf(c.w, fr, c.z), fr, c.y));
    if (rho > K.rho_max) Fv += dFv * (rho - K.rho_max);
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

// one atom's density row (TPA lanes), its embedding terms and q32 record
template <int TPA, bool ORTHO, class FR>
__device__ __forceinline__ void density_atom(const EamArgs& a, const Smem32& S, const Consts32& K, const FR& fr,
                                             int i, int lane, bool active, float& es, float& ec) {
    float acc = 0.f;
    int ei = 0;
    const Cut4 cut(S, a.ne);
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) {
        pi = __ldg(a.p32 + i);
        ei = a.elem[i];
        const int nn = __ldg(a.nnbr + i);
        const int* row = a.nbr + (size_t)i * a.maxnbr;
        for (int k = lane; k < nn; k += TPA) {
            const int e = __ldg(row + k);
            const int ej = entry_elem(e);
            const float4 q = __ldg(a.p32 + entry_j(e));
            float ox, oy, oz;
            code_offset(e, ox, oy, oz);
            float dx, dy, dz;
            cart<ORTHO>(fr, (pi.x - q.x) + ox, (pi.y - q.y) + oy, (pi.z - q.z) + oz, dx, dy, dz);
            const float rsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (rsq < cut(S, ei * a.ne + ej)) {
                const float r = rsq * inv_sqrt(rsq);
                float fr;
                const int m = knot32(fmaf(r, K.dri, r * K.dri_lo), a.nr - 2, fr);
                const float4 c = __ldg(a.rho32 + (size_t)(ej * a.ne + ei) * a.nr + m);
                acc += fmaf(fmaf(fmaf(c.w, fr, c.z), fr, c.y), fr, c.x);
            }
        }
    }
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPA);
    if (active && lane == 0) {
        float Fv, dFv;
        embed32(a, K, ei, acc, Fv, dFv);
        a.q32[i] = make_float4(pi.x, pi.y, pi.z, dFv);
        a.rho32out[i] = acc;
        kahan_add(es, ec, Fv);
    }
}

template <int TPA, bool ORTHO>
__global__ void __launch_bounds__(256, 8) k_density32(EamArgs a) {
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
        density_atom<TPA, ORTHO>(a, S, K, a.fr, i, lane, active, es, ec);
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
template <int TPA, bool ORTHO>
__global__ void __launch_bounds__(256, 8) k_density32b(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        const CellFrame fr = cell_frame<ORTHO>(a.cells + a.chunk_cell[ch]);
        float es = 0.f, ec = 0.f;
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            density_atom<TPA, ORTHO>(a, S, K, fr, i, lane, i < hi, es, ec);
        }
        chunk_store<1>([&](int) { return (double)es - (double)ec; }, a.chunk_part + (size_t)ch * kChunkSlots + 13);
    }
}

// one atom's force row (TPA lanes): force, pair energy, virial and (TAIL) the
// kinetic tensor of v + f dt/2m into the thread's shared slots ke[c*256]
template <int TPA, bool ORTHO, bool TAIL, class FR>
__device__ __forceinline__ void force_atom(const EamArgs& a, const Smem32& S, const Consts32& K, const FR& fr,
                                           int i, int lane, bool active, float& es, float& ec, float (&w)[6],
                                           float* ke) {
    float fx = 0.f, fy = 0.f, fz = 0.f, ep = 0.f;
    const Cut4 cut(S, a.ne);
    int ei = 0;
    if (active) {
        const float4 pi = __ldg(a.q32 + i);
        const float dFi = pi.w;
        ei = a.elem[i];
        const int nn = __ldg(a.nnbr + i);
        const int* row = a.nbr + (size_t)i * a.maxnbr;
        for (int k = lane; k < nn; k += TPA) {
            const int e = __ldg(row + k);
            const int t = ei * a.ne + entry_elem(e);
            const float4 q = __ldg(a.q32 + entry_j(e));
            float ox, oy, oz;
            code_offset(e, ox, oy, oz);
            float dx, dy, dz;
            cart<ORTHO>(fr, (pi.x - q.x) + ox, (pi.y - q.y) + oy, (pi.z - q.z) + oz, dx, dy, dz);
            const float rsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (rsq < cut(S, t)) {
                const float rinv = inv_sqrt(rsq);
                const float r = rsq * rinv;
                float fr;
                const int m = knot32(fmaf(r, K.dri, r * K.dri_lo), a.nr - 2, fr);
                const size_t kt = (size_t)t * a.nr + m;
                float4 r0, r1;
                ldg8(a.ftab + 2 * kt, r0, r1);
                const float der_i = fmaf(fmaf(r0.z, fr, r0.y), fr, r0.x);
                float der_j = der_i;
                if (entry_elem(e) != ei) {
                    const float4 r2 = __ldg(a.fjtab + kt);
                    der_j = fmaf(fmaf(r2.z, fr, r2.y), fr, r2.x);
                }
                const float zpoly = fmaf(fmaf(r1.z, fr, r1.y), fr, r1.x);
                const float z = r0.w + fmaf(fr, zpoly, r1.w);
                const float zp = fmaf(fmaf(3.0f * r1.z, fr, 2.0f * r1.y), fr, r1.x) * K.dri;
                const float phi = z * rinv;
                const float dphi = (zp - phi) * rinv;
                const float fp = -fmaf(dFi, der_i, fmaf(q.w, der_j, dphi)) * rinv;
                const float fdx = fp * dx, fdy = fp * dy, fdz = fp * dz;
                fx += fdx;
                fy += fdy;
                fz += fdz;
                ep += phi;
                w[0] = fmaf(fdx, dx, w[0]);
                w[1] = fmaf(fdx, dy, w[1]);
                w[2] = fmaf(fdx, dz, w[2]);
                w[3] = fmaf(fdy, dy, w[3]);
                w[4] = fmaf(fdy, dz, w[4]);
                w[5] = fmaf(fdz, dz, w[5]);
            }
        }
        kahan_add(es, ec, ep);
    }
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o, TPA);
        fy += __shfl_xor_sync(0xffffffffu, fy, o, TPA);
        fz += __shfl_xor_sync(0xffffffffu, fz, o, TPA);
    }
    if (active && lane == 0) {
        a.f32[i] = fx;
        a.f32[a.n + i] = fy;
        a.f32[2 * a.n + i] = fz;
        if (TAIL) {
            // kinetic tensor of the half-kicked velocity v + f dt/2m
            const float dtm = a.dtm32[ei], m = a.mass32[ei];
            const float vx = fmaf(fx, dtm, __ldg(a.v32 + i));
            const float vy = fmaf(fy, dtm, __ldg(a.v32 + a.n + i));
            const float vz = fmaf(fz, dtm, __ldg(a.v32 + 2 * a.n + i));
            const float mx = m * vx, my = m * vy, mz = m * vz;
            ke[0] = fmaf(mx, vx, ke[0]);
            ke[256] = fmaf(mx, vy, ke[256]);
            ke[512] = fmaf(mx, vz, ke[512]);
            ke[768] = fmaf(my, vy, ke[768]);
            ke[1024] = fmaf(my, vz, ke[1024]);
            ke[1280] = fmaf(mz, vz, ke[1280]);
        }
    }
}

template <int TPA, bool ORTHO, bool TAIL>
__global__ void __launch_bounds__(256, 5) k_force32(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    const int stride = (gridDim.x * blockDim.x) / TPA;
    float es = 0.f, ec = 0.f;  // pair energy, compensated
    float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    // kinetic tensor (TAIL): one private shared-memory slot per thread keeps
    // these six sums out of registers, so the MD variant runs at the same
    // occupancy as the plain one
    __shared__ float ke[TAIL ? 6 : 1][256];
    if (TAIL)
#pragma unroll
        for (int c = 0; c < 6; c++) ke[c][threadIdx.x] = 0.f;
    for (int base = 0;; base += stride) {
        const int i = gid + base;
        const bool active = i < a.n;
        if (!__any_sync(0xffffffffu, active)) break;
        force_atom<TPA, ORTHO, TAIL>(a, S, K, a.fr, i, lane, active, es, ec, w, &ke[0][threadIdx.x]);
    }
    constexpr int NS = TAIL ? 13 : 7;  // energy, virial[6], kinetic tensor[6]
    auto sum_k = [&](int k) -> double {
        switch (k) {
            case 0: return 0.5 * ((double)es - (double)ec);
            case 1: return 0.5 * (double)w[0];
            case 2: return 0.5 * (double)w[1];
            case 3: return 0.5 * (double)w[2];
            case 4: return 0.5 * (double)w[3];
            case 5: return 0.5 * (double)w[4];
            case 6: return 0.5 * (double)w[5];
            default: return (double)ke[TAIL ? k - 7 : 0][threadIdx.x];
        }
    };
    __shared__ double tot[NS];
    if (block_partials_fn<NS>(sum_k, a.partials, 0, &a.sc->counter[0]) && threadIdx.x < 32) {
        final_sums_smem<NS>(a.partials, gridDim.x, tot);
        if (threadIdx.x == 0) {
            DevScalars* sc = a.sc;
            sc->energy = tot[0] + sc->e_embed;
            for (int k = 0; k < 6; k++) sc->virial[k] = tot[k + 1];
            if (TAIL) {
                // update_x_d (md_nvt.cpp:106-128) then the closing half of the
                // thermostat (md_nvt.cpp:427-432)
                for (int k = 0; k < 6; k++) sc->mvv[k] = tot[7 + k];
                sc->T_part = (tot[7] + (tot[10] + tot[12])) / a.nhc.ndof_kB;
                sc->fac_close = thermo_half(a.nhc, sc);
                sc->pending_kick = 1;
                long long st = ++sc->step;
                if (st <= a.nsteps) write_thermo_row(a.thermo, sc, st);
                if (!(isfinite(sc->energy) && isfinite(sc->T_part))) sc->bad = 1;
            }
            sc->counter[0] = 0;
        }
    }
}

// batch: chunk slots 0 pair energy, 1-6 virial, 7-12 kinetic tensor (TAIL)
template <int TPA, bool ORTHO, bool TAIL>
__global__ void __launch_bounds__(256, 5) k_force32b(EamArgs a) {
    __shared__ Smem32 S;
    S.fill(a);
    const Consts32 K(a);
    const int lane = threadIdx.x % TPA;
    const int apb = blockDim.x / TPA;
    __shared__ float ke[TAIL ? 6 : 1][256];
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        const CellFrame fr = cell_frame<ORTHO>(a.cells + a.chunk_cell[ch]);
        float es = 0.f, ec = 0.f;
        float w[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (TAIL)
#pragma unroll
            for (int c = 0; c < 6; c++) ke[c][threadIdx.x] = 0.f;
        for (int i0 = lo; i0 < hi; i0 += apb) {
            const int i = i0 + (int)threadIdx.x / TPA;
            force_atom<TPA, ORTHO, TAIL>(a, S, K, fr, i, lane, i < hi, es, ec, w, &ke[0][threadIdx.x]);
        }
        constexpr int NS = TAIL ? 13 : 7;
        chunk_store<NS>(
            [&](int k) -> double {
                switch (k) {
                    case 0: return 0.5 * ((double)es - (double)ec);
                    case 1: return 0.5 * (double)w[0];
                    case 2: return 0.5 * (double)w[1];
                    case 3: return 0.5 * (double)w[2];
                    case 4: return 0.5 * (double)w[3];
                    case 5: return 0.5 * (double)w[4];
                    case 6: return 0.5 * (double)w[5];
                    default: return (double)ke[TAIL ? k - 7 : 0][threadIdx.x];
                }
            },
            a.chunk_part + (size_t)ch * kChunkSlots);
    }
}

// one atom's energy: density and pair terms in one pass, then F(rho_i)
template <int TPA, bool ORTHO, class FR>
__device__ __forceinline__ void energy_atom(const EamArgs& a, const Smem32& S, const Consts32& K, const FR& fr,
                                            int i, int lane, bool active, float& es, float& ec) {
    float acc = 0.f, ep = 0.f;
    int ei = 0;
    const Cut4 cut(S, a.ne);
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
            float ox, oy, oz;
            code_offset(e, ox, oy, oz);
            float dx, dy, dz;
            cart<ORTHO>(fr, (pi.x - q.x) + ox, (pi.y - q.y) + oy, (pi.z - q.z) + oz, dx, dy, dz);
            const float rsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (rsq < cut(S, t)) {
                const float rinv = inv_sqrt(rsq);
                const float r = rsq * rinv;
                float fr;
                const int m = knot32(fmaf(r, K.dri, r * K.dri_lo), a.nr - 2, fr);
                const float4 c = __ldg(a.rho32 + (size_t)(ej * a.ne + ei) * a.nr + m);
                acc += fmaf(fmaf(fmaf(c.w, fr, c.z), fr, c.y), fr, c.x);
                const float4* rec = a.ftab + 2 * ((size_t)t * a.nr + m);
                float4 r0, r1;
                ldg8(rec, r0, r1);
                const float z = r0.w + fmaf(fr, fmaf(fmaf(r1.z, fr, r1.y), fr, r1.x), r1.w);
                ep += 0.5f * z * rinv;
            }
        }
    }
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPA);
    if (active) kahan_add(es, ec, ep);
    if (active && lane == 0) {
        float Fv, dFv;
        embed32(a, K, ei, acc, Fv, dFv);
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
template <int TPA, bool ORTHO>
static void density_t(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_density32<TPA, ORTHO>, 256);
    k_density32<TPA, ORTHO><<<grid, 256, 0, s->stream>>>(a);
}

template <int TPA, bool ORTHO>
static void force_t(mappg_sys* s, const EamArgs& a) {
    static int grid = 0, grid_tail = 0;
    if (a.md_tail) {
        if (!grid_tail) grid_tail = occupancy_grid(s, k_force32<TPA, ORTHO, true>, 256);
        k_force32<TPA, ORTHO, true><<<grid_tail, 256, 0, s->stream>>>(a);
    } else {
        if (!grid) grid = occupancy_grid(s, k_force32<TPA, ORTHO, false>, 256);
        k_force32<TPA, ORTHO, false><<<grid, 256, 0, s->stream>>>(a);
    }
}

template <int TPA, bool ORTHO>
static void energy_t(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_energy32<TPA, ORTHO>, 256);
    k_energy32<TPA, ORTHO><<<grid, 256, 0, s->stream>>>(a);
}

#define MAPPG_TPA32(FN)                                  \
    do {                                                 \
        const bool o = a.fr.ortho != 0;                  \
        switch (s->tpa) {                                \
            case 4: o ? FN<4, true>(s, a) : FN<4, false>(s, a); break;    \
            case 16: o ? FN<16, true>(s, a) : FN<16, false>(s, a); break; \
            case 32: o ? FN<32, true>(s, a) : FN<32, false>(s, a); break; \
            default: o ? FN<8, true>(s, a) : FN<8, false>(s, a); break;   \
        }                                                \
        MAPPG_CUDA(cudaGetLastError());                  \
    } while (0)

template <int TPA, bool ORTHO>
static void density_b(mappg_sys* s, const EamArgs& a) {
    static int grid = 0;
    if (!grid) grid = occupancy_grid(s, k_density32b<TPA, ORTHO>, 256);
    k_density32b<TPA, ORTHO><<<std::min(grid, a.nchunk), 256, 0, s->stream>>>(a);
}

template <int TPA, bool ORTHO>
static void force_b(mappg_sys* s, const EamArgs& a) {
    static int grid = 0, grid_tail = 0;
    if (a.md_tail) {
        if (!grid_tail) grid_tail = occupancy_grid(s, k_force32b<TPA, ORTHO, true>, 256);
        k_force32b<TPA, ORTHO, true><<<std::min(grid_tail, a.nchunk), 256, 0, s->stream>>>(a);
    } else {
        if (!grid) grid = occupancy_grid(s, k_force32b<TPA, ORTHO, false>, 256);
        k_force32b<TPA, ORTHO, false><<<std::min(grid, a.nchunk), 256, 0, s->stream>>>(a);
    }
}

template <int TPA, bool ORTHO>
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

#define MAPPG_TPA32B(FN)                                 \
    do {                                                 \
        const bool o = all_ortho(s);                     \
        switch (s->tpa) {                                \
            case 4: o ? FN<4, true>(s, a) : FN<4, false>(s, a); break;    \
            case 16: o ? FN<16, true>(s, a) : FN<16, false>(s, a); break; \
            case 32: o ? FN<32, true>(s, a) : FN<32, false>(s, a); break; \
            default: o ? FN<8, true>(s, a) : FN<8, false>(s, a); break;   \
        }                                                \
        MAPPG_CUDA(cudaGetLastError());                  \
    } while (0)

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
void launch_force32(mappg_sys* s, const EamArgs& a) {
    if (s->ncell > 1) {
        MAPPG_TPA32B(force_b);
        cells_done(s, a, a.md_tail ? 2 : 0);
    } else {
        MAPPG_TPA32(force_t);
    }
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
