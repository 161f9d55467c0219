// NVT molecular dynamics on the device: md.nvt(T,dt).run(atoms,nsteps).
//
// One step of MDNVT::run (md_nvt.cpp:409-438) is a fixed kernel sequence,
// captured once into a CUDA graph and replayed.
//
// FP64 path (the reference's operation order, f*dt2/m with a division and no
// fused multiply-adds, so the trajectory follows the oracle to rounding):
//   k_step_open      fac_x_d *= chain(T/T0), the opening thermostat half
//   k_kick_drift64   v = v*fac_x_d + f*dt2/m; x += v*dt; sum of v*dt
//                    (update_x_d__x, md_nvt.cpp:70-102)
//   k_com_skin64     x -= mean displacement; skin test (DynamicMD::decide,
//                    dynamic_md.cpp:90-105) opens the rebuild gate
//   rebuild chain    (system.cu) only when the gate is open
//   density, force   (eam.cu)
//   k_kick2_64       v += f*dt2/m, kinetic tensor (update_x_d,
//                    md_nvt.cpp:106-128), closing thermostat half, thermo row
//
// Mixed path (FP64 state, fewer FP64 instructions; GB300 runs FP64 at a
// small fraction of FP32):
//   k_step_open32    opening half; the pending closing kick of the previous
//                    step and this step's kick fold into v <- A v + B f dt/2m
//                    (A = fc*fo, B = 1 + fc*fo; A = fo, B = 1 on the first)
//   k_integrate32    that kick, x += v dt (FP64), v32 = (float)v, the frame
//                    position p32 from x, the FP32 skin test and the
//                    displacement sum; the mean displacement is accumulated
//                    in sc->drift and removed from x at the next rebuild and
//                    at the end of the run (a uniform shift leaves forces and
//                    energies unchanged)
//   rebuild chain, k_density32, k_force32 with the MD tail (kinetic tensor of
//   v + f dt/2m, closing half, thermo row)
// Velocity scaling stays lazy as in the reference: the chain's factor is
// folded into the next kick and applied at the end of the run
// (update_x_d_final, md_nvt.cpp:51-56).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "eam_common.cuh"
#include "nhc.cuh"

namespace mappg {

void launch_cells_done(mappg_sys* s, const EamArgs& a, int what);  // eam32.cu
void lb_update(mappg_sys* s);                                       // lbfgs.cu

struct MdArgs {
    int n;
    double* x;
    double* v;
    const double* f;
    const float* f32;
    float* v32;
    const double* x0;
    const uint8_t* elem;
    const int* binc;
    float4* p32;
    const float4* p0;
    const uint8_t* dof;    // x_dof bits (null: every component free)
    int com_on[3];         // the mean displacement is removed along c (no frozen atom along c)
    double masses[kMaxElem];
    double dtm[kMaxElem];  // dt2/m
    float dtm32[kMaxElem];
    float m32[kMaxElem];   // masses as floats (the kinetic tensors' FP32 products)
    double dt, dt2, skin_sq;
    float dt32, skin_sq32;
    double bs[6];          // x -> scaled frame
    Frame fr;
    double* partials;
    double* thermo;  // rows of 14 or null (a batch: rows of ncell x (pe, T))
    long long nsteps;
    NhcParams nhc;
    DevScalars* sc;
    // batch of cells
    int ncell, nchunk;
    const CellGeo* cells;
    const int* cell_of;
    const int* chunk_begin;
    const int* chunk_cell;
    const int* cell_chunk;
    double* chunk_part;
    double* chunk_disp;
    CellMd* cmd;
    uint8_t* cell_reb;  // per cell: an atom moved beyond skin/2 (rebuild that cell)
};

// NHC parameters of one cell of a batch: its own target and dof
__device__ __forceinline__ NhcParams cell_nhc(const NhcParams& P0, const CellMd* m) {
    NhcParams P = P0;
    P.T = m->T;
    P.ndof = (int)m->ndof;
    P.ndof_kB = m->ndof_kB;
    return P;
}

template <int K>
__device__ bool md_block_partials(double (&v)[K], double* partials, unsigned* counter) {
    return block_partials<K>(v, partials, 0, counter);
}

// pre_init (md_nvt.cpp:256-340): kinetic tensor and temperature of the
// incoming velocities
__global__ void k_mvv_init(MdArgs a) {
    double d[6] = {0, 0, 0, 0, 0, 0};
    const int n = a.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double m = a.masses[a.elem[i]];
        double v0 = a.v[i], v1 = a.v[n + i], v2 = a.v[2 * n + i];
        if (a.dof) {
            const unsigned b = a.dof[i];
            if (!(b & 1u)) v0 = 0.0;
            if (!(b & 2u)) v1 = 0.0;
            if (!(b & 4u)) v2 = 0.0;
        }
        d[0] += __dmul_rn(__dmul_rn(v0, v0), m);
        d[1] += __dmul_rn(__dmul_rn(v0, v1), m);
        d[2] += __dmul_rn(__dmul_rn(v0, v2), m);
        d[3] += __dmul_rn(__dmul_rn(v1, v1), m);
        d[4] += __dmul_rn(__dmul_rn(v1, v2), m);
        d[5] += __dmul_rn(__dmul_rn(v2, v2), m);
    }
    if (md_block_partials<6>(d, a.partials, &a.sc->counter[3]) && threadIdx.x < 32) {
        double t[6];
        final_sums<6>(a.partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            for (int k = 0; k < 6; k++) a.sc->mvv[k] = t[k];
            a.sc->T_part = (t[0] + (t[3] + t[5])) / a.nhc.ndof_kB;
            a.sc->counter[3] = 0;
            a.sc->step = 0;
        }
    }
}

// run start: thermo row 0, no pending velocity scale or kick
__global__ void k_run_begin(MdArgs a) {
    write_thermo_row(a.thermo, a.sc, 0);
    a.sc->fac_x_d = 1.0;
    a.sc->pending_kick = 0;
}

// ------------------------------------------------------------------ FP64 path
__global__ void k_step_open(MdArgs a) { a.sc->fac_x_d *= thermo_half(a.nhc, a.sc); }

__global__ void __launch_bounds__(256) k_kick_drift64(MdArgs a) {
    const int n = a.n;
    const double fac = a.sc->fac_x_d;
    double dsum[3] = {0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int e = a.elem[i];
        const unsigned b = a.dof ? a.dof[i] : 7u;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double vv = a.v[c * n + i], ff = a.f[c * n + i], xx = a.x[c * n + i];
            // a frozen component keeps its velocity and still drifts
            // (update_x_d__x_w_dof, md_nvt.cpp:144-180)
            if ((b >> c) & 1u) vv = __dadd_rn(__dmul_rn(vv, fac), __ddiv_rn(__dmul_rn(ff, a.dt2), a.masses[e]));
            double dx = __dmul_rn(vv, a.dt);
            dsum[c] = __dadd_rn(dsum[c], dx);
            xx = __dadd_rn(xx, dx);
            a.v[c * n + i] = vv;
            a.x[c * n + i] = xx;
        }
    }
    if (md_block_partials<3>(dsum, a.partials, &a.sc->counter[4]) && threadIdx.x < 32) {
        double t[3];
        final_sums<3>(a.partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            double natms = (double)n;
            for (int c = 0; c < 3; c++) a.sc->com[c] = a.com_on[c] ? t[c] / natms : 0.0;
            a.sc->rebuild = 0;
            a.sc->counter[4] = 0;
        }
    }
}

__global__ void __launch_bounds__(256) k_com_skin64(MdArgs a) {
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
    }
    if (__syncthreads_or(moved) && threadIdx.x == 0) a.sc->rebuild = 1;
}

__global__ void __launch_bounds__(256) k_kick2_64(MdArgs a) {
    const int n = a.n;
    double d[6] = {0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int e = a.elem[i];
        const double m = a.masses[e];
        const unsigned b = a.dof ? a.dof[i] : 7u;
        double vv[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            // update_x_d_w_dof (md_nvt.cpp:184-215): frozen components are
            // neither kicked nor counted in the kinetic tensor
            if ((b >> c) & 1u) {
                double v0 = a.v[c * n + i], ff = a.f[c * n + i];
                v0 = __dadd_rn(v0, __ddiv_rn(__dmul_rn(ff, a.dt2), m));
                a.v[c * n + i] = v0;
                vv[c] = v0;
            } else {
                vv[c] = 0.0;
            }
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
        final_sums<6>(a.partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            DevScalars* sc = a.sc;
            for (int k = 0; k < 6; k++) sc->mvv[k] = t[k];
            sc->T_part = (t[0] + (t[3] + t[5])) / a.nhc.ndof_kB;
            sc->fac_x_d = thermo_half(a.nhc, sc);
            long long st = ++sc->step;
            if (st <= a.nsteps) write_thermo_row(a.thermo, sc, st);
            if (!(isfinite(sc->energy) && isfinite(sc->T_part))) sc->bad = 1;
            sc->counter[5] = 0;
        }
    }
}

__global__ void k_run_end64(MdArgs a) {
    const int n = a.n;
    const double fac = a.sc->fac_x_d;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += gridDim.x * blockDim.x)
        if (!a.dof || ((a.dof[i % n] >> (i / n)) & 1u)) a.v[i] = __dmul_rn(a.v[i], fac);
}

// ------------------------------------------------------------------ mixed path
__global__ void k_step_open32(MdArgs a) {
    DevScalars* sc = a.sc;
    const double fo = thermo_half(a.nhc, sc);
    if (sc->pending_kick) {
        const double F = sc->fac_close * fo;
        sc->kickA = F;
        sc->kickB = 1.0 + F;
    } else {
        sc->kickA = fo;
        sc->kickB = 1.0;
    }
    sc->rebuild = 0;
}

template <bool ORTHO>
__global__ void __launch_bounds__(256) k_integrate32(MdArgs a) {
    const int n = a.n;
    const double A = a.sc->kickA;
    const float B = (float)a.sc->kickB;
    float dsum0 = 0.f, dsum1 = 0.f, dsum2 = 0.f;
    int moved = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int e = a.elem[i];
        const float kf = a.dtm32[e] * B;
        const unsigned b = a.dof ? a.dof[i] : 7u;
        double xv[3];
        float vf[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            // a frozen component (atoms.x_dof) keeps its velocity and drifts
            double v = a.v[c * n + i];
            if ((b >> c) & 1u) v = fma(v, A, (double)(a.f32[c * n + i] * kf));
            double x = fma(v, a.dt, a.x[c * n + i]);
            a.v[c * n + i] = v;
            a.x[c * n + i] = x;
            xv[c] = x;
            vf[c] = (float)v;
            a.v32[c * n + i] = vf[c];
        }
        dsum0 = fmaf(vf[0], a.dt32, dsum0);
        dsum1 = fmaf(vf[1], a.dt32, dsum1);
        dsum2 = fmaf(vf[2], a.dt32, dsum2);
        // frame position and the skin test against the position at the build
        const int bc = a.binc[i];
        // the scaled frame; for an orthorhombic box one product per axis
        const double u0 = ORTHO ? a.bs[0] * xv[0] : a.bs[0] * xv[0] + (a.bs[1] * xv[1] + a.bs[2] * xv[2]);
        const double u1 = ORTHO ? a.bs[3] * xv[1] : a.bs[3] * xv[1] + a.bs[4] * xv[2];
        const double u2 = a.bs[5] * xv[2];
        float4 p;
        p.x = (float)(u0 - (double)(8 * (bc & 1023)));
        p.y = (float)(u1 - (double)(8 * ((bc >> 10) & 1023)));
        p.z = (float)(u2 - (double)(8 * ((bc >> 20) & 1023)));
        p.w = 0.f;
        a.p32[i] = p;
        const float4 q = a.p0[i];
        const float da = p.x - q.x, db = p.y - q.y, dc = p.z - q.z;
        float cx, cy, cz;
        if (ORTHO) {
            cx = da * a.fr.G[0][0];
            cy = db * a.fr.G[1][1];
            cz = dc * a.fr.G[2][2];
        } else {
            cx = da * a.fr.G[0][0] + db * a.fr.G[1][0] + dc * a.fr.G[2][0];
            cy = db * a.fr.G[1][1] + dc * a.fr.G[2][1];
            cz = dc * a.fr.G[2][2];
        }
        moved |= fmaf(cx, cx, fmaf(cy, cy, cz * cz)) > a.skin_sq32;
    }
    if (__syncthreads_or(moved) && threadIdx.x == 0) a.sc->rebuild = 1;
    const float dv[3] = {dsum0, dsum1, dsum2};
    if (block_partials_f32<3>(dv, a.partials, 0, &a.sc->counter[4]) && threadIdx.x < 32) {
        double t[3];
        final_sums<3>(a.partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            const double natms = (double)n;
            for (int c = 0; c < 3; c++) {
                a.sc->com[c] = a.com_on[c] ? t[c] / natms : 0.0;
                a.sc->drift[c] += a.sc->com[c];
            }
            a.sc->pending_kick = 0;
            a.sc->counter[4] = 0;
        }
    }
}

// update_x_d (md_nvt.cpp:106-128) and the closing half of the thermostat
// (md_nvt.cpp:427-432) of a mixed step: kinetic tensor of the half-kicked
// velocity v + f dt/2m (FP32 terms, FP64 sums), then in the last block the
// chain, the pending kick and the thermo row
__global__ void __launch_bounds__(256) k_close32(MdArgs a) {
    const int n = a.n;
    float k0 = 0.f, k1 = 0.f, k2 = 0.f, k3 = 0.f, k4 = 0.f, k5 = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int e = a.elem[i];
        const float dtm = a.dtm32[e], m = a.m32[e];
        float vx = fmaf(a.f32[i], dtm, a.v32[i]);
        float vy = fmaf(a.f32[n + i], dtm, a.v32[n + i]);
        float vz = fmaf(a.f32[2 * n + i], dtm, a.v32[2 * n + i]);
        if (a.dof) {  // frozen components leave the kinetic tensor
            const unsigned b = a.dof[i];
            if (!(b & 1u)) vx = 0.f;
            if (!(b & 2u)) vy = 0.f;
            if (!(b & 4u)) vz = 0.f;
        }
        const float mx = m * vx, my = m * vy, mz = m * vz;
        k0 = fmaf(mx, vx, k0);
        k1 = fmaf(mx, vy, k1);
        k2 = fmaf(mx, vz, k2);
        k3 = fmaf(my, vy, k3);
        k4 = fmaf(my, vz, k4);
        k5 = fmaf(mz, vz, k5);
    }
    const float d[6] = {k0, k1, k2, k3, k4, k5};
    if (block_partials_f32<6>(d, a.partials, 0, &a.sc->counter[5]) && threadIdx.x < 32) {
        double t[6];
        final_sums<6>(a.partials, gridDim.x, t);
        if (threadIdx.x == 0) {
            DevScalars* sc = a.sc;
            for (int k = 0; k < 6; k++) sc->mvv[k] = t[k];
            sc->T_part = (t[0] + (t[3] + t[5])) / a.nhc.ndof_kB;
            sc->fac_close = thermo_half(a.nhc, sc);
            sc->pending_kick = 1;
            long long st = ++sc->step;
            if (st <= a.nsteps) write_thermo_row(a.thermo, sc, st);
            if (!(isfinite(sc->energy) && isfinite(sc->T_part))) sc->bad = 1;
            sc->counter[5] = 0;
        }
    }
}

// the same kinetic tensor per chunk of a batch (slots 7-12), for the
// per-cell closing half in k_cells_done
__global__ void __launch_bounds__(256) k_ke32b(MdArgs a) {
    const int n = a.n;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        float k[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            const int e = a.elem[i];
            const float dtm = a.dtm32[e], m = a.m32[e];
            const float vx = fmaf(a.f32[i], dtm, a.v32[i]);
            const float vy = fmaf(a.f32[n + i], dtm, a.v32[n + i]);
            const float vz = fmaf(a.f32[2 * n + i], dtm, a.v32[2 * n + i]);
            const float mx = m * vx, my = m * vy, mz = m * vz;
            k[0] = fmaf(mx, vx, k[0]);
            k[1] = fmaf(mx, vy, k[1]);
            k[2] = fmaf(mx, vz, k[2]);
            k[3] = fmaf(my, vy, k[3]);
            k[4] = fmaf(my, vz, k[4]);
            k[5] = fmaf(mz, vz, k[5]);
        }
        chunk_store_f32<6>(k, a.chunk_part + (size_t)ch * kChunkSlots + 7);
    }
}

// end of a mixed run: the pending closing kick and scale, v = (v + f dt/2m) fc,
// and the accumulated mean displacement removed from x
__global__ void k_run_end32(MdArgs a) {
    const int n = a.n;
    const bool pend = a.sc->pending_kick != 0;
    const double fc = pend ? a.sc->fac_close : a.sc->fac_x_d;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * n; q += gridDim.x * blockDim.x) {
        const int i = q % n, c = q / n;
        a.x[q] -= a.sc->drift[c];
        if (a.dof && !((a.dof[i] >> c) & 1u)) continue;  // frozen: neither kicked nor scaled
        double v = a.v[q];
        if (pend) v += (double)a.f32[q] * a.dtm[a.elem[i]];
        a.v[q] = v * fc;
    }
}

__global__ void k_clear_drift(DevScalars* sc) {
    sc->drift[0] = sc->drift[1] = sc->drift[2] = 0.0;
    sc->pending_kick = 0;
}

// ------------------------------------------------------------------ batch of cells (mixed path)
// per-cell sums of chunk slots lo..lo+K-1 by one warp per cell, fixed order
template <int K>
__device__ __forceinline__ void cell_sums(const MdArgs& a, const double* part, int stride, int c, double (&t)[K]) {
    const int lane = threadIdx.x & 31;
    const int lo = a.cell_chunk[c], hi = a.cell_chunk[c + 1];
#pragma unroll
    for (int k = 0; k < K; k++) {
        double v = 0.0;
        for (int ch = lo + lane; ch < hi; ch += 32) v += part[(size_t)ch * stride + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        t[k] = v;
    }
}

// kinetic tensor of the incoming velocities per chunk (slots 7-12)
__global__ void __launch_bounds__(256) k_mvv_init_b(MdArgs a) {
    const int n = a.n;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        double d[6] = {0, 0, 0, 0, 0, 0};
        for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            double m = a.masses[a.elem[i]];
            double v0 = a.v[i], v1 = a.v[n + i], v2 = a.v[2 * n + i];
            d[0] += __dmul_rn(__dmul_rn(v0, v0), m);
            d[1] += __dmul_rn(__dmul_rn(v0, v1), m);
            d[2] += __dmul_rn(__dmul_rn(v0, v2), m);
            d[3] += __dmul_rn(__dmul_rn(v1, v1), m);
            d[4] += __dmul_rn(__dmul_rn(v1, v2), m);
            d[5] += __dmul_rn(__dmul_rn(v2, v2), m);
        }
        chunk_store<6>([&](int k) { return d[k]; }, a.chunk_part + (size_t)ch * kChunkSlots + 7);
    }
}

// run start per cell: kinetic tensor, T, thermo row 0, no pending scale/kick
__global__ void k_cells_begin(MdArgs a) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    double t[6];
    cell_sums<6>(a, a.chunk_part + 7, kChunkSlots, c, t);
    if ((threadIdx.x & 31) != 0) return;
    CellMd* m = a.cmd + c;
    for (int k = 0; k < 6; k++) m->mvv[k] = t[k];
    m->T_part = (t[0] + (t[3] + t[5])) / m->ndof_kB;
    m->step = 0;
    m->fac_x_d = 1.0;
    m->pending_kick = 0;
    if (a.thermo) {
        a.thermo[2 * c] = m->energy;
        a.thermo[2 * c + 1] = m->T_part;
    }
}

// opening half of every cell's chain and its kick factors (k_step_open32)
__global__ void k_cells_open(MdArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c == 0) a.sc->rebuild = 0;
    if (c >= a.ncell) return;
    CellMd* m = a.cmd + c;
    const NhcParams P = cell_nhc(a.nhc, m);
    const double fo = thermo_half(P, m);
    if (m->pending_kick) {
        const double F = m->fac_close * fo;
        m->kickA = F;
        m->kickB = 1.0 + F;
    } else {
        m->kickA = fo;
        m->kickB = 1.0;
    }
}

// k_integrate32 per chunk: the cell's kick factors and frame, displacement
// sums per chunk
__global__ void __launch_bounds__(256) k_integrate32b(MdArgs a) {
    const int n = a.n;
    int moved = 0;
    for (int ch = blockIdx.x; ch < a.nchunk; ch += gridDim.x) {
        int moved_ch = 0;
        const int lo = a.chunk_begin[ch], hi = a.chunk_begin[ch + 1];
        const int c = a.chunk_cell[ch];
        const CellGeo& g = a.cells[c];
        const double A = a.cmd[c].kickA;
        const float B = (float)a.cmd[c].kickB;
        float dsum0 = 0.f, dsum1 = 0.f, dsum2 = 0.f;
        for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            const int e = a.elem[i];
            const float kf = a.dtm32[e] * B;
            double xv[3];
            float vf[3];
#pragma unroll
            for (int q = 0; q < 3; q++) {
                double v = fma(a.v[q * n + i], A, (double)(a.f32[q * n + i] * kf));
                double x = fma(v, a.dt, a.x[q * n + i]);
                a.v[q * n + i] = v;
                a.x[q * n + i] = x;
                xv[q] = x;
                vf[q] = (float)v;
                a.v32[q * n + i] = vf[q];
            }
            dsum0 = fmaf(vf[0], a.dt32, dsum0);
            dsum1 = fmaf(vf[1], a.dt32, dsum1);
            dsum2 = fmaf(vf[2], a.dt32, dsum2);
            const int bc = a.binc[i];
            const bool orth = g.ortho != 0;  // uniform over the chunk
            const double u0 = orth ? g.bs[0] * xv[0] : g.bs[0] * xv[0] + (g.bs[1] * xv[1] + g.bs[2] * xv[2]);
            const double u1 = orth ? g.bs[3] * xv[1] : g.bs[3] * xv[1] + g.bs[4] * xv[2];
            const double u2 = g.bs[5] * xv[2];
            float4 p;
            p.x = (float)(u0 - (double)(8 * (bc & 1023)));
            p.y = (float)(u1 - (double)(8 * ((bc >> 10) & 1023)));
            p.z = (float)(u2 - (double)(8 * ((bc >> 20) & 1023)));
            p.w = 0.f;
            a.p32[i] = p;
            const float4 q = a.p0[i];
            const float da = p.x - q.x, db = p.y - q.y, dc = p.z - q.z;
            const float cx = da * g.G[0][0] + db * g.G[1][0] + dc * g.G[2][0];
            const float cy = db * g.G[1][1] + dc * g.G[2][1];
            const float cz = dc * g.G[2][2];
            moved_ch |= fmaf(cx, cx, fmaf(cy, cy, cz * cz)) > a.skin_sq32;
        }
        // the chunk's cell is rebuilt at the next list check
        if (__syncthreads_or(moved_ch)) {
            moved = 1;
            if (threadIdx.x == 0) a.cell_reb[c] = 1;
        }
        const float ds[3] = {dsum0, dsum1, dsum2};
        chunk_store_f32<3>(ds, a.chunk_disp + (size_t)ch * 4);
    }
    if (__syncthreads_or(moved) && threadIdx.x == 0) a.sc->rebuild = 1;
}

// per-cell mean displacement of the step, added to the cell's drift
__global__ void k_cells_com(MdArgs a) {
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.ncell) return;
    double t[3];
    cell_sums<3>(a, a.chunk_disp, 4, c, t);
    if ((threadIdx.x & 31) != 0) return;
    CellMd* m = a.cmd + c;
    const double natms = (double)(a.cells[c].end - a.cells[c].begin);
    for (int k = 0; k < 3; k++) {
        m->com[k] = t[k] / natms;
        m->drift[k] += m->com[k];
    }
    m->pending_kick = 0;
}

// end of a batch run: pending closing kick and scale, drift removed, per cell
__global__ void k_run_end32b(MdArgs a) {
    const int n = a.n;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * n; q += gridDim.x * blockDim.x) {
        const int i = q % n, k = q / n;
        const CellMd* m = a.cmd + a.cell_of[i];
        const bool pend = m->pending_kick != 0;
        const double fc = pend ? m->fac_close : m->fac_x_d;
        double v = a.v[q];
        if (pend) v += (double)a.f32[q] * a.dtm[a.elem[i]];
        a.v[q] = v * fc;
        a.x[q] -= m->drift[k];
    }
}

__global__ void k_cells_clear(MdArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncell) return;
    CellMd* m = a.cmd + c;
    m->drift[0] = m->drift[1] = m->drift[2] = 0.0;
    m->pending_kick = 0;
}

}  // namespace mappg

using namespace mappg;

namespace mappg {
void sys_build(mappg_sys* s);

static MdArgs md_args(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters,
                      long long nsteps, double* thermo_dev) {
    MdArgs a;
    memset(&a, 0, sizeof(a));
    a.n = s->n;
    a.x = s->x;
    a.v = s->v;
    a.f = s->f;
    a.f32 = s->f32;
    a.v32 = s->v32;
    a.x0 = s->x0;
    a.elem = s->elem;
    a.binc = s->binc;
    a.p32 = s->p32;
    a.p0 = s->p0;
    a.dt = dt;
    a.dt2 = dt / 2.0;
    a.dt32 = (float)dt;
    for (int e = 0; e < s->ne; e++) {
        a.masses[e] = s->masses[e];
        a.dtm[e] = a.dt2 / s->masses[e];
        a.dtm32[e] = (float)a.dtm[e];
        a.m32[e] = (float)a.masses[e];
    }
    a.skin_sq = 0.25 * s->skin * s->skin;
    // the FP32 skin test triggers a little early rather than late
    a.skin_sq32 = (float)(a.skin_sq * (1.0 - 1e-4));
    const double S[3] = {8.0 * s->nb[0], 8.0 * s->nb[1], 8.0 * s->nb[2]};
    const double* b6 = s->box.b6;
    a.bs[0] = b6[0] * S[0];
    a.bs[1] = b6[1] * S[0];
    a.bs[2] = b6[2] * S[0];
    a.bs[3] = b6[3] * S[1];
    a.bs[4] = b6[4] * S[1];
    a.bs[5] = b6[5] * S[2];
    a.fr = s->frame;
    a.partials = s->partials;
    a.thermo = thermo_dev;
    a.nsteps = nsteps;
    // ThermostatNHC(dt/2, t_relax, L, niters)  md_nvt.cpp:19, thermostat.cpp:20-36
    const double tdt = dt / 2.0;
    a.nhc.T = T;
    a.nhc.ddt = tdt / (double)niters;
    a.nhc.ddt2 = 0.5 * tdt / (double)niters;
    a.nhc.freq_sq = 1.0 / (t_relax * t_relax);
    a.nhc.kB = kB;
    // MDNVT::pre_init (md_nvt.cpp:264-291): frozen components leave the
    // degrees of freedom, and the mean displacement is kept along a
    // component in which any atom is frozen
    a.dof = s->dof;
    a.nhc.ndof = 3 * s->n - (s->dof_frozen[0] + s->dof_frozen[1] + s->dof_frozen[2]);
    for (int c = 0; c < 3; c++) a.com_on[c] = s->dof_frozen[c] == 0;
    a.nhc.ndof_kB = a.nhc.ndof * kB;
    a.nhc.L = L;
    a.nhc.niters = niters;
    a.sc = s->sc;
    a.ncell = s->ncell;
    a.nchunk = s->nchunk;
    a.cells = s->cells_dev;
    a.cell_of = s->cell_of;
    a.chunk_begin = s->chunk_begin;
    a.chunk_cell = s->chunk_cell;
    a.cell_chunk = s->cell_chunk;
    a.chunk_part = s->chunk_part;
    a.chunk_disp = s->chunk_disp;
    a.cmd = s->cmd;
    a.cell_reb = s->cell_reb;
    return a;
}

// mark: record s->ev_main once the step's positions are final (after the
// list check; the passes after it do not move the atoms)
static void launch_step64(mappg_sys* s, const MdArgs& a, bool mark = false) {
    int g = grid_for(s, s->n, 256);
    k_step_open<<<1, 1, 0, s->stream>>>(a);
    k_kick_drift64<<<g, 256, 0, s->stream>>>(a);
    k_com_skin64<<<g, 256, 0, s->stream>>>(a);
    launch_rebuild_chain(s);
    if (mark) MAPPG_CUDA(cudaEventRecord(s->ev_main, s->stream));
    launch_force(s);
    k_kick2_64<<<g, 256, 0, s->stream>>>(a);
}

static void launch_step32(mappg_sys* s, const MdArgs& a, bool mark = false) {
    // streaming kernels with a last-block reduction: four blocks per SM keep
    // loads in flight and the serial tail (the fixed-order sum over block
    // partials) short
    int g = std::min(grid_for(s, s->n, 256), 4 * s->sm_count);
    k_step_open32<<<1, 1, 0, s->stream>>>(a);
    if (a.fr.ortho)
        k_integrate32<true><<<g, 256, 0, s->stream>>>(a);
    else
        k_integrate32<false><<<g, 256, 0, s->stream>>>(a);
    launch_rebuild_chain(s);
    if (mark) MAPPG_CUDA(cudaEventRecord(s->ev_main, s->stream));
    EamArgs e = eam_args(s);
    launch_density32(s, e);
    launch_force32(s, e);
    k_close32<<<g, 256, 0, s->stream>>>(a);
}

static void launch_step32b(mappg_sys* s, const MdArgs& a) {
    const int nc = s->ncell;
    k_cells_open<<<(nc + 255) / 256, 256, 0, s->stream>>>(a);
    k_integrate32b<<<std::min(s->nchunk, s->sm_count * 8), 256, 0, s->stream>>>(a);
    k_cells_com<<<(nc * 32 + 255) / 256, 256, 0, s->stream>>>(a);
    launch_rebuild_chain(s);
    EamArgs e = eam_args(s);
    launch_density32(s, e);
    launch_force32(s, e);
    k_ke32b<<<std::min(s->nchunk, s->sm_count * 8), 256, 0, s->stream>>>(a);
    e.thermo = a.thermo;
    e.nsteps = a.nsteps;
    e.nhc = a.nhc;
    launch_cells_done(s, e, 2);  // kinetic tensors, each cell's closing half, thermo rows
}

struct NvtRun {
    MdArgs a;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    // batches: the planned steps (up to kBatchGraphSteps) as one graph, so a
    // whole run of every cell is one launch
    cudaGraphExec_t exec_many = nullptr;
    cudaGraph_t graph_many = nullptr;
    long long many = 0;
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
    if (r->exec_many) cudaGraphExecDestroy(r->exec_many);
    if (r->graph_many) cudaGraphDestroy(r->graph_many);
    delete r;
    s->run = nullptr;
}

void nvt_free(mappg_sys* s) { run_clear(s); }

void sys_join_side(mappg_sys* s);  // system.cu

// runs this short launch their steps' kernels directly: capturing and
// instantiating the step graph costs more than it saves over a few steps
constexpr long long kGraphMinSteps = 8;
// longest run of batch steps captured as one graph (about 14 nodes a step)
constexpr long long kBatchGraphSteps = 512;

// MDNVT::init + the opening force call of MDNVT::run, then the step graph
void nvt_begin(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, long long nsteps,
               const double* eta, bool thermo, const double* Tcell) {
    const bool batch = s->ncell > 1;
    if (batch && s->precision != MAPPG_MIXED) throw Error{MAPPG_ERR_UNSUPP, "batched MD runs in mixed precision"};
    if (batch && !Tcell) throw Error{MAPPG_ERR_ARG, "a batch needs one temperature per cell"};
    if (!batch && Tcell) throw Error{MAPPG_ERR_ARG, "per-cell temperatures need a batch of cells"};
    if (batch) {
        T = 1.0;
        for (int c = 0; c < s->ncell; c++)
            if (!(Tcell[c] > 0.0)) throw Error{MAPPG_ERR_ARG, "T must be positive"};
    }
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
        long long need = (batch ? 2LL * s->ncell : 14LL) * (nsteps + 1);
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
    r->a = md_args(s, T, dt, kB, t_relax, L, niters, nsteps, tdev);
    r->L = L;
    r->planned = nsteps;
    r->thermo = thermo;
    MdArgs& a = r->a;
    int g = grid_for(s, s->n, 256);
    if (batch) {
        // per-cell targets, degrees of freedom and chain state
        std::vector<CellMd> cm(s->ncell);
        MAPPG_CUDA(cudaMemcpyAsync(cm.data(), s->cmd, sizeof(CellMd) * s->ncell, cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        for (int c = 0; c < s->ncell; c++) {
            CellMd& m = cm[c];
            m.T = Tcell[c];
            m.ndof = 3.0 * (s->cell_begin[c + 1] - s->cell_begin[c]);
            m.ndof_kB = m.ndof * kB;
            for (int k = 0; k < kMaxChain; k++) m.eta[k] = (eta && k < L) ? eta[(size_t)c * L + k] : 0.0;
            m.drift[0] = m.drift[1] = m.drift[2] = 0.0;
            m.pending_kick = 0;
            m.step = 0;
        }
        MAPPG_CUDA(cudaMemcpyAsync(s->cmd, cm.data(), sizeof(CellMd) * s->ncell, cudaMemcpyHostToDevice, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        sys_build(s);
        launch_force(s);
        k_mvv_init_b<<<std::min(s->nchunk, s->sm_count * 8), 256, 0, s->stream>>>(a);
        k_cells_begin<<<(s->ncell * 32 + 255) / 256, 256, 0, s->stream>>>(a);
        MAPPG_CUDA(cudaGetLastError());
        auto capture = [&](long long k, cudaGraph_t* gr, cudaGraphExec_t* ex) {
            MAPPG_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            try {
                for (long long q = 0; q < k; q++) launch_step32b(s, a);
            } catch (...) {
                cudaGraph_t g2 = nullptr;
                cudaStreamEndCapture(s->stream, &g2);
                if (g2) cudaGraphDestroy(g2);
                throw;
            }
            MAPPG_CUDA(cudaStreamEndCapture(s->stream, gr));
            MAPPG_CUDA(cudaGraphInstantiate(ex, *gr, 0));
        };
        capture(1, &r->graph, &r->exec);
        r->many = std::min(nsteps, kBatchGraphSteps);
        if (r->many >= kGraphMinSteps) capture(r->many, &r->graph_many, &r->exec_many);
        return;
    }
    double eta_h[kMaxChain] = {0};
    if (eta)
        for (int k = 0; k < L; k++) eta_h[k] = eta[k];
    MAPPG_CUDA(cudaMemcpyAsync(s->sc->eta, eta_h, sizeof(double) * kMaxChain, cudaMemcpyHostToDevice, s->stream));
    k_clear_drift<<<1, 1, 0, s->stream>>>(s->sc);
    // MDNVT::run builds the list at its start.  A list built for this box
    // whose atoms all stayed within half the skin of their positions at that
    // build still holds every pair within the cutoff, so the skin test
    // decides here (the forces are the same; only their summation order can
    // differ from a fresh build's)
    if (s->list_box) {
        lb_update(s);
        s->built = true;
    } else {
        sys_build(s);
    }
    launch_force(s);
    // the list and the opening force do not read velocities: an upload of
    // them on the side stream (nvt_run_host) overlaps them and is joined here
    sys_join_side(s);
    k_mvv_init<<<g, 256, 0, s->stream>>>(a);
    k_run_begin<<<1, 1, 0, s->stream>>>(a);
    MAPPG_CUDA(cudaGetLastError());
    if (nsteps < kGraphMinSteps) return;  // nvt_steps launches the kernels itself
    MAPPG_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    try {
        if (s->precision == MAPPG_MIXED)
            launch_step32(s, a);
        else
            launch_step64(s, a);
    } catch (...) {
        cudaGraph_t g2 = nullptr;
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
    long long st = 0;
    if (r->exec_many)
        for (; nsteps - st >= r->many; st += r->many) MAPPG_CUDA(cudaGraphLaunch(r->exec_many, s->stream));
    for (; st < nsteps; st++) {
        if (r->exec)
            MAPPG_CUDA(cudaGraphLaunch(r->exec, s->stream));
        else if (s->precision == MAPPG_MIXED)
            launch_step32(s, r->a);
        else
            launch_step64(s, r->a);
    }
    r->done += nsteps;
}

// update_x_d_final, chain state out, thermo rows, checks
void nvt_end(mappg_sys* s, double* eta, double* thermo) {
    NvtRun* r = (NvtRun*)s->run;
    if (!r) throw Error{MAPPG_ERR_ARG, "no NVT run has begun on this system"};
    sys_join_side(s);  // a side-stream read of the positions (nvt_run_xout) comes first
    int g = grid_for(s, 3LL * s->n, 256);
    if (s->ncell > 1) {
        k_run_end32b<<<g, 256, 0, s->stream>>>(r->a);
        k_cells_clear<<<(s->ncell + 255) / 256, 256, 0, s->stream>>>(r->a);
        MAPPG_CUDA(cudaGetLastError());
        DevScalars h;
        std::vector<CellMd> cm(s->ncell);
        MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaMemcpyAsync(cm.data(), s->cmd, sizeof(CellMd) * s->ncell, cudaMemcpyDeviceToHost, s->stream));
        if (thermo && r->thermo)
            MAPPG_CUDA(cudaMemcpyAsync(thermo, r->a.thermo, sizeof(double) * 2 * s->ncell * (r->done + 1),
                                       cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        if (eta)
            for (int c = 0; c < s->ncell; c++)
                for (int k = 0; k < r->L; k++) eta[(size_t)c * r->L + k] = cm[c].eta[k];
        run_clear(s);
        if (h.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during the run"};
        if (h.bad) throw Error{MAPPG_ERR_NAN, "non-finite position, energy or temperature during the run"};
        return;
    }
    if (s->precision == MAPPG_MIXED) {
        k_run_end32<<<g, 256, 0, s->stream>>>(r->a);
        k_clear_drift<<<1, 1, 0, s->stream>>>(s->sc);
    } else {
        k_run_end64<<<g, 256, 0, s->stream>>>(r->a);
    }
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
    if (h.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during the run"};
    if (h.bad) throw Error{MAPPG_ERR_NAN, "non-finite position, energy or temperature during the run"};
}

// Positions (what = 0) or velocities (what = 1) of a run at a step boundary,
// written in the caller's atom order.  They are the state MDNVT::run exports
// between steps (md_nvt.cpp:390,436,470): after the closing kick, before the
// deferred thermostat scale.  The mixed path keeps the mean displacement in
// sc->drift and may hold the closing kick back (pending_kick); both are
// applied to the copy here, the run's own state is left as it is.
__global__ void k_snapshot(MdArgs a, const int* __restrict__ id, double* __restrict__ out, int what, int mixed) {
    const int n = a.n;
    const bool pend = mixed && a.sc->pending_kick != 0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * n; q += gridDim.x * blockDim.x) {
        const int i = q % n, c = q / n;
        double val;
        if (what == 0) {
            val = a.x[q];
            if (mixed) val -= a.sc->drift[c];
        } else {
            val = a.v[q];
            if (pend) val += (double)a.f32[q] * a.dtm[a.elem[i]];
        }
        out[3 * (size_t)id[i] + c] = val;
    }
}

void nvt_snapshot(mappg_sys* s, double* x, double* v) {
    NvtRun* r = (NvtRun*)s->run;
    if (!r) throw Error{MAPPG_ERR_ARG, "no NVT run has begun on this system"};
    if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "snapshots are taken of single-cell runs"};
    const int g = grid_for(s, 3LL * s->n, 256);
    const int mixed = s->precision == MAPPG_MIXED ? 1 : 0;
    double* out[2] = {x, v};
    for (int what = 0; what < 2; what++) {
        if (!out[what]) continue;
        k_snapshot<<<g, 256, 0, s->stream>>>(r->a, s->id, s->stage, what, mixed);
        MAPPG_CUDA(cudaGetLastError());
        MAPPG_CUDA(cudaMemcpyAsync(out[what], s->stage, sizeof(double) * 3 * (size_t)s->n, cudaMemcpyDeviceToHost,
                                   s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    }
    DevScalars h;
    MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    if (h.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded during the run"};
    if (h.bad) throw Error{MAPPG_ERR_NAN, "non-finite position, energy or temperature during the run"};
}

// positions in the caller's order less the mean displacement not yet
// removed (sc->drift; zero on the FP64 path): what the run's end leaves in x
__global__ void k_scatter_x_final(int n, const int* __restrict__ id, const double* __restrict__ x,
                                  const DevScalars* __restrict__ sc, double* __restrict__ out) {
    const double d0 = sc->drift[0], d1 = sc->drift[1], d2 = sc->drift[2];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const size_t u = 3 * (size_t)id[i];
        out[u] = x[i] - d0;
        out[u + 1] = x[n + i] - d1;
        out[u + 2] = x[2 * n + i] - d2;
    }
}

// nvt_run whose final positions go to the host array x_out during the last
// step: they are final once that step's list check is done, so the side
// stream gathers them then and copies them out under the density and force
// passes; the run's end (which removes sc->drift from x) waits for the
// gather only.  Needs the side stream (sys_upload_side made it).
void nvt_run_xout(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, int nsteps,
                  double* eta, double* thermo, double* x_out) {
    nvt_begin(s, T, dt, kB, t_relax, L, niters, nsteps, eta, thermo != nullptr, nullptr);
    NvtRun* r = (NvtRun*)s->run;
    if (nsteps > 0) {
        nvt_steps(s, nsteps - 1);
        if (s->precision == MAPPG_MIXED)
            launch_step32(s, r->a, true);
        else
            launch_step64(s, r->a, true);
        r->done += 1;
        MAPPG_CUDA(cudaStreamWaitEvent(s->side, s->ev_main, 0));
        k_scatter_x_final<<<grid_for(s, s->n, 256), 256, 0, s->side>>>(s->n, s->id, s->x, s->sc, s->stage2);
        MAPPG_CUDA(cudaGetLastError());
        MAPPG_CUDA(cudaEventRecord(s->ev_side, s->side));
        s->v_pending = true;
        MAPPG_CUDA(cudaMemcpyAsync(x_out, s->stage2, sizeof(double) * 3 * (size_t)s->n, cudaMemcpyDeviceToHost,
                                   s->side));
    }
    nvt_end(s, eta, thermo);
}

void nvt_run(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, int nsteps, double* eta,
             double* thermo, const double* Tcell) {
    nvt_begin(s, T, dt, kB, t_relax, L, niters, nsteps, eta, thermo != nullptr, Tcell);
    nvt_steps(s, nsteps);
    nvt_end(s, eta, thermo);
}

}  // namespace mappg
