// Device state of one periodic cell, coordinate transforms, binning and the
// full neighbour-list build.
//
// The list holds, for every atom i, every periodic image j' = x_j + n*H
// (j' != i) with |x_i - x_j'|^2 < (cut_ij + skin)^2, the same set that
// NeighborMD::create_list (neighbor_md.cpp:82-152) finds in full mode
// (pair_wise = false) over the ghost images of Update::list
// (exchange.h:833-875).  Candidates come from the 27 bins around atom i; an
// FP32 distance on bin-relative positions settles every pair outside a thin
// band around the cutoff, and pairs inside the band are decided with the
// reference's FP64 arithmetic: x = S2X(s) (xmath.h:2636-2658) of the wrapped
// fractional coordinate, images at S2X(s_j + n), RSQ = d0^2 + (d1^2 + d2^2)
// (xmath.h:2464-2510), no fused multiply-adds.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <type_traits>
#include <vector>

#include "system.h"

namespace mappg {

// ------------------------------------------------------------------ box
// Atoms::update_H  atoms.cpp:187-194 with the lower-triangular inverse,
// depth and determinant of xmath.h:1403-1480,2399-2415
static void box_from_H(Box& b, const double* H9) {
    memcpy(b.H, H9, sizeof(double) * 9);
    double(*H)[3] = b.H;
    double(*B)[3] = b.B;
    memset(B, 0, sizeof(double) * 9);
    B[0][0] = 1.0 / H[0][0];
    B[1][1] = 1.0 / H[1][1];
    B[1][0] = -B[1][1] * (B[0][0] * H[1][0]);
    B[2][2] = 1.0 / H[2][2];
    B[2][1] = -B[2][2] * (B[1][1] * H[2][1]);
    B[2][0] = -B[2][2] * (B[0][0] * H[2][0] + B[1][0] * H[2][1]);
    b.vol = H[0][0] * (H[1][1] * H[2][2]);
    b.depth_inv[0] = sqrt(B[0][0] * B[0][0] + (B[1][0] * B[1][0] + B[2][0] * B[2][0]));
    b.depth_inv[1] = sqrt(B[1][1] * B[1][1] + B[2][1] * B[2][1]);
    b.depth_inv[2] = fabs(B[2][2]);
    b.h6[0] = H[0][0]; b.h6[1] = H[1][0]; b.h6[2] = H[2][0];
    b.h6[3] = H[1][1]; b.h6[4] = H[2][1]; b.h6[5] = H[2][2];
    b.b6[0] = B[0][0]; b.b6[1] = B[1][0]; b.b6[2] = B[2][0];
    b.b6[3] = B[1][1]; b.b6[4] = B[2][1]; b.b6[5] = B[2][2];
}

void sys_set_box(mappg_sys* s, const double* H) {
    if (!(H[0] > 0 && H[4] > 0 && H[8] > 0) || H[1] != 0.0 || H[2] != 0.0 || H[5] != 0.0)
        throw Error{MAPPG_ERR_ARG, "H must be lower triangular with a positive diagonal"};
    box_from_H(s->box, H);
    double nbv[3];
    for (int d = 0; d < 3; d++) {
        double cs = s->max_cut * s->box.depth_inv[d];
        if (!(cs < 1.0))
            throw Error{MAPPG_ERR_GEOM, "box thinner than cutoff+skin along dimension " + std::to_string(d) +
                                            ": multi-layer periodic images are not supported"};
        int nb = (int)(1.0 / (cs * (1.0 + 1e-12)));
        nb = std::max(1, std::min(nb, 1023));
        s->nb[d] = nb;
        nbv[d] = 1.0 / nb;
    }
    s->nbins = s->nb[0] * s->nb[1] * s->nb[2];
    // scaled bin frame: s'_d = s_d * 8 nb_d; Cartesian dx = dx' G with
    // G_dk = H_dk / (8 nb_d), kept as head + tail
    Frame& fr = s->frame;
    fr.ortho = (H[3] == 0.0 && H[6] == 0.0 && H[7] == 0.0) ? 1 : 0;
    for (int d = 0; d < 3; d++)
        for (int k = 0; k < 3; k++) {
            double g = s->box.H[d][k] / (8.0 * s->nb[d]);
            fr.G[d][k] = (float)g;
            fr.Glo[d][k] = (float)(g - (double)fr.G[d][k]);
        }
    // neighbour code c = (d0+1)+3(d1+1)+9(d2+1): the image's bin is atom i's
    // bin + d; its frame offset is exactly -8 d
    for (int c = 0; c < 27; c++) {
        int d[3] = {c % 3 - 1, (c / 3) % 3 - 1, c / 9 - 1};
        for (int k = 0; k < 3; k++) {
            double sh = 0.0;
            for (int q = 0; q < 3; q++) sh += d[q] * s->box.H[q][k];
            fr.off[c][k] = -kBinW * d[k];
            s->shift[c][k] = sh;  // indexed by image code n instead of d
        }
        fr.off[c][3] = 0.f;
    }
    double pmax = s->skin;
    for (int q = 0; q < 3; q++) {
        double l = 0;
        for (int k = 0; k < 3; k++) l += s->box.H[q][k] * s->box.H[q][k];
        pmax += sqrt(l) * nbv[q];
    }
    double csk = 0;
    for (int i = 0; i < s->ne * s->ne; i++) csk = std::max(csk, s->cut_sk_sq[i]);
    s->band = 2e-5 * (csk + pmax * pmax);
    s->built = false;
    s->list_box = false;
}

// a batch: every cell gets its own box, bins (a block of global bin ids) and
// frame; the system-level box fields keep cell 0's for code that reads them
static void chunk_cells(mappg_sys* s);

void sys_set_cells(mappg_sys* s, int ncell, const int* natoms, const double* H) {
    s->ncell = ncell;
    s->cells.assign(ncell, CellGeo());
    s->cell_begin.assign(ncell + 1, 0);
    double band = 0.0;
    int bins = 0;
    bool all_ortho = true;
    for (int c = 0; c < ncell; c++) {
        sys_set_box(s, H + 9 * (size_t)c);
        CellGeo& g = s->cells[c];
        memcpy(g.h6, s->box.h6, sizeof(g.h6));
        memcpy(g.b6, s->box.b6, sizeof(g.b6));
        const double S[3] = {8.0 * s->nb[0], 8.0 * s->nb[1], 8.0 * s->nb[2]};
        g.bs[0] = g.b6[0] * S[0];
        g.bs[1] = g.b6[1] * S[0];
        g.bs[2] = g.b6[2] * S[0];
        g.bs[3] = g.b6[3] * S[1];
        g.bs[4] = g.b6[4] * S[1];
        g.bs[5] = g.b6[5] * S[2];
        memcpy(g.G, s->frame.G, sizeof(g.G));
        memcpy(g.Glo, s->frame.Glo, sizeof(g.Glo));
        for (int d = 0; d < 3; d++) g.nb[d] = s->nb[d];
        g.bin_base = bins;
        g.ortho = s->frame.ortho;
        all_ortho = all_ortho && g.ortho != 0;
        bins += s->nbins;
        band = std::max(band, s->band);
        s->cell_begin[c + 1] = s->cell_begin[c] + natoms[c];
        g.begin = s->cell_begin[c];
        g.end = s->cell_begin[c + 1];
    }
    sys_set_box(s, H);  // cell 0
    s->nbins = bins;
    s->band = band;
    s->cells_ortho = all_ortho;
    chunk_cells(s);
}

// chunks of at most s->chunk_atoms atoms, never across cells (host arrays)
static void chunk_cells(mappg_sys* s) {
    const int ncell = s->ncell;
    s->chunk_begin_h.clear();
    s->cell_chunk_h.assign(ncell + 1, 0);
    std::vector<int> chunk_cell;
    for (int c = 0; c < ncell; c++) {
        for (int a = s->cell_begin[c]; a < s->cell_begin[c + 1]; a += s->chunk_atoms) {
            s->chunk_begin_h.push_back(a);
            chunk_cell.push_back(c);
        }
        s->cell_chunk_h[c + 1] = (int)s->chunk_begin_h.size();
    }
    s->nchunk = (int)s->chunk_begin_h.size();
    s->chunk_begin_h.push_back(s->cell_begin[ncell]);
    s->cells_chunk_cell_h = chunk_cell;
}

// device copies of the chunk arrays and the per-chunk sums
static void upload_chunks(mappg_sys* s) {
    const int nc = s->ncell, nk = s->nchunk;
    void* old[] = {s->chunk_begin, s->chunk_cell, s->cell_chunk, s->chunk_part, s->chunk_disp};
    for (void* p : old)
        if (p) cudaFree(p);
    MAPPG_CUDA(cudaMalloc((void**)&s->chunk_begin, sizeof(int) * (nk + 1)));
    MAPPG_CUDA(cudaMalloc((void**)&s->chunk_cell, sizeof(int) * nk));
    MAPPG_CUDA(cudaMalloc((void**)&s->cell_chunk, sizeof(int) * (nc + 1)));
    MAPPG_CUDA(cudaMalloc((void**)&s->chunk_part, sizeof(double) * kChunkSlots * (size_t)nk));
    MAPPG_CUDA(cudaMalloc((void**)&s->chunk_disp, sizeof(double) * 4 * (size_t)nk));
    MAPPG_CUDA(cudaMemsetAsync(s->chunk_part, 0, sizeof(double) * kChunkSlots * (size_t)nk, s->stream));
    MAPPG_CUDA(cudaMemsetAsync(s->chunk_disp, 0, sizeof(double) * 4 * (size_t)nk, s->stream));
    MAPPG_CUDA(cudaMemcpyAsync(s->chunk_begin, s->chunk_begin_h.data(), sizeof(int) * (nk + 1), cudaMemcpyHostToDevice,
                               s->stream));
    MAPPG_CUDA(cudaMemcpyAsync(s->chunk_cell, s->cells_chunk_cell_h.data(), sizeof(int) * nk, cudaMemcpyHostToDevice,
                               s->stream));
    MAPPG_CUDA(cudaMemcpyAsync(s->cell_chunk, s->cell_chunk_h.data(), sizeof(int) * (nc + 1), cudaMemcpyHostToDevice,
                               s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
}

void sys_rechunk(mappg_sys* s, int chunk_atoms) {
    if (s->ncell <= 1) return;
    if (chunk_atoms < 32) throw Error{MAPPG_ERR_ARG, "chunks hold at least 32 atoms"};
    if (chunk_atoms == s->chunk_atoms) return;
    s->chunk_atoms = chunk_atoms;
    chunk_cells(s);
    upload_chunks(s);
}

int grid_for(mappg_sys* s, long long threads, int block) {
    long long g = (threads + block - 1) / block;
    long long cap = (long long)s->sm_count * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    if (g > kMaxBlocks) g = kMaxBlocks;
    return (int)g;
}

// ------------------------------------------------------------------ kernels
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

struct Geo {
    double h6[6], b6[6];
    double bs[6];  // b6 with each column scaled by 8 nb_d: x -> s' directly
    int nb[3];
};

static Geo make_geo(mappg_sys* s) {
    Geo g;
    memcpy(g.h6, s->box.h6, sizeof(g.h6));
    memcpy(g.b6, s->box.b6, sizeof(g.b6));
    for (int d = 0; d < 3; d++) g.nb[d] = s->nb[d];
    const double S0 = 8.0 * s->nb[0], S1 = 8.0 * s->nb[1], S2 = 8.0 * s->nb[2];
    g.bs[0] = g.b6[0] * S0;
    g.bs[1] = g.b6[1] * S0;
    g.bs[2] = g.b6[2] * S0;
    g.bs[3] = g.b6[3] * S1;
    g.bs[4] = g.b6[4] * S1;
    g.bs[5] = g.b6[5] * S2;
    return g;
}

// one wrap of X2S (xmath.h:2660-2700): ++/-- until in [0,1); bounded
__device__ __forceinline__ double wrap01(double v, int* bad) {
    int it = 0;
    while (v < 0.0 && it < 64) {
        v = dadd(v, 1.0);
        it++;
    }
    while (v >= 1.0 && it < 64) {
        v = dsub(v, 1.0);
        it++;
    }
    if (it >= 64 || v != v) {
        *bad = 1;
        v = 0.0;
    }
    return v;
}

__device__ __forceinline__ void s2x(const double* h, double s0, double s1, double s2, double& x0, double& x1,
                                    double& x2) {
    x0 = dadd(dmul(h[0], s0), dadd(dmul(h[1], s1), dmul(h[2], s2)));
    x1 = dadd(dmul(h[3], s1), dmul(h[4], s2));
    x2 = dmul(s2, h[5]);
}

// rebuild step 1: wrap x into the cell (x2s_lcl then s2x_all), bin, count
__global__ void k_wrap_bin(int n, double* __restrict__ x, double* __restrict__ s, Geo g, int* __restrict__ binc,
                           int* __restrict__ binid, int* __restrict__ bin_count, DevScalars* sc) {
    if (!sc->rebuild) return;
    int bad = 0;
    const double drift0 = sc->drift[0], drift1 = sc->drift[1], drift2 = sc->drift[2];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        // the mixed MD path defers its mean-displacement removal to here
        double x0 = dsub(x[i], drift0), x1 = dsub(x[n + i], drift1), x2 = dsub(x[2 * n + i], drift2);
        double s0 = dadd(dmul(g.b6[0], x0), dadd(dmul(g.b6[1], x1), dmul(g.b6[2], x2)));
        s0 = wrap01(s0, &bad);
        double s1 = dadd(dmul(g.b6[3], x1), dmul(g.b6[4], x2));
        s1 = wrap01(s1, &bad);
        double s2 = dmul(x2, g.b6[5]);
        s2 = wrap01(s2, &bad);
        s2x(g.h6, s0, s1, s2, x0, x1, x2);
        x[i] = x0;
        x[n + i] = x1;
        x[2 * n + i] = x2;
        s[i] = s0;
        s[n + i] = s1;
        s[2 * n + i] = s2;
        int b0 = min((int)(s0 * g.nb[0]), g.nb[0] - 1);
        int b1 = min((int)(s1 * g.nb[1]), g.nb[1] - 1);
        int b2 = min((int)(s2 * g.nb[2]), g.nb[2] - 1);
        binc[i] = b0 | (b1 << 10) | (b2 << 20);
        int b = b0 + g.nb[0] * (b1 + g.nb[1] * b2);
        binid[i] = b;
        atomicAdd(&bin_count[b], 1);
    }
    if (bad) sc->bad = 1;
}

// batch variant of step 1: each atom uses its cell's box, bins and drift
// (cells without their rebuild flag keep their wrap, bins and rows)
__global__ void k_wrap_bin_b(int n, double* __restrict__ x, double* __restrict__ s, const CellGeo* __restrict__ cells,
                             const int* __restrict__ cell_of, const CellMd* __restrict__ cmd, int* __restrict__ binc,
                             int* __restrict__ binid, int* __restrict__ bin_count, const uint8_t* __restrict__ cell_reb,
                             DevScalars* sc) {
    if (!sc->rebuild) return;
    int bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = cell_of[i];
        if (!cell_reb[c]) continue;
        const CellGeo& g = cells[c];
        const double* dr = cmd[c].drift;
        double x0 = dsub(x[i], dr[0]), x1 = dsub(x[n + i], dr[1]), x2 = dsub(x[2 * n + i], dr[2]);
        double s0 = dadd(dmul(g.b6[0], x0), dadd(dmul(g.b6[1], x1), dmul(g.b6[2], x2)));
        s0 = wrap01(s0, &bad);
        double s1 = dadd(dmul(g.b6[3], x1), dmul(g.b6[4], x2));
        s1 = wrap01(s1, &bad);
        double s2 = dmul(x2, g.b6[5]);
        s2 = wrap01(s2, &bad);
        s2x(g.h6, s0, s1, s2, x0, x1, x2);
        x[i] = x0;
        x[n + i] = x1;
        x[2 * n + i] = x2;
        s[i] = s0;
        s[n + i] = s1;
        s[2 * n + i] = s2;
        int b0 = min((int)(s0 * g.nb[0]), g.nb[0] - 1);
        int b1 = min((int)(s1 * g.nb[1]), g.nb[1] - 1);
        int b2 = min((int)(s2 * g.nb[2]), g.nb[2] - 1);
        binc[i] = b0 | (b1 << 10) | (b2 << 20);
        int b = g.bin_base + b0 + g.nb[0] * (b1 + g.nb[1] * b2);
        binid[i] = b;
        atomicAdd(&bin_count[b], 1);
    }
    if (bad) sc->bad = 1;
}

// rebuild step 2: exclusive scan of bin counts (one block), counts zeroed
__global__ void k_scan_bins(int nbins, int* __restrict__ bin_count, int* __restrict__ bin_start, DevScalars* sc) {
    if (!sc->rebuild) return;
    __shared__ int part[1024];
    int t = threadIdx.x, T = blockDim.x;
    int chunk = (nbins + T - 1) / T;
    int lo = min(t * chunk, nbins), hi = min(lo + chunk, nbins);
    int sum = 0;
    for (int b = lo; b < hi; b++) sum += bin_count[b];
    part[t] = sum;
    __syncthreads();
    for (int off = 1; off < T; off <<= 1) {
        int v = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - sum;
    for (int b = lo; b < hi; b++) {
        int c = bin_count[b];
        bin_start[b] = run;
        run += c;
        bin_count[b] = 0;
    }
    if (t == T - 1) bin_start[nbins] = part[T - 1];
    if (t == 0) {
        sc->maxrow = 0;
        sc->sumrow = 0;
    }
}

// batch variant of step 2: one warp per flagged cell scans its own bins,
// from the cell's first atom (a cell's bins hold exactly its atoms, so the
// other cells' bin starts stay valid)
__global__ void k_scan_bins_b(int ncell, int n, int nbins, const CellGeo* __restrict__ cells,
                              const uint8_t* __restrict__ cell_reb, int* __restrict__ bin_count,
                              int* __restrict__ bin_start, DevScalars* sc) {
    if (!sc->rebuild) return;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        bin_start[nbins] = n;
        sc->maxrow = 0;
        sc->sumrow = 0;
    }
    for (int c = warp; c < ncell; c += nw) {
        if (!cell_reb[c]) continue;
        const CellGeo& g = cells[c];
        const int nb = g.nb[0] * g.nb[1] * g.nb[2], base = g.bin_base;
        int run = g.begin;
        for (int k0 = 0; k0 < nb; k0 += 32) {
            const int k = k0 + lane;
            const int v = k < nb ? bin_count[base + k] : 0;
            int incl = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += u;
            }
            if (k < nb) {
                bin_start[base + k] = run + incl - v;
                bin_count[base + k] = 0;
            }
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

// rebuild step 3: scatter atom indices into their bins (order fixed next);
// a batch scatters the atoms of flagged cells only
__global__ void k_scatter_bins(int n, const int* __restrict__ binid, const int* __restrict__ bin_start,
                               int* __restrict__ bin_count, int* __restrict__ bin_tmp, const int* __restrict__ cell_of,
                               const uint8_t* __restrict__ cell_reb, DevScalars* sc) {
    if (!sc->rebuild) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (cell_reb && !cell_reb[cell_of[i]]) continue;
        int b = binid[i];
        int slot = atomicAdd(&bin_count[b], 1);
        bin_tmp[bin_start[b] + slot] = i;
    }
}

// rebuild step 4: one warp per bin ranks its atoms by index (deterministic
// order), counts zeroed for the next rebuild
__global__ void k_sort_bins(int nbins, const int* __restrict__ bin_start, const int* __restrict__ bin_tmp,
                            int* __restrict__ bin_atoms, int* __restrict__ bin_count, const int* __restrict__ cell_of,
                            const uint8_t* __restrict__ cell_reb, DevScalars* sc) {
    if (!sc->rebuild) return;
    int lane = threadIdx.x & 31;
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nw = (gridDim.x * blockDim.x) >> 5;
    for (int b = warp; b < nbins; b += nw) {
        int lo = bin_start[b], hi = bin_start[b + 1];
        // a batch bin's slots lie in its cell's atom range, so the cell of a
        // non-empty bin is the cell of atom index lo
        if (cell_reb && lo < hi && !cell_reb[cell_of[lo]]) continue;
        for (int k = lo + lane; k < hi; k += 32) {
            int a = bin_tmp[k];
            int r = 0;
            for (int q = lo; q < hi; q++) r += bin_tmp[q] < a;
            bin_atoms[lo + r] = a;
        }
        if (lane == 0) bin_count[b] = 0;
    }
}

// FP32 positions in the scaled bin frame, relative to the atom's bin corner:
// p'_d = (x B)_d * 8 nb_d - 8 b_d (x not wrapped between builds, so p' may
// leave [0,8) by the drift since the build); gated == true only in a rebuild
__device__ __forceinline__ float4 frame_pos(const Geo& g, double x0, double x1, double x2, int bc) {
    double u0 = g.bs[0] * x0 + (g.bs[1] * x1 + g.bs[2] * x2);
    double u1 = g.bs[3] * x1 + g.bs[4] * x2;
    double u2 = g.bs[5] * x2;
    float4 p;
    p.x = (float)(u0 - (double)(8 * (bc & 1023)));
    p.y = (float)(u1 - (double)(8 * ((bc >> 10) & 1023)));
    p.z = (float)(u2 - (double)(8 * ((bc >> 20) & 1023)));
    p.w = 0.f;
    return p;
}

__global__ void k_shadow(int n, const double* __restrict__ x, const int* __restrict__ binc, float4* __restrict__ p32,
                         float4* __restrict__ p0, Geo g, int gated, DevScalars* sc) {
    if (gated && !sc->rebuild) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = frame_pos(g, x[i], x[n + i], x[2 * n + i], binc[i]);
        p32[i] = p;
        if (gated) p0[i] = p;
    }
}

__global__ void k_shadow_b(int n, const double* __restrict__ x, const int* __restrict__ binc,
                           const CellGeo* __restrict__ cells, const int* __restrict__ cell_of,
                           float4* __restrict__ p32, float4* __restrict__ p0, int gated,
                           const uint8_t* __restrict__ cell_reb, DevScalars* sc) {
    if (gated && !sc->rebuild) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (gated && !cell_reb[cell_of[i]]) continue;
        const CellGeo& cg = cells[cell_of[i]];
        Geo g;
        for (int k = 0; k < 6; k++) g.bs[k] = cg.bs[k];
        float4 p = frame_pos(g, x[i], x[n + i], x[2 * n + i], binc[i]);
        p32[i] = p;
        if (gated) p0[i] = p;
    }
}

struct BuildArgs {
    int n, maxnbr, ne;
    const double* x;
    const double* s;
    const float4* p32;
    const uint8_t* elem;
    const int* bin_start;
    const int* bin_atoms;
    int* nbr;
    int* nnbr;
    double* x0;
    Geo g;
    Frame fr;
    float lo2[kMaxElem * kMaxElem], hi2[kMaxElem * kMaxElem];
    float in2[kMaxElem * kMaxElem];  // pair cutoff squared: entries below it lead their row
    double cut_sk_sq[kMaxElem * kMaxElem];
    const CellGeo* cells;  // batch: per-cell geometry, indexed by cell_of
    const int* cell_of;
    const uint8_t* cell_reb;  // batch: the cells to rebuild
};

// frame displacement to Cartesian: dx' G with G as head + tail
template <class FR>
__device__ __forceinline__ void frame_to_cart(const FR& fr, float a, float b, float c, float& x, float& y,
                                              float& z) {
    if (fr.ortho) {
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

// the reference's predicate for a pair inside the FP32 band: x_j' =
// S2X(s_j + n) in FP64 without fused multiply-adds, RSQ < (cut + skin)^2
__device__ __forceinline__ bool exact_keep(const BuildArgs& a, const double* h6, double xi0, double xi1, double xi2,
                                           int j, int im, int pe) {
    const int n = a.n;
    const int n0 = (im & 3) - 1, n1 = ((im >> 2) & 3) - 1, n2 = ((im >> 4) & 3) - 1;
    double s0 = a.s[j], s1 = a.s[n + j], s2 = a.s[2 * n + j];
    if (n0 > 0) s0 = dadd(s0, 1.0);
    if (n0 < 0) s0 = dsub(s0, 1.0);
    if (n1 > 0) s1 = dadd(s1, 1.0);
    if (n1 < 0) s1 = dsub(s1, 1.0);
    if (n2 > 0) s2 = dadd(s2, 1.0);
    if (n2 < 0) s2 = dsub(s2, 1.0);
    double xj0, xj1, xj2;
    s2x(h6, s0, s1, s2, xj0, xj1, xj2);
    double e0 = dsub(xi0, xj0), e1 = dsub(xi1, xj1), e2 = dsub(xi2, xj2);
    double rsq = dadd(dmul(e0, e0), dadd(dmul(e1, e1), dmul(e2, e2)));
    return rsq < a.cut_sk_sq[pe];
}

// rebuild step 5: one warp per bin.  The candidates of the bin's 27-bin
// stencil are read 32 at a time, once for all atoms of the bin, and every
// atom of the bin tests them in turn, so a candidate's gathers and its place
// in the bin sequence are paid once per bin instead of once per atom.  A
// row holds first its atom's neighbours inside the pair cutoff at build time,
// in (bin step, bin order) order, bin steps c = (d0+1) + 3(d1+1) + 9(d2+1),
// then those of the skin shell, in the reverse of that order: the shell's
// entries are written backwards from the row's end and moved behind the
// inner ones once the bin's candidates are done.  Lanes test candidates and
// ballots keep their order.  With the inner entries in front, the lanes of
// an atom (slots lane, lane + TPA, ...) get equal shares of the pairs inside
// the cutoff, and the density pass's lanes reach the shell together.  A
// batch finds the bin's cell through its first atom (the bins of a cell hold
// only that cell's atoms).
// ORTHO: every cell orthorhombic (one product per axis to Cartesian).
// UNI: every pair type has the same list cutoff (thresholds in registers).
template <bool BATCH, bool ORTHO, bool UNI>
__global__ void __launch_bounds__(256) k_build_bins(BuildArgs a, int nbins, DevScalars* sc) {
    if (!sc->rebuild) return;
    __shared__ float4 off[27];
    __shared__ int s_pre[8][32], s_lo[8][32], s_img[8][32];  // per warp: the bin's 27 stencil bins
    __shared__ float4 s_at[8][32];  // per warp: the bin's atoms (frame position, w = index << 3 | element)
    __shared__ float s_lo2[kMaxElem * kMaxElem], s_hi2[kMaxElem * kMaxElem], s_in2[kMaxElem * kMaxElem];
    if (threadIdx.x < 27)
        off[threadIdx.x] = make_float4(a.fr.off[threadIdx.x][0], a.fr.off[threadIdx.x][1], a.fr.off[threadIdx.x][2], 0.f);
    if (threadIdx.x < a.ne * a.ne) {
        s_lo2[threadIdx.x] = a.lo2[threadIdx.x];
        s_hi2[threadIdx.x] = a.hi2[threadIdx.x];
        s_in2[threadIdx.x] = a.in2[threadIdx.x];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int n = a.n;
    const float lo2u = a.lo2[0], hi2u = a.hi2[0], in2u = a.in2[0];
    int maxrow = 0, overflow = 0;
    long long sumrow = 0;
    for (int b = warp; b < nbins; b += nw) {
        const int a0 = a.bin_start[b];
        const int na = a.bin_start[b + 1] - a0;
        if (na == 0) continue;
        const int cell = BATCH ? a.cell_of[a0] : 0;  // a batch bin's slots lie in its cell's atom range
        if (BATCH && !a.cell_reb[cell]) continue;
        const CellGeo* cg = BATCH ? a.cells + cell : nullptr;
        const int nbx = BATCH ? cg->nb[0] : a.g.nb[0], nby = BATCH ? cg->nb[1] : a.g.nb[1],
                  nbz = BATCH ? cg->nb[2] : a.g.nb[2];
        const int bin_base = BATCH ? cg->bin_base : 0;
        const float G0 = BATCH ? cg->G[0][0] : a.fr.G[0][0], G1 = BATCH ? cg->G[1][1] : a.fr.G[1][1],
                    G2 = BATCH ? cg->G[2][2] : a.fr.G[2][2];
        double h6[6];
#pragma unroll
        for (int k = 0; k < 6; k++) h6[k] = BATCH ? cg->h6[k] : a.g.h6[k];
        const int bl = b - bin_base;
        const int b0 = bl % nbx, b1 = (bl / nbx) % nby, b2 = bl / (nbx * nby);
        int lo = 0, ncand = 0, img = 0;
        if (lane < 27) {
            const int c = lane;
            int u0 = b0 + c % 3 - 1, u1 = b1 + (c / 3) % 3 - 1, u2 = b2 + c / 9 - 1;
            int n0 = u0 < 0 ? -1 : (u0 >= nbx ? 1 : 0);
            int n1 = u1 < 0 ? -1 : (u1 >= nby ? 1 : 0);
            int n2 = u2 < 0 ? -1 : (u2 >= nbz ? 1 : 0);
            int w = bin_base + (u0 - n0 * nbx) + nbx * ((u1 - n1 * nby) + nby * (u2 - n2 * nbz));
            lo = a.bin_start[w];
            ncand = a.bin_start[w + 1] - lo;
            img = (n0 + 1) | ((n1 + 1) << 2) | ((n2 + 1) << 4);
        }
        int incl = ncand;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        s_pre[wib][lane] = incl - ncand;
        s_lo[wib][lane] = lo;
        s_img[wib][lane] = img;
        for (int g0 = 0; g0 < na; g0 += 32) {
            const int ng = min(32, na - g0);
            __syncwarp();  // the previous group's atoms are no longer read
            if (lane < ng) {
                const int i = a.bin_atoms[a0 + g0 + lane];
                float4 p = a.p32[i];
                p.w = __int_as_float((i << 3) | a.elem[i]);
                s_at[wib][lane] = p;
            }
            __syncwarp();
            int mycnt = 0;  // lane q: inner entries so far of the group's atom q (row front)
            int myout = 0;  // lane q: shell entries so far (row end, backwards)
            int c = 0, cpre = 0, cnext = s_pre[wib][1], clo = s_lo[wib][0], cimg = s_img[wib][0];
            for (int t0 = 0; t0 < total; t0 += 32) {
                const int t = t0 + lane;
                const bool valid = t < total;
                int j = -1, ej = 0, im = 21;
                int selfq = -1;  // the group atom this candidate is (its own bin, no image shift)
                float qx = 0.f, qy = 0.f, qz = 0.f;  // candidate minus its bin-step offset
                if (valid) {
                    while (t >= cnext) {
                        c++;
                        cpre = cnext;
                        cnext = c < 26 ? s_pre[wib][c + 1] : total;
                        clo = s_lo[wib][c];
                        cimg = s_img[wib][c];
                    }
                    j = a.bin_atoms[clo + (t - cpre)];
                    const float4 pj = a.p32[j];
                    const float4 o = off[c];
                    ej = a.elem[j];
                    im = cimg;
                    // the bin's own atoms appear once unshifted, as bin step 13
                    if (c == 13 && im == 21) selfq = (t - cpre) - g0;
                    qx = pj.x - o.x;
                    qy = pj.y - o.y;
                    qz = pj.z - o.z;
                }
                const int ent = valid ? make_entry(j, ej, c) : 0;
                for (int q = 0; q < ng; q++) {
                    const float4 pq = s_at[wib][q];
                    const int iw = __float_as_int(pq.w);
                    const int i = iw >> 3;
                    bool keep = false, inner = false;
                    if (valid && q != selfq) {
                        float dx, dy, dz;
                        if (ORTHO) {
                            dx = (pq.x - qx) * G0;
                            dy = (pq.y - qy) * G1;
                            dz = (pq.z - qz) * G2;
                        } else if (BATCH) {
                            frame_to_cart(*cg, pq.x - qx, pq.y - qy, pq.z - qz, dx, dy, dz);
                        } else {
                            frame_to_cart(a.fr, pq.x - qx, pq.y - qy, pq.z - qz, dx, dy, dz);
                        }
                        const float r2 = dx * dx + (dy * dy + dz * dz);
                        const int pe = UNI ? 0 : (iw & 7) * a.ne + ej;
                        if (r2 < (UNI ? lo2u : s_lo2[pe]))
                            keep = true;
                        else if (r2 <= (UNI ? hi2u : s_hi2[pe]))
                            keep = exact_keep(a, h6, a.x[i], a.x[n + i], a.x[2 * n + i], j, im,
                                              UNI ? (iw & 7) * a.ne + ej : pe);
                        inner = keep && r2 < (UNI ? in2u : s_in2[pe]);
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, keep);
                    if (m) {
                        const unsigned mi = __ballot_sync(0xffffffffu, inner);
                        const unsigned mo = m & ~mi;
                        const unsigned below = (1u << lane) - 1u;
                        const int cin = __shfl_sync(0xffffffffu, mycnt, q);
                        const int cout = __shfl_sync(0xffffffffu, myout, q);
                        if (keep) {
                            // both streams stay inside the row; where they
                            // meet the row has overflowed and is built again
                            // with a larger capacity
                            const int pos = inner ? cin + __popc(mi & below)
                                                  : a.maxnbr - 1 - (cout + __popc(mo & below));
                            if (pos >= 0 && pos < a.maxnbr) a.nbr[(size_t)i * a.maxnbr + pos] = ent;
                        }
                        if (lane == q) {
                            mycnt = cin + __popc(mi);
                            myout = cout + __popc(mo);
                        }
                    }
                }
            }
            // each row's shell entries move from the row's end to follow its
            // inner ones: a move to lower slots, 32 entries at a time, each
            // batch read before it is written (the gap is never negative)
            __syncwarp();
            for (int q = 0; q < ng; q++) {
                const int cin = __shfl_sync(0xffffffffu, mycnt, q);
                const int cout = __shfl_sync(0xffffffffu, myout, q);
                if (cout == 0 || cin + cout > a.maxnbr) continue;
                int* row = a.nbr + (size_t)(__float_as_int(s_at[wib][q].w) >> 3) * a.maxnbr;
                const int src = a.maxnbr - cout;
                for (int k0 = 0; k0 < cout; k0 += 32) {
                    const int k = k0 + lane;
                    const int v = k < cout ? row[src + k] : 0;
                    __syncwarp();
                    if (k < cout) row[cin + k] = v;
                    __syncwarp();
                }
            }
            if (lane < ng) {
                const int i = __float_as_int(s_at[wib][lane].w) >> 3;
                const int tot = mycnt + myout;
                a.nnbr[i] = min(tot, a.maxnbr);
                if (tot > a.maxnbr) overflow = 1;
                maxrow = max(maxrow, tot);
                sumrow += tot;
                a.x0[i] = a.x[i];
                a.x0[n + i] = a.x[n + i];
                a.x0[2 * n + i] = a.x[2 * n + i];
            }
        }
        __syncwarp();  // the stencil table is rewritten for the next bin
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        maxrow = max(maxrow, __shfl_xor_sync(0xffffffffu, maxrow, o));
        overflow |= __shfl_xor_sync(0xffffffffu, overflow, o);
        sumrow += __shfl_xor_sync(0xffffffffu, sumrow, o);
    }
    if (lane == 0) {
        if (overflow) sc->overflow = 1;
        if (maxrow) atomicMax(&sc->maxrow, maxrow);
        if (sumrow) atomicAdd(&sc->sumrow, (unsigned long long)sumrow);
    }
}

__global__ void k_rebuild_done(DevScalars* sc) {
    if (!sc->rebuild) return;
    sc->nrebuild++;
    sc->drift[0] = sc->drift[1] = sc->drift[2] = 0.0;
}

__global__ void k_rebuild_done_b(DevScalars* sc, CellMd* cmd, uint8_t* cell_reb, int ncell) {
    if (!sc->rebuild) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
        if (!cell_reb[c]) continue;
        cmd[c].drift[0] = cmd[c].drift[1] = cmd[c].drift[2] = 0.0;
        cell_reb[c] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->nrebuild++;
        sc->drift[0] = sc->drift[1] = sc->drift[2] = 0.0;
    }
}

// skin test of DynamicMD::decide (dynamic_md.cpp:90-105): rebuild when any
// |x - x0|^2 > skin^2/4, RSQ order, FP64
__global__ void k_skin(int n, const double* __restrict__ x, const double* __restrict__ x0, double skin_sq,
                       DevScalars* sc) {
    int moved = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d0 = dsub(x0[i], x[i]), d1 = dsub(x0[n + i], x[n + i]), d2 = dsub(x0[2 * n + i], x[2 * n + i]);
        double r = dadd(dmul(d0, d0), dadd(dmul(d1, d1), dmul(d2, d2)));
        moved |= r > skin_sq;
    }
    if (__syncthreads_or(moved) && threadIdx.x == 0) sc->rebuild = 1;
}

// batch: the same test, flagging the cells whose atoms moved
__global__ void k_skin_b(int n, const double* __restrict__ x, const double* __restrict__ x0, double skin_sq,
                         const int* __restrict__ cell_of, uint8_t* __restrict__ cell_reb, DevScalars* sc) {
    int moved = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d0 = dsub(x0[i], x[i]), d1 = dsub(x0[n + i], x[n + i]), d2 = dsub(x0[2 * n + i], x[2 * n + i]);
        double r = dadd(dmul(d0, d0), dadd(dmul(d1, d1), dmul(d2, d2)));
        if (r > skin_sq) {
            cell_reb[cell_of[i]] = 1;
            moved = 1;
        }
    }
    if (__syncthreads_or(moved) && threadIdx.x == 0) sc->rebuild = 1;
}

__global__ void k_set_rebuild(DevScalars* sc, int v) {
    sc->rebuild = v;
}

// caller order (AoS) <-> bin-sorted order (SoA)
__global__ void k_gather_aos(int n, const int* __restrict__ id, const double* __restrict__ src,
                             double* __restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int u = id[i];
        dst[i] = src[3 * (size_t)u];
        dst[n + i] = src[3 * (size_t)u + 1];
        dst[2 * n + i] = src[3 * (size_t)u + 2];
    }
}

__global__ void k_scatter_aos(int n, const int* __restrict__ id, const double* __restrict__ src,
                              double* __restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int u = id[i];
        dst[3 * (size_t)u] = src[i];
        dst[3 * (size_t)u + 1] = src[n + i];
        dst[3 * (size_t)u + 2] = src[2 * n + i];
    }
}

__global__ void k_f32_to_f64(int n3, const float* __restrict__ a, double* __restrict__ b) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) b[i] = (double)a[i];
}

// ------------------------------------------------------------------ launchers
void sync_forces64(mappg_sys* s) {
    if (!s->f_is_f32) return;
    k_f32_to_f64<<<grid_for(s, 3LL * s->n, 256), 256, 0, s->stream>>>(3 * s->n, s->f32, s->f);
    MAPPG_CUDA(cudaGetLastError());
    s->f_is_f32 = false;
}

void request_rebuild(mappg_sys* s) {
    k_set_rebuild<<<1, 1, 0, s->stream>>>(s->sc, 1);
    MAPPG_CUDA(cudaGetLastError());
    if (s->cell_reb) MAPPG_CUDA(cudaMemsetAsync(s->cell_reb, 1, s->ncell, s->stream));
}

void launch_shadow(mappg_sys* s, bool gated) {
    if (s->ncell > 1) {
        k_shadow_b<<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->x, s->binc, s->cells_dev, s->cell_of,
                                                                   s->p32, s->p0, gated ? 1 : 0, s->cell_reb, s->sc);
        MAPPG_CUDA(cudaGetLastError());
        return;
    }
    Geo g = make_geo(s);
    k_shadow<<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->x, s->binc, s->p32, s->p0, g, gated ? 1 : 0,
                                                            s->sc);
    MAPPG_CUDA(cudaGetLastError());
}

void launch_rebuild_chain(mappg_sys* s) {
    Geo g = make_geo(s);
    const int B = 256;
    int gb = grid_for(s, s->n, B);
    const bool batch = s->ncell > 1;
    // a batch rebuilds the cells whose flag is set (cell_reb), a single cell
    // all of its atoms
    const uint8_t* reb = batch ? s->cell_reb : nullptr;
    if (batch) {
        k_wrap_bin_b<<<gb, B, 0, s->stream>>>(s->n, s->x, s->s, s->cells_dev, s->cell_of, s->cmd, s->binc, s->binid,
                                              s->bin_count, s->cell_reb, s->sc);
        k_scan_bins_b<<<(s->ncell * 32 + B - 1) / B, B, 0, s->stream>>>(s->ncell, s->n, s->nbins, s->cells_dev,
                                                                         s->cell_reb, s->bin_count, s->bin_start,
                                                                         s->sc);
    } else {
        k_wrap_bin<<<gb, B, 0, s->stream>>>(s->n, s->x, s->s, g, s->binc, s->binid, s->bin_count, s->sc);
        k_scan_bins<<<1, 1024, 0, s->stream>>>(s->nbins, s->bin_count, s->bin_start, s->sc);
    }
    int* bin_tmp = s->bin_atoms + s->n;
    k_scatter_bins<<<gb, B, 0, s->stream>>>(s->n, s->binid, s->bin_start, s->bin_count, bin_tmp, s->cell_of, reb,
                                            s->sc);
    k_sort_bins<<<grid_for(s, (long long)s->nbins * 32, B), B, 0, s->stream>>>(
        s->nbins, s->bin_start, bin_tmp, s->bin_atoms, s->bin_count, s->cell_of, reb, s->sc);
    if (batch)
        k_shadow_b<<<gb, B, 0, s->stream>>>(s->n, s->x, s->binc, s->cells_dev, s->cell_of, s->p32, s->p0, 1,
                                            s->cell_reb, s->sc);
    else
        k_shadow<<<gb, B, 0, s->stream>>>(s->n, s->x, s->binc, s->p32, s->p0, g, 1, s->sc);
    BuildArgs a;
    a.n = s->n;
    a.maxnbr = s->maxnbr;
    a.ne = s->ne;
    a.x = s->x;
    a.s = s->s;
    a.p32 = s->p32;
    a.elem = s->elem;
    a.bin_start = s->bin_start;
    a.bin_atoms = s->bin_atoms;
    a.nbr = s->nbr;
    a.nnbr = s->nnbr;
    a.x0 = s->x0;
    a.g = g;
    for (int p = 0; p < s->ne * s->ne; p++) {
        a.cut_sk_sq[p] = s->cut_sk_sq[p];
        a.lo2[p] = (float)(s->cut_sk_sq[p] - s->band);
        a.hi2[p] = (float)(s->cut_sk_sq[p] + s->band);
        a.in2[p] = (float)s->cut_sq[p];
    }
    a.fr = s->frame;
    a.cells = s->cells_dev;
    a.cell_of = s->cell_of;
    a.cell_reb = reb;
    const int gbins = grid_for(s, (long long)s->nbins * 32, B);
    bool uni = true;
    for (int p = 1; p < s->ne * s->ne; p++) uni = uni && a.lo2[p] == a.lo2[0] && a.hi2[p] == a.hi2[0];
    auto launch = [&](auto BT, auto OT, auto UT) {
        k_build_bins<decltype(BT)::value, decltype(OT)::value, decltype(UT)::value>
            <<<gbins, B, 0, s->stream>>>(a, s->nbins, s->sc);
    };
    auto by_uni = [&](auto BT, auto OT) {
        if (uni)
            launch(BT, OT, std::true_type());
        else
            launch(BT, OT, std::false_type());
    };
    if (batch) {
        if (s->cells_ortho)
            by_uni(std::true_type(), std::true_type());
        else
            by_uni(std::true_type(), std::false_type());
        k_rebuild_done_b<<<(s->ncell + 255) / 256, 256, 0, s->stream>>>(s->sc, s->cmd, s->cell_reb, s->ncell);
    } else {
        if (s->frame.ortho)
            by_uni(std::false_type(), std::true_type());
        else
            by_uni(std::false_type(), std::false_type());
        k_rebuild_done<<<1, 1, 0, s->stream>>>(s->sc);
    }
    MAPPG_CUDA(cudaGetLastError());
}

void launch_skin_test(mappg_sys* s) {
    double skin_sq = 0.25 * s->skin * s->skin;
    if (s->cell_reb)
        k_skin_b<<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->x, s->x0, skin_sq, s->cell_of, s->cell_reb,
                                                                s->sc);
    else
        k_skin<<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->x, s->x0, skin_sq, s->sc);
    MAPPG_CUDA(cudaGetLastError());
}

EamArgs eam_args(mappg_sys* s) {
    const mappg_ff* ff = s->ff;
    EamArgs a;
    memset(&a, 0, sizeof(a));
    a.n = s->n;
    a.maxnbr = s->maxnbr;
    a.ne = s->ne;
    a.nr = ff->dev.nr;
    a.nrho = ff->dev.nrho;
    a.nbr = s->nbr;
    a.nnbr = s->nnbr;
    a.elem = s->elem;
    a.x = s->x;
    a.p32 = s->p32;
    a.binc = s->binc;
    a.rho64 = ff->dev.rho64;
    a.rphi64 = ff->dev.rphi64;
    a.F64 = ff->dev.F64;
    a.rho32 = ff->dev.rho32;
    a.ftab = ff->dev.ftab;
    a.fjtab = ff->dev.fjtab;
    a.F32 = ff->dev.F32;
    a.F32lo = ff->dev.F32lo;
    a.rho_ei = ff->dev.rho_ei;
    a.rho_ntab = a.rho_ei ? s->ne * s->ne : s->ne;
    a.rho_w = std::min(a.nr - 1, (int)(kDensSmemBytes / (sizeof(float) * 4 * a.rho_ntab)));
    a.rho_mlo = (a.nr - 1) - a.rho_w;  // knots up to nr - 2, the last one a pair can use
    a.dr_inv = ff->dev.dr_inv;
    a.drho_inv = ff->dev.drho_inv;
    a.rho_max = ff->dev.rho_max;
    a.cut_uniform = 1;
    for (int p = 0; p < s->ne * s->ne; p++) {
        a.cut_sq[p] = s->cut_sq[p];
        if ((float)s->cut_sq[p] != (float)s->cut_sq[0]) a.cut_uniform = 0;
    }
    memcpy(a.shift, s->shift, sizeof(a.shift));
    a.fr = s->frame;
    for (int d = 0; d < 3; d++) a.nb[d] = s->nb[d];
    a.q32 = s->q32;
    a.rho = s->rho;
    a.rho_keep = s->keep_rho64 ? s->rho : nullptr;
    a.rho0 = s->rho;
    a.h32 = s->h32;
    a.alpha = 0.0;
    a.cell_active = s->cell_active;
    a.cutmask = s->cutmask;
    a.fs_tab = s->fs_tab;
    a.fs_rec = s->fs_rec;
    a.fs_stride = s->fs_w;
    a.fs_w = s->fs_w;
    if (s->force_smem > 0 && s->fs_rec > 0) {
        const long long fit = (long long)s->force_smem * 1024 / ((long long)sizeof(float4) * s->fs_rec);
        a.fs_w = (int)std::min<long long>(s->fs_w, fit);
    }
    a.fs_off = s->fs_w - a.fs_w;
    a.fs_mlo = s->fs_mlo + a.fs_off;
    a.grp_atoms = s->grp_atoms;
    for (int g = 0; g <= s->ne; g++) a.grp_begin[g] = s->grp_begin[g];
    a.dF = s->dF;
    a.rho32out = s->rho32;
    a.f = s->f;
    a.f32 = s->f32;
    a.partials = s->partials;
    a.sc = s->sc;
    a.ncell = s->ncell;
    a.nchunk = s->nchunk;
    a.cells = s->cells_dev;
    a.chunk_begin = s->chunk_begin;
    a.chunk_cell = s->chunk_cell;
    a.chunk_part = s->chunk_part;
    return a;
}

// host check after a build: capacity, bad coordinates
void check_build(mappg_sys* s) {
    DevScalars h;
    MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    if (h.bad) throw Error{MAPPG_ERR_NAN, "non-finite or far out-of-cell position"};
    if (h.overflow) throw Error{MAPPG_ERR_NBR, "neighbour list capacity exceeded"};
}

}  // namespace mappg

using namespace mappg;

// ------------------------------------------------------------------ system lifecycle (called from api.cpp)
namespace mappg {

static void dev_alloc(void** p, size_t bytes) { MAPPG_CUDA(cudaMalloc(p, bytes > 0 ? bytes : 16)); }

void sys_free(mappg_sys* s) {
    void* ptrs[] = {s->x, s->v, s->f, s->x0, s->s, s->elem, s->id, s->inv, s->p32, s->q32, s->p0, s->f32, s->v32,
                    s->rho32, s->binc, s->binid, s->bin_count, s->bin_start, s->bin_atoms, s->nbr, s->nnbr,
                    s->rho, s->dF, s->partials, s->sc, s->stage, s->thermo_dev, s->cells_dev, s->cell_of,
                    s->chunk_begin, s->chunk_cell, s->cell_chunk, s->chunk_part, s->chunk_disp, s->cmd,
                    s->cell_out, s->dof, s->stage2, s->cutmask, s->fs_tab, s->grp_atoms, s->cell_reb};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s->ev_main) cudaEventDestroy(s->ev_main);
    if (s->ev_side) cudaEventDestroy(s->ev_side);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->stream) cudaStreamDestroy(s->stream);
}

static unsigned long long morton3(unsigned a, unsigned b, unsigned c) {
    auto spread = [](unsigned long long v) {
        v &= 0x1fffff;
        v = (v | v << 32) & 0x1f00000000ffffULL;
        v = (v | v << 16) & 0x1f0000ff0000ffULL;
        v = (v | v << 8) & 0x100f00f00f00f00fULL;
        v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
        v = (v | v << 2) & 0x1249249249249249ULL;
        return v;
    };
    return spread(a) | (spread(b) << 1) | (spread(c) << 2);
}

void sys_alloc(mappg_sys* s, const double* x_host) {
    const int n = s->n;
    MAPPG_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    // fixed atom order: Morton order of the initial bins, then caller index
    // (a batch: cell by cell, Morton order within each cell)
    std::vector<unsigned long long> key(n);
    for (int c = 0; c < s->ncell; c++) {
        const bool batch = s->ncell > 1;
        const double* b6 = batch ? s->cells[c].b6 : s->box.b6;
        const int* nb = batch ? s->cells[c].nb : s->nb;
        const int u0 = batch ? s->cell_begin[c] : 0, u1 = batch ? s->cell_begin[c + 1] : n;
        for (int u = u0; u < u1; u++) {
            const double* xu = x_host + 3 * (size_t)u;
            double sv[3] = {b6[0] * xu[0] + (b6[1] * xu[1] + b6[2] * xu[2]), b6[3] * xu[1] + b6[4] * xu[2],
                            xu[2] * b6[5]};
            unsigned b[3];
            for (int d = 0; d < 3; d++) {
                double w = sv[d] - floor(sv[d]);
                if (!(w >= 0.0 && w < 1.0)) w = 0.0;
                b[d] = (unsigned)std::min((int)(w * nb[d] * 2), 2 * nb[d] - 1);
            }
            key[u] = ((unsigned long long)c << 40) | morton3(b[0], b[1], b[2]);
        }
    }
    s->host_id.resize(n);
    std::iota(s->host_id.begin(), s->host_id.end(), 0);
    std::stable_sort(s->host_id.begin(), s->host_id.end(), [&](int a, int b) { return key[a] < key[b]; });
    std::vector<int> inv(n);
    for (int i = 0; i < n; i++) inv[s->host_id[i]] = i;

    size_t nd = (size_t)3 * n * sizeof(double);
    dev_alloc((void**)&s->x, nd);
    dev_alloc((void**)&s->v, nd);
    dev_alloc((void**)&s->f, nd);
    dev_alloc((void**)&s->x0, nd);
    dev_alloc((void**)&s->s, nd);
    dev_alloc((void**)&s->stage, nd);
    dev_alloc((void**)&s->elem, n);
    dev_alloc((void**)&s->id, sizeof(int) * n);
    dev_alloc((void**)&s->inv, sizeof(int) * n);
    dev_alloc((void**)&s->p32, sizeof(float4) * n);
    dev_alloc((void**)&s->q32, sizeof(float4) * n);
    dev_alloc((void**)&s->p0, sizeof(float4) * n);
    dev_alloc((void**)&s->f32, sizeof(float) * 3 * (size_t)n);
    dev_alloc((void**)&s->v32, sizeof(float) * 3 * (size_t)n);
    dev_alloc((void**)&s->rho32, sizeof(float) * n);
    if (s->precision == MAPPG_MIXED) dev_alloc((void**)&s->cutmask, sizeof(unsigned) * 32 * (size_t)n);
    dev_alloc((void**)&s->binc, sizeof(int) * n);
    dev_alloc((void**)&s->binid, sizeof(int) * n);
    dev_alloc((void**)&s->bin_atoms, sizeof(int) * 2 * (size_t)n);
    dev_alloc((void**)&s->nnbr, sizeof(int) * n);
    dev_alloc((void**)&s->rho, sizeof(double) * n);
    dev_alloc((void**)&s->dF, sizeof(double) * n);
    dev_alloc((void**)&s->partials, sizeof(double) * kRedSlots * kMaxBlocks);
    dev_alloc((void**)&s->sc, sizeof(DevScalars));
    MAPPG_CUDA(cudaMemsetAsync(s->sc, 0, sizeof(DevScalars), s->stream));
    MAPPG_CUDA(cudaMemsetAsync(s->v, 0, nd, s->stream));
    MAPPG_CUDA(cudaMemsetAsync(s->f, 0, nd, s->stream));
    MAPPG_CUDA(cudaMemcpyAsync(s->id, s->host_id.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->stream));
    MAPPG_CUDA(cudaMemcpyAsync(s->inv, inv.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->stream));
    if (s->ncell > 1) {
        const int nc = s->ncell, nk = s->nchunk;
        std::vector<int> cell_of(n);
        for (int c = 0; c < nc; c++)
            for (int i = s->cell_begin[c]; i < s->cell_begin[c + 1]; i++) cell_of[i] = c;
        dev_alloc((void**)&s->cells_dev, sizeof(CellGeo) * nc);
        dev_alloc((void**)&s->cell_of, sizeof(int) * n);
        dev_alloc((void**)&s->cmd, sizeof(CellMd) * nc);
        dev_alloc((void**)&s->cell_out, sizeof(double) * 8 * nc);
        dev_alloc((void**)&s->cell_reb, nc);
        MAPPG_CUDA(cudaMemsetAsync(s->cell_reb, 1, nc, s->stream));
        MAPPG_CUDA(cudaMemsetAsync(s->cmd, 0, sizeof(CellMd) * nc, s->stream));
        MAPPG_CUDA(cudaMemcpyAsync(s->cells_dev, s->cells.data(), sizeof(CellGeo) * nc, cudaMemcpyHostToDevice,
                                   s->stream));
        MAPPG_CUDA(cudaMemcpyAsync(s->cell_of, cell_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->stream));
        upload_chunks(s);
    }
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
}

void sys_alloc_bins(mappg_sys* s) {
    if (s->bin_count) cudaFree(s->bin_count);
    if (s->bin_start) cudaFree(s->bin_start);
    s->bin_count = nullptr;
    s->bin_start = nullptr;
    dev_alloc((void**)&s->bin_count, sizeof(int) * s->nbins);
    dev_alloc((void**)&s->bin_start, sizeof(int) * (s->nbins + 1));
    MAPPG_CUDA(cudaMemsetAsync(s->bin_count, 0, sizeof(int) * s->nbins, s->stream));
}

void sys_alloc_nbr(mappg_sys* s, int maxnbr) {
    if (s->nbr) cudaFree(s->nbr);
    s->nbr = nullptr;
    s->maxnbr = maxnbr;
    dev_alloc((void**)&s->nbr, sizeof(int) * (size_t)s->n * maxnbr);
}

// upload caller-order AoS doubles into a SoA device array
void sys_upload(mappg_sys* s, const double* host, double* dev) {
    MAPPG_CUDA(cudaMemcpyAsync(s->stage, host, sizeof(double) * 3 * (size_t)s->n, cudaMemcpyHostToDevice, s->stream));
    k_gather_aos<<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->id, s->stage, dev);
    MAPPG_CUDA(cudaGetLastError());
}

// upload on the side stream, after the work queued on s->stream so far;
// s->v_pending marks the target as unfinished until s->stream waits on it
void sys_upload_side(mappg_sys* s, const double* host, double* dev) {
    if (!s->side) {
        MAPPG_CUDA(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
        MAPPG_CUDA(cudaEventCreateWithFlags(&s->ev_main, cudaEventDisableTiming));
        MAPPG_CUDA(cudaEventCreateWithFlags(&s->ev_side, cudaEventDisableTiming));
        dev_alloc((void**)&s->stage2, sizeof(double) * 3 * (size_t)s->n);
    }
    MAPPG_CUDA(cudaEventRecord(s->ev_main, s->stream));
    MAPPG_CUDA(cudaStreamWaitEvent(s->side, s->ev_main, 0));
    MAPPG_CUDA(cudaMemcpyAsync(s->stage2, host, sizeof(double) * 3 * (size_t)s->n, cudaMemcpyHostToDevice, s->side));
    k_gather_aos<<<grid_for(s, s->n, 256), 256, 0, s->side>>>(s->n, s->id, s->stage2, dev);
    MAPPG_CUDA(cudaGetLastError());
    MAPPG_CUDA(cudaEventRecord(s->ev_side, s->side));
    s->v_pending = true;
}

// s->stream waits for the side-stream upload (if one is pending)
void sys_join_side(mappg_sys* s) {
    if (!s->v_pending) return;
    MAPPG_CUDA(cudaStreamWaitEvent(s->stream, s->ev_side, 0));
    s->v_pending = false;
}

// queue a caller-order download without waiting for it (the stage array is
// reused in stream order by the next one)
void sys_download_async(mappg_sys* s, const double* dev, double* host) {
    k_scatter_aos<<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->id, dev, s->stage);
    MAPPG_CUDA(cudaGetLastError());
    MAPPG_CUDA(cudaMemcpyAsync(host, s->stage, sizeof(double) * 3 * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream));
}

void sys_download(mappg_sys* s, const double* dev, double* host) {
    k_scatter_aos<<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->id, dev, s->stage);
    MAPPG_CUDA(cudaGetLastError());
    MAPPG_CUDA(cudaMemcpyAsync(host, s->stage, sizeof(double) * 3 * (size_t)s->n, cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
}

// full build with capacity growth: first build sizes the rows from a count
void sys_build(mappg_sys* s) {
    for (int attempt = 0; attempt < 4; attempt++) {
        request_rebuild(s);
        MAPPG_CUDA(cudaMemsetAsync(&s->sc->overflow, 0, sizeof(int), s->stream));
        launch_rebuild_chain(s);
        DevScalars h;
        MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        if (h.bad) throw Error{MAPPG_ERR_NAN, "non-finite or far out-of-cell position"};
        if (!h.overflow) {
            k_set_rebuild<<<1, 1, 0, s->stream>>>(s->sc, 0);
            s->built = true;
            s->list_box = true;
            return;
        }
        int need = (int)h.maxrow;
        int cap = ((need + need / 4 + 16) + 31) / 32 * 32;
        sys_alloc_nbr(s, cap);
    }
    throw Error{MAPPG_ERR_NBR, "neighbour list capacity could not be sized"};
}

// the cell of atom i (bin-sorted order) of a batch
static int cell_of_host(const mappg_sys* s, int i) {
    return (int)(std::upper_bound(s->cell_begin.begin(), s->cell_begin.end(), i) - s->cell_begin.begin()) - 1;
}

void sys_neighbors(mappg_sys* s, int* counts, int* entries, long long* total) {
    const int n = s->n;
    std::vector<int> nn(n), bc(n);
    MAPPG_CUDA(cudaMemcpyAsync(nn.data(), s->nnbr, sizeof(int) * n, cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaMemcpyAsync(bc.data(), s->binc, sizeof(int) * n, cudaMemcpyDeviceToHost, s->stream));
    std::vector<int> rows;
    if (entries) {
        rows.resize((size_t)n * s->maxnbr);
        MAPPG_CUDA(cudaMemcpyAsync(rows.data(), s->nbr, sizeof(int) * rows.size(), cudaMemcpyDeviceToHost, s->stream));
    }
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    long long tot = 0;
    std::vector<long long> off(n + 1, 0);
    for (int i = 0; i < n; i++) {
        int u = s->host_id[i];
        if (counts) counts[u] = nn[i];
        tot += nn[i];
    }
    if (total) *total = tot;
    if (!entries) return;
    // caller order offsets
    std::vector<long long> uoff(n + 1, 0);
    std::vector<int> ucount(n);
    for (int i = 0; i < n; i++) ucount[s->host_id[i]] = nn[i];
    for (int u = 0; u < n; u++) uoff[u + 1] = uoff[u] + ucount[u];
    for (int i = 0; i < n; i++) {
        int u = s->host_id[i];
        int b[3] = {bc[i] & 1023, (bc[i] >> 10) & 1023, (bc[i] >> 20) & 1023};
        int* out = entries + 4 * uoff[u];
        for (int k = 0; k < nn[i]; k++) {
            int e = rows[(size_t)i * s->maxnbr + k];
            int j = entry_j(e);
            int d[3] = {entry_step(e, 0), entry_step(e, 1), entry_step(e, 2)};
            out[4 * k] = s->host_id[j];
            const int* nbq = s->ncell > 1 ? s->cells[cell_of_host(s, i)].nb : s->nb;
            for (int q = 0; q < 3; q++) {
                int uq = b[q] + d[q];
                out[4 * k + 1 + q] = uq < 0 ? -1 : (uq >= nbq[q] ? 1 : 0);
            }
        }
    }
}

}  // namespace mappg
