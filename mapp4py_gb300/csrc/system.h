// Device-resident state of one periodic cell and the kernel argument blocks.
//
// HBM layout (atoms kept in a fixed bin-sorted order chosen at creation; id[]
// maps it back to the caller's order):
//   x, v, f, x0, s   FP64 structure-of-arrays, 3 planes of n doubles each
//   elem             uint8 per atom
//   p32              float4 per atom: position relative to its bin corner
//                    (FP32) and the element in .w; what the mixed-precision
//                    kernels gather per neighbour
//   binc             packed bin coordinates per atom (10 bits each)
//   nbr              full neighbour list, row i holds nnbr[i] entries
//                    (j << 5 | code), code = bin step (dx+1)+3(dy+1)+9(dz+1)
//                    from atom i's bin to the neighbour image's bin
//   rho, dF, dF32    per-atom host density and F'(rho)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace mappg {

constexpr int kRedSlots = 8;     // doubles per block partial
constexpr int kMaxBlocks = 4096; // partial slots
constexpr int kMaxChain = 16;    // NHC chain length

struct Box {
    double H[3][3], B[3][3], h6[6], b6[6], vol, depth_inv[3];
};

// scalars that live on the device so a whole MD step runs without the host
struct DevScalars {
    int rebuild;       // set: the rebuild kernels of this step do their work
    int overflow;      // a neighbour row ran out of capacity
    int bad;           // non-finite value seen
    int pad0;
    unsigned counter[8];  // last-block-done counters, one per reduction site
    double energy;     // last force/energy call
    double virial[6];  // F_H voigt
    double com[3];     // mean displacement of the step (removed from x)
    int maxrow;        // longest neighbour row of the last build
    int pad1;
    unsigned long long sumrow;  // total entries of the last build
    // NVT state (MDNVT / ThermostatNHC)
    double mvv[6];
    double T_part;
    double fac_x_d;    // pending velocity scale applied in the next kick
    double eta[kMaxChain];
    long long step;    // steps done in this run
    long long nrebuild;
};

struct NhcParams {
    double T, ddt, ddt2, freq_sq, kB, ndof_kB;
    int L, niters, ndof;
};

struct Sys;

// arguments of the EAM kernels (passed by value)
struct EamArgs {
    int n, maxnbr, ne, nr, nrho;
    const int* nbr;
    const int* nnbr;
    const uint8_t* elem;
    const double* x;   // SoA 3n
    const float4* p32;
    const int* binc;
    const double4* rho64;
    const double4* rphi64;
    const double4* F64;
    const float4* rho32;
    const float4* rphi32;
    const float4* F32;
    const float* rphi32_lo;
    double dr_inv, drho_inv, rho_max;
    double cut_sq[kMaxElem * kMaxElem];
    double shift[27][3];   // image shift n*H for image code (n0+1)+3(n1+1)+9(n2+1)
    float off32[27][4];    // bin-step offset for neighbour code (FP32 head)
    float off32lo[27][4];  // its FP32 tail: off = head + tail to ~1e-15
    int nb[3];
    double* rho;
    double* dF;
    float* dF32;
    double* f;             // SoA 3n
    double* partials;
    DevScalars* sc;
};

}  // namespace mappg

struct mappg_sys {
    const mappg_ff* ff = nullptr;
    int n = 0;
    int precision = MAPPG_FP64;
    int ne = 0;
    int device = 0;
    int sm_count = 0;
    int tpa = 8;
    double skin = 0.5;
    double max_cut = 0.0;  // max cut + skin
    double cut_sq[mappg::kMaxElem * mappg::kMaxElem];
    double cut_sk_sq[mappg::kMaxElem * mappg::kMaxElem];
    double masses[mappg::kMaxElem];
    mappg::Box box;
    int nb[3] = {1, 1, 1};
    int nbins = 1;
    float off32[27][4];
    float off32lo[27][4];
    double shift[27][3];
    double band = 0.0;  // half-width of the exact-arithmetic band of the list filter
    cudaStream_t stream = nullptr;

    // device arrays (bin-sorted order)
    double *x = nullptr, *v = nullptr, *f = nullptr, *x0 = nullptr, *s = nullptr;
    uint8_t* elem = nullptr;
    int* id = nullptr;   // sorted -> caller index
    int* inv = nullptr;  // caller -> sorted index
    float4* p32 = nullptr;
    int* binc = nullptr;
    int* binid = nullptr;
    int* bin_count = nullptr;
    int* bin_start = nullptr;
    int* bin_atoms = nullptr;
    int maxnbr = 0;
    int* nbr = nullptr;
    int* nnbr = nullptr;
    double *rho = nullptr, *dF = nullptr;
    float* dF32 = nullptr;
    double* partials = nullptr;
    mappg::DevScalars* sc = nullptr;
    double* stage = nullptr;      // device staging, 3n doubles (caller order)
    double* thermo_dev = nullptr; // per-step thermo rows of an NVT run
    long long thermo_cap = 0;

    void* run = nullptr;  // an NVT run in progress (md.cu)
    bool built = false;
    bool have_v = false;
    bool forces_valid = false;
    std::vector<int> host_id;  // sorted -> caller (host copy)
};

namespace mappg {

// system.cu
void sys_set_box(mappg_sys* s, const double* H);
void launch_rebuild_chain(mappg_sys* s);   // kernels gated by sc->rebuild
void request_rebuild(mappg_sys* s);        // host sets the gate
void launch_shadow(mappg_sys* s, bool gated);
void check_build(mappg_sys* s);            // host: overflow / capacity
void launch_skin_test(mappg_sys* s);       // sets sc->rebuild if needed
EamArgs eam_args(mappg_sys* s);
int grid_for(mappg_sys* s, long long threads, int block);

// eam.cu
void launch_force(mappg_sys* s);           // density+embed, force; totals in sc
void launch_energy(mappg_sys* s);          // energy only; total in sc->energy
void launch_density_only(mappg_sys* s);    // k_density alone (timing)
void launch_force_only(mappg_sys* s);      // k_force alone (timing; needs dF)

}  // namespace mappg
