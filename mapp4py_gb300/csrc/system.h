// Device-resident state of one periodic cell and the kernel argument blocks.
//
// HBM layout (atoms kept in a fixed bin-sorted order chosen at creation; id[]
// maps it back to the caller's order):
//   x, v, f, x0, s   FP64 structure-of-arrays, 3 planes of n doubles each
//   elem             uint8 per atom
//   binc             packed bin coordinates per atom (10 bits each)
//   p32              float4 per atom: the position in the scaled bin frame
//                    (below), relative to the atom's bin corner
//   q32              float4 per atom: p32.xyz and F'(rho) in .w, written by
//                    the mixed density kernel and gathered by the force kernel
//   nbr              full neighbour list, row i holds nnbr[i] entries
//                    (j << 9 | e_j << 6 | k), k = k0 | k1 << 2 | k2 << 4 with
//                    k_d = d_d + 1, d the bin step from atom i's bin to the
//                    neighbour image's bin (j < 2^23: the entry is read as
//                    unsigned)
//   f32, v32         FP32 copies for the mixed path (forces out of the force
//                    kernel; velocities for its kinetic-energy epilogue)
//
// Scaled bin frame: with nb_d bins along fractional axis d, the scaled
// coordinate is s'_d = s_d * 8 nb_d, so every bin is exactly 8 wide, bin
// steps are exact (+-8) and the periodic seam is exact (8 nb_d).  A pair's
// displacement in the frame, dx' = (p'_i - p'_j) - 8 d, is therefore free of
// rounded constants; it becomes Cartesian through G = diag(1/(8 nb)) H,
// applied as a head + tail pair so that its rounding is not shared by all
// pairs either.
#pragma once

#include <functional>

#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace mappg {

constexpr int kRedSlots = 16;    // doubles per block partial
constexpr int kMaxBlocks = 4096; // partial slots
constexpr int kMaxChain = 16;    // NHC chain length
constexpr int kEntryShift = 9;   // j << 9 | element << 6 | bin steps
constexpr int kMaxAtoms = 1 << 23;
constexpr float kBinW = 8.0f;    // bin width in the scaled frame

__host__ __device__ inline int entry_j(int e) { return (int)((unsigned)e >> kEntryShift); }
__host__ __device__ inline int entry_elem(int e) { return (e >> 6) & 7; }
// bin step d_q in {-1, 0, 1} along axis q
__host__ __device__ inline int entry_step(int e, int q) { return ((e >> (2 * q)) & 3) - 1; }
// the entry of neighbour j (element ej) reached by stencil bin c = (d0+1) +
// 3(d1+1) + 9(d2+1) of atom i's bin
__host__ __device__ inline int make_entry(int j, int ej, int c) {
    const unsigned k = (unsigned)(c % 3) | (unsigned)((c / 3) % 3) << 2 | (unsigned)(c / 9) << 4;
    return (int)((unsigned)j << kEntryShift | (unsigned)ej << 6 | k);
}

struct Box {
    double H[3][3], B[3][3], h6[6], b6[6], vol, depth_inv[3];
};

// scalars that live on the device so a whole MD step runs without the host
struct DevScalars {
    int rebuild;       // set: the rebuild kernels of this step do their work
    int overflow;      // a neighbour row ran out of capacity
    int bad;           // non-finite value seen
    int pending_kick;  // mixed MD: v still lacks the closing half kick
    unsigned counter[8];  // last-block-done counters, one per reduction site
    double energy;     // last force/energy call
    double e_embed;    // embedding energy of the last mixed density pass
    double de;         // last energy difference of a line-search trial (k_de32)
    double virial[6];  // F_H voigt
    double com[3];     // mean displacement of the step
    double drift[3];   // mixed MD: displacement not yet removed from x
    int maxrow;        // longest neighbour row of the last build
    int pad1;
    unsigned long long sumrow;  // total entries of the last build
    // NVT state (MDNVT / ThermostatNHC)
    double mvv[6];
    double T_part;
    double fac_x_d;    // pending velocity scale applied in the next kick
    double fac_close;  // mixed MD: closing factor of the last step
    double kickA;      // mixed MD: v <- A v + B f dt/2m
    double kickB;
    double eta[kMaxChain];
    long long step;    // steps done in this run
    long long nrebuild;
};

struct NhcParams {
    double T, ddt, ddt2, freq_sq, kB, ndof_kB;
    int L, niters, ndof;
};

// geometry of the scaled bin frame
struct Frame {
    float G[3][3];     // Cartesian = dx' G (row vector), head
    float Glo[3][3];   // tail
    float off[27][4];  // -8 d for code c (exact)
    int ortho;         // H has no off-diagonal terms
};

// one cell of a batch (several independent periodic cells in one system):
// its box, bins and scaled frame, read per atom by the batch kernels
struct CellGeo {
    double h6[6], b6[6];   // H and its inverse, lower-triangular packed
    double bs[6];          // b6 with column d scaled by 8 nb_d: x -> s'
    float G[3][3];         // scaled frame to Cartesian, head
    float Glo[3][3];       // tail
    int nb[3];             // bins per axis
    int bin_base;          // first global bin index of the cell
    int begin, end;        // atom range (bin-sorted order)
    int ortho;
    int pad;
};

// per-cell dynamic state of a batch (the DevScalars fields that are per cell)
struct CellMd {
    double T, ndof, ndof_kB;  // thermostat target and degrees of freedom
    double eta[kMaxChain];
    double mvv[6];
    double T_part;
    double fac_x_d, fac_close, kickA, kickB;
    double energy, e_embed, virial[6];
    double com[3], drift[3];
    long long step;           // steps done in this run
    int pending_kick, pad;
};

// a batch kernel walks chunks of at most kChunk atoms of one cell; each chunk
// leaves kChunkSlots block sums (energy, virial, kinetic tensor, embedding
// energy) that a per-cell kernel adds up in a fixed order
constexpr int kChunk = 256;
constexpr int kChunkSlots = 16;
constexpr int kMaxCells = 1 << 16;

// arguments of the EAM kernels (passed by value)
// shared memory given to the density tables of k_density32s: the rest of
// the SM's 256 KB stays L1 for the neighbour-position gathers
constexpr size_t kDensSmemBytes = 94 * 1024;
// static shared memory of k_force32s (frame offsets, cutoffs, block sums),
// kept out of its dynamic table budget
constexpr size_t kForceSmemReserve = 4 * 1024;

struct EamArgs {
    int n, maxnbr, ne, nr, nrho;
    const int* nbr;
    const int* nnbr;
    const uint8_t* elem;
    const double* x;   // SoA 3n
    const float4* p32;
    float4* q32;
    const int* binc;
    const Dbl4* rho64;
    const Dbl4* rphi64;
    const Dbl4* F64;
    const float4* rho32;
    const float4* ftab;     // mixed force records, 2 float4 per (pair type, knot)
    const float4* fjtab;    // rho_{i->j} derivative per (pair type, knot)
    const float4* F32;
    const float* F32lo;
    int rho_ei;              // 0: rho_{j->i} depends on e_j only (setfl, funcfl), read row e_j*ne
    // density tables held in shared memory by k_density32s: knots
    // rho_mlo .. rho_mlo + rho_w - 1 of each of rho_ntab tables
    int rho_mlo, rho_w, rho_ntab;
    int cut_uniform;         // every pair type has the same cutoff
    double dr_inv, drho_inv, rho_max;
    double cut_sq[kMaxElem * kMaxElem];
    double shift[27][3];   // image shift n*H for image code (n0+1)+3(n1+1)+9(n2+1)
    Frame fr;
    int nb[3];
    double* rho;
    double* dF;
    float* rho32out;
    double* f;             // SoA 3n (FP64 kernels)
    float* f32;            // SoA 3n (mixed kernels)
    double* partials;
    DevScalars* sc;
    // line searches of mixed-precision minimizers: the density pass also
    // writes the FP64 density here when non-null; the energy-difference pass
    // (k_de32) reads it with the search direction h (float4 per atom,
    // Cartesian) and the trial step alpha
    double* rho_keep;
    const double* rho0;
    const float4* h32;
    double alpha;
    // per-cell closing half of a batch MD step (k_cells_done)
    double* thermo;
    long long nsteps;
    NhcParams nhc;
    // batch of cells (ncell > 1): per-atom cell, chunks, per-chunk sums
    int ncell, nchunk;
    const CellGeo* cells;
    const int* chunk_begin;   // nchunk + 1 atom offsets
    const int* chunk_cell;
    double* chunk_part;       // nchunk x kChunkSlots
    const uint8_t* cell_active;  // batch minimizers: cells the chunk kernels work on (null: all)
    // mixed kernels: per atom and lane, bit t set when the lane's t-th row
    // entry is inside the cutoff (written by the density pass, read by the
    // force pass; rows longer than 32 x lanes are scanned in full)
    unsigned* cutmask;
    const double* cell_alpha;    // batch energy differences: trial step per cell
    // k_force32s: the force records of one element group at a time in shared
    // memory.  fs_tab holds, per group g (the element of atom i), fs_rec
    // records of fs_stride knots ending at the cutoff's knot, record-major:
    //   r <  ne       (z1, z2, z3, z0 head) of r*phi for the pair (g, r)
    //   r <  2 ne     (rho'_{r->g} x3, z0 tail of (g, r - ne))
    //   r >= 2 ne     rho'_{g->e} for e != g (per-pair densities only)
    // The kernel copies the top fs_w knots of each record (from fs_off in
    // its row; knots fs_mlo .. fs_mlo + fs_w - 1), as many as the shared
    // memory budget allows.  grp_atoms lists the atoms of each element in
    // bin order, group g at grp_begin[g] .. grp_begin[g + 1] (null for one
    // element)
    const float4* fs_tab;
    int fs_rec, fs_w, fs_mlo, fs_stride, fs_off;
    const int* grp_atoms;
    int grp_begin[kMaxElem + 1];
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
    int unroll = 1;  // neighbour entries per loop step of the mixed kernels (1 or 2)
    int unroll_force = 0;  // the force pass's own entries per loop step (0: unroll)
    double skin = 0.5;
    double max_cut = 0.0;  // max cut + skin
    double cut_sq[mappg::kMaxElem * mappg::kMaxElem];
    double cut_sk_sq[mappg::kMaxElem * mappg::kMaxElem];
    double masses[mappg::kMaxElem];
    mappg::Box box;
    int nb[3] = {1, 1, 1};
    int nbins = 1;
    mappg::Frame frame;
    double shift[27][3];
    double band = 0.0;  // half-width of the exact-arithmetic band of the list filter
    cudaStream_t stream = nullptr;

    // device arrays (bin-sorted order)
    double *x = nullptr, *v = nullptr, *f = nullptr, *x0 = nullptr, *s = nullptr;
    uint8_t* elem = nullptr;
    int* id = nullptr;   // sorted -> caller index
    int* inv = nullptr;  // caller -> sorted index
    float4* p32 = nullptr;
    float4* q32 = nullptr;
    float4* p0 = nullptr;  // p32 at the last build (mixed skin test)
    float* f32 = nullptr;
    float* v32 = nullptr;
    float* rho32 = nullptr;
    unsigned* cutmask = nullptr;  // mixed: 32 words per atom (any lanes-per-atom choice)
    // mixed force pass with the force records in shared memory (k_force32s):
    // force_smem is its budget in KB (0: the L1 kernel k_force32; set by the
    // autotuner); fs_tab is built on first use for the fs_w knots (from knot
    // fs_mlo) of fs_rec records per element group that the largest budget
    // holds
    int force_smem = 0;
    int smem_optin = 0;  // shared memory a block may opt in to
    float4* fs_tab = nullptr;
    int fs_rec = 0, fs_w = 0, fs_mlo = 0;
    int* grp_atoms = nullptr;
    int grp_begin[mappg::kMaxElem + 1] = {0};
    int* binc = nullptr;
    int* binid = nullptr;
    int* bin_count = nullptr;
    int* bin_start = nullptr;
    int* bin_atoms = nullptr;
    int maxnbr = 0;
    int* nbr = nullptr;
    int* nnbr = nullptr;
    double *rho = nullptr, *dF = nullptr;
    double* partials = nullptr;
    mappg::DevScalars* sc = nullptr;
    double* stage = nullptr;      // device staging, 3n doubles (caller order)
    double* thermo_dev = nullptr; // per-step thermo rows of an NVT run
    long long thermo_cap = 0;

    // batch of independent cells (ncell > 1); a single cell leaves these empty
    int ncell = 1;
    std::vector<mappg::CellGeo> cells;   // host copy
    std::vector<int> cell_begin;         // ncell + 1 atom offsets
    std::vector<int> chunk_begin_h;      // nchunk + 1
    std::vector<int> cell_chunk_h;       // ncell + 1 chunk offsets
    std::vector<int> cells_chunk_cell_h; // cell of each chunk
    int nchunk = 0;
    int chunk_atoms = mappg::kChunk;     // atoms per chunk (batch autotuner: 128, 256, 512)
    mappg::CellGeo* cells_dev = nullptr;
    int* cell_of = nullptr;              // per atom
    int* chunk_begin = nullptr;
    int* chunk_cell = nullptr;
    int* cell_chunk = nullptr;           // ncell + 1
    double* chunk_part = nullptr;
    uint8_t* cell_active = nullptr;      // batch minimizer in progress: cells still working (null: all)
    // batch: per cell, set when one of its atoms moved more than skin/2 since
    // the cell's last build (or a full build was requested); the rebuild
    // chain rebuilds only these cells and clears their flags
    uint8_t* cell_reb = nullptr;
    double* chunk_disp = nullptr;        // nchunk x 4 (integrator displacement sums)
    mappg::CellMd* cmd = nullptr;        // per-cell MD state
    double* cell_out = nullptr;          // ncell x 8 (pe, virial6, spare) staging

    void* run = nullptr;  // an NVT run in progress (md.cu)
    bool built = false;
    bool list_box = false;  // a neighbour list exists for the current box (skin test may reuse it)
    bool have_v = false;
    bool f_is_f32 = false;  // the newest forces are in f32 (mixed kernels)
    bool force64 = false;   // mixed system computing FP64 forces (end of a relaxation)
    // mixed minimizer in progress: the density pass keeps the FP64 density
    // (rho) and h32 holds the search direction for energy differences
    bool keep_rho64 = false;
    float4* h32 = nullptr;
    // learned preconditioner in progress: recompute its diagonal from the
    // current configuration every precond_every iterations (0: never)
    std::function<void()> precond_refresh;
    int precond_every = 0;
    // called by the minimizers after every hook_every-th iteration's force
    // call (mappg_sys_set_hook)
    int (*hook)(void* user, long long iteration) = nullptr;
    void* hook_user = nullptr;
    int hook_every = 0;
    std::vector<int> host_id;  // sorted -> caller (host copy)
    // atoms.x_dof: bit c of dof[i] set when component c of atom i (bin
    // order) is a degree of freedom; null when every component is
    uint8_t* dof = nullptr;
    int dof_frozen[3] = {0, 0, 0};  // atoms frozen per component
    bool cells_ortho = false;       // batch: every cell's box orthorhombic
    // second stream for an upload that runs under other work (nvt_run_host),
    // its staging array, and the events that order it with s->stream
    cudaStream_t side = nullptr;
    double* stage2 = nullptr;
    cudaEvent_t ev_main = nullptr, ev_side = nullptr;
    bool v_pending = false;  // s->v is being written on `side` until ev_side
};

namespace mappg {

// system.cu
void sys_set_box(mappg_sys* s, const double* H);
void sys_set_cells(mappg_sys* s, int ncell, const int* natoms, const double* H);  // a batch
void sys_rechunk(mappg_sys* s, int chunk_atoms);  // a batch's chunks of at most chunk_atoms atoms
void launch_rebuild_chain(mappg_sys* s);   // kernels gated by sc->rebuild
void request_rebuild(mappg_sys* s);        // host sets the gate
void launch_shadow(mappg_sys* s, bool gated);
void check_build(mappg_sys* s);            // host: overflow / capacity
void launch_skin_test(mappg_sys* s);       // sets sc->rebuild if needed
void sync_forces64(mappg_sys* s);          // f (FP64) from f32 when needed
EamArgs eam_args(mappg_sys* s);
int grid_for(mappg_sys* s, long long threads, int block);

// eam.cu (FP64 kernels; dispatches to eam32.cu in mixed mode)
void launch_force(mappg_sys* s);           // density+embed, force; totals in sc
void launch_energy(mappg_sys* s);          // energy only; total in sc->energy
void launch_density_only(mappg_sys* s);    // the density kernel alone (timing)
void launch_force_only(mappg_sys* s);      // the force kernel alone (timing; needs dF)

// eam32.cu (mixed kernels)
void launch_density32(mappg_sys* s, const EamArgs& a);
void launch_force32(mappg_sys* s, const EamArgs& a);
void launch_energy32(mappg_sys* s, const EamArgs& a);
bool force_smem_available(mappg_sys* s);   // builds the k_force32s records on first use
int force_smem_max_kb(const mappg_sys* s); // the largest shared-memory budget of k_force32s

}  // namespace mappg
