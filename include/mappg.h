/*
 * mappg.h -- C ABI of libmappg, the GB300 (sm_103a) EAM molecular-dynamics
 * and minimization engine.  It replaces the force-field and driver path of
 * MAPP (sinamoeini/mapp4py): ForceFieldEAM behind the ForceFieldMD contract,
 * its neighbour list, the NVT (Nose-Hoover chain) integrator and the L-BFGS
 * minimizer with back-tracking line search.
 *
 * Conventions
 *   - Every call returns 0 on success and a negative status on failure;
 *     mappg_last_error() returns the message of the last failure on the
 *     calling thread.  No C++ exception crosses this boundary.
 *   - Units are MAPP's: Angstrom, eV, amu; time in A*sqrt(amu/eV).
 *   - Boxes are 3x3 row-major, lower triangular, rows are the cell vectors
 *     (x = s*H with s the fractional coordinate), as Atoms::H.
 *   - Per-atom arrays are row-major [natoms][3] doubles in the caller's atom
 *     order; element indices are unsigned char as MAPP's elem_type.
 *   - Virial arrays are Voigt ordered (xx, xy, xz, yy, yz, zz) and hold
 *     F_H = sum over pairs of fpair*dx(x)dx, the quantity ForceFieldMD keeps
 *     in F_H (ff_md.cpp:125-144); the stress is S_pe = -F_H/volume.
 *   - One handle is used by one host thread at a time.  Each system owns
 *     its device buffers and one CUDA stream.
 */
#ifndef MAPPG_H
#define MAPPG_H

#ifdef __cplusplus
extern "C" {
#endif

#define MAPPG_OK 0
#define MAPPG_ERR_ARG -1      /* invalid argument                          */
#define MAPPG_ERR_CUDA -2     /* CUDA runtime failure                      */
#define MAPPG_ERR_FILE -3     /* potential file missing or malformed       */
#define MAPPG_ERR_GEOM -4     /* box too thin for cutoff + skin            */
#define MAPPG_ERR_NBR -5      /* neighbour capacity exceeded               */
#define MAPPG_ERR_NAN -6      /* non-finite position, force or energy      */
#define MAPPG_ERR_TIMEOUT -7  /* a bounded device wait gave up             */
#define MAPPG_ERR_UNSUPP -8   /* feature outside this engine's scope       */

#define MAPPG_LS_BT 0      /* back-tracking (ls_bt)            */
#define MAPPG_LS_GOLDEN 1  /* golden section (ls_golden)       */
#define MAPPG_LS_BRENT 2   /* Brent's method (ls_brent)        */

#define MAPPG_FP64 0  /* FP64 everywhere (the reference's arithmetic)       */
#define MAPPG_MIXED 1 /* FP32 pair math, FP64 state and global reductions   */

typedef struct mappg_ff mappg_ff;
typedef struct mappg_sys mappg_sys;

/* Message of the last failed call on this thread ("" if none). */
const char* mappg_last_error(void);

/* Device name and SM count of the current CUDA device. */
int mappg_device_info(char* name, int name_len, int* sm_count);

/* The current GPU's FP64 fused multiply-add rate in TFLOP/s (2 flops per
 * FMA), measured with a kernel of independent FMA chains and no memory
 * traffic: the arithmetic roof of the FP64 path (its kernels are bounded by
 * FP64 issue, not HBM).  No counterpart in the reference.  iters: FMA
 * iterations per thread per launch; reps: timed launches (best counts). */
int mappg_fp64_fma_rate(int iters, int reps, double* tflops);

/* ---------------------------------------------------------------- tables */

/* Read a DYNAMO setfl file.  Replaces ImportEAM::setfl (import_eam.h:348-613)
 * called by the Python constructor ff_eam_setfl (ff_eam.cpp:668-698).
 * nelems/elems select and order elements as the reference's optional element
 * list does; nelems = 0 keeps the file's order.  Splines are built as
 * ImportEAM::interpolate (import_eam.cpp:62-83) and the cutoff as
 * set_cuttoff (import_eam.h:52-64). */
int mappg_ff_setfl(const char* path, int nelems, const char* const* elems, mappg_ff** out);

/* Read a Finnis-Sinclair (eam/fs) file.  Replaces ImportEAM::fs
 * (import_eam.h:617-901) behind ff_eam_fs (ff_eam.cpp:700-801). */
int mappg_ff_fs(const char* path, int nelems, const char* const* elems, mappg_ff** out);

/* Read one DYNAMO funcfl file per element.  Replaces ImportEAM::funcfl
 * (import_eam.h:68-346) behind ff_eam_funcfl (ff_eam.cpp:594-666). */
int mappg_ff_funcfl(int nfiles, const char* const* paths, mappg_ff** out);

/* Tables from raw knot values (no file): F [nelem][nrho], rho
 * [nelem][nelem][nr] with rho[i][j] the reference's rho_arr[i][j], rphi
 * [nelem][nelem][nr] (only i >= j is read).  Same spline and cutoff rules as
 * mappg_ff_setfl. */
int mappg_ff_from_knots(int nelem, int nr, int nrho, double dr, double drho, const double* F,
                        const double* rho, const double* rphi, mappg_ff** out);

/* Table dimensions. */
int mappg_ff_info(const mappg_ff* ff, int* nelem, int* nr, int* nrho, double* dr, double* drho);

/* Host copies of the spline coefficients ([..][4] each, NULL to skip) and
 * of the derived cutoffs [nelem][nelem]. */
int mappg_ff_tables(const mappg_ff* ff, double* F, double* rho, double* rphi, double* cut);

/* Element name i (as read from the file, "" for knot tables). */
int mappg_ff_element_name(const mappg_ff* ff, int i, char* buf, int len);

void mappg_ff_destroy(mappg_ff* ff);

/* ---------------------------------------------------------------- system */

/* One periodic cell resident on the GPU.  Replaces the AtomsMD state that
 * ForceFieldEAM, NeighborMD and DynamicMD work on (atoms.h:462-580,
 * atoms_md.h:6-60).  masses has one entry per element.  skin is the
 * neighbour skin (Atoms skin, default 0.5).  precision is MAPPG_FP64 or
 * MAPPG_MIXED. */
int mappg_sys_create(const mappg_ff* ff, int natoms, const double* H, const double* x,
                     const unsigned char* elem, const double* masses, double skin, int precision,
                     mappg_sys** out);
void mappg_sys_destroy(mappg_sys* sys);

int mappg_sys_natoms(const mappg_sys* sys);
int mappg_sys_set_x(mappg_sys* sys, const double* x);
int mappg_sys_get_x(mappg_sys* sys, double* x);
int mappg_sys_set_v(mappg_sys* sys, const double* v);
int mappg_sys_get_v(mappg_sys* sys, double* v);
int mappg_sys_get_f(mappg_sys* sys, double* f);
int mappg_sys_set_box(mappg_sys* sys, const double* H);

/* Wrap positions into the cell, bin them and build the full neighbour list
 * within cut+skin.  Replaces DynamicMD::init's x2s_lcl / Update::list /
 * NeighborMD::create_list (dynamic_md.cpp:34-53, neighbor_md.cpp:82-152);
 * ghosts are replaced by periodic image shifts stored with each entry. */
int mappg_sys_build(mappg_sys* sys);

/* Skin test and rebuild when any atom moved more than skin/2 since the last
 * build (DynamicMD::decide/update_w_x, dynamic_md.cpp:90-105,
 * dynamic_md.h:37-68).  *rebuilt (may be NULL) tells which happened. */
int mappg_sys_update(mappg_sys* sys, int* rebuilt);

/* Forces, energy and virial (ForceFieldMD::force_calc / derivative,
 * ff_md.cpp:125-179 over ForceFieldEAM::__force_calc, ff_eam.cpp:65-240).
 * Builds the neighbour list first if none exists.  Forces stay on the device
 * (read them with mappg_sys_get_f).  pe, virial6 may be NULL. */
int mappg_sys_force(mappg_sys* sys, double* pe, double* virial6);

/* Energy only (ForceFieldMD::value, ff_md.cpp:148-155 over
 * ForceFieldEAM::__energy_calc, ff_eam.cpp:244-318). */
int mappg_sys_energy(mappg_sys* sys, double* pe);

/* Forces, energy and virial of an FP64 system, computed without allocating
 * any device memory: for callers whose memory pool owns the device, or that
 * must not let a library call cudaMalloc/cudaFree (which synchronise the
 * device) once they are running.  No counterpart in the reference.
 * f_dev: 3*natoms doubles of device memory, written as x, y, z per atom in
 * the caller's order; ev_dev: NULL or 7 doubles of device memory, written as
 * [pe, virial xx, xy, xz, yy, yz, zz].  The work is queued on the system's
 * stream and the call returns without waiting (mappg_sys_sync waits).
 * The system must be FP64, hold a neighbour list (mappg_sys_build or
 * mappg_sys_update) and have at most 262144 atoms; other calls are refused
 * with MAPPG_ERR_ARG.  Intermediate arrays live in one fixed device array of
 * about 11 MB (10.5 MiB) that every GPU using this call holds until the process
 * exits; the first call on each device looks up that array's address and
 * loads the kernels, so make it before any stream capture.  Calls share the
 * array: calls that overlap on the GPU race and must be serialised.  The
 * call runs on the system's device, which must be the calling thread's
 * current device (checked on every call).  Because it returns before the
 * work completes, it makes no finiteness check (mappg_sys_force returns
 * MAPPG_ERR_NAN for a non-finite energy): check ev_dev[0] after waiting. */
int mappg_sys_force_noalloc(mappg_sys* sys, double* f_dev, double* ev_dev);

/* Per-atom host density rho and F'(rho) from the last force call. */
int mappg_sys_get_rho(mappg_sys* sys, double* rho, double* dF);

/* The current full neighbour list in the caller's atom order: counts[i]
 * entries for atom i, each written as 4 ints (neighbour atom, image shift
 * n0, n1, n2) so that the neighbour sits at x_j + n*H.  Pass entries = NULL
 * to get *total only. */
int mappg_sys_neighbors(mappg_sys* sys, int* counts, int* entries, long long* total);

/* Counters: [0] rebuilds, [1] neighbour capacity per atom, [2] max list
 * length, [3] mean list length*1000, [4] bins, [5] precision. */
int mappg_sys_stats(mappg_sys* sys, long long* out6);

/* Gaussian velocities sqrt(kB*T/m) per component (AtomsMD::create_T,
 * atoms_md.cpp:130-162) from the Park-Miller generator and polar Box-Muller
 * of Random (random.cpp:32-68), seeded with seed.  Seed 0, on which the
 * reference's generator never returns, is rejected.  v is [natoms][3]. */
int mappg_create_temp(int natoms, const unsigned char* elem, const double* masses, double T, double kB, int seed,
                      double* v);

/* create_temp with atoms.x_dof (AtomsMD::create_T, atoms_md.cpp:138-149):
 * dof is [natoms][3], nonzero where the component is a degree of freedom;
 * only those components draw a sample (in order), the others keep the value
 * v holds.  dof NULL: as mappg_create_temp. */
int mappg_create_temp_dof(int natoms, const unsigned char* elem, const double* masses, const unsigned char* dof,
                          double T, double kB, int seed, double* v);

/* atoms.x_dof: per atom and component (caller order, [natoms][3]), nonzero
 * where it is a degree of freedom; NULL (or all nonzero) clears it.  Forces
 * on frozen components are zero in every force call (ForceFieldMD::
 * force_calc, ff_md.cpp:138-144), so the minimizers leave them in place.
 * NVT runs take the reference's _w_dof steps (md_nvt.cpp:144-215): a
 * frozen component is neither kicked nor thermostatted and keeps drifting
 * with its velocity, leaves the degrees of freedom and the kinetic tensor,
 * and the mean displacement is not removed along a component in which any
 * atom is frozen; mixed-precision MD takes the same branches in its FP32
 * kernels.  md.nst takes MDNST's handling (md_nst.cpp:259-279,374-476):
 * frozen components leave the degrees of freedom and carry no force, and a
 * stress along a direction in which an atom is frozen is refused.  Batches
 * refuse a mask. */
int mappg_sys_set_dof(mappg_sys* sys, const unsigned char* dof);

/* ---------------------------------------------------------------- drivers */

/* md.nvt(T,dt).run(atoms,nsteps): velocity Verlet with the Nose-Hoover
 * chain of ThermostatNHC (MDNVT::run, md_nvt.cpp:383-480,
 * thermostat.cpp:47-143), including the lazy velocity rescale and the
 * centre-of-mass displacement removal.  NVE is t_relax = +inf.  eta (L
 * doubles, may be NULL) carries the chain state in and out.  thermo (may be
 * NULL) receives nsteps+1 rows of 14 doubles: pe, T, mvv[6] (xx,xy,xz,yy,yz,
 * zz), virial[6].  Velocities must have been set. */
int mappg_nvt_run(mappg_sys* sys, double T, double dt, double kB, double t_relax, int L,
                  int niters, int nsteps, double* eta, double* thermo);

/* MDNVT::run with the atoms' host arrays (md_nvt.cpp:383-480): x_in and
 * v_in ([natoms][3], caller order) are uploaded, the run goes as
 * mappg_nvt_run, and the final positions, velocities and forces are written
 * to x_out, v_out, f_out (each may be NULL, and may be the input array).
 * The velocity upload overlaps the list check and the opening force call;
 * the downloads are queued together and the call returns once they are
 * done.  Pinned host memory makes the copies asynchronous.  Single cells. */
int mappg_nvt_run_host(mappg_sys* sys, const double* x_in, const double* v_in, double T, double dt, double kB,
                       double t_relax, int L, int niters, int nsteps, double* eta, double* thermo, double* x_out,
                       double* v_out, double* f_out);

/* The same run in three parts, for callers that time or interleave the
 * steps: mappg_nvt_begin does MDNVT::init and the opening force call (a
 * neighbour build, then the step is captured as a CUDA graph) for a run of
 * nsteps steps; mappg_nvt_steps enqueues steps on the system's stream
 * without waiting; mappg_nvt_end waits, applies the pending velocity scale,
 * returns eta and (if record_thermo was set) the thermo rows, and checks the
 * run's error flags. */
int mappg_nvt_begin(mappg_sys* sys, double T, double dt, double kB, double t_relax, int L, int niters,
                    long long nsteps, const double* eta, int record_thermo);
int mappg_nvt_steps(mappg_sys* sys, long long nsteps);
int mappg_nvt_end(mappg_sys* sys, double* eta, double* thermo);

/* md.nst(S,T,dt).run(atoms,nsteps): constant-stress MD (MDNST::run,
 * md_nst.cpp:374-450; update_V_H 315-341; update_x_d__x__x_d 70-145;
 * MDMath::calc 887-1000; pre_init 281-311).  S: 9 doubles, row-major, the
 * lower triangle read, NaN where the box entry has no degree of freedom;
 * tau: 9 relaxation times of the box (the reference's default 1000 dt).
 * The particle chain (t_relax, L, niters) is md.nvt's; the box chain
 * (t_relax_S, L_S, niters_S) is thermo_baro (default 1000 dt, 3, 1).
 * nreset > 0 renews the reference box every nreset steps.  Carried between
 * runs (in/out): V_H (9, the box velocity), eta (L), eta_S (L_S).  thermo
 * (NULL to skip): (nsteps+1) rows of 23 doubles: pe, T, mvv (6), F_H (6),
 * H (9).  The box moves every step and the neighbour list is rebuilt for it
 * each step; mixed-precision systems take the FP32 force passes.  Positions,
 * velocities and the box are read back with mappg_sys_get_x/get_v/get_box. */
int mappg_nst_run(mappg_sys* sys, const double* S, const double* tau, double T, double dt, double kB, double t_relax,
                  int L, int niters, double t_relax_S, int L_S, int niters_S, int nreset, int nsteps, double* V_H,
                  double* eta, double* eta_S, double* thermo);

/* Positions and velocities ([natoms][3] in the caller's order; either may
 * be NULL) of a begun run after the steps enqueued so far, as MDNVT::run
 * holds them when it writes its export (md_nvt.cpp:390,436,470): after the
 * closing kick, before the deferred thermostat scale.  Waits for the steps;
 * the run continues unchanged.  Single-cell systems only. */
int mappg_nvt_snapshot(mappg_sys* sys, double* x, double* x_d);

/* The system's CUDA stream (a cudaStream_t) and a wait on it. */
int mappg_sys_stream(mappg_sys* sys, void** stream);
int mappg_sys_sync(mappg_sys* sys);

/* Choose the lanes per atom (4, 8 or 16; 256/lanes atoms per block) and the
 * neighbour entries per loop step (1 or 2, mixed kernels) of the density and
 * force kernels by timing them on this system's atoms and neighbour list;
 * the two passes share the lanes per atom and each takes its own entries per
 * step; the choice is kept for the system.  tpa, unroll (may be NULL)
 * receive it (unroll: the density pass's), ms (7 doubles, may be NULL) the
 * density+force time of each candidate
 * (4,1) (8,1) (16,1) (4,2) (8,2) (16,2) (32,1); FP64 systems try the
 * one-entry forms only (the others stay 0).  Single mixed cells also time
 * each candidate with both force-record sources (mappg_sys_force_tables);
 * ms then holds the faster.  No counterpart in the reference. */
int mappg_sys_autotune(mappg_sys* sys, int* tpa, int* unroll, double* ms);

/* The kernel shape in use (set by mappg_sys_autotune / mappg_batch_autotune):
 * out[0] lanes per atom, out[1] entries per loop step of the density pass,
 * out[2] of the force pass, out[3] the force pass's shared-memory budget in
 * KB (mappg_sys_force_tables), out[4] atoms per chunk of a batch (0 for one
 * cell).  No counterpart in the reference. */
int mappg_sys_tuning(mappg_sys* sys, int* out);

/* The mixed force pass's record source: mode 0 reads the force records
 * through L1 (k_force32); mode k > 0 copies the records of one element group
 * at a time into k KB of shared memory (k_force32s; single cells of mixed
 * precision; the knots nearest the cutoff that fit, clamped to the largest
 * budget a block may opt in to; nearer pairs read global memory); mode -1
 * only queries.  *active receives the mode in use.  mappg_sys_autotune
 * times 0, 64 KB, 128 KB and the largest budget and keeps the fastest; the
 * forces are the same in every mode.  No counterpart in the reference. */
int mappg_sys_force_tables(mappg_sys* sys, int mode, int* active);

/* A batch of cells (mappg_batch_create): the atoms per chunk (128, 256 or
 * 512: the atoms a block of the batch kernels works through before it takes
 * another chunk) together with mappg_sys_autotune's lanes per atom and
 * entries per loop step, each of the 21 candidates timed on the batch's own
 * cells and neighbour lists; the fastest is kept.  No counterpart in the
 * reference (it runs one cell).  ms_out: NULL or 21 doubles, chunk-major. */
int mappg_batch_autotune(mappg_sys* sys, int* tpa, int* unroll, int* chunk_atoms, double* ms_out);

/* Enqueue one kernel launch on the system's stream without waiting, for
 * timing: 0 density + embedding, 1 force/virial (uses the last F'(rho)),
 * 2 energy only, 3 neighbour rebuild. */
int mappg_sys_enqueue(mappg_sys* sys, int what);

/* The energy change E(x + alpha h) - E(x) of a mixed-precision system, as
 * the line searches of its minimizers take it: formed pair by pair from the
 * displacement change (an FP32 difference of two FP32 energies would carry
 * rounding of the size of the decreases near convergence), the embedding
 * change in FP64.  No counterpart in the reference, whose line searches
 * compare FP64 energies (MinMDHandler::F, min_cg.h:260-267).  h is
 * [natoms][3] in the caller's order; atoms do not move.  Refused when
 * alpha*h would take an atom beyond half the neighbour list's skin. */
int mappg_sys_energy_delta(mappg_sys* sys, const double* h, double alpha, double* de);

/* md.min_lbfgs(m,e_tol,max_dx,ls=ls_bt(c,rho,min_alpha)).run(atoms,nsteps)
 * (MinLBFGS::__run, min_l-bfgs.h:113-219; LineSearchBackTrack::min,
 * ls.h:711-769) with an added stop at max|F| < f_tol (f_tol <= 0 disables
 * it).  stats (6 doubles): iterations, pe, max|F|, stop code, energy calls,
 * force calls.  Stop codes follow ls.h:9-22 (4 = energy tolerance, 5 = max
 * iterations) plus 100 = force tolerance. */
int mappg_lbfgs_run(mappg_sys* sys, int m, double e_tol, double max_dx, double f_tol, double c,
                    double rho, double min_alpha, int nsteps, double* stats);

/* md.min_cg(e_tol,max_dx,ls=ls_bt(c,rho,min_alpha)).run(atoms,nsteps):
 * Polak-Ribiere conjugate gradients (MinCG::__run, min_cg.h:454-536) over
 * the back-tracking line search with the previous-step cap (init_flag 1,
 * ls.h:711-769), with an added stop at max|F| < f_tol (f_tol <= 0 disables
 * it).  stats as mappg_lbfgs_run. */
int mappg_cg_run(mappg_sys* sys, double e_tol, double max_dx, double f_tol, double c, double rho,
                 double min_alpha, int nsteps, double* stats);

/* Line search of a minimizer (mapp4py.ls_bt / ls_golden / ls_brent,
 * ls.cpp:95-100,262-268,456-461 for the defaults): kind is MAPPG_LS_*; c,
 * rho, min_alpha are the back-tracking's (0.4, 0.5, 0); tol (sqrt(2 eps)),
 * max_iter (5), bracket (1) and zeps (1e-3 eps, Brent only) the others'. */
typedef struct mappg_ls {
    int kind;
    double c, rho, min_alpha;
    double tol;
    int max_iter;
    int bracket;
    double zeps;
} mappg_ls;

/* mappg_lbfgs_run and mappg_cg_run with any of the three line searches
 * (LineSearchGoldenSection::min ls.h:340-515, LineSearchBrent::min
 * ls.h:524-706, both after LineSearch::bracket ls.h:214-335 unless
 * bracket = 0; back-tracking as mappg_lbfgs_run).  Stop codes add
 * 8 = the bracketing found no lower energy (B_F_DOWNHILL). */
int mappg_lbfgs_run_ls(mappg_sys* sys, int m, double e_tol, double max_dx, double f_tol, const mappg_ls* ls,
                       int nsteps, double* stats);
int mappg_cg_run_ls(mappg_sys* sys, double e_tol, double max_dx, double f_tol, const mappg_ls* ls, int nsteps,
                    double* stats);

/* md.min_lbfgs / md.min_cg with box degrees of freedom (MinLBFGS::__run
 * min_l-bfgs.h:113-219, MinCG::__run min_cg.h:454-536, with MinMDHandler
 * min_cg.h:89-331 for BC = true or X = false).  method 0 is L-BFGS with m
 * history pairs, 1 conjugate gradients.  H_dof: 9 ints, row-major; the
 * lower triangle says which entries of the box may relax (as the Python
 * H_dof).  affine != 0 moves the atoms only with the box.  Each vector of
 * the method carries a box part, the lower triangle of a 3x3 tensor, whose
 * force is F_H masked by H_dof; a direction h moves the atoms along
 * h + x0 h.A and the box along H0 h.A, and every line-search trial rebuilds
 * the neighbour list for its box.  Stops as the reference's (energy
 * tolerance, iterations, line-search failures; no force tolerance).  stats
 * as mappg_lbfgs_run; the relaxed box is read with mappg_sys_get_box. */
int mappg_min_box_run(mappg_sys* sys, int method, int m, double e_tol, double max_dx, const int* H_dof, int affine,
                      const mappg_ls* ls, int nsteps, double* stats);

/* The system's box (9 doubles, rows are the cell vectors; Atoms::H). */
int mappg_sys_get_box(mappg_sys* sys, double* H);

/* A function that mappg_lbfgs_run, mappg_lbfgs_run_precond and mappg_cg_run
 * call after every nevery-th iteration's force call, with the number of
 * iterations done; the system's positions and forces are then that
 * iteration's and may be read from it (mappg_sys_get_x/get_f).  This is
 * where the reference writes its periodic export (ExportHandler::print,
 * min.h:216-220).  mappg_nst_run calls it after every nevery-th step and
 * after its last step, with positions, velocities (before the run's final
 * velocity scale), forces and box of that step (MDNST::run's exports).  A
 * non-zero return stops the run with MAPPG_ERR_ARG.  hook NULL or
 * nevery <= 0 removes it. */
int mappg_sys_set_hook(mappg_sys* sys, int (*hook)(void* user, long long iteration), void* user, int nevery);

/* The exchange-energy hooks of ForceFieldMD that grand-canonical Monte Carlo
 * (GCMC) calls (init_xchng / fin_xchng / pre_xchng_energy / xchng_energy /
 * post_xchng_energy, ff_md.h:19-21,49-50).  GCMC is outside this engine:
 * each returns MAPPG_ERR_UNSUPP with a message, whatever its arguments
 * (gcmc stands for the caller's GCMC object and is not read). */
int mappg_sys_init_xchng(mappg_sys* sys);
int mappg_sys_fin_xchng(mappg_sys* sys);
int mappg_sys_pre_xchng_energy(mappg_sys* sys, void* gcmc);
int mappg_sys_xchng_energy(mappg_sys* sys, void* gcmc, double* de);
int mappg_sys_post_xchng_energy(mappg_sys* sys, void* gcmc);

/* --------------------------------------------------------- CFG snapshots */

typedef struct mappg_cfg mappg_cfg;

/* Read an AtomEye CFG file, standard or extended, as md.atoms.import_cfg
 * (ImportCFGMD::operator(), import_cfg.cpp:496-595; header rules
 * read_header 32-191; bodies read_body_ext 196-372 and read_body_std
 * 377-478; Python entry 597-652).  The box is (H0 Transform) times
 * sqrt(1 + 2 eta) when eta is given, made lower triangular (same row
 * lengths and angles) and scaled by A; x = s H with s wrapped into [0,1);
 * velocities, when the file has them, are x_d = s_d R H.  Elements are
 * numbered in order of first appearance; a repeated name keeps its first
 * mass.  Failures are MAPPG_ERR_FILE with the reference's messages. */
int mappg_cfg_read(const char* path, mappg_cfg** out);
/* Atom and element counts, whether velocities were read, the box (9). */
int mappg_cfg_info(const mappg_cfg* cfg, int* natoms, int* nelem, int* has_vel, double* H);
/* Mass and name of element i (name_len bytes including the terminator). */
int mappg_cfg_element(const mappg_cfg* cfg, int i, double* mass, char* name, int name_len);
/* Positions, velocities (NULL to skip) [natoms][3] and elements in file order. */
int mappg_cfg_atoms(const mappg_cfg* cfg, double* x, double* x_d, unsigned char* elem);
int mappg_cfg_destroy(mappg_cfg* cfg);

/* Write an extended CFG file as ExportCFGMD::write (export_cfg_md.cpp:26-113,
 * 167-193): A = 1, H0 = H (lower triangular), s = x H^-1 wrapped into
 * [0,1), a mass and name line whenever the element changes along the atom
 * order, then per atom s and the extra vectors (vec_dims[k] doubles each,
 * [natoms][dim]) in the given order, all as "%.16lf ".  An extra vector
 * named "x_d" is written as s_d = x_d H^-1 and the header then says
 * "R = 1.0" instead of ".NO_VELOCITY."; the others are listed as
 * auxiliary[k] = name_d. */
int mappg_cfg_write(const char* path, int natoms, const double* H, const double* x, const unsigned char* elem,
                    int nelem, const double* masses, const char* const* names, int nvec,
                    const char* const* vec_names, const int* vec_dims, const double* const* vecs);

/* ------------------------------------------------------- batches of cells */

/* Several independent periodic cells (ncell >= 2) in one system, for runs
 * over many small cells: every kernel of a step covers all cells at once.
 * The reference runs one cell per process (its drivers take one Atoms); a
 * batch is the same per-cell computation as mappg_sys_create's, cell by
 * cell.  natoms[c] atoms per cell, H is ncell boxes of 9 doubles, x and
 * elem hold the cells' atoms one cell after the other.  Mixed precision
 * only.  The per-atom calls (set/get x, v, f, build, update, neighbours)
 * work on the concatenated atoms; energies and MD state are per cell. */
int mappg_batch_create(const mappg_ff* ff, int ncell, const int* natoms, const double* H, const double* x,
                       const unsigned char* elem, const double* masses, double skin, int precision,
                       mappg_sys** out);
int mappg_batch_ncell(const mappg_sys* sys);

/* Per-cell energy (pe[ncell]) and virial (virial[ncell][6], may be NULL)
 * after a force pass over all cells; forces via mappg_sys_get_f. */
int mappg_batch_force(mappg_sys* sys, double* pe, double* virial);
int mappg_batch_energy(mappg_sys* sys, double* pe);

/* md.nvt run of every cell at its own temperature T[c] (MDNVT::run,
 * md_nvt.cpp:383-480, one chain per cell), one CUDA graph per step over all
 * cells.  eta: ncell x L doubles in/out (may be NULL); thermo: NULL or
 * (nsteps+1) x ncell x 2 doubles (pe, T per cell per step).  begin/end as
 * mappg_nvt_begin/end; mappg_nvt_steps enqueues steps of either. */
int mappg_batch_nvt_begin(mappg_sys* sys, const double* T, double dt, double kB, double t_relax, int L, int niters,
                          long long nsteps, const double* eta, int record_thermo);
int mappg_batch_nvt_end(mappg_sys* sys, double* eta, double* thermo);
int mappg_batch_nvt_run(mappg_sys* sys, const double* T, double dt, double kB, double t_relax, int L, int niters,
                        int nsteps, double* eta, double* thermo);

/* ------------------------------------------- learned L-BFGS preconditioner */

/* A small network predicts each atom's three diagonal Hessian elements from
 * 33 local features; their inverses replace the scalar initial inverse
 * Hessian of the L-BFGS two-loop recursion.  No counterpart in the
 * reference (MinLBFGS uses gamma*I, min_l-bfgs.h:148-170).
 * Network: 33 -> 64 -> 64 -> 3, tanh hidden units, softplus outputs, BF16
 * tensor-core forward/backward with FP32 accumulation, AdamW on FP32
 * master weights.  Parameters: W1 [64][64] | W2 [64][80] | W3 [16][80]
 * row-major [unit][input] (input 33 of W1 and input 64 of W2/W3 are the
 * biases); norm: 33 feature means then 33 standard deviations. */
typedef struct mappg_mlp mappg_mlp;
int mappg_mlp_nparams(void);
int mappg_mlp_create(int seed, mappg_mlp** out);
void mappg_mlp_destroy(mappg_mlp* net);
/* training rows: feat [n][33], target [n][3] (Hessian diagonals, eV/A^2);
 * sets the feature standardisation from these rows and shuffles them */
int mappg_mlp_set_data(mappg_mlp* net, const float* feat, const float* target, int n, int seed);
/* minibatch AdamW; losses[epochs] (may be NULL) = mean squared log error */
int mappg_mlp_train(mappg_mlp* net, int epochs, int batch, double lr, double wd, double* losses);
/* loss and gradient over the given rows (grad: nparams floats) */
int mappg_mlp_grad(mappg_mlp* net, const float* feat, const float* target, int n, float* grad, double* loss);
int mappg_mlp_predict(mappg_mlp* net, const float* feat, int n, float* out);
int mappg_mlp_get_params(mappg_mlp* net, float* w, float* norm);
int mappg_mlp_set_params(mappg_mlp* net, const float* w, const float* norm);

/* Features of a system's atoms, [natoms][33] in caller order: 16 Gaussian
 * radial functions (centres 2.0..5.5 A, width 0.3 A, cosine cutoff 5.5 A)
 * per neighbour species (A, B), then the host density rho_i. */
int mappg_sys_descriptors(mappg_sys* sys, float* feat);

/* Diagonal Hessian elements [natoms][3] by central differences of the
 * forces with step h; atoms of one colour (color[natoms], caller order)
 * move together, so same-coloured atoms must be further apart than twice
 * the cutoff.  FP64 systems. */
int mappg_sys_hessian_diag(mappg_sys* sys, const int* color, double h, double* out);

/* With a learned preconditioner, recompute its diagonal from the current
 * configuration every `every` L-BFGS iterations (0, the default: once, at
 * the start).  Applies to mappg_lbfgs_run_precond and
 * mappg_batch_lbfgs_run_precond.  No counterpart in the reference. */
int mappg_mlp_set_refresh(mappg_mlp* net, int every);

/* mappg_lbfgs_run with H0 = diag(1/y), y the network's prediction for the
 * starting configuration; a non-descent direction falls back to plain
 * L-BFGS (gamma*I) for that iteration.  stats: 7 doubles, the six of
 * mappg_lbfgs_run then the number of fallbacks. */
int mappg_lbfgs_run_precond(mappg_sys* sys, mappg_mlp* net, int m, double e_tol, double max_dx, double f_tol,
                            double c, double rho, double min_alpha, int nsteps, double* stats);

/* mappg_lbfgs_run (one cell) or mappg_batch_lbfgs_run (a batch) with
 * H0 = diag(1/d), d the caller's Hessian diagonal (n x 3 in the caller's
 * atom order, eV/A^2, every entry positive and finite), scaled each
 * iteration by (s.y)/(y.P.y) of the newest pair as the learned diagonal
 * is; a non-descent direction falls back to plain L-BFGS.  For a diagonal
 * from elsewhere (finite differences, a model of one's own), and the bound
 * the network's prediction is measured against.  stats as
 * mappg_lbfgs_run_precond (a batch: ncell x 7).  No counterpart in the
 * reference. */
int mappg_lbfgs_run_diag(mappg_sys* sys, const double* hdiag, int m, double e_tol, double max_dx, double f_tol,
                         double c, double rho, double min_alpha, int nsteps, double* stats);

/* L-BFGS over a batch of cells: every cell runs mappg_lbfgs_run's
 * iteration with its own history, line search and stopping state; the
 * kernels of each phase cover all cells.  m in 1..32.  stats: ncell x 7
 * doubles (iterations, pe, max|F|, stop code, energy calls, force calls,
 * learned-direction fallbacks). */
int mappg_batch_lbfgs_run(mappg_sys* sys, int m, double e_tol, double max_dx, double f_tol, double c, double rho,
                          double min_alpha, int nsteps, double* stats);
int mappg_batch_lbfgs_run_precond(mappg_sys* sys, mappg_mlp* net, int m, double e_tol, double max_dx,
                                  double f_tol, double c, double rho, double min_alpha, int nsteps, double* stats);

/* ------------------------------------------------------------ diagnostics */

/* D[128][64] = A[128][64] * Bt[64][64]^T through the tensor-core path the
 * learned preconditioner uses (tcgen05 MMA, BF16 operands as raw 16-bit
 * patterns, FP32 result), for checking it against plain arithmetic.  No
 * counterpart in the reference. */
int mappg_tc_gemm_check(const unsigned short* A, const unsigned short* Bt, float* D);

#ifdef __cplusplus
}
#endif
#endif /* MAPPG_H */
