// extern "C" entry points of libmappg (declared in include/mappg.h).
// Every entry point catches all exceptions, records the message for
// mappg_last_error() and returns a negative status.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "linesearch.h"
#include "system.h"

namespace mappg {

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
const char* get_error() { return g_err.c_str(); }

void sys_alloc(mappg_sys* s, const double* x_host);
void sys_alloc_bins(mappg_sys* s);
void sys_alloc_nbr(mappg_sys* s, int maxnbr);
void sys_free(mappg_sys* s);
void sys_upload(mappg_sys* s, const double* host, double* dev);
void sys_download(mappg_sys* s, const double* dev, double* host);
void sys_upload_side(mappg_sys* s, const double* host, double* dev);
void sys_join_side(mappg_sys* s);
void sys_download_async(mappg_sys* s, const double* dev, double* host);
void nvt_run_xout(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, int nsteps,
                  double* eta, double* thermo, double* x_out);
void sys_build(mappg_sys* s);
void sys_neighbors(mappg_sys* s, int* counts, int* entries, long long* total);
void nvt_run(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, int nsteps, double* eta,
             double* thermo, const double* Tcell);
void lbfgs_run(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, const LsParams& ls, int nsteps,
               double* stats, const double* P, long long* n_fallback);
void lb_update(mappg_sys* s);
void nvt_begin(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, long long nsteps,
               const double* eta, bool thermo, const double* Tcell);
void nvt_steps(mappg_sys* s, long long nsteps);
void nvt_end(mappg_sys* s, double* eta, double* thermo);
void nvt_snapshot(mappg_sys* s, double* x, double* v);
void nst_run(mappg_sys* s, const double* S, const double* tau, double T, double dt, double kB, double t_relax, int L,
             int niters, double t_relax_S, int L_S, int niters_S, int nreset, int nsteps, double* V_H, double* eta,
             double* eta_S, double* thermo);
void nvt_free(mappg_sys* s);
void batch_lbfgs_run(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, double c_ls, double rho_ls,
                     double min_alpha, int nsteps, const double* P, double* stats);
void cg_run(mappg_sys* s, double e_tol, double max_dx, double f_tol, const LsParams& ls, int nsteps, double* stats);
void box_min_run(mappg_sys* s, int method, int m, double e_tol, double max_dx, const int* H_dof, bool affine,
                 const LsParams& ls, int nsteps, double* stats);
void launch_density_only(mappg_sys* s);
void launch_force_only(mappg_sys* s);


void upload_tables(mappg_ff* ff) {
    HostTables& t = ff->host;
    DevTables& d = ff->dev;
    const int ne = t.nelem;
    d.nelem = ne;
    d.nr = t.nr;
    d.nrho = t.nrho;
    d.dr_inv = 1.0 / t.dr;
    d.drho_inv = 1.0 / t.drho;
    d.rho_max = (double)t.nrho * t.drho;
    d.max_cut = 0.0;
    for (int i = 0; i < ne * ne; i++) {
        d.cut[i] = t.cut[i];
        d.max_cut = std::max(d.max_cut, t.cut[i]);
    }
    MAPPG_CUDA(cudaGetDevice(&ff->device));
    size_t nrt = (size_t)ne * ne * t.nr, nFt = (size_t)ne * t.nrho;
    auto up64 = [](Dbl4** dst, const std::vector<double>& src, size_t n) {
        MAPPG_CUDA(cudaMalloc(dst, sizeof(Dbl4) * n));
        MAPPG_CUDA(cudaMemcpy(*dst, src.data(), sizeof(Dbl4) * n, cudaMemcpyHostToDevice));
    };
    auto up32 = [](float4** dst, const std::vector<double>& src, size_t n) {
        std::vector<float> f(4 * n);
        for (size_t k = 0; k < 4 * n; k++) f[k] = (float)src[k];
        MAPPG_CUDA(cudaMalloc(dst, sizeof(float4) * n));
        MAPPG_CUDA(cudaMemcpy(*dst, f.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    };
    // setfl and funcfl density functions depend on the neighbour's element
    // only (the reference aliases rho_arr[i][j] to rho_arr[i][0],
    // import_eam.h:499-504); the kernels then read one row per e_j, which
    // halves the density tables' share of the L1 cache for two elements
    d.rho_ei = 0;
    for (int ej = 0; ej < ne && !d.rho_ei; ej++)
        for (int ei = 1; ei < ne; ei++)
            if (memcmp(t.rho_at(ej, ei), t.rho_at(ej, 0), sizeof(double) * 4 * t.nr) != 0) {
                d.rho_ei = 1;
                break;
            }
    up64(&d.rho64, t.rho, nrt);
    up64(&d.rphi64, t.rphi, nrt);
    up64(&d.F64, t.F, nFt);
    up32(&d.rho32, t.rho, nrt);
    up32(&d.F32, t.F, nFt);
    std::vector<float> lo(nFt);
    for (size_t k = 0; k < nFt; k++) lo[k] = (float)(t.F[4 * k] - (double)(float)t.F[4 * k]);
    MAPPG_CUDA(cudaMalloc(&d.F32lo, sizeof(float) * nFt));
    MAPPG_CUDA(cudaMemcpy(d.F32lo, lo.data(), sizeof(float) * nFt, cudaMemcpyHostToDevice));
    // force records of the mixed force kernel: one 32-byte sector per
    // (pair type, knot) holds rho'_{j->i} and r*phi; rho'_{i->j} sits in a
    // second table that only pairs of unlike elements read (for like
    // elements the two derivatives are the same function)
    const double dri = 1.0 / t.dr;
    std::vector<float> rec((size_t)8 * nrt), recj((size_t)4 * nrt);
    for (int ei = 0; ei < ne; ei++)
        for (int ej = 0; ej < ne; ej++)
            for (int m = 0; m < t.nr; m++) {
                const double* ci = t.rho_at(ej, ei) + 4 * (size_t)m;  // density at i from j
                const double* cj = t.rho_at(ei, ej) + 4 * (size_t)m;  // density at j from i
                const double* cz = t.rphi_at(ei, ej) + 4 * (size_t)m;
                const size_t k = (size_t)(ei * ne + ej) * t.nr + m;
                float* r = rec.data() + 8 * k;
                r[0] = (float)(ci[1] * dri);
                r[1] = (float)(2.0 * ci[2] * dri);
                r[2] = (float)(3.0 * ci[3] * dri);
                r[3] = (float)cz[0];
                r[4] = (float)cz[1];
                r[5] = (float)cz[2];
                r[6] = (float)cz[3];
                r[7] = (float)(cz[0] - (double)r[3]);
                float* q = recj.data() + 4 * k;
                q[0] = (float)(cj[1] * dri);
                q[1] = (float)(2.0 * cj[2] * dri);
                q[2] = (float)(3.0 * cj[3] * dri);
                q[3] = 0.f;
            }
    MAPPG_CUDA(cudaMalloc(&d.ftab, sizeof(float) * rec.size()));
    MAPPG_CUDA(cudaMemcpy(d.ftab, rec.data(), sizeof(float) * rec.size(), cudaMemcpyHostToDevice));
    MAPPG_CUDA(cudaMalloc(&d.fjtab, sizeof(float) * recj.size()));
    MAPPG_CUDA(cudaMemcpy(d.fjtab, recj.data(), sizeof(float) * recj.size(), cudaMemcpyHostToDevice));
}

void free_tables(mappg_ff* ff) {
    DevTables& d = ff->dev;
    void* p[] = {d.rho64, d.rphi64, d.F64, d.rho32, d.ftab, d.fjtab, d.F32, d.F32lo};
    for (void* q : p)
        if (q) cudaFree(q);
}

}  // namespace mappg

using namespace mappg;

// tables reach the device when the first system uses them, so the host-side
// readers work (and can be tested) without a GPU
static mappg_ff* finish_ff(mappg_ff* ff) { return ff; }

static void ensure_uploaded(const mappg_ff* cff) {
    mappg_ff* ff = const_cast<mappg_ff*>(cff);
    if (ff->dev.rho64) return;
    try {
        upload_tables(ff);
    } catch (...) {
        free_tables(ff);
        ff->dev = DevTables();
        throw;
    }
}

extern "C" {

const char* mappg_last_error(void) { return get_error(); }

int mappg_device_info(char* name, int name_len, int* sm_count) {
    return guard([&] {
        int dev;
        MAPPG_CUDA(cudaGetDevice(&dev));
        cudaDeviceProp p;
        MAPPG_CUDA(cudaGetDeviceProperties(&p, dev));
        if (name && name_len > 0) {
            strncpy(name, p.name, name_len - 1);
            name[name_len - 1] = 0;
        }
        if (sm_count) *sm_count = p.multiProcessorCount;
    });
}

int mappg_ff_setfl(const char* path, int nelems, const char* const* elems, mappg_ff** out) {
    return guard([&] {
        if (!path || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        mappg_ff* ff = new mappg_ff();
        try {
            read_setfl(path, nelems, elems, ff->host);
        } catch (...) {
            delete ff;
            throw;
        }
        *out = finish_ff(ff);
    });
}

int mappg_ff_fs(const char* path, int nelems, const char* const* elems, mappg_ff** out) {
    return guard([&] {
        if (!path || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        mappg_ff* ff = new mappg_ff();
        try {
            read_fs(path, nelems, elems, ff->host);
        } catch (...) {
            delete ff;
            throw;
        }
        *out = finish_ff(ff);
    });
}

int mappg_ff_funcfl(int nfiles, const char* const* paths, mappg_ff** out) {
    return guard([&] {
        if (!paths || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        mappg_ff* ff = new mappg_ff();
        try {
            read_funcfl(nfiles, paths, ff->host);
        } catch (...) {
            delete ff;
            throw;
        }
        *out = finish_ff(ff);
    });
}

int mappg_ff_from_knots(int nelem, int nr, int nrho, double dr, double drho, const double* F, const double* rho,
                        const double* rphi, mappg_ff** out) {
    return guard([&] {
        if (!F || !rho || !rphi || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (nr < 5 || nrho < 5) throw Error{MAPPG_ERR_ARG, "nr and nrho must be at least 5"};
        if (!(dr > 0.0) || !(drho > 0.0)) throw Error{MAPPG_ERR_ARG, "dr and drho must be positive"};
        mappg_ff* ff = new mappg_ff();
        try {
            HostTables& t = ff->host;
            t.alloc(nelem, nr, nrho, dr, drho);
            t.names.assign(nelem, "");
            for (int i = 0; i < nelem; i++)
                for (int k = 0; k < nrho; k++) t.F_at(i)[4 * k] = F[(size_t)i * nrho + k];
            for (int i = 0; i < nelem; i++)
                for (int j = 0; j < nelem; j++)
                    for (int k = 0; k < nr; k++) t.rho_at(i, j)[4 * k] = rho[((size_t)i * nelem + j) * nr + k];
            for (int i = 0; i < nelem; i++)
                for (int j = 0; j <= i; j++)
                    for (int k = 0; k < nr; k++) t.rphi_at(i, j)[4 * k] = rphi[((size_t)i * nelem + j) * nr + k];
            t.finish_splines(true);
        } catch (...) {
            delete ff;
            throw;
        }
        *out = finish_ff(ff);
    });
}

int mappg_ff_info(const mappg_ff* ff, int* nelem, int* nr, int* nrho, double* dr, double* drho) {
    return guard([&] {
        if (!ff) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (nelem) *nelem = ff->host.nelem;
        if (nr) *nr = ff->host.nr;
        if (nrho) *nrho = ff->host.nrho;
        if (dr) *dr = ff->host.dr;
        if (drho) *drho = ff->host.drho;
    });
}

int mappg_ff_tables(const mappg_ff* ff, double* F, double* rho, double* rphi, double* cut) {
    return guard([&] {
        if (!ff) throw Error{MAPPG_ERR_ARG, "null handle"};
        const HostTables& t = ff->host;
        if (F) memcpy(F, t.F.data(), sizeof(double) * t.F.size());
        if (rho) memcpy(rho, t.rho.data(), sizeof(double) * t.rho.size());
        if (rphi) memcpy(rphi, t.rphi.data(), sizeof(double) * t.rphi.size());
        if (cut) memcpy(cut, t.cut.data(), sizeof(double) * t.cut.size());
    });
}

int mappg_ff_element_name(const mappg_ff* ff, int i, char* buf, int len) {
    return guard([&] {
        if (!ff || !buf || len < 1) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (i < 0 || i >= ff->host.nelem) throw Error{MAPPG_ERR_ARG, "element index out of range"};
        const std::string& nm = i < (int)ff->host.names.size() ? ff->host.names[i] : std::string();
        strncpy(buf, nm.c_str(), len - 1);
        buf[len - 1] = 0;
    });
}

void mappg_ff_destroy(mappg_ff* ff) {
    if (!ff) return;
    free_tables(ff);
    delete ff;
}

int mappg_sys_create(const mappg_ff* ff, int natoms, const double* H, const double* x, const unsigned char* elem,
                     const double* masses, double skin, int precision, mappg_sys** out) {
    return guard([&] {
        if (!ff || !H || !x || !elem || !masses || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (natoms < 1 || natoms > kMaxAtoms)
            throw Error{MAPPG_ERR_ARG, "natoms out of range (1.." + std::to_string(kMaxAtoms) + " per system)"};
        if (precision != MAPPG_FP64 && precision != MAPPG_MIXED) throw Error{MAPPG_ERR_ARG, "unknown precision mode"};
        if (!(skin >= 0.0)) throw Error{MAPPG_ERR_ARG, "skin must be >= 0"};
        const int ne = ff->host.nelem;
        for (int i = 0; i < natoms; i++)
            if (elem[i] >= ne) throw Error{MAPPG_ERR_ARG, "element index beyond the force field's elements"};
        for (int e = 0; e < ne; e++)
            if (!(masses[e] > 0.0)) throw Error{MAPPG_ERR_ARG, "masses must be positive"};
        for (int i = 0; i < 3 * natoms; i++)
            if (!std::isfinite(x[i])) throw Error{MAPPG_ERR_NAN, "non-finite position"};
        ensure_uploaded(ff);
        mappg_sys* s = new mappg_sys();
        try {
            s->ff = ff;
            s->n = natoms;
            s->precision = precision;
            s->ne = ne;
            s->skin = skin;
            for (int e = 0; e < ne; e++) s->masses[e] = masses[e];
            // ForceFieldMD::pre_init (ff_md.cpp:80-94) and max_cut = cut + skin
            double mc = 0.0;
            for (int i = 0; i < ne; i++)
                for (int j = 0; j < ne; j++) {
                    double c = ff->host.cut[i * ne + j];
                    mc = std::max(mc, c);
                    s->cut_sq[i * ne + j] = c * c;
                    double ck = c + skin;
                    s->cut_sk_sq[i * ne + j] = ck * ck;
                }
            s->max_cut = mc + skin;
            MAPPG_CUDA(cudaGetDevice(&s->device));
            cudaDeviceProp p;
            MAPPG_CUDA(cudaGetDeviceProperties(&p, s->device));
            s->sm_count = p.multiProcessorCount;
            s->smem_optin = (int)p.sharedMemPerBlockOptin;
            sys_set_box(s, H);
            sys_alloc(s, x);
            sys_alloc_bins(s);
            // row capacity from the mean density, refined by the first build
            double dens = natoms / s->box.vol;
            double est = dens * 4.18879 * s->max_cut * s->max_cut * s->max_cut;
            int cap = ((int)(est * 1.35) + 32 + 31) / 32 * 32;
            sys_alloc_nbr(s, std::min(cap, 4096));
            sys_upload(s, x, s->x);
            std::vector<uint8_t> es(natoms);
            for (int i = 0; i < natoms; i++) es[i] = elem[s->host_id[i]];
            MAPPG_CUDA(cudaMemcpyAsync(s->elem, es.data(), natoms, cudaMemcpyHostToDevice, s->stream));
            // the atoms of each element in bin order (k_force32s works one
            // element's force records at a time)
            s->grp_begin[0] = 0;
            for (int g = 0; g < ne; g++)
                s->grp_begin[g + 1] = s->grp_begin[g] + (int)std::count(es.begin(), es.end(), (uint8_t)g);
            std::vector<int> grp;
            if (ne > 1) {
                grp.reserve(natoms);
                for (int g = 0; g < ne; g++)
                    for (int i = 0; i < natoms; i++)
                        if (es[i] == g) grp.push_back(i);
                MAPPG_CUDA(cudaMalloc(&s->grp_atoms, sizeof(int) * (size_t)natoms));
                MAPPG_CUDA(cudaMemcpyAsync(s->grp_atoms, grp.data(), sizeof(int) * (size_t)natoms,
                                           cudaMemcpyHostToDevice, s->stream));
            }
            MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        } catch (...) {
            sys_free(s);
            delete s;
            throw;
        }
        *out = s;
    });
}

void mappg_sys_destroy(mappg_sys* s) {
    if (!s) return;
    nvt_free(s);
    sys_free(s);
    delete s;
}

int mappg_sys_natoms(const mappg_sys* s) { return s ? s->n : 0; }

int mappg_sys_set_x(mappg_sys* s, const double* x) {
    return guard([&] {
        if (!s || !x) throw Error{MAPPG_ERR_ARG, "null argument"};
        sys_upload(s, x, s->x);
        s->built = false;
    });
}

int mappg_sys_get_x(mappg_sys* s, double* x) {
    return guard([&] {
        if (!s || !x) throw Error{MAPPG_ERR_ARG, "null argument"};
        sys_download(s, s->x, x);
    });
}

int mappg_sys_set_v(mappg_sys* s, const double* v) {
    return guard([&] {
        if (!s || !v) throw Error{MAPPG_ERR_ARG, "null argument"};
        sys_upload(s, v, s->v);
        s->have_v = true;
    });
}

int mappg_sys_get_v(mappg_sys* s, double* v) {
    return guard([&] {
        if (!s || !v) throw Error{MAPPG_ERR_ARG, "null argument"};
        sys_download(s, s->v, v);
    });
}

int mappg_sys_get_f(mappg_sys* s, double* f) {
    return guard([&] {
        if (!s || !f) throw Error{MAPPG_ERR_ARG, "null argument"};
        sync_forces64(s);
        sys_download(s, s->f, f);
    });
}

int mappg_sys_set_box(mappg_sys* s, const double* H) {
    return guard([&] {
        if (!s || !H) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "the boxes of a batch are fixed at creation"};
        int nb_old = s->nbins;
        sys_set_box(s, H);
        if (s->nbins != nb_old) sys_alloc_bins(s);
        s->built = false;
    });
}

int mappg_sys_build(mappg_sys* s) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        sys_build(s);
    });
}

int mappg_sys_update(mappg_sys* s, int* rebuilt) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (!s->built) {
            sys_build(s);
            if (rebuilt) *rebuilt = 1;
            return;
        }
        long long before;
        MAPPG_CUDA(cudaMemcpyAsync(&before, &s->sc->nrebuild, sizeof(long long), cudaMemcpyDeviceToHost, s->stream));
        lb_update(s);
        check_build(s);
        long long after;
        MAPPG_CUDA(cudaMemcpyAsync(&after, &s->sc->nrebuild, sizeof(long long), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        if (rebuilt) *rebuilt = after != before;
    });
}

int mappg_sys_force(mappg_sys* s, double* pe, double* virial6) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_ARG, "a batch of cells reports per cell: mappg_batch_force"};
        if (!s->built) sys_build(s);
        launch_force(s);
        DevScalars h;
        MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        if (pe) *pe = h.energy;
        if (virial6)
            for (int k = 0; k < 6; k++) virial6[k] = h.virial[k];
        if (!std::isfinite(h.energy)) throw Error{MAPPG_ERR_NAN, "non-finite energy"};
    });
}

int mappg_sys_energy(mappg_sys* s, double* pe) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_ARG, "a batch of cells reports per cell: mappg_batch_energy"};
        if (!s->built) sys_build(s);
        launch_energy(s);
        double e;
        MAPPG_CUDA(cudaMemcpyAsync(&e, &s->sc->energy, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        if (pe) *pe = e;
    });
}

int mappg_sys_get_rho(mappg_sys* s, double* rho, double* dF) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        std::vector<double> a(s->n), b(s->n);
        if (s->precision == MAPPG_MIXED) {
            std::vector<float> r32(s->n);
            std::vector<float4> q(s->n);
            MAPPG_CUDA(cudaMemcpyAsync(r32.data(), s->rho32, sizeof(float) * s->n, cudaMemcpyDeviceToHost, s->stream));
            MAPPG_CUDA(cudaMemcpyAsync(q.data(), s->q32, sizeof(float4) * s->n, cudaMemcpyDeviceToHost, s->stream));
            MAPPG_CUDA(cudaStreamSynchronize(s->stream));
            for (int i = 0; i < s->n; i++) {
                a[i] = r32[i];
                b[i] = q[i].w;
            }
        } else {
            MAPPG_CUDA(cudaMemcpyAsync(a.data(), s->rho, sizeof(double) * s->n, cudaMemcpyDeviceToHost, s->stream));
            MAPPG_CUDA(cudaMemcpyAsync(b.data(), s->dF, sizeof(double) * s->n, cudaMemcpyDeviceToHost, s->stream));
            MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        }
        for (int i = 0; i < s->n; i++) {
            int u = s->host_id[i];
            if (rho) rho[u] = a[i];
            if (dF) dF[u] = b[i];
        }
    });
}

int mappg_sys_neighbors(mappg_sys* s, int* counts, int* entries, long long* total) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (!s->built) sys_build(s);
        sys_neighbors(s, counts, entries, total);
    });
}

int mappg_sys_stats(mappg_sys* s, long long* out6) {
    return guard([&] {
        if (!s || !out6) throw Error{MAPPG_ERR_ARG, "null argument"};
        DevScalars h;
        MAPPG_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        out6[0] = h.nrebuild;
        out6[1] = s->maxnbr;
        out6[2] = h.maxrow;
        out6[3] = s->n ? (long long)(1000.0 * (double)h.sumrow / s->n) : 0;
        out6[4] = s->nbins;
        out6[5] = s->precision;
    });
}

// lanes per atom (atoms per block) and neighbour entries per loop step of
// the density and force kernels: both passes on the system's own atoms and
// neighbour list, timed with CUDA events for each candidate; the fastest is
// kept for the system's later launches
int mappg_sys_autotune(mappg_sys* s, int* tpa_out, int* unroll_out, double* ms_out) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->run) throw Error{MAPPG_ERR_ARG, "an NVT run is in progress"};
        if (!s->built) sys_build(s);
        const int cand[7][2] = {{4, 1}, {8, 1}, {16, 1}, {4, 2}, {8, 2}, {16, 2}, {32, 1}};
        // the FP64 kernels have no unrolled form; 32 lanes per atom spread a
        // small system's FP64 work over more of the SMs
        const bool mixed = s->precision == MAPPG_MIXED;
        cudaEvent_t e0, e1;
        MAPPG_CUDA(cudaEventCreate(&e0));
        MAPPG_CUDA(cudaEventCreate(&e1));
        // density and force are timed apart: they share the lanes per atom
        // (the force pass walks the density pass's per-lane cutoff bits) but
        // each keeps its own entries per loop step; a single mixed cell also
        // tries the force pass with its records in shared memory
        // (k_force32s) at three budgets
        int modes[4] = {0, 0, 0, 0}, nmodes = 1;
        if (mixed && force_smem_available(s)) {
            const int mx = force_smem_max_kb(s);
            for (int kb : {64, 128, mx})
                if (kb <= mx && kb > modes[nmodes - 1]) modes[nmodes++] = kb;
        }
        const int tpa0 = s->tpa, u0 = s->unroll, uf0 = s->unroll_force, sm0 = s->force_smem;
        double td[7], tf[7];
        int tf_mode[7];
        auto time_ms = [&](auto&& launch) {
            launch();  // warm-up (and first-use set-up)
            MAPPG_CUDA(cudaEventRecord(e0, s->stream));
            for (int r = 0; r < 3; r++) launch();
            MAPPG_CUDA(cudaEventRecord(e1, s->stream));
            MAPPG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            MAPPG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            return ms / 3.0;
        };
        try {
            for (int c = 0; c < 7; c++) {
                td[c] = tf[c] = 0.0;
                tf_mode[c] = 0;
                if (!mixed && cand[c][1] != 1) continue;
                s->tpa = cand[c][0];
                s->unroll = cand[c][1];
                s->unroll_force = 0;
                td[c] = time_ms([&] { launch_density_only(s); });
                tf[c] = 1e30;
                for (int mi = 0; mi < nmodes; mi++) {
                    s->force_smem = modes[mi];
                    const double t = time_ms([&] { launch_force_only(s); });
                    if (t < tf[c]) {
                        tf[c] = t;
                        tf_mode[c] = modes[mi];
                    }
                }
                if (ms_out) ms_out[c] = td[c] + tf[c];
            }
        } catch (...) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            s->tpa = tpa0;
            s->unroll = u0;
            s->unroll_force = uf0;
            s->force_smem = sm0;
            throw;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        // per lanes per atom: the best density unroll plus the best force
        // unroll and record source
        double best = 1e30;
        int best_tpa = tpa0, best_u = u0, best_uf = 0, best_sm = sm0;
        for (int c = 0; c < 7; c++) {
            if (td[c] <= 0.0) continue;
            for (int c2 = 0; c2 < 7; c2++) {
                if (tf[c2] <= 0.0 || cand[c2][0] != cand[c][0]) continue;
                if (td[c] + tf[c2] < best) {
                    best = td[c] + tf[c2];
                    best_tpa = cand[c][0];
                    best_u = cand[c][1];
                    best_uf = cand[c2][1];
                    best_sm = tf_mode[c2];
                }
            }
        }
        s->tpa = best_tpa;
        s->unroll = best_u;
        s->unroll_force = best_uf == best_u ? 0 : best_uf;
        s->force_smem = best_sm;
        if (tpa_out) *tpa_out = best_tpa;
        if (unroll_out) *unroll_out = best_u;
    });
}

int mappg_sys_tuning(mappg_sys* s, int* out) {
    return guard([&] {
        if (!s || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        out[0] = s->tpa;
        out[1] = s->unroll;
        out[2] = s->unroll_force ? s->unroll_force : s->unroll;
        out[3] = s->force_smem;
        out[4] = s->ncell > 1 ? s->chunk_atoms : 0;
    });
}

int mappg_sys_force_tables(mappg_sys* s, int mode, int* active) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (mode < -1) throw Error{MAPPG_ERR_ARG, "mode must be -1, 0 or a budget in KB"};
        if (mode > 0) {
            if (!force_smem_available(s))
                throw Error{MAPPG_ERR_UNSUPP, "shared-memory force records need a single mixed-precision cell"};
            s->force_smem = std::min(mode, force_smem_max_kb(s));
        } else if (mode == 0) {
            s->force_smem = 0;
        }
        if (active) *active = s->force_smem;
    });
}

// a batch of cells: atoms per chunk (the atoms one block works through
// before it takes the next chunk: 128, 256, 512) together with the lanes
// per atom and entries per loop step of mappg_sys_autotune, each candidate
// timed on the batch's own cells and lists; ms_out: 3 x 7 timings
int mappg_batch_autotune(mappg_sys* s, int* tpa_out, int* unroll_out, int* chunk_out, double* ms_out) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell <= 1) throw Error{MAPPG_ERR_ARG, "mappg_batch_autotune takes a batch of cells"};
        const int chunks[3] = {128, 256, 512};
        double best = 1e30;
        int bt = s->tpa, bu = s->unroll, bf = s->unroll_force, bc = s->chunk_atoms;
        for (int k = 0; k < 3; k++) {
            sys_rechunk(s, chunks[k]);
            double ms[7] = {0, 0, 0, 0, 0, 0, 0};
            int t = 0, u = 0;
            int rc = mappg_sys_autotune(s, &t, &u, ms);
            if (rc != MAPPG_OK) throw Error{rc, mappg_last_error()};
            for (int c = 0; c < 7; c++) {
                if (ms_out) ms_out[7 * k + c] = ms[c];
                if (ms[c] > 0.0 && ms[c] < best) {
                    best = ms[c];
                    bc = chunks[k];
                }
            }
            if (bc == chunks[k]) {
                bt = t;
                bu = u;
                bf = s->unroll_force;
            }
        }
        sys_rechunk(s, bc);
        s->tpa = bt;
        s->unroll = bu;
        s->unroll_force = bf;
        if (tpa_out) *tpa_out = bt;
        if (unroll_out) *unroll_out = bu;
        if (chunk_out) *chunk_out = bc;
    });
}

int mappg_create_temp(int natoms, const unsigned char* elem, const double* masses, double T, double kB, int seed,
                      double* v) {
    return mappg_create_temp_dof(natoms, elem, masses, nullptr, T, kB, seed, v);
}

int mappg_create_temp_dof(int natoms, const unsigned char* elem, const double* masses, const unsigned char* dof,
                          double T, double kB, int seed, double* v) {
    return guard([&] {
        if (!elem || !masses || !v || natoms < 0) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (seed == 0) throw Error{MAPPG_ERR_ARG, "seed 0 never yields a Gaussian sample"};
        if (!(kB == kB)) throw Error{MAPPG_ERR_ARG, "boltzmann constant should be set prior to create_temp"};
        int sd = seed;
        auto uniform = [&sd]() {
            int first = sd / 127773, second = sd % 127773;
            int rnd = 16807 * second - 2836 * first;
            sd = rnd > 0 ? rnd : rnd + 2147483647;
            return sd * 1.0 / 2147483647;
        };
        bool gchk = false;
        double reserved = 0.0;
        for (int i = 0; i < natoms; i++) {
            double fac = sqrt(kB * T / masses[elem[i]]);
            for (int j = 0; j < 3; j++) {
                if (dof && !dof[3 * (size_t)i + j]) continue;  // kept (atoms_md.cpp:138-149)
                double g;
                if (gchk) {
                    gchk = false;
                    g = reserved;
                } else {
                    gchk = true;
                    double u = 0.0, w = 0.0, s2 = 1.0;
                    while (s2 >= 1.0) {
                        u = 2.0 * uniform() - 1.0;
                        w = 2.0 * uniform() - 1.0;
                        s2 = u * u + w * w;
                    }
                    double r = sqrt(-2.0 * log(s2) / s2);
                    reserved = w * r;
                    g = u * r;
                }
                v[3 * (size_t)i + j] = g * fac;
            }
        }
    });
}

int mappg_nvt_run(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters, int nsteps,
                  double* eta, double* thermo) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (!s->have_v) throw Error{MAPPG_ERR_ARG, "velocities must be set before MD"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_ARG, "a batch of cells runs with mappg_batch_nvt_run"};
        nvt_run(s, T, dt, kB, t_relax, L, niters, nsteps, eta, thermo, nullptr);
    });
}

int mappg_nvt_run_host(mappg_sys* s, const double* x_in, const double* v_in, double T, double dt, double kB,
                       double t_relax, int L, int niters, int nsteps, double* eta, double* thermo, double* x_out,
                       double* v_out, double* f_out) {
    return guard([&] {
        if (!s || !x_in || !v_in) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_ARG, "a batch of cells runs with mappg_batch_nvt_run"};
        try {
            sys_upload(s, x_in, s->x);
            s->built = false;
            sys_upload_side(s, v_in, s->v);  // joined before the run reads velocities
            s->have_v = true;
            if (x_out && nsteps > 0)
                nvt_run_xout(s, T, dt, kB, t_relax, L, niters, nsteps, eta, thermo, x_out);
            else
                nvt_run(s, T, dt, kB, t_relax, L, niters, nsteps, eta, thermo, nullptr);
        } catch (...) {
            if (s->side) cudaStreamSynchronize(s->side);
            s->v_pending = false;
            throw;
        }
        if (x_out && nsteps == 0) sys_download_async(s, s->x, x_out);
        if (v_out) sys_download_async(s, s->v, v_out);
        if (f_out) {
            sync_forces64(s);
            sys_download_async(s, s->f, f_out);
        }
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->side));  // the positions' copy
    });
}

int mappg_nvt_begin(mappg_sys* s, double T, double dt, double kB, double t_relax, int L, int niters,
                    long long nsteps, const double* eta, int record_thermo) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_ARG, "a batch of cells runs with mappg_batch_nvt_begin"};
        nvt_begin(s, T, dt, kB, t_relax, L, niters, nsteps, eta, record_thermo != 0, nullptr);
    });
}

int mappg_nvt_steps(mappg_sys* s, long long nsteps) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (nsteps < 0) throw Error{MAPPG_ERR_ARG, "nsteps must be >= 0"};
        nvt_steps(s, nsteps);
    });
}

int mappg_nvt_end(mappg_sys* s, double* eta, double* thermo) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        nvt_end(s, eta, thermo);
    });
}

int mappg_nst_run(mappg_sys* s, const double* S, const double* tau, double T, double dt, double kB, double t_relax,
                  int L, int niters, double t_relax_S, int L_S, int niters_S, int nreset, int nsteps, double* V_H,
                  double* eta, double* eta_S, double* thermo) {
    return guard([&] {
        if (!s || !S || !tau || !V_H || !eta || !eta_S) throw Error{MAPPG_ERR_ARG, "null argument"};
        nst_run(s, S, tau, T, dt, kB, t_relax, L, niters, t_relax_S, L_S, niters_S, nreset, nsteps, V_H, eta, eta_S,
                thermo);
    });
}

// GCMC exchange energies: outside this engine (ff_md.h:19-21,49-50)
static int xchng_unsupported() {
    return guard([] {
        throw Error{MAPPG_ERR_UNSUPP, "GCMC exchange energies (ForceFieldMD::xchng_energy) are outside this engine"};
    });
}
int mappg_sys_init_xchng(mappg_sys*) { return xchng_unsupported(); }
int mappg_sys_fin_xchng(mappg_sys*) { return xchng_unsupported(); }
int mappg_sys_pre_xchng_energy(mappg_sys*, void*) { return xchng_unsupported(); }
int mappg_sys_xchng_energy(mappg_sys*, void*, double*) { return xchng_unsupported(); }
int mappg_sys_post_xchng_energy(mappg_sys*, void*) { return xchng_unsupported(); }

int mappg_sys_set_dof(mappg_sys* s, const unsigned char* dof) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "frozen components (x_dof) are per single cell"};
        if (s->run) throw Error{MAPPG_ERR_ARG, "an NVT run is in progress"};
        if (s->dof) cudaFree(s->dof);
        s->dof = nullptr;
        for (int c = 0; c < 3; c++) s->dof_frozen[c] = 0;
        if (!dof) return;
        const int n = s->n;
        std::vector<uint8_t> bits(n);
        bool any = false;
        for (int i = 0; i < n; i++) {
            const int u = s->host_id[i];  // caller index of the atom at bin-order position i
            uint8_t b = 0;
            for (int c = 0; c < 3; c++) {
                if (dof[3 * (size_t)u + c])
                    b |= (uint8_t)(1u << c);
                else
                    s->dof_frozen[c]++;
            }
            bits[i] = b;
            any |= b != 7;
        }
        if (!any) return;  // every component free: no mask
        MAPPG_CUDA(cudaMalloc(&s->dof, n));
        MAPPG_CUDA(cudaMemcpyAsync(s->dof, bits.data(), n, cudaMemcpyHostToDevice, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    });
}

int mappg_nvt_snapshot(mappg_sys* s, double* x, double* x_d) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        nvt_snapshot(s, x, x_d);
    });
}

int mappg_sys_set_hook(mappg_sys* s, int (*hook)(void*, long long), void* user, int nevery) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (hook && nevery > 0) {
            s->hook = hook;
            s->hook_user = user;
            s->hook_every = nevery;
        } else {
            s->hook = nullptr;
            s->hook_user = nullptr;
            s->hook_every = 0;
        }
    });
}

// ------------------------------------------------------------------ batches of cells
int mappg_batch_create(const mappg_ff* ff, int ncell, const int* natoms, const double* H, const double* x,
                       const unsigned char* elem, const double* masses, double skin, int precision, mappg_sys** out) {
    return guard([&] {
        if (!ff || !natoms || !H || !x || !elem || !masses || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (ncell < 2 || ncell > kMaxCells)
            throw Error{MAPPG_ERR_ARG, "a batch holds 2.." + std::to_string(kMaxCells) + " cells"};
        if (precision != MAPPG_MIXED) throw Error{MAPPG_ERR_UNSUPP, "batches run in mixed precision"};
        if (!(skin >= 0.0)) throw Error{MAPPG_ERR_ARG, "skin must be >= 0"};
        long long total = 0;
        for (int c = 0; c < ncell; c++) {
            if (natoms[c] < 1) throw Error{MAPPG_ERR_ARG, "every cell needs at least one atom"};
            total += natoms[c];
        }
        if (total > kMaxAtoms) throw Error{MAPPG_ERR_ARG, "too many atoms in the batch"};
        const int n = (int)total;
        const int ne = ff->host.nelem;
        for (int i = 0; i < n; i++)
            if (elem[i] >= ne) throw Error{MAPPG_ERR_ARG, "element index beyond the force field's elements"};
        for (int e = 0; e < ne; e++)
            if (!(masses[e] > 0.0)) throw Error{MAPPG_ERR_ARG, "masses must be positive"};
        for (long long i = 0; i < 3 * total; i++)
            if (!std::isfinite(x[i])) throw Error{MAPPG_ERR_NAN, "non-finite position"};
        ensure_uploaded(ff);
        mappg_sys* s = new mappg_sys();
        try {
            s->ff = ff;
            s->n = n;
            s->precision = precision;
            s->ne = ne;
            s->skin = skin;
            for (int e = 0; e < ne; e++) s->masses[e] = masses[e];
            double mc = 0.0;
            for (int i = 0; i < ne; i++)
                for (int j = 0; j < ne; j++) {
                    double c = ff->host.cut[i * ne + j];
                    mc = std::max(mc, c);
                    s->cut_sq[i * ne + j] = c * c;
                    double ck = c + skin;
                    s->cut_sk_sq[i * ne + j] = ck * ck;
                }
            s->max_cut = mc + skin;
            MAPPG_CUDA(cudaGetDevice(&s->device));
            cudaDeviceProp p;
            MAPPG_CUDA(cudaGetDeviceProperties(&p, s->device));
            s->sm_count = p.multiProcessorCount;
            sys_set_cells(s, ncell, natoms, H);
            sys_alloc(s, x);
            sys_alloc_bins(s);
            double vol = 0.0;
            for (const CellGeo& g : s->cells) vol += g.h6[0] * g.h6[3] * g.h6[5];
            double est = (n / vol) * 4.18879 * s->max_cut * s->max_cut * s->max_cut;
            int cap = ((int)(est * 1.35) + 32 + 31) / 32 * 32;
            sys_alloc_nbr(s, std::min(cap, 4096));
            sys_upload(s, x, s->x);
            std::vector<uint8_t> es(n);
            for (int i = 0; i < n; i++) es[i] = elem[s->host_id[i]];
            MAPPG_CUDA(cudaMemcpyAsync(s->elem, es.data(), n, cudaMemcpyHostToDevice, s->stream));
            MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        } catch (...) {
            sys_free(s);
            delete s;
            throw;
        }
        *out = s;
    });
}

int mappg_batch_ncell(const mappg_sys* s) { return s ? s->ncell : 0; }

static void batch_cells_out(mappg_sys* s, double* pe, double* virial) {
    std::vector<CellMd> cm(s->ncell);
    MAPPG_CUDA(cudaMemcpyAsync(cm.data(), s->cmd, sizeof(CellMd) * s->ncell, cudaMemcpyDeviceToHost, s->stream));
    MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    for (int c = 0; c < s->ncell; c++) {
        if (!std::isfinite(cm[c].energy)) throw Error{MAPPG_ERR_NAN, "non-finite energy"};
        if (pe) pe[c] = cm[c].energy;
        if (virial)
            for (int k = 0; k < 6; k++) virial[6 * (size_t)c + k] = cm[c].virial[k];
    }
}

int mappg_batch_force(mappg_sys* s, double* pe, double* virial) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell < 2) throw Error{MAPPG_ERR_ARG, "not a batch of cells"};
        if (!s->built) sys_build(s);
        launch_force(s);
        batch_cells_out(s, pe, virial);
    });
}

int mappg_batch_energy(mappg_sys* s, double* pe) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell < 2) throw Error{MAPPG_ERR_ARG, "not a batch of cells"};
        if (!s->built) sys_build(s);
        launch_energy(s);
        batch_cells_out(s, pe, nullptr);
    });
}

int mappg_batch_nvt_begin(mappg_sys* s, const double* T, double dt, double kB, double t_relax, int L, int niters,
                          long long nsteps, const double* eta, int record_thermo) {
    return guard([&] {
        if (!s || !T) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->ncell < 2) throw Error{MAPPG_ERR_ARG, "not a batch of cells"};
        nvt_begin(s, 1.0, dt, kB, t_relax, L, niters, nsteps, eta, record_thermo != 0, T);
    });
}

int mappg_batch_lbfgs_run(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, double c, double rho,
                          double min_alpha, int nsteps, double* stats) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell < 2) throw Error{MAPPG_ERR_ARG, "not a batch of cells"};
        batch_lbfgs_run(s, m, e_tol, max_dx, f_tol, c, rho, min_alpha, nsteps, nullptr, stats);
    });
}

int mappg_batch_nvt_end(mappg_sys* s, double* eta, double* thermo) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell < 2) throw Error{MAPPG_ERR_ARG, "not a batch of cells"};
        nvt_end(s, eta, thermo);
    });
}

int mappg_batch_nvt_run(mappg_sys* s, const double* T, double dt, double kB, double t_relax, int L, int niters,
                        int nsteps, double* eta, double* thermo) {
    return guard([&] {
        if (!s || !T) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->ncell < 2) throw Error{MAPPG_ERR_ARG, "not a batch of cells"};
        if (!s->have_v) throw Error{MAPPG_ERR_ARG, "velocities must be set before MD"};
        nvt_run(s, 1.0, dt, kB, t_relax, L, niters, nsteps, eta, thermo, T);
    });
}

int mappg_sys_stream(mappg_sys* s, void** stream) {
    return guard([&] {
        if (!s || !stream) throw Error{MAPPG_ERR_ARG, "null argument"};
        *stream = (void*)s->stream;
    });
}

int mappg_sys_sync(mappg_sys* s) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
    });
}

int mappg_sys_enqueue(mappg_sys* s, int what) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (!s->built) throw Error{MAPPG_ERR_ARG, "build the neighbour list first"};
        switch (what) {
            case 0: launch_density_only(s); break;
            case 1: launch_force_only(s); break;
            case 2: launch_energy(s); break;
            case 3:
                request_rebuild(s);
                launch_rebuild_chain(s);
                break;
            default: throw Error{MAPPG_ERR_ARG, "unknown kernel selector"};
        }
    });
}

// line-search parameters as the Python types accept them (ls.cpp:190-260,
// 358-450, 560-620)
static LsParams ls_params(const mappg_ls* q) {
    if (!q) throw Error{MAPPG_ERR_ARG, "null line search"};
    LsParams p;
    p.kind = q->kind;
    p.c = q->c;
    p.rho = q->rho;
    p.min_alpha = q->min_alpha;
    p.tol = q->tol;
    p.max_iter = q->max_iter;
    p.bracket = q->bracket != 0;
    p.zeps = q->zeps;
    if (p.kind == MAPPG_LS_BT) {
        if (!(p.c > 0.0 && p.c < 1.0)) throw Error{MAPPG_ERR_ARG, "c must be in (0,1)"};
        if (!(p.rho > 0.0 && p.rho < 1.0)) throw Error{MAPPG_ERR_ARG, "rho must be in (0,1)"};
        if (!(p.min_alpha >= 0.0)) throw Error{MAPPG_ERR_ARG, "min_alpha must be >= 0"};
    } else if (p.kind == MAPPG_LS_GOLDEN || p.kind == MAPPG_LS_BRENT) {
        if (!(p.tol > 0.0)) throw Error{MAPPG_ERR_ARG, "tol must be > 0"};
        if (p.max_iter <= 0) throw Error{MAPPG_ERR_ARG, "max_iter must be > 0"};
        if (p.kind == MAPPG_LS_BRENT && !(p.zeps > 0.0)) throw Error{MAPPG_ERR_ARG, "zeps must be > 0"};
    } else {
        throw Error{MAPPG_ERR_ARG, "unknown line search"};
    }
    return p;
}

static LsParams bt_params(double c, double rho, double min_alpha) {
    mappg_ls q{MAPPG_LS_BT, c, rho, min_alpha, 0.0, 0, 0, 0.0};
    return ls_params(&q);
}

int mappg_cg_run(mappg_sys* s, double e_tol, double max_dx, double f_tol, double c, double rho, double min_alpha,
                 int nsteps, double* stats) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "conjugate gradients run per single cell"};
        cg_run(s, e_tol, max_dx, f_tol, bt_params(c, rho, min_alpha), nsteps, stats);
    });
}

int mappg_lbfgs_run(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, double c, double rho,
                    double min_alpha, int nsteps, double* stats) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "L-BFGS on a batch of cells runs with mappg_batch_lbfgs_run"};
        lbfgs_run(s, m, e_tol, max_dx, f_tol, bt_params(c, rho, min_alpha), nsteps, stats, nullptr, nullptr);
    });
}

int mappg_cg_run_ls(mappg_sys* s, double e_tol, double max_dx, double f_tol, const mappg_ls* ls, int nsteps,
                    double* stats) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "conjugate gradients run per single cell"};
        cg_run(s, e_tol, max_dx, f_tol, ls_params(ls), nsteps, stats);
    });
}

int mappg_min_box_run(mappg_sys* s, int method, int m, double e_tol, double max_dx, const int* H_dof, int affine,
                      const mappg_ls* ls, int nsteps, double* stats) {
    return guard([&] {
        if (!s || !H_dof) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "box degrees of freedom are per single cell"};
        box_min_run(s, method, m, e_tol, max_dx, H_dof, affine != 0, ls_params(ls), nsteps, stats);
    });
}

int mappg_sys_get_box(mappg_sys* s, double* H) {
    return guard([&] {
        if (!s || !H) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "the boxes of a batch are those it was created with"};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) H[3 * i + j] = s->box.H[i][j];
    });
}

int mappg_lbfgs_run_ls(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, const mappg_ls* ls,
                       int nsteps, double* stats) {
    return guard([&] {
        if (!s) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "L-BFGS on a batch of cells runs with mappg_batch_lbfgs_run"};
        lbfgs_run(s, m, e_tol, max_dx, f_tol, ls_params(ls), nsteps, stats, nullptr, nullptr);
    });
}

}  // extern "C"
