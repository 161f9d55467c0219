/*
 * oracle.c -- CPU restatement of MAPP's EAM molecular-dynamics and
 * minimization path (sinamoeini/mapp4py), FP64, single rank.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (mapp4py_gb300/, the
 * libmappg C ABI) links, loads or calls this file.  Only tests/, the smoke
 * check and the CPU-baseline leg of bench.py use it, as the checker.
 *
 * Parity status: pinned to the reference itself.  The reference ships no
 * test vectors for this path; it is compiled from its own sources with a
 * single-rank MPI stand-in (ref.mk, refshim/), and the fixtures
 * tests/golden/ref_*.npz hold its forces, energies, stresses, NVT/NVE
 * trajectories, L-BFGS iterates and create_temp draws on the analytic
 * potential and on the four potential files of its examples.  This file
 * restates the cited reference code step by step in the reference's own
 * operation order and reproduces those fixtures to 1e-14 (bit for bit for
 * NVE and create_temp); it is also cross-checked by finite differences,
 * lattice symmetry, Newton's third law and energy conservation.
 *
 * Reference files cited below are relative to the mapp4py source tree.
 * Build with -ffp-contract=off: the reference's own x86 build never fuses
 * multiply-adds, and the neighbour predicate is compared bit for bit.
 */
#include <ctype.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OMIN(a, b) ((a) < (b) ? (a) : (b))
#define OMAX(a, b) ((a) > (b) ? (a) : (b))

#include <time.h>
static double now_seconds(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static char orc_err[512];
const char* orc_last_error(void) { return orc_err; }
static int fail(const char* msg) {
    snprintf(orc_err, sizeof(orc_err), "%s", msg);
    return -1;
}

/* ------------------------------------------------------------------------ */
/* EAM tables                                                               */
/* ------------------------------------------------------------------------ */
typedef struct {
    int nelem, nr, nrho;
    double dr, drho, dr_inv, drho_inv, rho_max;
    double* F;    /* [nelem][nrho][4]                                   */
    double* rho;  /* [nelem][nelem][nr][4]  == reference rho_arr[i][j]  */
    double* rphi; /* [nelem][nelem][nr][4]  symmetric                     */
    double* cut;  /* [nelem][nelem]                                       */
} orc_eam;

/* ImportEAM::interpolate(size_t,type0,type0(*)[4])  import_eam.cpp:62-83 */
static void interpolate4(size_t n, double (*s)[4]) {
    s[0][1] = s[1][0] - s[0][0];
    s[1][1] = 0.5 * (s[2][0] - s[0][0]);
    s[n - 2][1] = 0.5 * (s[n - 1][0] - s[n - 3][0]);
    s[n - 1][1] = s[n - 1][0] - s[n - 2][0];
    for (size_t i = 2; i < n - 2; i++)
        s[i][1] = ((s[i - 2][0] - s[i + 2][0]) + 8.0 * (s[i + 1][0] - s[i - 1][0])) / 12.0;
    for (size_t i = 0; i < n - 1; i++) {
        s[i][2] = 3.0 * (s[i + 1][0] - s[i][0]) - 2.0 * s[i][1] - s[i + 1][1];
        s[i][3] = s[i][1] + s[i + 1][1] - 2.0 * (s[i + 1][0] - s[i][0]);
    }
    s[n - 1][2] = 0.0;
    s[n - 1][3] = 0.0;
}

#define RHO(e, i, j) ((double(*)[4])((e)->rho + ((size_t)((i) * (e)->nelem + (j)) * (e)->nr) * 4))
#define RPHI(e, i, j) ((double(*)[4])((e)->rphi + ((size_t)((i) * (e)->nelem + (j)) * (e)->nr) * 4))
#define FTAB(e, i) ((double(*)[4])((e)->F + ((size_t)(i) * (e)->nrho) * 4))

/* ImportEAM::set_cuttoff  import_eam.h:52-64 */
static void set_cutoff(orc_eam* e) {
    for (int i = 0; i < e->nelem; i++)
        for (int j = 0; j < i + 1; j++) {
            size_t n_ = (size_t)e->nr - 1;
            while ((RPHI(e, i, j)[n_][0] == 0.0 && RHO(e, i, j)[n_][0] == 0.0 &&
                    RHO(e, j, i)[n_][0] == 0.0) && n_ >= 1)
                n_--;
            e->cut[i * e->nelem + j] = e->cut[j * e->nelem + i] = (double)n_ * e->dr;
        }
}

static orc_eam* eam_alloc(int nelem, int nr, int nrho, double dr, double drho) {
    orc_eam* e = (orc_eam*)calloc(1, sizeof(orc_eam));
    e->nelem = nelem;
    e->nr = nr;
    e->nrho = nrho;
    e->dr = dr;
    e->drho = drho;
    e->F = (double*)calloc((size_t)nelem * nrho * 4, sizeof(double));
    e->rho = (double*)calloc((size_t)nelem * nelem * nr * 4, sizeof(double));
    e->rphi = (double*)calloc((size_t)nelem * nelem * nr * 4, sizeof(double));
    e->cut = (double*)calloc((size_t)nelem * nelem, sizeof(double));
    return e;
}

/* ForceFieldEAM::ForceFieldEAM  ff_eam.cpp:14-50 (derived constants) */
static void eam_finish(orc_eam* e) {
    for (int i = 0; i < e->nelem; i++) interpolate4((size_t)e->nrho, FTAB(e, i));
    for (int i = 0; i < e->nelem; i++)
        for (int j = 0; j < e->nelem; j++) interpolate4((size_t)e->nr, RHO(e, i, j));
    for (int i = 0; i < e->nelem; i++)
        for (int j = 0; j <= i; j++) {
            interpolate4((size_t)e->nr, RPHI(e, i, j));
            if (i != j) memcpy(RPHI(e, j, i), RPHI(e, i, j), sizeof(double) * 4 * e->nr);
        }
    set_cutoff(e);
    e->dr_inv = 1.0 / e->dr;
    e->drho_inv = 1.0 / e->drho;
    e->rho_max = (double)e->nrho * e->drho;
}

/*
 * Build tables from raw knot values.  F: [nelem][nrho]; rho: [nelem][nelem][nr]
 * (rho[i][j] is the reference's rho_arr[i][j]: the density that an atom of
 * element i deposits on an atom of element j); rphi: [nelem][nelem][nr], only
 * i>=j is read.
 */
void* orc_eam_from_knots(int nelem, int nr, int nrho, double dr, double drho, const double* F,
                         const double* rho, const double* rphi) {
    if (nr < 5 || nrho < 5 || dr <= 0.0 || drho <= 0.0 || nelem < 1) {
        fail("invalid table dimensions");
        return NULL;
    }
    orc_eam* e = eam_alloc(nelem, nr, nrho, dr, drho);
    for (int i = 0; i < nelem; i++)
        for (int k = 0; k < nrho; k++) FTAB(e, i)[k][0] = F[(size_t)i * nrho + k];
    for (int i = 0; i < nelem; i++)
        for (int j = 0; j < nelem; j++)
            for (int k = 0; k < nr; k++) RHO(e, i, j)[k][0] = rho[((size_t)i * nelem + j) * nr + k];
    for (int i = 0; i < nelem; i++)
        for (int j = 0; j <= i; j++)
            for (int k = 0; k < nr; k++) RPHI(e, i, j)[k][0] = rphi[((size_t)i * nelem + j) * nr + k];
    eam_finish(e);
    return e;
}

void orc_eam_free(void* p) {
    orc_eam* e = (orc_eam*)p;
    if (!e) return;
    free(e->F);
    free(e->rho);
    free(e->rphi);
    free(e->cut);
    free(e);
}

void orc_eam_info(void* p, int* nelem, int* nr, int* nrho, double* dr, double* drho) {
    orc_eam* e = (orc_eam*)p;
    *nelem = e->nelem;
    *nr = e->nr;
    *nrho = e->nrho;
    *dr = e->dr;
    *drho = e->drho;
}

/* copies of the coefficient arrays, layouts as in orc_eam */
void orc_eam_tables(void* p, double* F, double* rho, double* rphi, double* cut) {
    orc_eam* e = (orc_eam*)p;
    if (F) memcpy(F, e->F, sizeof(double) * 4 * e->nelem * e->nrho);
    if (rho) memcpy(rho, e->rho, sizeof(double) * 4 * e->nelem * e->nelem * e->nr);
    if (rphi) memcpy(rphi, e->rphi, sizeof(double) * 4 * e->nelem * e->nelem * e->nr);
    if (cut) memcpy(cut, e->cut, sizeof(double) * e->nelem * e->nelem);
}

/* ------------------------------------------------------------------------ */
/* setfl reader: ImportEAM::setfl  import_eam.h:348-613, with the line       */
/* handling of FileReader  import.cpp:92-119,133-143,208-240 and            */
/* ImportEAM::read_double  import_eam.cpp:154-170.                           */
/* ------------------------------------------------------------------------ */
typedef struct {
    FILE* f;
    char* line;
    size_t cap;
    int finished;
} freader;

/* FileReader::operator() -- returns 1 when finished.  A last line without a
   trailing newline counts as end of file, as std::getline + eof() does. */
static int fr_line(freader* r) {
    if (r->finished) return 1;
    size_t n = 0;
    int c;
    while ((c = fgetc(r->f)) != EOF && c != '\n') {
        if (n + 2 > r->cap) {
            r->cap = r->cap ? 2 * r->cap : 1024;
            r->line = (char*)realloc(r->line, r->cap);
        }
        r->line[n++] = (char)c;
    }
    if (c == EOF) {
        r->finished = 1;
        return 1;
    }
    if (!r->line) {
        r->cap = 16;
        r->line = (char*)malloc(r->cap);
    }
    r->line[n] = '\0';
    return 0;
}

/* FileReader::skip(n) */
static int fr_skip(freader* r, int n) {
    for (int i = 0; i < n && !r->finished; i++) {
        int c;
        while ((c = fgetc(r->f)) != EOF && c != '\n') {
        }
        if (c == EOF) r->finished = 1;
    }
    /* std::istream::ignore sets eof only when it hits the end */
    if (!r->finished) {
        int c = fgetc(r->f);
        if (c == EOF)
            r->finished = 1;
        else
            ungetc(c, r->f);
    }
    return r->finished;
}

/* FileReader::parse_line: strip after '#', split on whitespace */
static int fr_parse(char* s, char*** args, int* acap) {
    char* last = s;
    while (*last != '#' && *last != '\0' && *last != '\n') last++;
    *last = '\0';
    int n = 0;
    char* p = s;
    while (p != last) {
        while (p != last && isspace((unsigned char)*p)) p++;
        if (p == last) continue;
        if (n + 1 > *acap) {
            *acap = *acap ? 2 * *acap : 16;
            *args = (char**)realloc(*args, sizeof(char*) * (*acap));
        }
        (*args)[n++] = p;
        while (p != last && !isspace((unsigned char)*p)) p++;
        if (p == last) continue;
        *p = '\0';
        p++;
    }
    return n;
}

static int read_double(freader* r, double* buf, size_t n, char*** args, int* acap) {
    size_t i = 0;
    while (i < n) {
        if (fr_line(r)) return fail("file ended immaturely");
        int na = fr_parse(r->line, args, acap);
        if ((size_t)na + i > n) return fail("file has extra arguments");
        for (int j = 0; j < na; j++) buf[i++] = atof((*args)[j]);
    }
    return 0;
}

void* orc_eam_read_setfl(const char* path) {
    freader r = {0};
    r.f = fopen(path, "r");
    if (!r.f) {
        fail("failed to open file");
        return NULL;
    }
    char** args = NULL;
    int acap = 0;
    orc_eam* e = NULL;
    double* buf = NULL;
    if (fr_skip(&r, 3)) {
        fail("file ended immaturely");
        goto done;
    }
    if (fr_line(&r)) {
        fail("file ended immaturely");
        goto done;
    }
    int na = fr_parse(r.line, &args, &acap);
    if (na < 2) {
        fail("invalid element line");
        goto done;
    }
    int nelem = na - 1;
    if (fr_line(&r)) {
        fail("file ended immaturely");
        goto done;
    }
    size_t nrho, nr;
    double drho, dr, rc;
    if (sscanf(r.line, " %zu %lf %zu %lf %lf", &nrho, &drho, &nr, &dr, &rc) != 5) {
        fail("invalid nrho/drho/nr/dr/rc line");
        goto done;
    }
    if (nrho < 5 || nr < 5 || drho <= 0.0 || dr <= 0.0) {
        fail("invalid table dimensions");
        goto done;
    }
    e = eam_alloc(nelem, (int)nr, (int)nrho, dr, drho);
    size_t npair = (size_t)nelem * (nelem + 1) / 2 * nr;
    buf = (double*)malloc(sizeof(double) * OMAX(nr + nrho, npair));
    for (int i = 0; i < nelem; i++) {
        if (fr_skip(&r, 1)) {
            fail("file ended immaturely");
            goto bad;
        }
        if (read_double(&r, buf, nrho + nr, &args, &acap)) goto bad;
        for (size_t k = 0; k < nrho; k++) FTAB(e, i)[k][0] = buf[k];
        for (int j = 0; j < nelem; j++)
            for (size_t k = 0; k < nr; k++) RHO(e, i, j)[k][0] = buf[k + nrho];
    }
    if (read_double(&r, buf, npair, &args, &acap)) goto bad;
    size_t ipos = 0;
    for (int i = 0; i < nelem; i++)
        for (int j = 0; j < i + 1; j++)
            for (size_t k = 0; k < nr; k++) RPHI(e, i, j)[k][0] = buf[ipos++];
    eam_finish(e);
    goto done;
bad:
    orc_eam_free(e);
    e = NULL;
done:
    free(buf);
    free(args);
    free(r.line);
    fclose(r.f);
    return e;
}

/* ------------------------------------------------------------------------ */
/* System state, coordinates and ghosts                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
    int natms, nghost, cap;
    double H[3][3], B[3][3], vol, depth_inv[3], h6[6], b6[6];
    double* x;           /* cap*3, locals then ghosts               */
    unsigned char* elem; /* cap                                       */
    int* src;            /* ghost g: index it was copied from (cap)   */
    int* gdim;           /* ghost g: dimension of its shift           */
    int* gsgn;           /* ghost g: +1 (s+1) or -1 (s-1)             */
    int* owner;          /* ghost g: local owner                      */
    int* img;            /* cap*3: integer image shift vs owner        */
    double *v, *f, *x0;
    double* masses;
    double skin, max_cut;
    double *cut_sq, *cut_sk_sq;
    orc_eam* eam;
    int pair_wise;
    int* nl_off;
    int* nl_cnt;
    int* nl;
    long nl_cap, no_pairs;
    double *rho, *dF, *drhoi, *drhoj;
    long dr_cap;
    double vec[7];
    double pe, F_H[3][3], S_pe[3][3];
    int nrebuild;
    unsigned char* dof; /* natms*3, nonzero: the component is a degree of freedom; NULL: all are */
} orc_sys;

/* Atoms::update_H  atoms.cpp:187-194 with MLT_inv / MLT_depth / MLT_det
   xmath.h:1403-1480,2399-2415 */
static void update_H(orc_sys* s) {
    double(*H)[3] = s->H;
    double(*B)[3] = s->B;
    memset(B, 0, sizeof(double) * 9);
    B[0][0] = 1.0 / H[0][0];
    B[1][1] = 1.0 / H[1][1];
    B[1][0] = -B[1][1] * (B[0][0] * H[1][0]);
    B[2][2] = 1.0 / H[2][2];
    B[2][1] = -B[2][2] * (B[1][1] * H[2][1]);
    B[2][0] = -B[2][2] * (B[0][0] * H[2][0] + B[1][0] * H[2][1]);
    s->vol = H[0][0] * (H[1][1] * H[2][2]);
    s->depth_inv[0] = sqrt(B[0][0] * B[0][0] + (B[1][0] * B[1][0] + B[2][0] * B[2][0]));
    s->depth_inv[1] = sqrt(B[1][1] * B[1][1] + B[2][1] * B[2][1]);
    s->depth_inv[2] = fabs(B[2][2]);
    /* MLT_2_V  xmath.h:1741-1770: column-wise lower triangle */
    s->h6[0] = H[0][0]; s->h6[1] = H[1][0]; s->h6[2] = H[2][0];
    s->h6[3] = H[1][1]; s->h6[4] = H[2][1]; s->h6[5] = H[2][2];
    s->b6[0] = B[0][0]; s->b6[1] = B[1][0]; s->b6[2] = B[2][0];
    s->b6[3] = B[1][1]; s->b6[4] = B[2][1]; s->b6[5] = B[2][2];
}

/* __X2S  xmath.h:2660-2700 (in place, with wrap into [0,1)) */
static void x2s_one(const double* b, double* x) {
    x[0] = b[0] * x[0] + (b[1] * x[1] + b[2] * x[2]);
    while (x[0] < 0.0) ++x[0];
    while (x[0] >= 1.0) --x[0];
    x[1] = b[3] * x[1] + b[4] * x[2];
    while (x[1] < 0.0) ++x[1];
    while (x[1] >= 1.0) --x[1];
    x[2] *= b[5];
    while (x[2] < 0.0) ++x[2];
    while (x[2] >= 1.0) --x[2];
}

/* __S2X  xmath.h:2636-2658 (in place) */
static void s2x_one(const double* h, double* s) {
    s[0] = h[0] * s[0] + (h[1] * s[1] + h[2] * s[2]);
    s[1] = h[3] * s[1] + h[4] * s[2];
    s[2] *= h[5];
}

static void sys_reserve(orc_sys* s, int cap) {
    if (cap <= s->cap) return;
    s->x = (double*)realloc(s->x, sizeof(double) * 3 * cap);
    s->elem = (unsigned char*)realloc(s->elem, cap);
    s->src = (int*)realloc(s->src, sizeof(int) * cap);
    s->gdim = (int*)realloc(s->gdim, sizeof(int) * cap);
    s->gsgn = (int*)realloc(s->gsgn, sizeof(int) * cap);
    s->owner = (int*)realloc(s->owner, sizeof(int) * cap);
    s->img = (int*)realloc(s->img, sizeof(int) * 3 * cap);
    s->f = (double*)realloc(s->f, sizeof(double) * 3 * cap);
    s->rho = (double*)realloc(s->rho, sizeof(double) * cap);
    s->dF = (double*)realloc(s->dF, sizeof(double) * cap);
    s->cap = cap;
}

void* orc_sys_new(int natms, const double* H9, const double* x, const unsigned char* elem,
                  const double* masses, double skin, void* eam) {
    orc_sys* s = (orc_sys*)calloc(1, sizeof(orc_sys));
    orc_eam* e = (orc_eam*)eam;
    s->eam = e;
    s->natms = natms;
    memcpy(s->H, H9, sizeof(double) * 9);
    update_H(s);
    sys_reserve(s, natms > 16 ? 2 * natms : 64);
    memcpy(s->x, x, sizeof(double) * 3 * natms);
    memcpy(s->elem, elem, natms);
    for (int i = 0; i < natms; i++) {
        s->owner[i] = i;
        s->img[3 * i] = s->img[3 * i + 1] = s->img[3 * i + 2] = 0;
    }
    s->v = (double*)calloc((size_t)3 * natms, sizeof(double));
    s->x0 = (double*)calloc((size_t)3 * natms, sizeof(double));
    s->masses = (double*)malloc(sizeof(double) * e->nelem);
    memcpy(s->masses, masses, sizeof(double) * e->nelem);
    s->skin = skin;
    s->pair_wise = 1;
    int ne = e->nelem;
    s->cut_sq = (double*)malloc(sizeof(double) * ne * ne);
    s->cut_sk_sq = (double*)malloc(sizeof(double) * ne * ne);
    return s;
}

void orc_sys_free(void* p) {
    orc_sys* s = (orc_sys*)p;
    if (!s) return;
    free(s->x); free(s->elem); free(s->src); free(s->gdim); free(s->gsgn); free(s->owner);
    free(s->img); free(s->v); free(s->f); free(s->x0); free(s->masses); free(s->cut_sq);
    free(s->cut_sk_sq); free(s->nl_off); free(s->nl_cnt); free(s->nl); free(s->rho);
    free(s->dF); free(s->drhoi); free(s->drhoj); free(s->dof);
    free(s);
}

void orc_sys_set_x(void* p, const double* x) { memcpy(((orc_sys*)p)->x, x, sizeof(double) * 3 * ((orc_sys*)p)->natms); }
void orc_sys_get_x(void* p, double* x) { memcpy(x, ((orc_sys*)p)->x, sizeof(double) * 3 * ((orc_sys*)p)->natms); }
void orc_sys_set_v(void* p, const double* v) { memcpy(((orc_sys*)p)->v, v, sizeof(double) * 3 * ((orc_sys*)p)->natms); }
void orc_sys_get_v(void* p, double* v) { memcpy(v, ((orc_sys*)p)->v, sizeof(double) * 3 * ((orc_sys*)p)->natms); }
void orc_sys_get_f(void* p, double* f) { memcpy(f, ((orc_sys*)p)->f, sizeof(double) * 3 * ((orc_sys*)p)->natms); }
void orc_sys_set_pair_wise(void* p, int pw) { ((orc_sys*)p)->pair_wise = pw; }
/* atoms.x_dof: per atom and component, nonzero when it is a degree of
   freedom; NULL clears it (every component free) */
void orc_sys_set_dof(void* p, const unsigned char* dof) {
    orc_sys* s = (orc_sys*)p;
    free(s->dof);
    s->dof = NULL;
    if (!dof) return;
    s->dof = (unsigned char*)malloc((size_t)3 * s->natms);
    memcpy(s->dof, dof, (size_t)3 * s->natms);
}
int orc_sys_nghost(void* p) { return ((orc_sys*)p)->nghost; }
int orc_sys_nrebuild(void* p) { return ((orc_sys*)p)->nrebuild; }

/* ForceFieldMD::pre_init  ff_md.cpp:80-94 */
static void ff_pre_init(orc_sys* s) {
    orc_eam* e = s->eam;
    int ne = e->nelem;
    double mc = 0.0;
    for (int i = 0; i < ne; i++)
        for (int j = 0; j < i + 1; j++) {
            double t = e->cut[i * ne + j];
            mc = OMAX(mc, t);
            s->cut_sq[i * ne + j] = s->cut_sq[j * ne + i] = t * t;
            t += s->skin;
            s->cut_sk_sq[i * ne + j] = s->cut_sk_sq[j * ne + i] = t * t;
        }
    /* DynamicMD::init  dynamic_md.cpp:41 */
    s->max_cut = mc + s->skin;
}

/* Update::list on one rank  exchange.h:833-875 (self communication,
   exchange.h:720,785-793).  Ghosts are made in s space, one dimension at a
   time: dir 0 images atoms with s < s_lo + max_cut_s to s+1, dir 1 images
   atoms with s >= s_hi - max_cut_s to s-1. */
static int ghost_list(orc_sys* s) {
    int n = s->natms;
    for (int d = 0; d < 3; d++) {
        double mcs = s->max_cut * s->depth_inv[d];
        /* Update::__reset  exchange.h:613-636 */
        int ncomms = (int)(mcs / 1.0) + 1;
        if (ncomms != 1) return fail("box thinner than cutoff+skin: multi-layer images are not supported");
        double bnd[2] = {0.0 + mcs, 1.0 - mcs};
        int last = n;
        for (int dir = 0; dir < 2; dir++) {
            int lo = 0, hi = last;
            for (int ic = 0; ic < ncomms; ic++) {
                int start = n;
                for (int a = lo; a < hi; a++) {
                    double sv = s->x[3 * a + d];
                    int take = dir == 0 ? (sv < bnd[0]) : (sv >= bnd[1]);
                    if (!take) continue;
                    sys_reserve(s, n + 1 > s->cap ? 2 * s->cap : s->cap);
                    memcpy(s->x + 3 * n, s->x + 3 * a, sizeof(double) * 3);
                    s->elem[n] = s->elem[a];
                    s->src[n] = a;
                    s->gdim[n] = d;
                    s->gsgn[n] = dir == 0 ? 1 : -1;
                    s->owner[n] = s->owner[a];
                    memcpy(s->img + 3 * n, s->img + 3 * a, sizeof(int) * 3);
                    n++;
                }
                lo = start;
                hi = n;
                for (int g = lo; g < hi; g++) {
                    if (dir == 0) {
                        ++s->x[3 * g + d];
                        s->img[3 * g + d] += 1;
                    } else {
                        --s->x[3 * g + d];
                        s->img[3 * g + d] -= 1;
                    }
                }
            }
        }
    }
    s->nghost = n - s->natms;
    return 0;
}

/* Update::update_w_x  exchange.h:796-813,880-887: ghost x = source x plus or
   minus the first d+1 components of row d of H, in creation order. */
static void ghost_refresh(orc_sys* s) {
    int n = s->natms + s->nghost;
    for (int g = s->natms; g < n; g++) {
        const double* src = s->x + 3 * s->src[g];
        double* xg = s->x + 3 * g;
        xg[0] = src[0];
        xg[1] = src[1];
        xg[2] = src[2];
        int d = s->gdim[g];
        for (int k = 0; k <= d; k++) {
            if (s->gsgn[g] > 0)
                xg[k] += s->H[d][k];
            else
                xg[k] -= s->H[d][k];
        }
    }
}

/* RSQ  xmath.h:2464-2510,3066: d0^2 + (d1^2 + d2^2) */
static inline double rsq3(const double* a, const double* b) {
    double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
    return d0 * d0 + (d1 * d1 + d2 * d2);
}

/* Cell<1>::setup / DO  cell.h:125-233 and NeighborMD::create_list
   neighbor_md.cpp:82-152.  Positions arrive in s; the cells are built in s,
   then s2x_all converts every position back to x and the lists are built. */
static int create_list(orc_sys* s) {
    const int M = 1;
    int nl = s->natms, nall = s->natms + s->nghost;
    double cut_s[3], cell_size[3];
    int npd[3], denom[3], ncells = 1;
    for (int d = 0; d < 3; d++) {
        cut_s[d] = s->max_cut * s->depth_inv[d];
        cell_size[d] = cut_s[d] / (double)M;
        npd[d] = (int)((1.0 - 0.0) / cell_size[d]) + 1 + 2 * M;
        denom[d] = ncells;
        ncells *= npd[d];
    }
    /* stencil order: countr[0] fastest  cell.h:38-78 */
    int rel[27], nrel = 0;
    for (int c2 = -1; c2 <= 1; c2++)
        for (int c1 = -1; c1 <= 1; c1++)
            for (int c0 = -1; c0 <= 1; c0++) rel[nrel++] = c0 * denom[0] + c1 * denom[1] + c2 * denom[2];
    int* head = (int*)malloc(sizeof(int) * ncells);
    for (int i = 0; i < ncells; i++) head[i] = -1;
    int* next = (int*)malloc(sizeof(int) * (nall ? nall : 1));
    int* cellv = (int*)malloc(sizeof(int) * (nall ? nall : 1));
    for (int i = nall - 1; i > nl - 1; i--) {
        const double* sv = s->x + 3 * i;
        int cn = 0;
        for (int d = 0; d < 3; d++) {
            int c;
            if (sv[d] < 0.0)
                c = OMIN((int)((sv[d] - (0.0 - cut_s[d])) / cell_size[d]), M - 1);
            else if (1.0 <= sv[d])
                c = OMIN(OMAX((int)((sv[d] - 0.0) / cell_size[d]), npd[d] - 2 * M - 1), npd[d] - 1 - M) + M;
            else
                c = OMIN((int)((sv[d] - 0.0) / cell_size[d]), npd[d] - 2 * M - 1) + M;
            cn += denom[d] * c;
        }
        cellv[i] = cn;
        next[i] = head[cn];
        head[cn] = i;
    }
    for (int i = nl - 1; i > -1; i--) {
        const double* sv = s->x + 3 * i;
        int cn = 0;
        for (int d = 0; d < 3; d++) cn += denom[d] * (OMIN((int)((sv[d] - 0.0) / cell_size[d]), npd[d] - 2 * M - 1) + M);
        cellv[i] = cn;
        next[i] = head[cn];
        head[cn] = i;
    }
    /* s2x_all */
    for (int i = 0; i < nall; i++) s2x_one(s->h6, s->x + 3 * i);

    free(s->nl_off);
    free(s->nl_cnt);
    s->nl_off = (int*)malloc(sizeof(int) * (nl + 1));
    s->nl_cnt = (int*)malloc(sizeof(int) * (nl ? nl : 1));
    long pos = 0;
    int ne = s->eam->nelem;
    for (int i = 0; i < nl; i++) {
        const double* xi = s->x + 3 * i;
        int ei = s->elem[i];
        s->nl_off[i] = (int)pos;
        int cnt = 0;
        for (int k = 0; k < nrel; k++) {
            int jc = cellv[i] + rel[k];
            for (int j = head[jc]; j != -1; j = next[j]) {
                if (i == j) continue;
                int keep = s->pair_wise ? (i < j) : 1;
                if (keep && rsq3(xi, s->x + 3 * j) < s->cut_sk_sq[ei * ne + s->elem[j]]) {
                    if (pos + 1 > s->nl_cap) {
                        s->nl_cap = s->nl_cap ? 2 * s->nl_cap : 1 << 16;
                        s->nl = (int*)realloc(s->nl, sizeof(int) * s->nl_cap);
                    }
                    s->nl[pos++] = j;
                    cnt++;
                }
            }
        }
        s->nl_cnt[i] = cnt;
    }
    s->nl_off[nl] = (int)pos;
    s->no_pairs = s->pair_wise ? pos : pos / 2;
    free(head);
    free(next);
    free(cellv);
    s->nrebuild++;
    return 0;
}

static void store_x0(orc_sys* s) { memcpy(s->x0, s->x, sizeof(double) * 3 * s->natms); }

/* x2s_lcl -> (full_xchng is a no-op on one rank) -> Update::list -> create_list */
static int rebuild(orc_sys* s) {
    for (int i = 0; i < s->natms; i++) x2s_one(s->b6, s->x + 3 * i);
    s->nghost = 0;
    if (ghost_list(s)) return -1;
    if (create_list(s)) return -1;
    store_x0(s);
    return 0;
}

/* DynamicMD::init  dynamic_md.cpp:34-53 */
int orc_sys_init_dynamic(void* p) {
    orc_sys* s = (orc_sys*)p;
    ff_pre_init(s);
    s->nrebuild = 0;
    return rebuild(s);
}

/* DynamicMD::decide  dynamic_md.cpp:90-105 (true: no rebuild needed) */
static int decide(orc_sys* s) {
    double skin_sq = 0.25 * s->skin * s->skin;
    for (int i = 0; i < s->natms; i++)
        if (rsq3(s->x0 + 3 * i, s->x + 3 * i) > skin_sq) return 0;
    return 1;
}

/* DynamicMD::update_w_x  dynamic_md.h:37-68 (box fixed) */
static int dynamic_update(orc_sys* s) {
    if (decide(s)) {
        ghost_refresh(s);
        return 0;
    }
    return rebuild(s);
}
int orc_sys_update(void* p) { return dynamic_update((orc_sys*)p); }

/* full neighbour set of every local atom, as (owner id, image shift):
   entries are written as 4 ints per neighbour: owner, n0, n1, n2 */
long orc_sys_neighbors(void* p, int* counts, int* entries) {
    orc_sys* s = (orc_sys*)p;
    long w = 0;
    for (int i = 0; i < s->natms; i++) {
        counts[i] = s->nl_cnt[i];
        for (int k = s->nl_off[i]; k < s->nl_off[i] + s->nl_cnt[i]; k++) {
            int j = s->nl[k];
            if (entries) {
                entries[4 * w] = s->owner[j];
                entries[4 * w + 1] = s->img[3 * j];
                entries[4 * w + 2] = s->img[3 * j + 1];
                entries[4 * w + 3] = s->img[3 * j + 2];
            }
            w++;
        }
    }
    return w;
}

/* ------------------------------------------------------------------------ */
/* EAM force and energy                                                      */
/* ------------------------------------------------------------------------ */
/* ForceFieldEAM::__force_calc  ff_eam.cpp:65-240 (half list, ghost rule) */
static void eam_force_half(orc_sys* s) {
    orc_eam* e = s->eam;
    const int ne = e->nelem, nlc = s->natms;
    if (s->dr_cap < s->no_pairs) {
        free(s->drhoi);
        free(s->drhoj);
        s->dr_cap = s->no_pairs;
        s->drhoi = (double*)malloc(sizeof(double) * (s->dr_cap ? s->dr_cap : 1));
        s->drhoj = (double*)malloc(sizeof(double) * (s->dr_cap ? s->dr_cap : 1));
    }
    double* x = s->x;
    double* f = s->f;
    double* rho = s->rho;
    double* dF = s->dF;
    double* v = s->vec;
    for (int i = 0; i < nlc; i++) rho[i] = 0.0;
    long ist = 0;
    for (int i = 0; i < nlc; i++) {
        int ei = s->elem[i];
        for (int jj = 0; jj < s->nl_cnt[i]; jj++) {
            int j = s->nl[s->nl_off[i] + jj];
            int ej = s->elem[j];
            double dx0 = x[3 * i] - x[3 * j];
            double dx1 = x[3 * i + 1] - x[3 * j + 1];
            double dx2 = x[3 * i + 2] - x[3 * j + 2];
            double rsq = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
            s->drhoi[ist] = s->drhoj[ist] = 0.0;
            if (rsq >= s->cut_sq[ei * ne + ej]) {
                ist++;
                continue;
            }
            double r = sqrt(rsq);
            double r_inv = 1.0 / r;
            double pp = r * e->dr_inv;
            size_t m = (size_t)pp;
            m = OMIN(m, (size_t)e->nr - 2);
            pp -= (double)m;
            pp = OMIN(pp, 1.0);
            double* c = RHO(e, ej, ei)[m];
            double rho_i = ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
            double drho_i_dr = ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->dr_inv;
            c = RHO(e, ei, ej)[m];
            double rho_j = ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
            double drho_j_dr = ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->dr_inv;
            c = RPHI(e, ei, ej)[m];
            double z2p = ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->dr_inv;
            double z2 = ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
            double phi = z2 * r_inv;
            double dphi_dr = z2p * r_inv - phi * r_inv;
            rho[i] += rho_i;
            if (j < nlc) rho[j] += rho_j;
            double fpair = -dphi_dr * r_inv;
            f[3 * i] += fpair * dx0;
            f[3 * i + 1] += fpair * dx1;
            f[3 * i + 2] += fpair * dx2;
            if (j < nlc) {
                f[3 * j] -= fpair * dx0;
                f[3 * j + 1] -= fpair * dx1;
                f[3 * j + 2] -= fpair * dx2;
            }
            if (j >= nlc) {
                fpair *= 0.5;
                phi *= 0.5;
            }
            v[0] += phi;
            v[1] -= fpair * dx0 * dx0;
            v[2] -= fpair * dx0 * dx1;
            v[3] -= fpair * dx0 * dx2;
            v[4] -= fpair * dx1 * dx1;
            v[5] -= fpair * dx1 * dx2;
            v[6] -= fpair * dx2 * dx2;
            s->drhoi[ist] = -drho_i_dr * r_inv;
            s->drhoj[ist] = -drho_j_dr * r_inv;
            ist++;
        }
        double pp = rho[i] * e->drho_inv;
        size_t m = (size_t)pp;
        m = OMIN(m, (size_t)e->nrho - 2);
        pp -= (double)m;
        pp = OMIN(pp, 1.0);
        double* c = FTAB(e, ei)[m];
        double tmp1 = ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->drho_inv;
        double tmp0 = ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
        if (rho[i] > e->rho_max) tmp0 += tmp1 * (rho[i] - e->rho_max);
        v[0] += tmp0;
        dF[i] = tmp1;
    }
    /* update(dF_ptr): forward F'(rho) of each owner to its ghosts */
    for (int g = nlc; g < nlc + s->nghost; g++) dF[g] = dF[s->src[g]];
    ist = 0;
    for (int i = 0; i < nlc; i++) {
        for (int jj = 0; jj < s->nl_cnt[i]; jj++) {
            if (s->drhoi[ist] != 0.0 || s->drhoj[ist] != 0.0) {
                int j = s->nl[s->nl_off[i] + jj];
                double fpair = dF[i] * s->drhoi[ist] + dF[j] * s->drhoj[ist];
                double dx0 = x[3 * i] - x[3 * j];
                double dx1 = x[3 * i + 1] - x[3 * j + 1];
                double dx2 = x[3 * i + 2] - x[3 * j + 2];
                f[3 * i] += dx0 * fpair;
                f[3 * i + 1] += dx1 * fpair;
                f[3 * i + 2] += dx2 * fpair;
                if (j < nlc) {
                    f[3 * j] -= dx0 * fpair;
                    f[3 * j + 1] -= dx1 * fpair;
                    f[3 * j + 2] -= dx2 * fpair;
                }
                if (j >= nlc) fpair *= 0.5;
                v[1] -= fpair * dx0 * dx0;
                v[2] -= fpair * dx0 * dx1;
                v[3] -= fpair * dx0 * dx2;
                v[4] -= fpair * dx1 * dx1;
                v[5] -= fpair * dx1 * dx2;
                v[6] -= fpair * dx2 * dx2;
            }
            ist++;
        }
    }
}

/* ForceFieldEAM::__energy_calc  ff_eam.cpp:244-318 */
static double eam_energy_half(orc_sys* s) {
    orc_eam* e = s->eam;
    const int ne = e->nelem, nlc = s->natms;
    double* x = s->x;
    double* rho = s->rho;
    double en = 0.0;
    for (int i = 0; i < nlc; i++) rho[i] = 0.0;
    for (int i = 0; i < nlc; i++) {
        int ei = s->elem[i];
        for (int jj = 0; jj < s->nl_cnt[i]; jj++) {
            int j = s->nl[s->nl_off[i] + jj];
            int ej = s->elem[j];
            double dx0 = x[3 * i] - x[3 * j];
            double dx1 = x[3 * i + 1] - x[3 * j + 1];
            double dx2 = x[3 * i + 2] - x[3 * j + 2];
            double rsq = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
            if (rsq < s->cut_sq[ei * ne + ej]) {
                double r = sqrt(rsq);
                double pp = r * e->dr_inv;
                size_t m = (size_t)pp;
                m = OMIN(m, (size_t)e->nr - 2);
                pp -= (double)m;
                pp = OMIN(pp, 1.0);
                double* c = RPHI(e, ei, ej)[m];
                double phi = (((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0]) / r;
                c = RHO(e, ej, ei)[m];
                rho[i] += ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
                if (j < nlc) {
                    c = RHO(e, ei, ej)[m];
                    rho[j] += ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
                    en += phi;
                } else
                    en += 0.5 * phi;
            }
        }
        double pp = rho[i] * e->drho_inv;
        size_t m = (size_t)pp;
        m = OMIN(m, (size_t)e->nrho - 2);
        pp -= (double)m;
        pp = OMIN(pp, 1.0);
        double* c = FTAB(e, ei)[m];
        double tmp0 = ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
        if (rho[i] > e->rho_max) tmp0 += ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->drho_inv * (rho[i] - e->rho_max);
        en += tmp0;
    }
    return en;
}

/* ForceFieldMD::force_calc / derivative  ff_md.cpp:70-77,125-144,159-179
   (no dof mask: every coordinate is free) */
static void force_calc(orc_sys* s) {
    int n = s->natms + s->nghost;
    memset(s->f, 0, sizeof(double) * 3 * n);
    memset(s->vec, 0, sizeof(s->vec));
    eam_force_half(s);
    double* vv = s->vec;
    for (int i = 0; i < 6; i++) vv[i + 1] *= -1.0;
    /* DyadicV_2_MSY: voigt [xx,xy,xz,yy,yz,zz] */
    static const int ia[6] = {0, 0, 0, 1, 1, 2}, ja[6] = {0, 1, 2, 1, 2, 2};
    for (int k = 0; k < 6; k++) s->F_H[ia[k]][ja[k]] = s->F_H[ja[k]][ia[k]] = vv[k + 1];
    s->pe = vv[0];
    double vol_neg = -s->vol;
    for (int i = 0; i < 6; i++) vv[i + 1] /= vol_neg;
    for (int k = 0; k < 6; k++) s->S_pe[ia[k]][ja[k]] = s->S_pe[ja[k]][ia[k]] = vv[k + 1];
    /* components without a degree of freedom carry no force  ff_md.cpp:138-144 */
    if (s->dof)
        for (int q = 0; q < 3 * s->natms; q++)
            if (!s->dof[q]) s->f[q] = 0.0;
}

/* force_calc over the full list with nthreads threads (timing baseline);
   the sign and volume conventions of ForceFieldMD::force_calc */
double orc_sys_force_full(void* p, double* out7, int nthreads);
static void force_calc_threads(orc_sys* s, int nthreads) {
    double o[7];
    orc_sys_force_full(s, o, nthreads);
    static const int ia[6] = {0, 0, 0, 1, 1, 2}, ja[6] = {0, 1, 2, 1, 2, 2};
    s->pe = o[0];
    for (int k = 0; k < 6; k++) {
        s->F_H[ia[k]][ja[k]] = s->F_H[ja[k]][ia[k]] = o[k + 1];
        s->S_pe[ia[k]][ja[k]] = s->S_pe[ja[k]][ia[k]] = o[k + 1] / -s->vol;
    }
}

/* returns pe; out7 = [pe, F_H voigt (xx,xy,xz,yy,yz,zz)] */
double orc_sys_force(void* p, double* out7) {
    orc_sys* s = (orc_sys*)p;
    force_calc(s);
    if (out7) {
        out7[0] = s->pe;
        out7[1] = s->F_H[0][0];
        out7[2] = s->F_H[0][1];
        out7[3] = s->F_H[0][2];
        out7[4] = s->F_H[1][1];
        out7[5] = s->F_H[1][2];
        out7[6] = s->F_H[2][2];
    }
    return s->pe;
}

/* ForceFieldMD::value  ff_md.cpp:148-155 */
double orc_sys_energy(void* p) { return eam_energy_half((orc_sys*)p); }

void orc_sys_get_rho(void* p, double* rho, double* dF) {
    orc_sys* s = (orc_sys*)p;
    if (rho) memcpy(rho, s->rho, sizeof(double) * s->natms);
    if (dF) memcpy(dF, s->dF, sizeof(double) * s->natms);
}

/* ------------------------------------------------------------------------ */
/* Full-list, multi-threaded restatement used only as the timed CPU         */
/* baseline: each atom sums over its full neighbour list (same arithmetic    */
/* per pair as ff_eam.cpp:109-160), so threads need no atomics.              */
/* Requires orc_sys_set_pair_wise(sys, 0) before orc_sys_init_dynamic.       */
/* ------------------------------------------------------------------------ */
double orc_sys_force_full(void* p, double* out7, int nthreads) {
    orc_sys* s = (orc_sys*)p;
    orc_eam* e = s->eam;
    const int ne = e->nelem, nlc = s->natms;
    double* x = s->x;
    double e_tot = 0.0, w[6] = {0, 0, 0, 0, 0, 0};
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static) reduction(+ : e_tot)
    for (int i = 0; i < nlc; i++) {
        int ei = s->elem[i];
        double ri = 0.0, ep = 0.0;
        for (int jj = 0; jj < s->nl_cnt[i]; jj++) {
            int j = s->nl[s->nl_off[i] + jj];
            int ej = s->elem[j];
            double dx0 = x[3 * i] - x[3 * j], dx1 = x[3 * i + 1] - x[3 * j + 1], dx2 = x[3 * i + 2] - x[3 * j + 2];
            double rsq = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
            if (rsq >= s->cut_sq[ei * ne + ej]) continue;
            double r = sqrt(rsq), pp = r * e->dr_inv;
            size_t m = OMIN((size_t)pp, (size_t)e->nr - 2);
            pp = OMIN(pp - (double)m, 1.0);
            double* c = RHO(e, ej, ei)[m];
            ri += ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
            c = RPHI(e, ei, ej)[m];
            ep += 0.5 * ((((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0]) / r);
        }
        s->rho[i] = ri;
        double pp = ri * e->drho_inv;
        size_t m = OMIN((size_t)pp, (size_t)e->nrho - 2);
        pp = OMIN(pp - (double)m, 1.0);
        double* c = FTAB(e, ei)[m];
        double t1 = ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->drho_inv;
        double t0 = ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
        if (ri > e->rho_max) t0 += t1 * (ri - e->rho_max);
        s->dF[i] = t1;
        e_tot += t0 + ep;
    }
#pragma omp parallel for schedule(static) reduction(+ : w[:6])
    for (int i = 0; i < nlc; i++) {
        int ei = s->elem[i];
        double fi0 = 0, fi1 = 0, fi2 = 0;
        for (int jj = 0; jj < s->nl_cnt[i]; jj++) {
            int j = s->nl[s->nl_off[i] + jj];
            int ej = s->elem[j];
            int jo = s->owner[j];
            double dx0 = x[3 * i] - x[3 * j], dx1 = x[3 * i + 1] - x[3 * j + 1], dx2 = x[3 * i + 2] - x[3 * j + 2];
            double rsq = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
            if (rsq >= s->cut_sq[ei * ne + ej]) continue;
            double r = sqrt(rsq), r_inv = 1.0 / r, pp = r * e->dr_inv;
            size_t m = OMIN((size_t)pp, (size_t)e->nr - 2);
            pp = OMIN(pp - (double)m, 1.0);
            double* c = RHO(e, ej, ei)[m];
            double dri = ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->dr_inv;
            c = RHO(e, ei, ej)[m];
            double drj = ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->dr_inv;
            c = RPHI(e, ei, ej)[m];
            double z2p = ((3.0 * c[3] * pp + 2.0 * c[2]) * pp + c[1]) * e->dr_inv;
            double z2 = ((c[3] * pp + c[2]) * pp + c[1]) * pp + c[0];
            double phi = z2 * r_inv, dphi = z2p * r_inv - phi * r_inv;
            double fp = -(dphi + s->dF[i] * dri + s->dF[jo] * drj) * r_inv;
            fi0 += fp * dx0;
            fi1 += fp * dx1;
            fi2 += fp * dx2;
            fp *= 0.5;
            w[0] += fp * dx0 * dx0;
            w[1] += fp * dx0 * dx1;
            w[2] += fp * dx0 * dx2;
            w[3] += fp * dx1 * dx1;
            w[4] += fp * dx1 * dx2;
            w[5] += fp * dx2 * dx2;
        }
        s->f[3 * i] = fi0;
        s->f[3 * i + 1] = fi1;
        s->f[3 * i + 2] = fi2;
    }
    if (out7) {
        out7[0] = e_tot;
        for (int k = 0; k < 6; k++) out7[k + 1] = w[k];
    }
    return e_tot;
}

/* ------------------------------------------------------------------------ */
/* NVT molecular dynamics: MDNVT  md_nvt.cpp:51-141,256-340,383-480 and     */
/* ThermostatNHC  thermostat.cpp:20-143                                      */
/* ------------------------------------------------------------------------ */
typedef struct {
    double ddt, ddt2, freq_sq, t_relax;
    int L, niters;
    double eta_d[16];
} nhc_t;

static void nhc_init(nhc_t* t, double dt, double t_relax, int L, int niters) {
    t->ddt = dt / (double)niters;
    t->ddt2 = 0.5 * dt / (double)niters;
    t->freq_sq = 1.0 / (t_relax * t_relax);
    t->t_relax = t_relax;
    t->L = L;
    t->niters = niters;
    for (int i = 0; i < 16; i++) t->eta_d[i] = 0.0;
}

static double nhc_f(double x) {
    if (fabs(x) < 0.015625) return 1.0 + x / 2.0 + x * x / 6.0 + x * x * x / 24.0;
    return (exp(x) - 1.0) / x;
}

static double nhc_step(nhc_t* t, double T_r, int ndof) {
    double rescale = 1.0, prev_fac, tmp;
    double* eta = t->eta_d;
    int L = t->L;
    if (L == 1) {
        for (int it = 0; it < t->niters; it++) {
            eta[0] += t->ddt2 * t->freq_sq * (T_r - 1.0);
            prev_fac = exp(-t->ddt * eta[0]);
            rescale *= prev_fac;
            T_r *= prev_fac * prev_fac;
            eta[0] += t->ddt2 * t->freq_sq * (T_r - 1.0);
        }
        return rescale;
    }
    for (int it = 0; it < t->niters; it++) {
        eta[L - 1] += t->ddt2 * (eta[L - 2] * eta[L - 2] - t->freq_sq);
        prev_fac = -eta[L - 1];
        for (int ich = L - 2; ich > 0; ich--) {
            eta[ich] += t->ddt2 * nhc_f(prev_fac * t->ddt2) * (prev_fac * eta[ich] + eta[ich - 1] * eta[ich - 1] - t->freq_sq);
            prev_fac = -eta[ich];
        }
        eta[0] += t->ddt2 * nhc_f(prev_fac * t->ddt2) * (prev_fac * eta[0] + t->freq_sq * (T_r - 1.0));
        prev_fac = -eta[0];
        tmp = exp(t->ddt * prev_fac);
        rescale *= tmp;
        T_r *= tmp * tmp;
        prev_fac = (T_r - 1.0) * t->freq_sq;
        eta[0] += t->ddt2 * nhc_f(-eta[1] * t->ddt2) * (-eta[1] * eta[0] + prev_fac);
        prev_fac = ndof * eta[0] * eta[0] - t->freq_sq;
        for (int ich = 1; ich < L - 1; ich++) {
            eta[ich] += t->ddt2 * nhc_f(-eta[ich + 1] * t->ddt2) * (-eta[ich + 1] * eta[ich] + prev_fac);
            prev_fac = eta[ich] * eta[ich] - t->freq_sq;
        }
        eta[L - 1] += t->ddt2 * prev_fac;
    }
    return rescale;
}

/* Algebra::DyadicV(scl,x,dyad)  xmath.h:2131-2200 */
static void dyadic_add(double m, const double* v, double* d) {
    d[0] += v[0] * v[0] * m;
    d[1] += v[0] * v[1] * m;
    d[2] += v[0] * v[2] * m;
    d[3] += v[1] * v[1] * m;
    d[4] += v[1] * v[2] * m;
    d[5] += v[2] * v[2] * m;
}

/*
 * md.nvt(T,dt).run(atoms,nsteps) for an atoms object whose velocities are
 * already set.  eta_d (length L, in/out) is the chain state carried between
 * runs.  If thermo is not NULL, it receives per step (nsteps+1 rows, row 0 =
 * before the first step): [pe, T_part, mvv xx..zz (6), virial F_H (6)].
 * Returns the number of neighbour-list rebuilds, or -1.
 */
int orc_md_nvt_run(void* p, double T, double dt, double kB, double t_relax, int L, int niters,
                   int nsteps, double* eta_io, double* thermo, int threads, double* loop_seconds) {
    orc_sys* s = (orc_sys*)p;
    /* threads > 0: full-list force and integrator loops on that many
       threads (the timed CPU baseline); otherwise the reference's serial
       half-list algorithm */
    if (threads > 0) s->pair_wise = 0;
#define FORCE_CALC() (threads > 0 ? force_calc_threads(s, threads) : force_calc(s))
    if (isnan(kB)) return fail("boltzmann constant should be set prior to MD");
    if (L < 1 || L > 16 || niters < 1) return fail("invalid thermostat parameters");
    nhc_t th;
    nhc_init(&th, dt / 2.0, t_relax, L, niters);
    if (eta_io)
        for (int i = 0; i < L; i++) th.eta_d[i] = eta_io[i];
    const int n = s->natms;
    const double dt2 = dt / 2.0;
    /* pre_init  md_nvt.cpp:256-340 (with x_dof: the frozen components leave
       the degrees of freedom and the kinetic tensor) */
    const unsigned char* dof = s->dof;
    if (dof && threads > 0) return fail("x_dof is restated on the serial path only");
    int ndof_part = n * 3;
    int dofs[3] = {1, 1, 1};
    if (dof)
        for (int i = 0; i < n; i++)
            for (int j = 0; j < 3; j++)
                if (!dof[3 * i + j]) {
                    ndof_part--;
                    dofs[j] = 0;
                }
    double mvv[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; i++) {
        double w[3];
        for (int j = 0; j < 3; j++) w[j] = (!dof || dof[3 * i + j]) ? s->v[3 * i + j] : 0.0;
        dyadic_add(s->masses[s->elem[i]], w, mvv);
    }
    double T_part = (mvv[0] + (mvv[3] + mvv[5])) / (ndof_part * kB);
    /* DynamicMD::init */
    if (orc_sys_init_dynamic(s)) return -1;
    /* run  md_nvt.cpp:383-480 */
    FORCE_CALC();
    int row = 0;
#define THERMO_ROW()                                                         \
    if (thermo) {                                                            \
        double* tr = thermo + (size_t)14 * row;                              \
        tr[0] = s->pe;                                                       \
        tr[1] = T_part;                                                      \
        for (int k = 0; k < 6; k++) tr[2 + k] = mvv[k];                      \
        tr[8] = s->F_H[0][0]; tr[9] = s->F_H[0][1]; tr[10] = s->F_H[0][2];   \
        tr[11] = s->F_H[1][1]; tr[12] = s->F_H[1][2]; tr[13] = s->F_H[2][2]; \
    }                                                                        \
    row++;
    THERMO_ROW();
    double fac, fac_x_d = 1.0;
    double t0 = now_seconds();
    for (int istep = 0; istep < nsteps; istep++) {
        fac_x_d *= fac = nhc_step(&th, T_part / T, ndof_part);
        fac *= fac;
        for (int k = 0; k < 6; k++) mvv[k] *= fac;
        T_part *= fac;
        /* update_x_d__x  md_nvt.cpp:70-102 */
        double dxl[3] = {0, 0, 0};
        if (threads > 0) {
            double d0 = 0, d1 = 0, d2 = 0;
#pragma omp parallel for schedule(static) num_threads(threads) reduction(+ : d0, d1, d2)
            for (int i = 0; i < n; i++) {
                double mi = s->masses[s->elem[i]];
                double* xd = s->v + 3 * i;
                double* xx = s->x + 3 * i;
                double* ff = s->f + 3 * i;
                double dd[3];
                for (int j = 0; j < 3; j++) {
                    xd[j] = xd[j] * fac_x_d + ff[j] * dt2 / mi;
                    dd[j] = xd[j] * dt;
                    xx[j] += dd[j];
                }
                d0 += dd[0];
                d1 += dd[1];
                d2 += dd[2];
            }
            dxl[0] = d0;
            dxl[1] = d1;
            dxl[2] = d2;
        } else {
            /* update_x_d__x(_w_dof)  md_nvt.cpp:70-102,144-180: a frozen
               component keeps its velocity and still drifts */
            for (int i = 0; i < n; i++) {
                double mi = s->masses[s->elem[i]];
                double* xd = s->v + 3 * i;
                double* xx = s->x + 3 * i;
                double* ff = s->f + 3 * i;
                for (int j = 0; j < 3; j++) {
                    if (!dof || dof[3 * i + j]) xd[j] = xd[j] * fac_x_d + ff[j] * dt2 / mi;
                    dxl[j] += xd[j] * dt;
                    xx[j] += xd[j] * dt;
                }
            }
        }
        double natms = (double)n;
        for (int j = 0; j < 3; j++) dxl[j] = dofs[j] ? dxl[j] / natms : 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < 3; j++) s->x[3 * i + j] -= dxl[j];
        if (dynamic_update(s)) return -1;
        FORCE_CALC();
        /* update_x_d(_w_dof)  md_nvt.cpp:106-128,184-215 */
        for (int k = 0; k < 6; k++) mvv[k] = 0.0;
        for (int i = 0; i < n; i++) {
            double mi = s->masses[s->elem[i]];
            double* xd = s->v + 3 * i;
            double* ff = s->f + 3 * i;
            double w[3];
            for (int j = 0; j < 3; j++) {
                if (!dof || dof[3 * i + j]) {
                    xd[j] += ff[j] * dt2 / mi;
                    w[j] = xd[j];
                } else {
                    w[j] = 0.0;
                }
            }
            dyadic_add(mi, w, mvv);
        }
        T_part = (mvv[0] + (mvv[3] + mvv[5])) / (ndof_part * kB);
        fac_x_d = fac = nhc_step(&th, T_part / T, ndof_part);
        fac *= fac;
        for (int k = 0; k < 6; k++) mvv[k] *= fac;
        T_part *= fac;
        THERMO_ROW();
    }
    if (loop_seconds) *loop_seconds = now_seconds() - t0;
    /* update_x_d_final(_w_dof)  md_nvt.cpp:51-66 */
    for (int i = 0; i < 3 * n; i++)
        if (!dof || dof[i]) s->v[i] *= fac_x_d;
    if (eta_io)
        for (int i = 0; i < L; i++) eta_io[i] = th.eta_d[i];
#undef THERMO_ROW
#undef FORCE_CALC
    return s->nrebuild;
}

/* ------------------------------------------------------------------------ */
/* NST molecular dynamics: MDNST::run  md_nst.cpp:374-450                    */
/* ------------------------------------------------------------------------ */
/* MDMath f, df, ddf  md_nst.cpp:848-873 */
static double mdm_f(double x) {
    if (fabs(x) < 0.015625) return 1.0 + x / 2.0 + x * x / 6.0 + x * x * x / 24.0;
    return (exp(x) - 1.0) / x;
}
static double mdm_df(double x) {
    if (fabs(x) < 0.015625) return 0.5 + x / 3.0 + x * x / 8.0 + x * x * x / 30.0;
    double e = exp(x);
    return (e - (e - 1.0) / x) / x;
}
static double mdm_ddf(double x) {
    if (fabs(x) < 0.015625) return 1.0 / 3.0 + x / 4.0 + x * x / 10.0 + x * x * x / 36.0;
    double e = exp(x);
    return (e - 2.0 * ((e - (e - 1.0) / x) / x)) / x;
}
static double dd_exp(double x, double y, double fx, double fy) {
    if (fabs(x - y) < sqrt(DBL_EPSILON)) return exp(0.5 * (x + y));
    return (fx - fy) / (x - y);
}
static double dd_f(double x, double y, double fx, double fy) {
    if (fabs(x - y) < sqrt(DBL_EPSILON * mdm_f(0.5 * (x + y)) / mdm_ddf(0.5 * (x + y)))) return mdm_df(0.5 * (x + y));
    return (fx - fy) / (x - y);
}
static double dd_f3(double x, double y, double z, double f_yz, double f_zx, double f_xy) {
    double d = mdm_ddf((x + y + z) / 3.0);
    double lim = sqrt(DBL_EPSILON * mdm_f((x + y + z) / 3.0) / d);
    if (fabs(x - z) > lim) return (f_xy - f_yz) / (x - z);
    if (fabs(y - x) > lim) return (f_yz - f_zx) / (y - x);
    if (fabs(z - y) > lim) return (f_zx - f_xy) / (z - y);
    return d;
}
static double dd_exp3(double x, double y, double z, double f_yz, double f_zx, double f_xy) {
    const double se = sqrt(DBL_EPSILON);
    if (fabs(x - z) > se) return (f_xy - f_yz) / (x - z);
    if (fabs(y - x) > se) return (f_yz - f_zx) / (y - x);
    if (fabs(z - y) > se) return (f_zx - f_xy) / (z - y);
    return exp((x + y + z) / 3.0);
}

/* MDMath::calc (3x3)  md_nst.cpp:887-1000: functions of the lower-
   triangular A through divided differences: E = exp(-dt2 (A + a)),
   F0 = dt2 f(-dt2 (A + a)) (off-diagonal sign as there), F1 = dt f(dt A) */
static void mdm_calc(double a, double dt, double dt2, double A[3][3], double E[3][3], double F0[3][3],
                     double F1[3][3]) {
    double x = -dt2 * (A[0][0] + a), y = -dt2 * (A[1][1] + a), z = -dt2 * (A[2][2] + a);
    double X = dt * A[0][0], Y = dt * A[1][1], Z = dt * A[2][2];
    memset(E, 0, sizeof(double) * 9);
    memset(F0, 0, sizeof(double) * 9);
    memset(F1, 0, sizeof(double) * 9);
    F0[0][0] = mdm_f(x); F0[1][1] = mdm_f(y); F0[2][2] = mdm_f(z);
    F1[0][0] = mdm_f(X); F1[1][1] = mdm_f(Y); F1[2][2] = mdm_f(Z);
    E[0][0] = exp(x); E[1][1] = exp(y); E[2][2] = exp(z);
    double f_yz = 0, f_zx = 0, f_xy = 0, F_yz = 0, F_zx = 0, F_xy = 0, g_yz = 0, g_zx = 0, g_xy = 0;
    if (A[2][1] != 0.0) {
        f_yz = dd_f(y, z, F0[1][1], F0[2][2]);
        F_yz = dd_f(Y, Z, F1[1][1], F1[2][2]);
        g_yz = dd_exp(y, z, E[1][1], E[2][2]);
    }
    if (A[2][0] != 0.0) {
        f_zx = dd_f(z, x, F0[2][2], F0[0][0]);
        F_zx = dd_f(Z, X, F1[2][2], F1[0][0]);
        g_zx = dd_exp(z, x, E[2][2], E[0][0]);
    }
    if (A[1][0] != 0.0) {
        f_xy = dd_f(x, y, F0[0][0], F0[1][1]);
        F_xy = dd_f(X, Y, F1[0][0], F1[1][1]);
        g_xy = dd_exp(x, y, E[0][0], E[1][1]);
    }
    F0[0][0] *= dt2; F0[1][1] *= dt2; F0[2][2] *= dt2;
    F0[2][1] = -A[2][1] * dt2 * dt2 * f_yz;
    F0[2][0] = -A[2][0] * dt2 * dt2 * f_zx;
    F0[1][0] = -A[1][0] * dt2 * dt2 * f_xy;
    F1[0][0] *= dt; F1[1][1] *= dt; F1[2][2] *= dt;
    F1[2][1] = A[2][1] * dt * dt * F_yz;
    F1[2][0] = A[2][0] * dt * dt * F_zx;
    F1[1][0] = A[1][0] * dt * dt * F_xy;
    E[2][1] = -A[2][1] * dt2 * g_yz;
    E[2][0] = -A[2][0] * dt2 * g_zx;
    E[1][0] = -A[1][0] * dt2 * g_xy;
    if (A[1][0] == 0.0 || A[2][1] == 0.0) return;
    F0[2][0] += dt2 * dt2 * dt2 * A[2][1] * A[1][0] * dd_f3(x, y, z, f_yz, f_zx, f_xy);
    F1[2][0] += dt * dt * dt * A[2][1] * A[1][0] * dd_f3(X, Y, Z, F_yz, F_zx, F_xy);
    E[2][0] += dt2 * dt2 * A[2][1] * A[1][0] * dd_exp3(x, y, z, g_yz, g_zx, g_xy);
}

/* row vector times lower-triangular matrix, V_mul_MLT order */
static void v_mlt(const double* v, double M[3][3], double* out) {
    double o0 = M[0][0] * v[0] + (M[1][0] * v[1] + M[2][0] * v[2]);
    double o1 = M[1][1] * v[1] + M[2][1] * v[2];
    double o2 = M[2][2] * v[2];
    out[0] = o0; out[1] = o1; out[2] = o2;
}
/* C = L R (lower triangular), MLT_mul_MLT order */
static void mlt_mul(double L[3][3], double R[3][3], double C[3][3]) {
    double T[3][3] = {{0}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j <= i; j++) {
            double t = R[i][j] * L[i][i];
            for (int k = i - 1; k >= j; k--) t = R[k][j] * L[i][k] + t;
            T[i][j] = t;
        }
    memcpy(C, T, sizeof(T));
}

typedef struct {
    double T, dt, dt2, kB;
    int ndof_part, ndof_baro;
    double S[3][3], S_dev[3][3], s_hyd, tau[3][3], V_H[3][3], V_H_prefac[3][3];
    int S_dof[3][3];
    double B_ref[3][3], vol_ref, T_baro, T_part, mvv[6];
} nst_t;

/* MDNST::update_V_H  md_nst.cpp:315-341 */
static void nst_update_V_H(nst_t* q, orc_sys* s) {
    double M0[3][3], M1[3][3], M2[3][3];
    mlt_mul(q->B_ref, s->H, M0);
    /* MUT_mul_MSY_mul_MLT: M1 = S_dev M0, M2 = M0^T M1 */
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double t = 0.0;
            for (int k = j; k < 3; k++) t += q->S_dev[i][k] * M0[k][j];
            M1[i][j] = t;
        }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double t = 0.0;
            for (int k = i; k < 3; k++) t += M0[k][i] * M1[k][j];
            M2[i][j] = t;
        }
    for (int i = 0; i < 3; i++)
        if (q->S_dof[i][i]) q->V_H[i][i] += (q->kB * q->T_part + s->vol * q->s_hyd) * q->V_H_prefac[i][i] * q->dt2;
    q->T_baro = 0.0;
    static const int vo[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j <= i; j++)
            if (q->S_dof[i][j]) {
                q->V_H[i][j] += (q->vol_ref * M2[i][j] - s->vol * s->S_pe[i][j] + q->mvv[vo[i][j]]) *
                                q->V_H_prefac[i][j] * q->dt2;
                q->T_baro += q->V_H[i][j] * q->V_H[i][j] * q->tau[i][j] * q->tau[i][j];
            }
    q->T_baro *= q->ndof_part * q->T / q->ndof_baro;
}

/* MDNST::update_x_d__x__x_d  md_nst.cpp:70-145 (no per-atom dof mask) */
static int nst_step_x(nst_t* q, orc_sys* s, double xi) {
    double M0[3][3], M1[3][3], M2[3][3];
    double tr = q->V_H[0][0] + q->V_H[1][1] + q->V_H[2][2];
    mdm_calc(tr / q->ndof_part, q->dt, q->dt2, q->V_H, M0, M1, M2);
    const int n = s->natms;
    double dx[3] = {0, 0, 0};
    for (int i = 0; i < n; i++) {
        double m_inv = 1.0 / s->masses[s->elem[i]];
        double* xd = s->v + 3 * i;
        double* xx = s->x + 3 * i;
        double* ff = s->f + 3 * i;
        double a[3], b[3], v0[3], w[3];
        /* SCL_V_mul_MLT(xi, x_d, MLT0) in place (xmath.h:1049-1053,1077-1080)
           applies xi to the last component only */
        v_mlt(xd, M0, a);
        a[2] = xi * xd[2] * M0[2][2];
        v_mlt(ff, M1, b);
        for (int k = 0; k < 3; k++) xd[k] = a[k] + m_inv * b[k];
        v_mlt(xx, q->V_H, v0);
        for (int k = 0; k < 3; k++) v0[k] += xd[k];
        v_mlt(v0, M2, w);
        for (int k = 0; k < 3; k++) {
            xx[k] += w[k];
            dx[k] += w[k];
        }
    }
    for (int k = 0; k < 3; k++) dx[k] /= (double)n;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) s->x[3 * i + k] -= dx[k];
    /* H <- H (I + M2 V_H) */
    double G[3][3];
    mlt_mul(M2, q->V_H, G);
    for (int k = 0; k < 3; k++) G[k][k] += 1.0;
    mlt_mul(s->H, G, s->H);
    update_H(s);
    if (rebuild(s)) return -1;
    force_calc(s);
    for (int k = 0; k < 6; k++) q->mvv[k] = 0.0;
    for (int i = 0; i < n; i++) {
        double mi = s->masses[s->elem[i]], m_inv = 1.0 / mi;
        double* xd = s->v + 3 * i;
        double a[3], b[3];
        v_mlt(xd, M0, a);
        v_mlt(s->f + 3 * i, M1, b);
        for (int k = 0; k < 3; k++) xd[k] = a[k] + m_inv * b[k];
        dyadic_add(mi, xd, q->mvv);
    }
    q->T_part = (q->mvv[0] + (q->mvv[3] + q->mvv[5])) / (q->ndof_part * q->kB);
    return 0;
}

/*
 * md.nst(S,T,dt).run(atoms,nsteps).  S[9] row-major, NaN where the stress
 * component is free (S_dof false); tau[9] the barostat relaxation times;
 * t_relax_S and L_S/niters_S the barostat chain.  V_H[9] (box velocity),
 * eta[L] and eta_S[L_S] are carried between runs (in/out).  thermo (may be
 * NULL): nsteps+1 rows [pe, T_part, mvv(6), F_H(6), H(9)].
 */
int orc_md_nst_run(void* p, const double* S, const double* tau, double T, double dt, double kB, double t_relax,
                   int L, int niters, double t_relax_S, int L_S, int niters_S, int nreset, int nsteps,
                   double* V_H, double* eta, double* eta_S, double* thermo) {
    orc_sys* s = (orc_sys*)p;
    if (isnan(kB)) return fail("boltzmann constant should be set prior to MD");
    nst_t q;
    memset(&q, 0, sizeof(q));
    q.T = T; q.dt = dt; q.dt2 = dt / 2.0; q.kB = kB;
    const int n = s->natms;
    /* x_dof (MDNVT::pre_init md_nvt.cpp:265-291): frozen components leave
     * the degrees of freedom; MDNST::run itself keeps the plain updates */
    int frozen[3] = {0, 0, 0};
    if (s->dof)
        for (int i = 0; i < n; i++)
            for (int c = 0; c < 3; c++)
                if (!s->dof[3 * i + c]) frozen[c]++;
    q.ndof_part = 3 * n - (frozen[0] + frozen[1] + frozen[2]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            q.S_dof[i][j] = !isnan(S[3 * i + j]);
            q.S[i][j] = q.S_dof[i][j] ? S[3 * i + j] : NAN;
            q.tau[i][j] = tau[3 * i + j];
            q.V_H[i][j] = j <= i ? V_H[3 * i + j] : 0.0;
        }
    /* MDNST::pre_run_chk md_nst.cpp:259-279 */
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++)
            if (q.S_dof[i][j] && frozen[i])
                return fail("cannot impose stress component while any of the atoms do not have degree freedom "
                            "in its direction");
    nhc_t tp, tb;
    nhc_init(&tp, dt / 2.0, t_relax, L, niters);
    nhc_init(&tb, dt / 2.0, t_relax_S, L_S, niters_S);
    for (int i = 0; i < L; i++) tp.eta_d[i] = eta[i];
    for (int i = 0; i < L_S; i++) tb.eta_d[i] = eta_S[i];
    /* MDNVT::pre_init: mvv (frozen components left out, md_nvt.cpp:318-330), T_part */
    for (int i = 0; i < n; i++) {
        double v[3];
        for (int c = 0; c < 3; c++) v[c] = (!s->dof || s->dof[3 * i + c]) ? s->v[3 * i + c] : 0.0;
        dyadic_add(s->masses[s->elem[i]], v, q.mvv);
    }
    q.T_part = (q.mvv[0] + (q.mvv[3] + q.mvv[5])) / (q.ndof_part * kB);
    /* MDNST::pre_init  md_nst.cpp:281-311 */
    q.ndof_baro = 0;
    q.T_baro = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j <= i; j++) {
            if (q.S_dof[i][j]) {
                q.V_H_prefac[i][j] = 1.0 / (q.tau[i][j] * q.tau[i][j] * q.ndof_part * kB * T);
                q.ndof_baro++;
                q.T_baro += q.V_H[i][j] * q.V_H[i][j] * q.tau[i][j] * q.tau[i][j];
            } else {
                q.S[i][j] = 0.0;
                q.V_H[i][j] = 0.0;
            }
            q.S_dev[i][j] = q.S[i][j];
        }
    if (q.ndof_baro == 0) return fail("no stress component is set");
    q.T_baro *= T * q.ndof_part * kB / q.ndof_baro;
    q.s_hyd = (q.S[0][0] + q.S[1][1] + q.S[2][2]) / 3.0;
    for (int i = 0; i < 3; i++) q.S_dev[i][i] = q.S[i][i] - q.s_hyd;
    /* S_dev keeps only its lower triangle (pre_init fills it with DoLT), and
       the stress product of update_V_H reads it as a square matrix */
    /* DynamicMD::init, then run */
    if (orc_sys_init_dynamic(s)) return -1;
    force_calc(s);
    int row = 0;
#define NST_ROW()                                                              \
    if (thermo) {                                                              \
        double* tr = thermo + (size_t)23 * row;                                \
        tr[0] = s->pe;                                                         \
        tr[1] = q.T_part;                                                      \
        for (int k = 0; k < 6; k++) tr[2 + k] = q.mvv[k];                      \
        tr[8] = s->F_H[0][0]; tr[9] = s->F_H[0][1]; tr[10] = s->F_H[0][2];     \
        tr[11] = s->F_H[1][1]; tr[12] = s->F_H[1][2]; tr[13] = s->F_H[2][2];   \
        for (int k = 0; k < 9; k++) tr[14 + k] = s->H[k / 3][k % 3];           \
    }                                                                          \
    row++;
    NST_ROW();
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) q.B_ref[i][j] = j <= i ? s->B[i][j] : 0.0;
    q.vol_ref = s->vol;
    double fac, fac_x_d = 1.0;
    for (int istep = 0; istep < nsteps; istep++) {
        fac = nhc_step(&tb, q.T_baro / T, q.ndof_baro);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j <= i; j++) q.V_H[i][j] *= fac;
        q.T_baro *= fac * fac;
        fac_x_d *= fac = nhc_step(&tp, q.T_part / T, q.ndof_part);
        fac *= fac;
        for (int k = 0; k < 6; k++) q.mvv[k] *= fac;
        q.T_part *= fac;
        nst_update_V_H(&q, s);
        if (nst_step_x(&q, s, fac_x_d)) return -1;
        nst_update_V_H(&q, s);
        fac_x_d = fac = nhc_step(&tp, q.T_part / T, q.ndof_part);
        fac *= fac;
        for (int k = 0; k < 6; k++) q.mvv[k] *= fac;
        q.T_part *= fac;
        fac = nhc_step(&tb, q.T_baro / T, q.ndof_baro);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j <= i; j++) q.V_H[i][j] *= fac;
        q.T_baro *= fac * fac;
        if (nreset && (istep + 1) % nreset == 0) {
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) q.B_ref[i][j] = j <= i ? s->B[i][j] : 0.0;
            q.vol_ref = s->vol;
        }
        NST_ROW();
    }
#undef NST_ROW
    /* update_x_d_final */
    for (int i = 0; i < 3 * n; i++) s->v[i] *= fac_x_d;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) V_H[3 * i + j] = q.V_H[i][j];
    for (int i = 0; i < L; i++) eta[i] = tp.eta_d[i];
    for (int i = 0; i < L_S; i++) eta_S[i] = tb.eta_d[i];
    return 0;
}

/* ------------------------------------------------------------------------ */
/* L-BFGS with back-tracking line search: MinLBFGS::__run                    */
/* min_l-bfgs.h:113-219, MinMDHandler<false,true>  min_cg.h:215-309,          */
/* LineSearchBackTrack::min  ls.h:711-769 (defaults ls.cpp:456-461)          */
/* ------------------------------------------------------------------------ */
static double vdot(const double* a, const double* b, int n) {
    double r = 0.0;
    for (int i = 0; i < n; i++) r += a[i] * b[i];
    return r;
}

/* line-search function object: x = x0 + alpha*h, skin test, energy */
static double ls_F(orc_sys* s, const double* x0, const double* h, double alpha) {
    int n3 = 3 * s->natms;
    for (int i = 0; i < n3; i++) s->x[i] = x0[i] + alpha * h[i];
    dynamic_update(s);
    return eam_energy_half(s);
}

static double max_abs_f(orc_sys* s) {
    double m = 0.0;
    for (int i = 0; i < 3 * s->natms; i++) m = OMAX(m, fabs(s->f[i]));
    return m;
}

/* ---------------------------------------------------------------- line searches
 * LineSearchBackTrack::min   ls.h:711-769
 * LineSearch::bracket        ls.h:214-335
 * LineSearchGoldenSection::min ls.h:340-515
 * LineSearchBrent::min       ls.h:524-706
 * Defaults: ls.cpp:7-11 (constants), 95-100, 262-268, 456-461.  The caller
 * does MinMDHandler::ls_prep (min_cg.h:230-256) and its three early exits. */
enum { LS_S, LS_F_DOWNHILL, LS_F_GRAD0, LS_MIN_ALPHA, MIN_S_TOLERANCE, MIN_F_MAX_ITER, B_S, B_F_MAX_ALPHA,
       B_F_DOWNHILL, MIN_S_FTOL = 100 };

typedef struct {
    int kind; /* 0 back-tracking, 1 golden section, 2 Brent */
    double c, rho, min_alpha, tol;
    int max_iter, bracket;
    double zeps;
} orc_ls;

/* the line-search function object (MinMDHandler::F / F_reset,
   min_cg.h:260-276); F and reset null: atoms only, x = x0 + alpha h */
typedef struct orc_line {
    orc_sys* s;
    const double* x0;
    const double* h;
    long* n_en;
    double prev_val;
    double (*F)(struct orc_line*, double);
    void (*reset)(struct orc_line*);
    void* ctx;
} orc_line;

static double lineF(orc_line* L, double a) {
    (*L->n_en)++;
    if (L->F) return L->F(L, a);
    return ls_F(L->s, L->x0, L->h, a);
}

static void line_reset(orc_line* L) {
    if (L->reset) {
        L->reset(L);
        return;
    }
    memcpy(L->s->x, L->x0, sizeof(double) * 3 * L->s->natms);
    dynamic_update(L->s);
}

static int ls_backtrack(const orc_ls* p, orc_line* L, double dfa, double max_a, double* nrgy, double* alpha,
                        int init_flag) {
    double init_energy = *nrgy;
    if (init_flag == 0) {
        max_a = OMIN(max_a, 1.0);
    } else if (init_flag == 1) {
        if (L->prev_val > 0.0 && dfa < 0.0) max_a = OMIN(max_a, -L->prev_val / dfa);
        L->prev_val = -dfa;
    }
    if (max_a <= p->min_alpha) return LS_MIN_ALPHA;
    double a = max_a;
    for (;;) {
        double ideal = *nrgy + a * p->c * dfa;
        double cur = lineF(L, a);
        if (cur <= ideal) {
            if (init_flag == 1) L->prev_val *= a;
            *nrgy = cur;
            *alpha = a;
            return LS_S;
        }
        a *= p->rho;
        if (a <= p->min_alpha) {
            *nrgy = init_energy;
            *alpha = a;
            line_reset(L);
            return LS_MIN_ALPHA;
        }
    }
}

static int ls_bracket(orc_line* L, double dfa, double max_a, double* pa, double* pb, double* pc, double* pfa,
                      double* pfb, double* pfc) {
    const double golden = 0.5 + 0.5 * sqrt(5.0), sqrt_eps = sqrt(DBL_EPSILON);
    double a = *pa, b, c, fa = *pfa, fb, fc, u, fu, r, q;
    int ret = B_S;
    q = 1.0e-14 / (max_a * fabs(dfa));
    if (0.01 < q && q < 1.0)
        b = q * max_a;
    else if (q >= 1.0)
        b = max_a;
    else
        b = 0.01 * max_a;
    fb = lineF(L, b);
    c = b;
    fc = fb;
    if (fb >= fa) {
        int iter = 20;
        r = (fa - fc) / (c * dfa);
        b = c * 0.5 / (1.0 + r);
        while (fb >= fa && iter && b > DBL_EPSILON) {
            fb = lineF(L, b);
            if (fb < fa) continue;
            c = b;
            fc = fb;
            iter--;
            r = (fa - fc) / (c * dfa);
            b = c * 0.5 / (1.0 + r);
        }
        if (fb >= fa) {
            b = sqrt_eps < max_a ? sqrt_eps : max_a;
            fb = lineF(L, b);
            if (fb >= fa) ret = B_F_DOWNHILL;
        }
        goto done;
    }
    while (fb >= fc) {
        c = b + golden * (b - a);
        if (c >= max_a) {
            c = max_a;
            fc = lineF(L, c);
            goto done;
        }
        fc = lineF(L, c);
        if (fc > fb) continue;
        double ulim = max_a;
        r = (b - a) * (fb - fc);
        q = (b - c) * (fb - fa);
        u = b - ((b - c) * q - (b - a) * r) / (2.0 * (q - r));
        if (b < u && u < c) {
            fu = lineF(L, u);
            if (fu < fc) {
                a = b; b = u; fa = fb; fb = fu;
                goto done;
            } else if (fu > fb) {
                c = u; fc = fu;
                goto done;
            }
            a = b; b = c; fa = fb; fb = fc;
        } else if (u > c) {
            u = OMIN(u, ulim);
            fu = lineF(L, u);
            a = b; b = c; c = u; fa = fb; fb = fc; fc = fu;
        } else {
            a = b; b = c; fa = fb; fb = fc;
        }
    }
done:
    *pa = a; *pb = b; *pc = c; *pfa = fa; *pfb = fb; *pfc = fc;
    return ret;
}

static int ls_golden(const orc_ls* p, orc_line* L, double dfa, double max_a, double* nrgy, double* alpha) {
    const double gold = 0.61803399, cgold = 0.38196601;
    int calc = 0;
    double a = 0.0, b, c, fa = *nrgy, fb, fc, x0, x1, x2, x3, f1, f2;
    if (p->bracket) {
        int chk = ls_bracket(L, dfa, max_a, &a, &b, &c, &fa, &fb, &fc);
        if (chk != B_S) {
            line_reset(L);
            return chk;
        }
        x0 = a;
        x3 = c;
        if (c - b > b - a) {
            x1 = b; x2 = b + cgold * (c - b); f1 = fb; f2 = lineF(L, x2); calc = 2;
        } else {
            x1 = b + cgold * (a - b); x2 = b; f1 = lineF(L, x1); f2 = fb; calc = 1;
        }
        int iter = p->max_iter;
        while (x3 - x0 > p->tol * (x1 + x2) && x3 - x0 > DBL_EPSILON && iter) {
            if (f2 < f1) {
                x0 = x1; x1 = x2; x2 = gold * x2 + cgold * x3; f1 = f2; f2 = lineF(L, x2); calc = 2;
            } else {
                x3 = x2; x2 = x1; x1 = gold * x1 + cgold * x0; f2 = f1; f1 = lineF(L, x1); calc = 1;
            }
            iter--;
        }
    } else {
        double delta, f0, f3;
        f1 = f2 = 0.0;
        x0 = x1 = x2 = 0.0;
        f0 = fa;
        x3 = max_a;
        f3 = lineF(L, x3);
        int iter = p->max_iter, set_left = 0, set_right = 0;
        while (x3 - x0 > p->tol * (x1 + x2) && x3 - x0 > DBL_EPSILON && iter) {
            delta = cgold * (x3 - x0);
            if (!set_left) { x1 = x0 + delta; f1 = lineF(L, x1); calc = 1; set_left = 1; }
            if (!set_right) { x2 = x3 - delta; f2 = lineF(L, x2); calc = 2; set_right = 1; }
            if ((f0 < f2 && f0 < f3) || (f1 < f2 && f1 < f3)) {
                set_left = 0; x3 = x2; x2 = x1; f3 = f2; f2 = f1;
            } else {
                set_right = 0; x0 = x1; x1 = x2; f0 = f1; f1 = f2;
            }
            iter--;
        }
        if (!set_left) {
            if (f0 < f1) {
                if (x0 == 0.0) {
                    line_reset(L);
                    *alpha = 0.0;
                    return LS_MIN_ALPHA;
                }
                x1 = x0; f1 = lineF(L, x1); calc = 1;
            }
        }
        if (!set_right) {
            if (f3 < f2) { x2 = x3; f2 = lineF(L, x2); calc = 2; }
        }
    }
    if (f1 < f2) {
        if (calc == 2) f1 = lineF(L, x1);
        *nrgy = f1;
        *alpha = x1;
    } else {
        if (calc == 1) f2 = lineF(L, x2);
        *nrgy = f2;
        *alpha = x2;
    }
    L->prev_val = -dfa * *alpha;
    return LS_S;
}

static int ls_brent(const orc_ls* p, orc_line* L, double dfa, double max_a, double* nrgy, double* alpha) {
    const double cgold = 0.38196601;
    double a = 0.0, b = 0.0, fa = *nrgy, fb = 0.0, x = 0.0, fx = 0.0;
    double d = 0.0, e = 0.0, etemp, fu = 0.0, fv, fw, r, q, pp, tol1, tol2, u = 0.0, v, w, xm;
    if (p->bracket) {
        int chk = ls_bracket(L, dfa, max_a, &a, &x, &b, &fa, &fx, &fb);
        if (chk != B_S) {
            line_reset(L);
            return chk;
        }
    } else {
        a = 0.0;
        b = max_a;
        x = cgold * (b - a);
        fx = lineF(L, x);
    }
    w = v = x;
    fw = fv = fx;
    for (int iter = 0; iter < p->max_iter; iter++) {
        xm = 0.5 * (a + b);
        tol1 = p->tol * fabs(x) + p->zeps;
        tol2 = 2.0 * tol1;
        if (fabs(x - xm) <= (tol2 - 0.5 * (b - a))) {
            if (u != x) lineF(L, x);
            *nrgy = fx;
            *alpha = x;
            L->prev_val = x;
            return LS_S;
        }
        if (fabs(e) > tol1) {
            r = (x - w) * (fx - fv);
            q = (x - v) * (fx - fw);
            pp = (x - v) * q - (x - w) * r;
            q = 2.0 * (q - r);
            if (q > 0.0) pp = -pp;
            q = fabs(q);
            etemp = e;
            e = d;
            if (fabs(pp) >= fabs(0.5 * q * etemp) || pp <= q * (a - x) || pp >= q * (b - x)) {
                e = x >= xm ? a - x : b - x;
                d = cgold * e;
            } else {
                d = pp / q;
                u = x + d;
                if (u - a < tol2 || b - u < tol2) d = (xm - x >= 0.0) ? fabs(tol1) : -fabs(tol1);
            }
        } else {
            e = x >= xm ? a - x : b - x;
            d = cgold * e;
        }
        if (fabs(d) >= tol1)
            u = x + d;
        else
            u = d >= 0.0 ? x + fabs(tol1) : x - fabs(tol1);
        fu = lineF(L, u);
        if (fu <= fx) {
            if (u >= x) a = x; else b = x;
            v = w; w = x; x = u;
            fv = fw; fw = fx; fx = fu;
        } else {
            if (u < x) a = u; else b = u;
            if (fu <= fw || w == x) {
                v = w; w = u; fv = fw; fw = fu;
            } else if (fu <= fv || v == x || v == w) {
                v = u; fv = fu;
            }
        }
    }
    if (fa < fx) {
        line_reset(L);
        *alpha = 0.0;
        return LS_MIN_ALPHA;
    }
    if (u != x) lineF(L, x);
    *nrgy = fx;
    *alpha = x;
    L->prev_val = x;
    return LS_S;
}

static int ls_min(const orc_ls* p, orc_line* L, double dfa, double max_a, double* nrgy, double* alpha,
                  int init_flag) {
    if (p->kind == 1) return ls_golden(p, L, dfa, max_a, nrgy, alpha);
    if (p->kind == 2) return ls_brent(p, L, dfa, max_a, nrgy, alpha);
    return ls_backtrack(p, L, dfa, max_a, nrgy, alpha, init_flag);
}

/*
 * md.min_lbfgs(m,e_tol,max_dx,ls=ls_bt(c,rho,min_alpha)).run(atoms,nsteps),
 * plus the max|F| stop (f_tol > 0: stop once max_i |F_i,a| < f_tol, checked
 * after each accepted step).  stats out: [niter, pe, max|F|, err, n_energy,
 * n_force].  Returns 0 on success.
 */
static int lbfgs_core(orc_sys* s, int m, double e_tol, double max_dx, double f_tol, const orc_ls* ls, int nsteps,
                      double* stats, const double* P, long* n_fallback);

int orc_lbfgs_run_ls(void* p, int m, double e_tol, double max_dx, double f_tol, const orc_ls* ls, int nsteps,
                     double* stats) {
    return lbfgs_core((orc_sys*)p, m, e_tol, max_dx, f_tol, ls, nsteps, stats, NULL, NULL);
}

/*
 * L-BFGS with a diagonal initial inverse Hessian, as the library's
 * mappg_lbfgs_run_diag runs it (the learned-preconditioner path; no
 * counterpart in the reference): hdiag is the per-component Hessian
 * diagonal in atom order (x, y, z per atom), P = 1/hdiag, and the two-loop
 * recursion's middle step is h <- tau P h instead of gamma h, with tau =
 * (s.y)/(y.P.y) of the newest pair (1 before the first).  A direction that
 * is not a descent direction is recomputed with gamma (counted in
 * stats[6]), then replaced by f as in the plain run.  A pair without
 * positive curvature takes no part in the recursion (rho = 0) and leaves
 * gamma and tau as they were.  hdiag must be positive and finite.
 * stats out: [niter, pe, max|F|, err, n_energy, n_force, fallbacks].
 */
int orc_lbfgs_run_diag(void* p, const double* hdiag, int m, double e_tol, double max_dx, double f_tol, double c_ls,
                       double rho_ls, double min_alpha, int nsteps, double* stats) {
    orc_sys* s = (orc_sys*)p;
    int n3 = 3 * s->natms;
    double* P = (double*)malloc(sizeof(double) * (n3 ? n3 : 1));
    for (int q = 0; q < n3; q++) {
        if (!(hdiag[q] > 0.0) || !isfinite(hdiag[q])) {
            free(P);
            return fail("the Hessian diagonal must be positive and finite");
        }
        P[q] = 1.0 / hdiag[q];
    }
    orc_ls ls = {0, c_ls, rho_ls, min_alpha, 0.0, 0, 0, 0.0};
    long nfb = 0;
    double st[6];
    int r = lbfgs_core(s, m, e_tol, max_dx, f_tol, &ls, nsteps, st, P, &nfb);
    free(P);
    if (stats && r == 0) {
        for (int k = 0; k < 6; k++) stats[k] = st[k];
        stats[6] = (double)nfb;
    }
    return r;
}

static int lbfgs_core(orc_sys* s, int m, double e_tol, double max_dx, double f_tol, const orc_ls* ls, int nsteps,
                      double* stats, const double* P, long* n_fallback) {
    int n3 = 3 * s->natms;
    if (orc_sys_init_dynamic(s)) return -1;
    double* f0 = (double*)malloc(sizeof(double) * n3);
    double* h = (double*)malloc(sizeof(double) * n3);
    double* x0 = (double*)malloc(sizeof(double) * n3);
    double** sv = (double**)malloc(sizeof(double*) * (m ? m : 1));
    double** yv = (double**)malloc(sizeof(double*) * (m ? m : 1));
    for (int i = 0; i < m; i++) {
        sv[i] = (double*)calloc(n3, sizeof(double));
        yv[i] = (double*)calloc(n3, sizeof(double));
    }
    double* rho = (double*)calloc(m ? m : 1, sizeof(double));
    double* alpha = (double*)calloc(m ? m : 1, sizeof(double));
    long n_en = 0, n_fc = 1;
    force_calc(s);
    double e_prev, e_curr = s->pe, alpha_m = 0.0, gamma = 1.0, tau = 1.0;
    int k = 0;
    int err = nsteps == 0 ? MIN_F_MAX_ITER : LS_S;
    if (err == LS_S && f_tol > 0.0 && max_abs_f(s) < f_tol) err = MIN_S_FTOL;
    orc_line line = {s, x0, h, &n_en, -1.0};
    int istep = 0;
    for (; err == LS_S; istep++) {
        memcpy(x0, s->x, sizeof(double) * n3);
        memcpy(f0, s->f, sizeof(double) * n3);
        /* the two-loop recursion, min_l-bfgs.h:148-170; a diagonal P
           replaces gamma*I by tau*diag(P) */
        for (int pass = P ? 0 : 1; pass < 2; pass++) {
            memcpy(h, s->f, sizeof(double) * n3);
            for (int i = 0; i < k; i++) {
                alpha[i] = -rho[i] * vdot(sv[i], h, n3);
                for (int q = 0; q < n3; q++) h[q] += alpha[i] * yv[i][q];
            }
            if (pass == 0)
                for (int q = 0; q < n3; q++) h[q] *= tau * P[q];
            else
                for (int q = 0; q < n3; q++) h[q] *= gamma;
            for (int i = k - 1; i > -1; i--) {
                double scl0 = -alpha[i] - rho[i] * vdot(yv[i], h, n3);
                for (int q = 0; q < n3; q++) h[q] += scl0 * sv[i][q];
            }
            if (pass == 1 || vdot(s->f, h, n3) >= 0.0) break;
            if (n_fallback) (*n_fallback)++; /* not a descent direction: gamma instead */
        }
        e_prev = e_curr;
        double f_h = vdot(s->f, h, n3);
        if (f_h < 0.0) {
            memcpy(h, s->f, sizeof(double) * n3);
            k = 0;
            f_h = vdot(s->f, s->f, n3);
        }
        /* ls->min(&handler, e_curr, alpha_m, 0)  min_l-bfgs.h:173 */
        {
            double h_norm = vdot(h, h, n3), dfa = -f_h, max_a;
            int lerr = LS_S;
            if (h_norm == 0.0) {
                max_a = 0.0;
                dfa = 0.0;
            } else if (dfa >= 0.0) {
                max_a = 0.0;
                dfa = 1.0;
            } else {
                double mx = 0.0;
                for (int q = 0; q < n3; q++) mx = OMAX(mx, fabs(h[q]));
                max_a = OMIN(fabs(max_dx / mx), INFINITY);
            }
            if (dfa == 0.0)
                lerr = LS_F_GRAD0;
            else if (max_a == 0.0)
                lerr = LS_MIN_ALPHA;
            else if (dfa >= 0.0)
                lerr = LS_F_DOWNHILL;
            else
                lerr = ls_min(ls, &line, dfa, max_a, &e_curr, &alpha_m, 0);
            err = lerr;
        }
        if (err != LS_S) {
            istep--;
            continue;
        }
        force_calc(s);
        n_fc++;
        if (e_prev - e_curr < e_tol) err = MIN_S_TOLERANCE;
        if (f_tol > 0.0 && max_abs_f(s) < f_tol) err = MIN_S_FTOL;
        if (istep + 1 == nsteps) err = MIN_F_MAX_ITER;
        if (err) continue;
        if (m) {
            if (k != m) k++;
            /* cyclic_shift: s[i] <- s[i-1] for i = k-1..1 (buffer rotation) */
            double* ts = sv[k - 1];
            double* ty = yv[k - 1];
            for (int i = k - 1; i > 0; i--) {
                sv[i] = sv[i - 1];
                yv[i] = yv[i - 1];
            }
            sv[0] = ts;
            yv[0] = ty;
            for (int i = m - 1; i > 0; i--) rho[i] = rho[i - 1];
            for (int q = 0; q < n3; q++) {
                sv[0][q] = alpha_m * h[q];
                yv[0][q] = f0[q] - s->f[q];
            }
            double inner0 = vdot(sv[0], yv[0], n3);
            double inner1 = vdot(yv[0], yv[0], n3);
            if (!P) {
                gamma = inner0 / inner1;
                rho[0] = 1.0 / inner0;
            } else if (inner0 > 0.0 && inner1 > 0.0) {
                double inner2 = 0.0;
                for (int q = 0; q < n3; q++) inner2 += yv[0][q] * yv[0][q] * P[q];
                gamma = inner0 / inner1;
                rho[0] = 1.0 / inner0;
                if (inner2 > 0.0) tau = inner0 / inner2;
            } else {
                rho[0] = 0.0;
            }
        } else {
            gamma = alpha_m * (vdot(h, f0, n3) - vdot(h, s->f, n3)) /
                    (vdot(s->f, s->f, n3) + vdot(f0, f0, n3) - 2.0 * vdot(s->f, f0, n3));
        }
    }
    if (stats) {
        stats[0] = istep;
        stats[1] = s->pe;
        stats[2] = max_abs_f(s);
        stats[3] = err;
        stats[4] = (double)n_en;
        stats[5] = (double)n_fc;
    }
    for (int i = 0; i < m; i++) {
        free(sv[i]);
        free(yv[i]);
    }
    free(sv); free(yv); free(rho); free(alpha); free(f0); free(h); free(x0);
    return 0;
}

/* MinCG::__run  min_cg.h:454-536 (Polak-Ribiere conjugate gradient) over
 * LineSearchBackTrack::min with init_flag 1  ls.h:711-769 (the first trial
 * step is capped by the previous step's decrease; LineSearch::reset sets
 * prev_val = -1, ls.h:42), plus the added stop at max|F| < f_tol. */
int orc_cg_run_ls(void* p, double e_tol, double max_dx, double f_tol, const orc_ls* ls, int nsteps, double* stats) {
    orc_sys* s = (orc_sys*)p;
    int n3 = 3 * s->natms;
    if (orc_sys_init_dynamic(s)) return -1;
    double* f0 = (double*)malloc(sizeof(double) * n3);
    double* h = (double*)malloc(sizeof(double) * n3);
    double* x0 = (double*)malloc(sizeof(double) * n3);
    long n_en = 0, n_fc = 1;
    orc_line line = {s, x0, h, &n_en, -1.0}; /* prev_val = -1 (LineSearch::reset) */
    double alpha = 0.0;
    force_calc(s);
    double e_prev, e_curr = s->pe;
    int err = nsteps == 0 ? MIN_F_MAX_ITER : LS_S;
    if (err == LS_S && f_tol > 0.0 && max_abs_f(s) < f_tol) err = MIN_S_FTOL;
    memcpy(h, s->f, sizeof(double) * n3);
    double f0_f0 = vdot(s->f, s->f, n3);
    int istep = 0;
    for (; err == LS_S; istep++) {
        if (f0_f0 == 0.0) {
            err = LS_F_GRAD0;
            continue;
        }
        memcpy(x0, s->x, sizeof(double) * n3);
        memcpy(f0, s->f, sizeof(double) * n3);
        e_prev = e_curr;
        double f_h = vdot(s->f, h, n3);
        if (f_h < 0.0) {
            memcpy(h, s->f, sizeof(double) * n3);
            f_h = f0_f0;
        }
        {
            double h_norm = vdot(h, h, n3), dfa = -f_h, max_a;
            int lerr = LS_S;
            if (h_norm == 0.0) {
                max_a = 0.0;
                dfa = 0.0;
            } else if (dfa >= 0.0) {
                max_a = 0.0;
                dfa = 1.0;
            } else {
                double mx = 0.0;
                for (int q = 0; q < n3; q++) mx = OMAX(mx, fabs(h[q]));
                max_a = fabs(max_dx / mx);
            }
            if (dfa == 0.0)
                lerr = LS_F_GRAD0;
            else if (max_a == 0.0)
                lerr = LS_MIN_ALPHA;
            else if (dfa >= 0.0)
                lerr = LS_F_DOWNHILL;
            else
                lerr = ls_min(ls, &line, dfa, max_a, &e_curr, &alpha, 1); /* min_cg.h:504 */
            err = lerr;
        }
        if (err != LS_S) {
            istep--;
            continue;
        }
        force_calc(s);
        n_fc++;
        if (e_prev - e_curr < e_tol) err = MIN_S_TOLERANCE;
        if (f_tol > 0.0 && max_abs_f(s) < f_tol) err = MIN_S_FTOL;
        if (istep + 1 == nsteps) err = MIN_F_MAX_ITER;
        if (err) continue;
        double f_f = vdot(s->f, s->f, n3), f_f0 = vdot(s->f, f0, n3);
        double ratio = (f_f - f_f0) / f0_f0;
        for (int q = 0; q < n3; q++) h[q] = ratio * h[q] + s->f[q];
        f0_f0 = f_f;
    }
    if (stats) {
        stats[0] = istep;
        stats[1] = s->pe;
        stats[2] = max_abs_f(s);
        stats[3] = err;
        stats[4] = (double)n_en;
        stats[5] = (double)n_fc;
    }
    free(f0);
    free(h);
    free(x0);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Box degrees of freedom                                                    */
/* ------------------------------------------------------------------------ */
/* MinLBFGS::__run  min_l-bfgs.h:113-219 and MinCG::__run  min_cg.h:454-536
 * with BC = true or X = false: MinMDHandler  min_cg.h:89-331 (init 164-198,
 * ls_prep 230-256, F 260-267, F_reset 271-276, prep_x_d 298-309,
 * prep_x_d_affine 313-321, post_force_calc_box 324-329) and the vector-tensor
 * algebra of new_min_vec.h (dot product 596-606: atoms first, then the lower
 * triangle (0,0),(1,0),(1,1),(2,0),(2,1),(2,2), TOP 224-322).  A trial
 * rebuilds the lists for its box (NewDynamicMD<true,true>::update,
 * dynamic_md.h:200-206, rebuilds only past the skin; a rebuild at every
 * trial gives the same energies while no pair crosses the cutoff unseen). */
typedef struct {
    double* v; /* 3n, or NULL when the atoms move affinely */
    double A[3][3];
} orc_vt;

static const int LT[6][2] = {{0, 0}, {1, 0}, {1, 1}, {2, 0}, {2, 1}, {2, 2}};

static double vt_dot(const orc_vt* a, const orc_vt* b, int n3) {
    double r = a->v ? vdot(a->v, b->v, n3) : 0.0;
    for (int k = 0; k < 6; k++) r += a->A[LT[k][0]][LT[k][1]] * b->A[LT[k][0]][LT[k][1]];
    return r;
}
static void vt_lin(orc_vt* y, double cy, const orc_vt* x, double cx, int n3) {
    if (y->v)
        for (int q = 0; q < n3; q++) y->v[q] = cy * y->v[q] + cx * x->v[q];
    for (int k = 0; k < 6; k++) {
        int i = LT[k][0], j = LT[k][1];
        y->A[i][j] = cy * y->A[i][j] + cx * x->A[i][j];
    }
}
static void vt_scale(orc_vt* y, double c, int n3) {
    if (y->v)
        for (int q = 0; q < n3; q++) y->v[q] *= c;
    for (int k = 0; k < 6; k++) y->A[LT[k][0]][LT[k][1]] *= c;
}
static void vt_copy(orc_vt* y, const orc_vt* x, int n3) {
    if (y->v) memcpy(y->v, x->v, sizeof(double) * n3);
    memcpy(y->A, x->A, sizeof(y->A));
}

typedef struct {
    orc_sys* s;
    int n3;
    double *x0, *xd;
    double H0[3][3], xdA[3][3];
} orc_box;

static int box_rebuild(orc_sys* s) {
    update_H(s);
    return rebuild(s);
}
static double box_F(orc_line* L, double a) {
    orc_box* b = (orc_box*)L->ctx;
    orc_sys* s = b->s;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) s->H[i][j] = b->H0[i][j] + a * b->xdA[i][j];
    for (int q = 0; q < b->n3; q++) s->x[q] = b->x0[q] + a * b->xd[q];
    if (box_rebuild(s)) return NAN;
    return eam_energy_half(s);
}
static void box_reset(orc_line* L) {
    orc_box* b = (orc_box*)L->ctx;
    orc_sys* s = b->s;
    memcpy(s->H, b->H0, sizeof(s->H));
    memcpy(s->x, b->x0, sizeof(double) * b->n3);
    box_rebuild(s);
}

/* handler.force_calc(): forces, pe and F_H masked by H_dof */
static void box_force(orc_sys* s, orc_vt* f, const int* hdof) {
    force_calc(s);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) f->A[i][j] = (j <= i && hdof[3 * i + j]) ? s->F_H[i][j] : 0.0;
    if (f->v) memcpy(f->v, s->f, sizeof(double) * 3 * s->natms);
}

/* prep_x_d / prep_x_d_affine: x_d = h + x0 h.A (affine: x0 h.A), box part
   H0 h.A (MLT_mul_MLT); returns max|x_d| */
static double box_prep(orc_box* b, const orc_vt* h) {
    int n = b->n3 / 3;
    const double(*A)[3] = h->A;
    double mx = 0.0;
    for (int i = 0; i < n; i++) {
        const double* p = b->x0 + 3 * i;
        double d[3] = {A[0][0] * p[0] + (A[1][0] * p[1] + A[2][0] * p[2]), A[1][1] * p[1] + A[2][1] * p[2],
                       A[2][2] * p[2]};
        for (int c = 0; c < 3; c++) {
            double v = h->v ? h->v[3 * i + c] + d[c] : d[c];
            b->xd[3 * i + c] = v;
            mx = OMAX(mx, fabs(v));
        }
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double t = 0.0;
            if (j <= i) {
                t = b->H0[i][i] * A[i][j];
                for (int k = i - 1; k >= j; k--) t = b->H0[i][k] * A[k][j] + t;
            }
            b->xdA[i][j] = t;
        }
    return mx;
}

/* method 0 L-BFGS, 1 CG; hdof[9] row-major (lower triangle read); stats as
   orc_lbfgs_run; the relaxed box is left in the system (orc_sys_get_box) */
int orc_min_box_run(void* p, int method, int m, double e_tol, double max_dx, const int* hdof, int affine,
                    const orc_ls* ls, int nsteps, double* stats) {
    orc_sys* s = (orc_sys*)p;
    int n3 = 3 * s->natms, X = !affine;
    if (orc_sys_init_dynamic(s)) return -1;
    orc_box box = {s, n3, (double*)malloc(sizeof(double) * n3), (double*)malloc(sizeof(double) * n3), {{0}}, {{0}}};
    int nv = 3 + (method == 0 ? 2 * m : 0);
    double* pool = X ? (double*)calloc((size_t)nv * n3, sizeof(double)) : NULL;
    orc_vt f = {X ? pool : NULL, {{0}}}, f0 = {X ? pool + n3 : NULL, {{0}}}, h = {X ? pool + 2 * n3 : NULL, {{0}}};
    orc_vt* sv = (orc_vt*)calloc(m ? m : 1, sizeof(orc_vt));
    orc_vt* yv = (orc_vt*)calloc(m ? m : 1, sizeof(orc_vt));
    if (method == 0)
        for (int i = 0; i < m; i++) {
            sv[i].v = X ? pool + (size_t)(3 + 2 * i) * n3 : NULL;
            yv[i].v = X ? pool + (size_t)(4 + 2 * i) * n3 : NULL;
        }
    double* rho = (double*)calloc(m ? m : 1, sizeof(double));
    double* alph = (double*)calloc(m ? m : 1, sizeof(double));
    long n_en = 0, n_fc = 1;
    orc_line line = {s, box.x0, box.xd, &n_en, -1.0, box_F, box_reset, &box};
    box_force(s, &f, hdof);
    double e_curr = s->pe, e_prev, f_h, alpha_m = 0.0, gamma = 1.0, f0_f0 = 0.0;
    int k = 0, err = nsteps == 0 ? MIN_F_MAX_ITER : LS_S, istep = 0;
    if (method == 1) {
        vt_copy(&h, &f, n3);
        f0_f0 = vt_dot(&f, &f, n3);
    }
    for (; err == LS_S; istep++) {
        if (method == 1 && f0_f0 == 0.0) {
            err = LS_F_GRAD0;
            continue;
        }
        memcpy(box.x0, s->x, sizeof(double) * n3);
        memcpy(box.H0, s->H, sizeof(box.H0));
        vt_copy(&f0, &f, n3);
        if (method == 0) {
            vt_copy(&h, &f, n3);
            for (int i = 0; i < k; i++) {
                alph[i] = -rho[i] * vt_dot(&sv[i], &h, n3);
                vt_lin(&h, 1.0, &yv[i], alph[i], n3);
            }
            vt_scale(&h, gamma, n3);
            for (int i = k - 1; i > -1; i--) {
                double scl0 = -alph[i] - rho[i] * vt_dot(&yv[i], &h, n3);
                vt_lin(&h, 1.0, &sv[i], scl0, n3);
            }
        }
        e_prev = e_curr;
        f_h = vt_dot(&f, &h, n3);
        if (f_h < 0.0) {
            vt_copy(&h, &f, n3);
            if (method == 0) {
                k = 0;
                f_h = vt_dot(&f, &f, n3);
            } else {
                f_h = f0_f0;
            }
        }
        double max_xd = box_prep(&box, &h);
        double h_norm = vt_dot(&h, &h, n3), dfa = -f_h, max_a;
        int lerr;
        if (h_norm == 0.0) {
            max_a = 0.0;
            dfa = 0.0;
        } else if (dfa >= 0.0) {
            max_a = 0.0;
            dfa = 1.0;
        } else {
            max_a = fabs(max_dx / max_xd);
        }
        if (dfa == 0.0)
            lerr = LS_F_GRAD0;
        else if (max_a == 0.0)
            lerr = LS_MIN_ALPHA;
        else if (dfa >= 0.0)
            lerr = LS_F_DOWNHILL;
        else
            lerr = ls_min(ls, &line, dfa, max_a, &e_curr, &alpha_m, method == 0 ? 0 : 1);
        err = lerr;
        if (err != LS_S) {
            istep--;
            continue;
        }
        box_force(s, &f, hdof);
        n_fc++;
        if (e_prev - e_curr < e_tol) err = MIN_S_TOLERANCE;
        if (istep + 1 == nsteps) err = MIN_F_MAX_ITER;
        if (err) continue;
        if (method == 1) {
            double f_f = vt_dot(&f, &f, n3), f_f0 = vt_dot(&f, &f0, n3);
            double ratio = (f_f - f_f0) / f0_f0;
            vt_lin(&h, ratio, &f, 1.0, n3);
            f0_f0 = f_f;
        } else if (m) {
            if (k != m) k++;
            orc_vt ts = sv[k - 1], ty = yv[k - 1];
            for (int i = k - 1; i > 0; i--) {
                sv[i] = sv[i - 1];
                yv[i] = yv[i - 1];
            }
            sv[0] = ts;
            yv[0] = ty;
            for (int i = m - 1; i > 0; i--) rho[i] = rho[i - 1];
            vt_lin(&sv[0], 0.0, &h, alpha_m, n3);
            vt_copy(&yv[0], &f0, n3);
            vt_lin(&yv[0], 1.0, &f, -1.0, n3);
            double inner0 = vt_dot(&sv[0], &yv[0], n3);
            double inner1 = vt_dot(&yv[0], &yv[0], n3);
            gamma = inner0 / inner1;
            rho[0] = 1.0 / inner0;
        } else {
            gamma = alpha_m * (vt_dot(&h, &f0, n3) - vt_dot(&h, &f, n3)) /
                    (vt_dot(&f, &f, n3) + vt_dot(&f0, &f0, n3) - 2.0 * vt_dot(&f, &f0, n3));
        }
    }
    if (stats) {
        stats[0] = istep;
        stats[1] = s->pe;
        stats[2] = max_abs_f(s);
        stats[3] = err;
        stats[4] = (double)n_en;
        stats[5] = (double)n_fc;
    }
    free(box.x0); free(box.xd); free(pool); free(sv); free(yv); free(rho); free(alph);
    return 0;
}

void orc_sys_get_box(void* p, double* H) { memcpy(H, ((orc_sys*)p)->H, sizeof(double) * 9); }

/* Park-Miller + polar Box-Muller  random.cpp:32-68, AtomsMD::create_T
   atoms_md.cpp:130-162.  Seed 0 makes the reference loop forever; here it is
   rejected. */
int orc_create_temp_dof(int natms, const unsigned char* elem, const double* masses, const unsigned char* dof,
                        double T, double kB, int seed, double* v);
int orc_create_temp(int natms, const unsigned char* elem, const double* masses, double T, double kB,
                    int seed, double* v) {
    return orc_create_temp_dof(natms, elem, masses, NULL, T, kB, seed, v);
}
/* AtomsMD::create_T with x_dof (atoms_md.cpp:138-149): only the free
   components draw a sample; the others keep their value */
int orc_create_temp_dof(int natms, const unsigned char* elem, const double* masses, const unsigned char* dof,
                        double T, double kB, int seed, double* v) {
    if (seed == 0) return fail("seed 0 never yields a Gaussian sample");
    int sd = seed, gchk = 0;
    double reserved = 0.0;
#define UNIF()                                     \
    ({                                             \
        int first = sd / 127773, second = sd % 127773; \
        int rnd = 16807 * second - 2836 * first;   \
        sd = rnd > 0 ? rnd : rnd + 2147483647;     \
        sd * 1.0 / 2147483647;                     \
    })
    for (int i = 0; i < natms; i++) {
        double fac = sqrt(kB * T / masses[elem[i]]);
        for (int j = 0; j < 3; j++) {
            if (dof && !dof[3 * i + j]) continue;
            double g;
            if (gchk) {
                gchk = 0;
                g = reserved;
            } else {
                gchk = 1;
                double u = 0.0, vv = 0.0, s2 = 1.0;
                while (s2 >= 1.0) {
                    u = 2.0 * UNIF() - 1.0;
                    vv = 2.0 * UNIF() - 1.0;
                    s2 = u * u + vv * vv;
                }
                double r = sqrt(-2.0 * log(s2) / s2);
                reserved = vv * r;
                g = u * r;
            }
            v[3 * i + j] = g * fac;
        }
    }
#undef UNIF
    return 0;
}

/* the back-tracking entry points (ls_bt) */
int orc_lbfgs_run(void* p, int m, double e_tol, double max_dx, double f_tol, double c_ls, double rho_ls,
                  double min_alpha, int nsteps, double* stats) {
    orc_ls ls = {0, c_ls, rho_ls, min_alpha, 0.0, 0, 0, 0.0};
    return orc_lbfgs_run_ls(p, m, e_tol, max_dx, f_tol, &ls, nsteps, stats);
}

int orc_cg_run(void* p, double e_tol, double max_dx, double f_tol, double c_ls, double rho_ls, double min_alpha,
               int nsteps, double* stats) {
    orc_ls ls = {0, c_ls, rho_ls, min_alpha, 0.0, 0, 0, 0.0};
    return orc_cg_run_ls(p, e_tol, max_dx, f_tol, &ls, nsteps, stats);
}
