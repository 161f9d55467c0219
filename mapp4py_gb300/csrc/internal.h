// Internal declarations shared by the libmappg translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "mappg.h"

namespace mappg {

// one cubic-spline interval of an FP64 table (c0, c1, c2, c3)
struct alignas(32) Dbl4 {
    double x, y, z, w;
};

constexpr int kMaxElem = 8;   // elements supported by the device kernels

// thread-local error message behind mappg_last_error()
void set_error(const std::string& msg);
const char* get_error();

struct Error {
    int code;
    std::string msg;
};

// Runs f; an exception becomes a negative status and the message of
// mappg_last_error().  Every extern "C" entry point goes through it.
template <class F>
int guard(F&& f) {
    try {
        f();
        return MAPPG_OK;
    } catch (const Error& e) {
        set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        return MAPPG_ERR_ARG;
    } catch (const std::exception& e) {
        set_error(e.what());
        return MAPPG_ERR_ARG;
    } catch (...) {
        set_error("unknown failure");
        return MAPPG_ERR_ARG;
    }
}

#define MAPPG_CUDA(call)                                                                     \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            throw ::mappg::Error{MAPPG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

// ------------------------------------------------------------------ tables
// Host copy of the EAM tables in the reference's layout (ForceFieldEAM).
struct HostTables {
    int nelem = 0, nr = 0, nrho = 0;
    double dr = 0, drho = 0;
    std::vector<double> F;     // [nelem][nrho][4]
    std::vector<double> rho;   // [nelem][nelem][nr][4]: rho_arr[i][j]
    std::vector<double> rphi;  // [nelem][nelem][nr][4]: symmetric
    std::vector<double> cut;   // [nelem][nelem]
    std::vector<std::string> names;
    double* rho_at(int i, int j) { return rho.data() + ((size_t)(i * nelem + j) * nr) * 4; }
    double* rphi_at(int i, int j) { return rphi.data() + ((size_t)(i * nelem + j) * nr) * 4; }
    double* F_at(int i) { return F.data() + ((size_t)i * nrho) * 4; }
    void alloc(int ne, int nr_, int nrho_, double dr_, double drho_);
    void finish_splines(bool per_pair_rho);
};

void interpolate4(size_t n, double (*s)[4]);
void read_setfl(const char* path, int nreq, const char* const* req, HostTables& t);
void read_fs(const char* path, int nreq, const char* const* req, HostTables& t);
void read_funcfl(int nfiles, const char* const* paths, HostTables& t);

// ------------------------------------------------------------------ device tables
struct DevTables {
    int nelem = 0, nr = 0, nrho = 0;
    double dr_inv = 0, drho_inv = 0, rho_max = 0, max_cut = 0;
    double cut[kMaxElem * kMaxElem];
    Dbl4* rho64 = nullptr;   // [ne*ne][nr]
    Dbl4* rphi64 = nullptr;  // [ne*ne][nr]
    Dbl4* F64 = nullptr;     // [ne][nrho]
    float4* rho32 = nullptr;    // rho value coefficients, [ne*ne][nr]
    float4* ftab = nullptr;     // force records, 2 float4 per (ei*ne+ej, knot):
                                // (d1i,d2i,d3i,z0) (z1,z2,z3,z0lo)
    float4* fjtab = nullptr;    // (d1j,d2j,d3j,0) per (ei*ne+ej, knot)
                                // d = (c1, 2c2, 3c3)/dr of rho_{j->i} / rho_{i->j}
    float4* F32 = nullptr;      // embedding coefficients, [ne][nrho]
    float* F32lo = nullptr;     // c0 - (float)c0 of the embedding table
    int rho_ei = 1;             // 0 when rho_{j->i} is the same table for every e_i
};

}  // namespace mappg

struct mappg_ff {
    mappg::HostTables host;
    mappg::DevTables dev;
    int device = -1;
};

namespace mappg {
void upload_tables(mappg_ff* ff);
void free_tables(mappg_ff* ff);
}  // namespace mappg
