// Internal declarations shared by the libmappg translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "mappg.h"

namespace mappg {

constexpr int kMaxElem = 8;   // elements supported by the device kernels
constexpr int kCodeBits = 5;  // low bits of a neighbour entry: image code

// thread-local error message behind mappg_last_error()
void set_error(const std::string& msg);
const char* get_error();

struct Error {
    int code;
    std::string msg;
};

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
    double4* rho64 = nullptr;   // [ne*ne][nr]
    double4* rphi64 = nullptr;  // [ne*ne][nr]
    double4* F64 = nullptr;     // [ne][nrho]
    float4* rho32 = nullptr;
    float4* rphi32 = nullptr;
    float4* F32 = nullptr;
    float* rphi32_lo = nullptr;  // c0 - (float)c0 of the r*phi table
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
