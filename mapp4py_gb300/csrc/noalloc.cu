// mappg_sys_force_noalloc: the FP64 force call for callers that must not
// allocate device memory.
//
// Some callers cannot let a library allocate: a host framework whose memory
// pool owns the whole device and counts every byte, a serving process that
// must not block on the allocator (cudaMalloc and cudaFree synchronise the
// device), or code that has to keep its footprint fixed after start-up.  The
// other force entry points write into per-system buffers that exist already,
// but nothing stops a later call from growing them.  This one never
// allocates: the caller passes the output buffers, and the intermediate
// arrays (per-atom density, F'(rho), forces in bin order, per-block partial
// sums and the reduction counters) live in one fixed array declared below.
//
// The array is a file-scope __device__ variable of kScratchBytes bytes
// (about 11.0 MB, 10.5 MiB, for kScratchAtoms = 262144 atoms).  Every GPU on
// which this file's code is loaded holds it until the process exits.  All calls share it and it
// keeps what the last call left there, so each call clears the counters that
// must start at zero before it launches anything; calls whose work overlaps
// on the GPU (two systems on two streams, say) race on it and give wrong
// results, so order them on one stream or wait between them.
#include <mutex>

#include "system.h"

namespace mappg {

void launch_force64_args(mappg_sys* s, const EamArgs& a);  // eam.cu
void preload_force64();                                    // eam.cu

constexpr int kScratchAtoms = 1 << 18;

// byte offsets inside the scratch array, each a multiple of 256
constexpr size_t kOffF = 0;                                           // 3n doubles
constexpr size_t kOffRho = kOffF + sizeof(double) * 3 * kScratchAtoms;  // n doubles
constexpr size_t kOffDF = kOffRho + sizeof(double) * kScratchAtoms;     // n doubles
constexpr size_t kOffPart = kOffDF + sizeof(double) * kScratchAtoms;    // partial sums
constexpr size_t kOffScal = kOffPart + sizeof(double) * kRedSlots * kMaxBlocks;
constexpr size_t kScratchBytes = kOffScal + ((sizeof(DevScalars) + 255) / 256) * 256;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// device address of g_scratch, looked up once per device
constexpr int kMaxDevices = 64;
static unsigned char* g_scratch_dev[kMaxDevices];
static std::mutex g_scratch_mu;

static unsigned char* scratch_on(int device) {
    if (device < 0 || device >= kMaxDevices) throw Error{MAPPG_ERR_ARG, "device ordinal out of range"};
    int cur = -1;
    MAPPG_CUDA(cudaGetDevice(&cur));
    if (cur != device)
        throw Error{MAPPG_ERR_ARG, "mappg_sys_force_noalloc: the system lives on device " + std::to_string(device) +
                                       " but the calling thread's current device is " + std::to_string(cur)};
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_dev[device]) {
        void* p = nullptr;
        MAPPG_CUDA(cudaGetSymbolAddress(&p, g_scratch));
        preload_force64();
        g_scratch_dev[device] = static_cast<unsigned char*>(p);
    }
    return g_scratch_dev[device];
}

// forces from bin order (structure of arrays) to the caller's order (x, y, z
// per atom), zero on components frozen by atoms.x_dof (dof null: none),
// energy and virial to the caller's 7 doubles
__global__ void k_noalloc_out(int n, const int* __restrict__ id, const double* __restrict__ f_bin,
                              const uint8_t* __restrict__ dof, const DevScalars* __restrict__ sc,
                              double* __restrict__ f_out, double* __restrict__ ev_out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const size_t u = 3 * (size_t)id[i];
        const unsigned d = dof ? dof[i] : 7u;
        f_out[u] = (d & 1u) ? f_bin[i] : 0.0;
        f_out[u + 1] = (d & 2u) ? f_bin[n + i] : 0.0;
        f_out[u + 2] = (d & 4u) ? f_bin[2 * n + i] : 0.0;
    }
    if (ev_out && blockIdx.x == 0 && threadIdx.x < 7)
        ev_out[threadIdx.x] = threadIdx.x == 0 ? sc->energy : sc->virial[threadIdx.x - 1];
}

}  // namespace mappg

using namespace mappg;

extern "C" int mappg_sys_force_noalloc(mappg_sys* s, double* f_dev, double* ev_dev) {
    try {
        if (!s || !f_dev) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->precision != MAPPG_FP64) throw Error{MAPPG_ERR_ARG, "mappg_sys_force_noalloc takes FP64 systems only"};
        if (s->n > kScratchAtoms)
            throw Error{MAPPG_ERR_ARG, "mappg_sys_force_noalloc: " + std::to_string(s->n) +
                                           " atoms exceed its scratch limit of " + std::to_string(kScratchAtoms)};
        if (!s->built)
            throw Error{MAPPG_ERR_ARG, "mappg_sys_force_noalloc: the system has no neighbour list "
                                       "(call mappg_sys_build or mappg_sys_update first)"};
        unsigned char* base = scratch_on(s->device);
        DevScalars* sc = reinterpret_cast<DevScalars*>(base + kOffScal);
        MAPPG_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), s->stream));
        EamArgs a = eam_args(s);
        a.f = reinterpret_cast<double*>(base + kOffF);
        a.rho = reinterpret_cast<double*>(base + kOffRho);
        a.dF = reinterpret_cast<double*>(base + kOffDF);
        a.partials = reinterpret_cast<double*>(base + kOffPart);
        a.sc = sc;
        launch_force64_args(s, a);
        k_noalloc_out<<<grid_for(s, s->n, 256), 256, 0, s->stream>>>(s->n, s->id, a.f, s->dof, sc, f_dev, ev_dev);
        MAPPG_CUDA(cudaGetLastError());
        return MAPPG_OK;
    } catch (const Error& e) {
        set_error(e.msg);
        return e.code;
    } catch (const std::exception& e) {
        set_error(e.what());
        return MAPPG_ERR_ARG;
    }
}
