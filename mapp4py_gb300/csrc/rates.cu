// Arithmetic-rate measurement for the FP64 path's roofline: the sustained
// FP64 fused multiply-add rate of this GPU, from a kernel of independent
// dependent-FMA chains (no memory traffic) timed with CUDA events.  GB300
// runs FP64 at a small fraction of its FP32 rate, and the FP64 EAM kernels
// are bounded by it rather than by HBM; a copy-bandwidth peak says nothing
// about them.
#include "system.h"

namespace mappg {

// kChains independent chains per thread keep the FP64 pipe busy; each
// iteration is one FMA per chain (2 flops)
constexpr int kChains = 8;

__global__ void k_fma64(int iters, double b, double c, double* sink) {
    double v[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) v[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < kChains; k++) v[k] = fma(v[k], b, c);
    }
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; k++) t += v[k];
    if (t == 12345.678) sink[0] = t;  // keeps the chains live; never true for these inputs
}

}  // namespace mappg

using namespace mappg;

// FP64 FMA throughput in TFLOP/s (2 flops per FMA): `reps` timed launches
// of `iters` iterations over every SM (8 blocks of 256 threads per SM),
// after one untimed launch; the best launch counts.
extern "C" int mappg_fp64_fma_rate(int iters, int reps, double* tflops) {
    try {
        if (!tflops || iters <= 0 || reps <= 0) throw Error{MAPPG_ERR_ARG, "bad argument"};
        int dev = 0, sms = 0;
        MAPPG_CUDA(cudaGetDevice(&dev));
        MAPPG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        // released on every return, including a failed CUDA call
        struct Held {
            double* sink = nullptr;
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            ~Held() {
                if (e0) cudaEventDestroy(e0);
                if (e1) cudaEventDestroy(e1);
                if (sink) cudaFree(sink);
            }
        } held;
        MAPPG_CUDA(cudaMalloc(&held.sink, sizeof(double)));
        MAPPG_CUDA(cudaEventCreate(&held.e0));
        MAPPG_CUDA(cudaEventCreate(&held.e1));
        double* sink = held.sink;
        cudaEvent_t e0 = held.e0, e1 = held.e1;
        const int grid = sms * 8, block = 256;
        k_fma64<<<grid, block>>>(iters, 0.999999, 1e-7, sink);
        MAPPG_CUDA(cudaGetLastError());
        float best = 1e30f;
        for (int r = 0; r < reps; r++) {
            MAPPG_CUDA(cudaEventRecord(e0));
            k_fma64<<<grid, block>>>(iters, 0.999999, 1e-7, sink);
            MAPPG_CUDA(cudaEventRecord(e1));
            MAPPG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            MAPPG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
        const double flops = 2.0 * kChains * (double)iters * grid * block;
        *tflops = flops / (best * 1e-3) / 1e12;
        return MAPPG_OK;
    } catch (const Error& e) {
        set_error(e.msg);
        return e.code;
    }
}
