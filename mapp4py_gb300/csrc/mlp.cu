// Tensor-core kernels of the learned L-BFGS preconditioner (tcgen05, BF16
// operands, FP32 accumulation in TMEM), and the check of the MMA building
// blocks against plain arithmetic.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <vector>

#include "linesearch.h"
#include "system.h"
#include "tc.cuh"

namespace mappg {

// D[128 x 64] = A[128 x 64] * Bt[64 x 64]^T with one CTA: the smallest use of
// every tcgen05 piece the MLP kernels rely on (operand layout, descriptors,
// MMA chain over K, commit, TMEM read-back)
// Both operand regions are twice the size the MMAs read and zero-filled
// beyond it, and 256 TMEM columns are held for a 64-column result, so that
// even a misread descriptor stays inside this CTA's memory.
constexpr int kCheckSmem = 64 * 1024;

__global__ void __launch_bounds__(128) k_tc_gemm_check(const uint16_t* __restrict__ A, const uint16_t* __restrict__ Bt,
                                                       float* __restrict__ D, int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t dyn[];
    uint8_t* sA = dyn;                // 32 KB, 16 KB used
    uint8_t* sB = dyn + 32 * 1024;    // 32 KB, 8 KB used
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    const int t = threadIdx.x, w = t >> 5;
    for (int q = t; q < kCheckSmem / 16; q += 128) ((uint4*)dyn)[q] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    for (int q = t; q < 128 * 8; q += 128) {
        const int r = q >> 3, kc = q & 7;
        *(uint4*)(sA + kmajor_off(r, kc * 8, 64)) = *(const uint4*)(A + r * 64 + kc * 8);
    }
    for (int q = t; q < 64 * 8; q += 128) {
        const int r = q >> 3, kc = q & 7;
        *(uint4*)(sB + kmajor_off(r, kc * 8, 64)) = *(const uint4*)(Bt + r * 64 + kc * 8);
    }
    if (t == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (w == 0) tmem_alloc(&tbase, 256);
    fence_smem_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = tbase;
    if (t == 0) {
        for (int kk = 0; kk < 4; kk++) {
            const uint64_t ad = smem_desc(smem_u32(sA) + kk * 256, 128, 64 * 16);
            const uint64_t bd = smem_desc(smem_u32(sB) + kk * 256, 128, 64 * 16);
            tc_mma(tm, ad, bd, idesc_bf16(128, 64), kk > 0 ? 1u : 0u);
        }
        tc_commit(&bar);
    }
    bool ok = mbar_wait(&bar, 0);
    ok = __syncthreads_and(ok);
    tc_fence_after();
    if (ok) {
        for (int c0 = 0; c0 < 64; c0 += 16) {
            float v[16];
            tmem_ld16(tm + ((uint32_t)(32 * w) << 16) + (uint32_t)c0, v);
            for (int i = 0; i < 16; i++) D[(32 * w + (t & 31)) * 64 + c0 + i] = v[i];
        }
    } else {
        if (t == 0) *err = 1;
        mbar_wait(&bar, 0);  // give in-flight MMAs a last bounded chance
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (w == 0) tmem_dealloc(tm, 256);
}

}  // namespace mappg

using namespace mappg;

extern "C" int mappg_tc_gemm_check(const uint16_t* A, const uint16_t* Bt, float* D) {
    uint16_t *dA = nullptr, *dB = nullptr;
    float* dD = nullptr;
    int* dErr = nullptr;
    auto release = [&] {
        if (dA) cudaFree(dA);
        if (dB) cudaFree(dB);
        if (dD) cudaFree(dD);
        if (dErr) cudaFree(dErr);
    };
    try {
        if (!A || !Bt || !D) throw Error{MAPPG_ERR_ARG, "null argument"};
        MAPPG_CUDA(cudaMalloc(&dA, 128 * 64 * 2));
        MAPPG_CUDA(cudaMalloc(&dB, 64 * 64 * 2));
        MAPPG_CUDA(cudaMalloc(&dD, 128 * 64 * 4));
        MAPPG_CUDA(cudaMalloc(&dErr, 4));
        MAPPG_CUDA(cudaMemcpy(dA, A, 128 * 64 * 2, cudaMemcpyHostToDevice));
        MAPPG_CUDA(cudaMemcpy(dB, Bt, 64 * 64 * 2, cudaMemcpyHostToDevice));
        MAPPG_CUDA(cudaMemset(dErr, 0, 4));
        MAPPG_CUDA(cudaFuncSetAttribute(k_tc_gemm_check, cudaFuncAttributeMaxDynamicSharedMemorySize, kCheckSmem));
        k_tc_gemm_check<<<1, 128, kCheckSmem>>>(dA, dB, dD, dErr);
        MAPPG_CUDA(cudaGetLastError());
        int err = 0;
        MAPPG_CUDA(cudaMemcpy(&err, dErr, 4, cudaMemcpyDeviceToHost));
        MAPPG_CUDA(cudaMemcpy(D, dD, 128 * 64 * 4, cudaMemcpyDeviceToHost));
        if (err) throw Error{MAPPG_ERR_TIMEOUT, "tensor-core MMA did not complete"};
        release();
        return MAPPG_OK;
    } catch (const Error& e) {
        release();
        set_error(e.msg);
        return e.code;
    }
}

// =====================================================================
// The preconditioner network: 33 inputs (16 Gaussian radial functions per
// neighbour species and the host density, standardised) -> 64 -> 64 -> 3,
// tanh hidden units, softplus outputs: an estimate of the three diagonal
// Hessian elements of an atom, whose inverses are L-BFGS's initial inverse
// Hessian.  Biases ride as weights on a constant-one input (feature 33 of
// the input, unit 64 of each hidden layer), so every layer is one GEMM.
//
// One CTA of 128 threads takes tiles of 128 atoms; thread t owns atom row t
// in every epilogue.  All products run on the tensor cores:
//   forward   Z1 = X W1^T, Z2 = H1 W2^T, Z3 = H2 W3^T       (M = 128 atoms)
//   backward  dH2 = dZ3 W3, dH1 = dZ2 W2                   (M = 128 atoms)
//   gradients G3 += dZ3^T H2, G2 += dZ2^T H1, G1 += dZ1^T X (K = 128 atoms)
// The gradient sums stay in TMEM over all tiles of a CTA and are written
// once as that CTA's partial; a fixed-order reduction and AdamW follow.
// =====================================================================
namespace mappg {

constexpr int kIn = 64;     // input width (33 features, the constant, zero pad)
constexpr int kHid = 64;    // hidden units per layer
constexpr int kHidK = 80;   // hidden layer as the next layer's K (units, constant, pad)
constexpr int kOut = 16;    // output width (3 used)
constexpr int kTile = 128;  // atoms per tile
constexpr int kNW1 = kHid * kIn, kNW2 = kHid * kHidK, kNW3 = kOut * kHidK;
constexpr int kNParam = kNW1 + kNW2 + kNW3;  // 10496
constexpr int kPartStride = kNParam + 32;    // per-CTA partial: gradients then loss

// dynamic shared memory layout of the training kernel (bytes)
constexpr int kSmXa = 0;                            // [128][64]  A: X
constexpr int kSmH1a = kSmXa + kTile * kIn * 2;     // [128][80]  A: H1
constexpr int kSmH2a = kSmH1a + kTile * kHidK * 2;  // [128][80]  A: H2
constexpr int kSmDZ3a = kSmH2a + kTile * kHidK * 2; // [128][16]  A: dZ3
constexpr int kSmDZ2a = kSmDZ3a + kTile * kOut * 2; // [128][64]  A: dZ2
constexpr int kSmW1 = kSmDZ2a + kTile * kHid * 2;   // [64][64]   B: W1
constexpr int kSmW2 = kSmW1 + kHid * kIn * 2;       // [64][80]   B: W2
constexpr int kSmW3 = kSmW2 + kHid * kHidK * 2;     // [16][80]   B: W3
constexpr int kSmW3t = kSmW3 + kOut * kHidK * 2;    // [64][16]   B: W3^T (hidden 2 x out)
constexpr int kSmW2t = kSmW3t + kHid * kOut * 2;    // [64][64]   B: W2^T without the bias column
constexpr int kSmAT = kSmW2t + kHid * kHid * 2;     // [128][128] A: dZ^T (64 rows used)
constexpr int kSmXT = kSmAT + 128 * kTile * 2;      // [64][128]  B: X^T
constexpr int kSmH1T = kSmXT + kIn * kTile * 2;     // [80][128]  B: H1^T
constexpr int kSmH2T = kSmH1T + kHidK * kTile * 2;  // [80][128]  B: H2^T
constexpr int kSmTrain = kSmH2T + kHidK * kTile * 2;
constexpr int kSmInfer = kSmW3 + kOut * kHidK * 2;  // the forward pass uses X, H1, H2 and W1..W3

// TMEM columns
constexpr uint32_t kTmD = 0, kTmG1 = 64, kTmG2 = 128, kTmG3 = 224, kTmCols = 512;

struct Norm33 {
    float mean[33], sdev[33];
};

struct MlpArgs {
    const uint16_t* X;   // [n][64] bf16 inputs
    const float* Y;      // [n][3] targets (training), may be null
    float* out;          // [n][3] predictions (inference), may be null
    const uint16_t* w1;  // [64][64] bf16
    const uint16_t* w2;  // [64][80]
    const uint16_t* w3;  // [16][80]
    const uint16_t* w3t; // [64][16]
    const uint16_t* w2t; // [64][64]
    float* part;         // [grid][kPartStride] per-CTA gradients and loss
    int* err;
    int n;
    float inv_count;     // 1 / (3 n): the loss is a mean over outputs
};

__device__ __forceinline__ uint16_t f2bf(float f) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}
__device__ __forceinline__ float bf2f(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// copy a [rows][K] row-major bf16 matrix into the K-major operand layout
__device__ __forceinline__ void stage_rows(uint8_t* dst, const uint16_t* src, int rows, int K) {
    const int chunks = rows * (K / 8);
    for (int q = threadIdx.x; q < chunks; q += blockDim.x) {
        const int r = q / (K / 8), kc = q % (K / 8);
        *(uint4*)(dst + kmajor_off(r, kc * 8, K)) = *(const uint4*)(src + (size_t)r * K + kc * 8);
    }
}

__device__ __forceinline__ float softplus(float z) { return z > 20.f ? z : log1pf(expf(z)); }
__device__ __forceinline__ float sigmoid(float z) { return 1.f / (1.f + expf(-z)); }

// issue D (+)= A[128 x K] B[N x K]^T as K/16 MMAs (one thread)
__device__ __forceinline__ void mma_chain(uint32_t tmem_d, uint32_t a, int lda_k, uint32_t b, int ldb_k, int K, int N,
                                          bool accumulate) {
    for (int kk = 0; kk < K / 16; kk++) {
        const uint64_t ad = smem_desc(a + kk * 256, 128, lda_k * 16);
        const uint64_t bd = smem_desc(b + kk * 256, 128, ldb_k * 16);
        tc_mma(tmem_d, ad, bd, idesc_bf16(128, N), (accumulate || kk > 0) ? 1u : 0u);
    }
}

// make this thread's shared-memory writes visible to the MMA, then run body
// on thread 0 and wait for the MMAs it commits; false on timeout
template <class F>
__device__ __forceinline__ bool mma_stage(uint64_t* bar, uint32_t& phase, F body) {
    fence_smem_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0) {
        body();
        tc_commit(bar);
    }
    bool ok = mbar_wait(bar, phase);
    phase ^= 1u;
    ok = __syncthreads_and(ok);
    tc_fence_after();
    return ok;
}

// one row of 16 TMEM columns of this thread's lane
__device__ __forceinline__ void row16(uint32_t tbase, uint32_t col, float (&v)[16]) {
    tmem_ld16(tbase + ((uint32_t)(threadIdx.x & ~31) << 16) + col, v);
}

template <bool TRAIN>
__global__ void __launch_bounds__(128, 1) k_mlp(MlpArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase_s;
    const int t = threadIdx.x;
    const uint32_t s0 = smem_u32(sm);
    // zero everything once (the padding rows and columns stay zero)
    const int bytes = TRAIN ? kSmTrain : kSmInfer;
    for (int q = t; q < bytes / 16; q += blockDim.x) ((uint4*)sm)[q] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    stage_rows(sm + kSmW1, a.w1, kHid, kIn);
    stage_rows(sm + kSmW2, a.w2, kHid, kHidK);
    stage_rows(sm + kSmW3, a.w3, kOut, kHidK);
    if (TRAIN) {
        stage_rows(sm + kSmW3t, a.w3t, kHid, kOut);
        stage_rows(sm + kSmW2t, a.w2t, kHid, kHid);
    }
    if (t == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // the forward pass uses the first 64 columns only
    constexpr uint32_t cols = TRAIN ? kTmCols : 64u;
    if (t < 32) tmem_alloc(&tbase_s, cols);
    fence_smem_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tb = tbase_s;
    uint32_t phase = 0;
    bool ok = true, first = true;
    float loss = 0.f;
    const int ntiles = (a.n + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int m = tile * kTile + t;
        const bool valid = m < a.n;
        // ---- X tile: row t of Xa and column t of XT
        uint16_t xrow[kIn];
        if (valid) {
            const uint4* src = (const uint4*)(a.X + (size_t)m * kIn);
#pragma unroll
            for (int c = 0; c < kIn / 8; c++) *(uint4*)(xrow + 8 * c) = src[c];
        } else {
#pragma unroll
            for (int c = 0; c < kIn; c++) xrow[c] = 0;
        }
#pragma unroll
        for (int c = 0; c < kIn / 8; c++) *(uint4*)(sm + kSmXa + kmajor_off(t, c * 8, kIn)) = *(uint4*)(xrow + 8 * c);
        if (TRAIN)
            for (int k = 0; k < kIn; k++) *(uint16_t*)(sm + kSmXT + kmajor_off(k, t, kTile)) = xrow[k];
        // ---- layer 1
        ok = mma_stage(&bar, phase, [&] { mma_chain(tb + kTmD, s0 + kSmXa, kIn, s0 + kSmW1, kIn, kIn, kHid, false); });
        if (!ok) break;
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            row16(tb, kTmD + c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const uint16_t h = f2bf(tanhf(v[i]));
                *(uint16_t*)(sm + kSmH1a + kmajor_off(t, c0 + i, kHidK)) = h;
                if (TRAIN) *(uint16_t*)(sm + kSmH1T + kmajor_off(c0 + i, t, kTile)) = h;
            }
        }
        const uint16_t one = f2bf(1.f);
        *(uint16_t*)(sm + kSmH1a + kmajor_off(t, kHid, kHidK)) = one;
        if (TRAIN) *(uint16_t*)(sm + kSmH1T + kmajor_off(kHid, t, kTile)) = one;
        // ---- layer 2
        ok = mma_stage(&bar, phase,
                       [&] { mma_chain(tb + kTmD, s0 + kSmH1a, kHidK, s0 + kSmW2, kHidK, kHidK, kHid, false); });
        if (!ok) break;
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            row16(tb, kTmD + c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const uint16_t h = f2bf(tanhf(v[i]));
                *(uint16_t*)(sm + kSmH2a + kmajor_off(t, c0 + i, kHidK)) = h;
                if (TRAIN) *(uint16_t*)(sm + kSmH2T + kmajor_off(c0 + i, t, kTile)) = h;
            }
        }
        *(uint16_t*)(sm + kSmH2a + kmajor_off(t, kHid, kHidK)) = one;
        if (TRAIN) *(uint16_t*)(sm + kSmH2T + kmajor_off(kHid, t, kTile)) = one;
        // ---- layer 3
        ok = mma_stage(&bar, phase,
                       [&] { mma_chain(tb + kTmD, s0 + kSmH2a, kHidK, s0 + kSmW3, kHidK, kHidK, kOut, false); });
        if (!ok) break;
        float z[16];
        row16(tb, kTmD, z);
        if (!TRAIN) {
            if (valid)
                for (int o = 0; o < 3; o++) a.out[(size_t)m * 3 + o] = softplus(z[o]);
            continue;
        }
        // ---- loss (mean squared log error) and dZ3
        float dz3[3] = {0.f, 0.f, 0.f};
        if (valid) {
            for (int o = 0; o < 3; o++) {
                const float y = softplus(z[o]);
                const float r = logf(y) - logf(a.Y[(size_t)m * 3 + o]);
                loss += r * r;
                dz3[o] = 2.f * r / y * sigmoid(z[o]) * a.inv_count;
            }
        }
        for (int o = 0; o < kOut; o++) {
            const uint16_t d = f2bf(o < 3 ? dz3[o] : 0.f);
            *(uint16_t*)(sm + kSmDZ3a + kmajor_off(t, o, kOut)) = d;
        }
        for (int r = 0; r < kHid; r++)
            *(uint16_t*)(sm + kSmAT + kmajor_off(r, t, kTile)) = f2bf(r < 3 ? dz3[r] : 0.f);
        // ---- G3 += dZ3^T H2 ; dH2 = dZ3 W3
        ok = mma_stage(&bar, phase, [&] {
            mma_chain(tb + kTmG3, s0 + kSmAT, kTile, s0 + kSmH2T, kTile, kTile, kHidK, !first);
            mma_chain(tb + kTmD, s0 + kSmDZ3a, kOut, s0 + kSmW3t, kOut, kOut, kHid, false);
        });
        if (!ok) break;
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            row16(tb, kTmD + c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const float h = bf2f(*(uint16_t*)(sm + kSmH2a + kmajor_off(t, c0 + i, kHidK)));
                const uint16_t d = f2bf(valid ? v[i] * (1.f - h * h) : 0.f);
                *(uint16_t*)(sm + kSmDZ2a + kmajor_off(t, c0 + i, kHid)) = d;
                *(uint16_t*)(sm + kSmAT + kmajor_off(c0 + i, t, kTile)) = d;
            }
        }
        // ---- G2 += dZ2^T H1 ; dH1 = dZ2 W2
        ok = mma_stage(&bar, phase, [&] {
            mma_chain(tb + kTmG2, s0 + kSmAT, kTile, s0 + kSmH1T, kTile, kTile, kHidK, !first);
            mma_chain(tb + kTmD, s0 + kSmDZ2a, kHid, s0 + kSmW2t, kHid, kHid, kHid, false);
        });
        if (!ok) break;
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            row16(tb, kTmD + c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const float h = bf2f(*(uint16_t*)(sm + kSmH1a + kmajor_off(t, c0 + i, kHidK)));
                *(uint16_t*)(sm + kSmAT + kmajor_off(c0 + i, t, kTile)) = f2bf(valid ? v[i] * (1.f - h * h) : 0.f);
            }
        }
        // ---- G1 += dZ1^T X
        ok = mma_stage(&bar, phase,
                       [&] { mma_chain(tb + kTmG1, s0 + kSmAT, kTile, s0 + kSmXT, kTile, kTile, kIn, !first); });
        first = false;
    }
    if (!ok) {
        if (t == 0) atomicExch(a.err, 1);
        mbar_wait(&bar, phase);  // a last bounded wait for MMAs in flight
    }
    if (TRAIN && ok) {
        // this CTA's gradient sums: row t of G1 (t < 64), G2 (t < 64), G3 (t < 16)
        float* P = a.part + (size_t)blockIdx.x * kPartStride;
        for (int c0 = 0; c0 < kHidK; c0 += 16) {
            float v1[16], v2[16], v3[16];
            const bool has = !first;  // false: this CTA saw no tile
            if (c0 < kIn) row16(tb, kTmG1 + c0, v1);
            row16(tb, kTmG2 + c0, v2);
            row16(tb, kTmG3 + c0, v3);
            for (int i = 0; i < 16; i++) {
                if (c0 < kIn && t < kHid) P[t * kIn + c0 + i] = has ? v1[i] : 0.f;
                if (t < kHid) P[kNW1 + t * kHidK + c0 + i] = has ? v2[i] : 0.f;
                if (t < kOut) P[kNW1 + kNW2 + t * kHidK + c0 + i] = has ? v3[i] : 0.f;
            }
        }
        // loss: block sum in a fixed order
        __shared__ float red[128];
        red[t] = loss;
        __syncthreads();
        if (t == 0) {
            float s = 0.f;
            for (int q = 0; q < 128; q++) s += red[q];
            P[kNParam] = s;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (t < 32) tmem_dealloc(tb, cols);
}

// sum of the per-CTA partials in a fixed order: grad[p] = sum_b part[b][p]
__global__ void k_mlp_reduce(const float* __restrict__ part, int nblk, float* __restrict__ grad) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p <= kNParam; p += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblk; b++) s += part[(size_t)b * kPartStride + p];
        grad[p] = s;
    }
}

// AdamW on the FP32 master weights, then the BF16 operand copies
struct AdamArgs {
    float* w;       // kNParam master weights (W1 | W2 | W3, row-major [n][k])
    float* m;
    float* v;
    const float* g;
    uint16_t *w1, *w2, *w3, *w3t, *w2t;
    float lr, beta1, beta2, eps, wd, bc1, bc2;  // bc = 1 - beta^t
    int step;  // 0: only refresh the BF16 copies
};

__device__ __forceinline__ bool is_bias(int p) {
    if (p < kNW1) return p % kIn == 33;
    if (p < kNW1 + kNW2) return (p - kNW1) % kHidK == kHid;
    return (p - kNW1 - kNW2) % kHidK == kHid;
}

__global__ void k_adamw(AdamArgs a) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kNParam; p += gridDim.x * blockDim.x) {
        float w = a.w[p];
        if (a.step > 0) {
            const float g = a.g[p];
            const float m = a.beta1 * a.m[p] + (1.f - a.beta1) * g;
            const float v = a.beta2 * a.v[p] + (1.f - a.beta2) * g * g;
            a.m[p] = m;
            a.v[p] = v;
            const float mh = m / a.bc1, vh = v / a.bc2;
            if (!is_bias(p)) w -= a.lr * a.wd * w;  // decoupled weight decay, not on biases
            w -= a.lr * mh / (sqrtf(vh) + a.eps);
            a.w[p] = w;
        }
        const uint16_t b = f2bf(w);
        if (p < kNW1) {
            a.w1[p] = b;
        } else if (p < kNW1 + kNW2) {
            const int q = p - kNW1, n = q / kHidK, k = q % kHidK;
            a.w2[q] = b;
            if (k < kHid) a.w2t[k * kHid + n] = b;  // [hidden 1][hidden 2]
        } else {
            const int q = p - kNW1 - kNW2, n = q / kHidK, k = q % kHidK;
            a.w3[q] = b;
            if (k < kHid) a.w3t[k * kOut + n] = b;  // [hidden 2][out]
        }
    }
}

}  // namespace mappg

// ---------------------------------------------------------------------------
// host side: the network handle, training, inference, and the features and
// finite-difference Hessian diagonals it is trained on
// ---------------------------------------------------------------------------
struct mappg_mlp {
    int device = 0, sm_count = 0;
    cudaStream_t stream = nullptr;
    float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr, *part = nullptr, *loss = nullptr;
    int* err = nullptr;
    uint16_t *w1 = nullptr, *w2 = nullptr, *w3 = nullptr, *w3t = nullptr, *w2t = nullptr;
    float mean[33], sdev[33];
    bool have_norm = false;
    long long step = 0;
    uint16_t* X = nullptr;  // training inputs, [n][64] bf16
    float* Y = nullptr;     // training targets, [n][3]
    int n = 0;
    int refresh_every = 0;  // L-BFGS: recompute the diagonal every this many iterations (0: once)
};

namespace mappg {

void launch_descriptors(mappg_sys* s, float* out);  // eam.cu
void launch_force(mappg_sys* s);
void sys_build(mappg_sys* s);
void lbfgs_run(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, const LsParams& ls, int nsteps,
               double* stats, const double* P, long long* n_fallback);
void batch_lbfgs_run(mappg_sys* s, int m, double e_tol, double max_dx, double f_tol, double c_ls, double rho_ls,
                     double min_alpha, int nsteps, const double* P, double* stats);

constexpr int kMlpGridMax = 148;
constexpr int kSmTrainBytes = kSmTrain, kSmInferBytes = kSmInfer;
constexpr float kYmin = 0.25f, kYmax = 200.f;  // clip of the Hessian estimate (eV/A^2)

static int mlp_grid(const mappg_mlp* net, int n) {
    int tiles = (n + kTile - 1) / kTile;
    return std::max(1, std::min(tiles, std::min(kMlpGridMax, net->sm_count)));
}

static void mlp_args(const mappg_mlp* net, MlpArgs& a) {
    memset(&a, 0, sizeof(a));
    a.w1 = net->w1;
    a.w2 = net->w2;
    a.w3 = net->w3;
    a.w3t = net->w3t;
    a.w2t = net->w2t;
    a.part = net->part;
    a.err = net->err;
}

static void mlp_check_err(mappg_mlp* net) {
    int e = 0;
    MAPPG_CUDA(cudaMemcpyAsync(&e, net->err, sizeof(int), cudaMemcpyDeviceToHost, net->stream));
    MAPPG_CUDA(cudaStreamSynchronize(net->stream));
    if (e) {
        MAPPG_CUDA(cudaMemsetAsync(net->err, 0, sizeof(int), net->stream));
        throw Error{MAPPG_ERR_TIMEOUT, "tensor-core MMA did not complete"};
    }
}

// forward pass: y = softplus(MLP(X)) for n rows of X (device), into out
static void mlp_forward(mappg_mlp* net, const uint16_t* X, int n, float* out, cudaStream_t st) {
    MlpArgs a;
    mlp_args(net, a);
    a.X = X;
    a.out = out;
    a.n = n;
    k_mlp<false><<<mlp_grid(net, n), 128, kSmInferBytes, st>>>(a);
    MAPPG_CUDA(cudaGetLastError());
}

// gradient of the mean squared log error over n rows into net->g (plus the
// loss sum in g[kNParam])
static void mlp_gradient(mappg_mlp* net, const uint16_t* X, const float* Y, int n, int count) {
    MlpArgs a;
    mlp_args(net, a);
    a.X = X;
    a.Y = Y;
    a.n = n;
    a.inv_count = 1.f / (3.f * (float)count);
    const int grid = mlp_grid(net, n);
    k_mlp<true><<<grid, 128, kSmTrainBytes, net->stream>>>(a);
    k_mlp_reduce<<<(kNParam + 256) / 256, 256, 0, net->stream>>>(net->part, grid, net->g);
    MAPPG_CUDA(cudaGetLastError());
}

static void mlp_adamw(mappg_mlp* net, float lr, float wd, bool update) {
    AdamArgs a;
    a.w = net->w;
    a.m = net->m;
    a.v = net->v;
    a.g = net->g;
    a.w1 = net->w1;
    a.w2 = net->w2;
    a.w3 = net->w3;
    a.w3t = net->w3t;
    a.w2t = net->w2t;
    a.lr = lr;
    a.beta1 = 0.9f;
    a.beta2 = 0.999f;
    a.eps = 1e-8f;
    a.wd = wd;
    if (update) net->step++;
    a.step = update ? (int)std::min<long long>(net->step, 1 << 30) : 0;
    a.bc1 = (float)(1.0 - pow(0.9, (double)net->step));
    a.bc2 = (float)(1.0 - pow(0.999, (double)net->step));
    k_adamw<<<(kNParam + 255) / 256, 256, 0, net->stream>>>(a);
    MAPPG_CUDA(cudaGetLastError());
}

// standardised features -> bf16 input rows (feature 33 is the constant 1)
__global__ void k_pack_inputs(int n, const float* __restrict__ feat, const int* __restrict__ order, Norm33 nrm,
                              uint16_t* __restrict__ X) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* f = feat + (size_t)(order ? order[i] : i) * 33;
        uint16_t* x = X + (size_t)i * kIn;
        for (int q = 0; q < kIn; q++) {
            float v = 0.f;
            if (q < 33) v = (f[q] - nrm.mean[q]) / nrm.sdev[q];
            if (q == 33) v = 1.f;
            x[q] = f2bf(v);
        }
    }
}

// preconditioner from the predicted Hessian diagonal: P = 1/clip(y), SoA
// 3n doubles in bin order
__global__ void k_precond(int n, const float* __restrict__ y, double* __restrict__ P) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int c = 0; c < 3; c++) P[(size_t)c * n + i] = 1.0 / (double)fminf(fmaxf(y[(size_t)i * 3 + c], kYmin), kYmax);
}

// finite-difference Hessian diagonal: displace the atoms of one colour along
// one axis, and accumulate -f/(2h) with the sign of the displacement
__global__ void k_fd_move(int n, double* __restrict__ x, const double* __restrict__ x_ref, const int* __restrict__ col,
                          int c, int axis, double d) {
    // every component from the reference, so the previous move is undone
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int k = 0; k < 3; k++) {
            const size_t q = (size_t)k * n + i;
            x[q] = (col[i] == c && k == axis) ? x_ref[q] + d : x_ref[q];
        }
}

__global__ void k_fd_acc(int n, const double* __restrict__ f, const int* __restrict__ col, int c, int axis,
                         double scale, double* __restrict__ H) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (col[i] == c) H[(size_t)axis * n + i] += scale * f[(size_t)axis * n + i];
}

}  // namespace mappg

using namespace mappg;

namespace {

template <class F>
int guarded(F&& f) {
    try {
        f();
        return MAPPG_OK;
    } catch (const Error& e) {
        set_error(e.msg);
        return e.code;
    } catch (const std::exception& e) {
        set_error(e.what());
        return MAPPG_ERR_ARG;
    }
}

void mlp_free(mappg_mlp* net) {
    void* p[] = {net->w, net->m, net->v, net->g, net->part, net->loss, net->err, net->w1, net->w2, net->w3,
                 net->w3t, net->w2t, net->X, net->Y};
    for (void* q : p)
        if (q) cudaFree(q);
    if (net->stream) cudaStreamDestroy(net->stream);
}

Norm33 norm_of(const mappg_mlp* net) {
    Norm33 n;
    for (int q = 0; q < 33; q++) {
        n.mean[q] = net->have_norm ? net->mean[q] : 0.f;
        n.sdev[q] = net->have_norm ? net->sdev[q] : 1.f;
    }
    return n;
}

// features (host, n x 33) -> standardised bf16 rows on the device
uint16_t* upload_inputs(mappg_mlp* net, const float* feat, int n, const std::vector<int>* order) {
    float* df = nullptr;
    int* dord = nullptr;
    uint16_t* X = nullptr;
    // the staging arrays go on every return; X only on a failed one (the
    // caller owns it otherwise)
    struct Held {
        float*& df;
        int*& dord;
        uint16_t*& X;
        bool keep_x = false;
        ~Held() {
            if (df) cudaFree(df);
            if (dord) cudaFree(dord);
            if (X && !keep_x) cudaFree(X);
        }
    } held{df, dord, X};
    MAPPG_CUDA(cudaMalloc(&df, sizeof(float) * 33 * (size_t)n));
    MAPPG_CUDA(cudaMalloc(&X, sizeof(uint16_t) * kIn * (size_t)n));
    MAPPG_CUDA(cudaMemcpyAsync(df, feat, sizeof(float) * 33 * (size_t)n, cudaMemcpyHostToDevice, net->stream));
    if (order) {
        MAPPG_CUDA(cudaMalloc(&dord, sizeof(int) * (size_t)n));
        MAPPG_CUDA(cudaMemcpyAsync(dord, order->data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, net->stream));
    }
    k_pack_inputs<<<std::max(1, std::min(1024, (n + 255) / 256)), 256, 0, net->stream>>>(n, df, dord, norm_of(net), X);
    MAPPG_CUDA(cudaGetLastError());
    MAPPG_CUDA(cudaStreamSynchronize(net->stream));
    held.keep_x = true;
    return X;
}

}  // namespace

extern "C" {

int mappg_mlp_nparams(void) { return kNParam; }

int mappg_mlp_create(int seed, mappg_mlp** out) {
    return guarded([&] {
        if (!out) throw Error{MAPPG_ERR_ARG, "null argument"};
        mappg_mlp* net = new mappg_mlp();
        try {
            MAPPG_CUDA(cudaGetDevice(&net->device));
            cudaDeviceProp p;
            MAPPG_CUDA(cudaGetDeviceProperties(&p, net->device));
            net->sm_count = p.multiProcessorCount;
            MAPPG_CUDA(cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking));
            MAPPG_CUDA(cudaFuncSetAttribute(k_mlp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmTrainBytes));
            MAPPG_CUDA(cudaFuncSetAttribute(k_mlp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmInferBytes));
            MAPPG_CUDA(cudaMalloc(&net->w, sizeof(float) * kNParam));
            MAPPG_CUDA(cudaMalloc(&net->m, sizeof(float) * kNParam));
            MAPPG_CUDA(cudaMalloc(&net->v, sizeof(float) * kNParam));
            MAPPG_CUDA(cudaMalloc(&net->g, sizeof(float) * (kNParam + 1)));
            MAPPG_CUDA(cudaMalloc(&net->part, sizeof(float) * kPartStride * kMlpGridMax));
            MAPPG_CUDA(cudaMalloc(&net->loss, sizeof(float) * 4));
            MAPPG_CUDA(cudaMalloc(&net->err, sizeof(int)));
            MAPPG_CUDA(cudaMalloc(&net->w1, 2 * kNW1));
            MAPPG_CUDA(cudaMalloc(&net->w2, 2 * kNW2));
            MAPPG_CUDA(cudaMalloc(&net->w3, 2 * kNW3));
            MAPPG_CUDA(cudaMalloc(&net->w3t, 2 * kHid * kOut));
            MAPPG_CUDA(cudaMalloc(&net->w2t, 2 * kHid * kHid));
            MAPPG_CUDA(cudaMemsetAsync(net->m, 0, sizeof(float) * kNParam, net->stream));
            MAPPG_CUDA(cudaMemsetAsync(net->v, 0, sizeof(float) * kNParam, net->stream));
            MAPPG_CUDA(cudaMemsetAsync(net->err, 0, sizeof(int), net->stream));
            MAPPG_CUDA(cudaMemsetAsync(net->w3t, 0, 2 * kHid * kOut, net->stream));
            // Glorot-uniform weights, zero biases; the output bias starts at
            // softplus^-1(5 eV/A^2), a typical diagonal Hessian element
            std::mt19937 rng((unsigned)seed);
            std::vector<float> w(kNParam, 0.f);
            auto fill = [&](int off, int rows, int K, int fan_in, int real_rows, int bias_col) {
                std::uniform_real_distribution<float> U(-1.f, 1.f);
                const float a = sqrtf(6.f / (float)(fan_in + real_rows));
                for (int r = 0; r < rows; r++)
                    for (int k = 0; k < K; k++) {
                        float v = 0.f;
                        if (r < real_rows && k < fan_in) v = a * U(rng);
                        if (k == bias_col) v = 0.f;
                        w[off + r * K + k] = v;
                    }
            };
            fill(0, kHid, kIn, 33, kHid, 33);
            fill(kNW1, kHid, kHidK, kHid, kHid, kHid);
            fill(kNW1 + kNW2, kOut, kHidK, kHid, 3, kHid);
            for (int o = 0; o < 3; o++) w[kNW1 + kNW2 + o * kHidK + kHid] = logf(expf(5.f) - 1.f);
            MAPPG_CUDA(cudaMemcpyAsync(net->w, w.data(), sizeof(float) * kNParam, cudaMemcpyHostToDevice, net->stream));
            mlp_adamw(net, 0.f, 0.f, false);
            MAPPG_CUDA(cudaStreamSynchronize(net->stream));
        } catch (...) {
            mlp_free(net);
            delete net;
            throw;
        }
        *out = net;
    });
}

void mappg_mlp_destroy(mappg_mlp* net) {
    if (!net) return;
    mlp_free(net);
    delete net;
}

int mappg_mlp_set_data(mappg_mlp* net, const float* feat, const float* target, int n, int seed) {
    return guarded([&] {
        if (!net || !feat || !target) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (n < 1) throw Error{MAPPG_ERR_ARG, "no training rows"};
        // standardisation of each feature over the training set
        for (int q = 0; q < 33; q++) {
            double s1 = 0.0, s2 = 0.0;
            for (int i = 0; i < n; i++) {
                const double v = feat[(size_t)i * 33 + q];
                s1 += v;
                s2 += v * v;
            }
            const double mu = s1 / n, var = std::max(s2 / n - mu * mu, 0.0);
            net->mean[q] = (float)mu;
            net->sdev[q] = (float)std::max(sqrt(var), 1e-6);
        }
        net->have_norm = true;
        std::vector<int> order(n);
        for (int i = 0; i < n; i++) order[i] = i;
        std::mt19937 rng((unsigned)seed);
        std::shuffle(order.begin(), order.end(), rng);
        std::vector<float> y(3 * (size_t)n);
        for (int i = 0; i < n; i++)
            for (int c = 0; c < 3; c++) {
                const float v = target[(size_t)order[i] * 3 + c];
                if (!(v == v)) throw Error{MAPPG_ERR_NAN, "non-finite target"};
                y[(size_t)i * 3 + c] = std::min(std::max(v, kYmin), kYmax);
            }
        if (net->X) cudaFree(net->X);
        if (net->Y) cudaFree(net->Y);
        net->X = nullptr;
        net->Y = nullptr;
        net->X = upload_inputs(net, feat, n, &order);
        MAPPG_CUDA(cudaMalloc(&net->Y, sizeof(float) * 3 * (size_t)n));
        MAPPG_CUDA(cudaMemcpy(net->Y, y.data(), sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice));
        net->n = n;
    });
}

// minibatch AdamW over the stored set; losses[e] = mean squared log error
// of epoch e (measured on the batches as they were trained)
int mappg_mlp_train(mappg_mlp* net, int epochs, int batch, double lr, double wd, double* losses) {
    return guarded([&] {
        if (!net) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (!net->X) throw Error{MAPPG_ERR_ARG, "no training data (mappg_mlp_set_data)"};
        if (epochs < 0 || batch < kTile) throw Error{MAPPG_ERR_ARG, "epochs >= 0 and batch >= 128 required"};
        batch = batch / kTile * kTile;
        for (int e = 0; e < epochs; e++) {
            double lsum = 0.0;
            for (int b0 = 0; b0 < net->n; b0 += batch) {
                const int nb = std::min(batch, net->n - b0);
                mlp_gradient(net, net->X + (size_t)b0 * kIn, net->Y + (size_t)b0 * 3, nb, nb);
                mlp_adamw(net, (float)lr, (float)wd, true);
                float l = 0.f;
                MAPPG_CUDA(cudaMemcpyAsync(&l, net->g + kNParam, sizeof(float), cudaMemcpyDeviceToHost, net->stream));
                MAPPG_CUDA(cudaStreamSynchronize(net->stream));
                lsum += l;
            }
            mlp_check_err(net);
            if (losses) losses[e] = lsum / (3.0 * net->n);
        }
    });
}

int mappg_mlp_grad(mappg_mlp* net, const float* feat, const float* target, int n, float* grad, double* loss) {
    return guarded([&] {
        if (!net || !feat || !target || !grad) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (n < 1) throw Error{MAPPG_ERR_ARG, "no rows"};
        uint16_t* X = upload_inputs(net, feat, n, nullptr);
        float* Y = nullptr;
        try {
            MAPPG_CUDA(cudaMalloc(&Y, sizeof(float) * 3 * (size_t)n));
            MAPPG_CUDA(cudaMemcpy(Y, target, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice));
            mlp_gradient(net, X, Y, n, n);
            MAPPG_CUDA(cudaMemcpyAsync(grad, net->g, sizeof(float) * kNParam, cudaMemcpyDeviceToHost, net->stream));
            float l = 0.f;
            MAPPG_CUDA(cudaMemcpyAsync(&l, net->g + kNParam, sizeof(float), cudaMemcpyDeviceToHost, net->stream));
            mlp_check_err(net);
            if (loss) *loss = l / (3.0 * n);
        } catch (...) {
            cudaFree(X);
            if (Y) cudaFree(Y);
            throw;
        }
        cudaFree(X);
        cudaFree(Y);
    });
}

int mappg_mlp_predict(mappg_mlp* net, const float* feat, int n, float* out) {
    return guarded([&] {
        if (!net || !feat || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (n < 1) throw Error{MAPPG_ERR_ARG, "no rows"};
        uint16_t* X = upload_inputs(net, feat, n, nullptr);
        float* dout = nullptr;
        try {
            MAPPG_CUDA(cudaMalloc(&dout, sizeof(float) * 3 * (size_t)n));
            mlp_forward(net, X, n, dout, net->stream);
            MAPPG_CUDA(cudaMemcpyAsync(out, dout, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, net->stream));
            mlp_check_err(net);
        } catch (...) {
            cudaFree(X);
            if (dout) cudaFree(dout);
            throw;
        }
        cudaFree(X);
        cudaFree(dout);
    });
}

// parameters: W1 [64][64] | W2 [64][80] | W3 [16][80], row-major [unit][input];
// norm: 33 means then 33 standard deviations
int mappg_mlp_get_params(mappg_mlp* net, float* w, float* norm) {
    return guarded([&] {
        if (!net) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (w) {
            MAPPG_CUDA(cudaMemcpyAsync(w, net->w, sizeof(float) * kNParam, cudaMemcpyDeviceToHost, net->stream));
            MAPPG_CUDA(cudaStreamSynchronize(net->stream));
        }
        if (norm) {
            const Norm33 nr = norm_of(net);
            for (int q = 0; q < 33; q++) {
                norm[q] = nr.mean[q];
                norm[33 + q] = nr.sdev[q];
            }
        }
    });
}

int mappg_mlp_set_params(mappg_mlp* net, const float* w, const float* norm) {
    return guarded([&] {
        if (!net) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (w) {
            MAPPG_CUDA(cudaMemcpyAsync(net->w, w, sizeof(float) * kNParam, cudaMemcpyHostToDevice, net->stream));
            mlp_adamw(net, 0.f, 0.f, false);
            MAPPG_CUDA(cudaStreamSynchronize(net->stream));
        }
        if (norm) {
            for (int q = 0; q < 33; q++) {
                if (!(norm[33 + q] > 0.f)) throw Error{MAPPG_ERR_ARG, "standard deviations must be positive"};
                net->mean[q] = norm[q];
                net->sdev[q] = norm[33 + q];
            }
            net->have_norm = true;
        }
    });
}

// preconditioner features of the system's atoms, n x 33 in caller order
int mappg_sys_descriptors(mappg_sys* s, float* feat) {
    return guarded([&] {
        if (!s || !feat) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (!s->built) sys_build(s);
        float* d = nullptr;
        MAPPG_CUDA(cudaMalloc(&d, sizeof(float) * 33 * (size_t)s->n));
        std::vector<float> tmp(33 * (size_t)s->n);
        try {
            launch_descriptors(s, d);
            MAPPG_CUDA(cudaMemcpyAsync(tmp.data(), d, sizeof(float) * tmp.size(), cudaMemcpyDeviceToHost, s->stream));
            MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        } catch (...) {
            cudaFree(d);
            throw;
        }
        cudaFree(d);
        for (int i = 0; i < s->n; i++)
            memcpy(feat + (size_t)s->host_id[i] * 33, tmp.data() + (size_t)i * 33, sizeof(float) * 33);
    });
}

// diagonal Hessian elements by central differences of the forces: atoms of
// one colour (color[], caller order; same-coloured atoms must sit further
// apart than twice the cutoff) move together by +-h along one axis
int mappg_sys_hessian_diag(mappg_sys* s, const int* color, double h, double* out) {
    return guarded([&] {
        if (!s || !color || !out) throw Error{MAPPG_ERR_ARG, "null argument"};
        if (s->precision != MAPPG_FP64) throw Error{MAPPG_ERR_ARG, "finite differences run on FP64 systems"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "finite differences run per single cell"};
        if (!(h > 0.0 && h < 0.25 * s->skin)) throw Error{MAPPG_ERR_ARG, "h must be in (0, skin/4)"};
        const int n = s->n;
        int ncol = 0;
        std::vector<int> col(n);
        for (int i = 0; i < n; i++) {
            const int c = color[s->host_id[i]];
            if (c < 0) throw Error{MAPPG_ERR_ARG, "colours must be >= 0"};
            col[i] = c;
            ncol = std::max(ncol, c + 1);
        }
        if (!s->built) sys_build(s);
        int* dcol = nullptr;
        double *xref = nullptr, *H = nullptr;
        auto release = [&] {
            if (dcol) cudaFree(dcol);
            if (xref) cudaFree(xref);
            if (H) cudaFree(H);
        };
        try {
            MAPPG_CUDA(cudaMalloc(&dcol, sizeof(int) * n));
            MAPPG_CUDA(cudaMalloc(&xref, sizeof(double) * 3 * (size_t)n));
            MAPPG_CUDA(cudaMalloc(&H, sizeof(double) * 3 * (size_t)n));
            cudaStream_t st = s->stream;
            MAPPG_CUDA(cudaMemcpyAsync(dcol, col.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
            MAPPG_CUDA(cudaMemcpyAsync(xref, s->x, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToDevice, st));
            MAPPG_CUDA(cudaMemsetAsync(H, 0, sizeof(double) * 3 * (size_t)n, st));
            const int g = std::max(1, std::min(1024, (n + 255) / 256));
            for (int c = 0; c < ncol; c++)
                for (int ax = 0; ax < 3; ax++)
                    for (int sg = -1; sg <= 1; sg += 2) {
                        k_fd_move<<<g, 256, 0, st>>>(n, s->x, xref, dcol, c, ax, sg * h);
                        launch_force(s);
                        k_fd_acc<<<g, 256, 0, st>>>(n, s->f, dcol, c, ax, -sg / (2.0 * h), H);
                    }
            MAPPG_CUDA(cudaMemcpyAsync(s->x, xref, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToDevice, st));
            MAPPG_CUDA(cudaGetLastError());
            std::vector<double> Hh(3 * (size_t)n);
            MAPPG_CUDA(cudaMemcpyAsync(Hh.data(), H, sizeof(double) * Hh.size(), cudaMemcpyDeviceToHost, st));
            MAPPG_CUDA(cudaStreamSynchronize(st));
            for (int i = 0; i < n; i++)
                for (int c = 0; c < 3; c++) out[3 * (size_t)s->host_id[i] + c] = Hh[(size_t)c * n + i];
        } catch (...) {
            release();
            throw;
        }
        release();
    });
}

// L-BFGS with the learned diagonal initial inverse Hessian: features and the
// network's prediction are computed once on the device at the start
static void run_precond(mappg_sys* s, mappg_mlp* net, int m, double e_tol, double max_dx, double f_tol, double c,
                        double rho, double min_alpha, int nsteps, double* stats, bool batch) {
        if (!net->have_norm) throw Error{MAPPG_ERR_ARG, "the network has no input standardisation (train it first)"};
        const int n = s->n;
        float *feat = nullptr, *y = nullptr;
        uint16_t* X = nullptr;
        double* P = nullptr;
        auto release = [&] {
            if (feat) cudaFree(feat);
            if (y) cudaFree(y);
            if (X) cudaFree(X);
            if (P) cudaFree(P);
        };
        try {
            sys_build(s);
            MAPPG_CUDA(cudaMalloc(&feat, sizeof(float) * 33 * (size_t)n));
            MAPPG_CUDA(cudaMalloc(&y, sizeof(float) * 3 * (size_t)n));
            MAPPG_CUDA(cudaMalloc(&X, sizeof(uint16_t) * kIn * (size_t)n));
            MAPPG_CUDA(cudaMalloc(&P, sizeof(double) * 3 * (size_t)n));
            // features of the current configuration -> network -> diagonal
            auto predict = [&] {
                launch_descriptors(s, feat);
                const int g = std::max(1, std::min(1024, (n + 255) / 256));
                k_pack_inputs<<<g, 256, 0, s->stream>>>(n, feat, nullptr, norm_of(net), X);
                MAPPG_CUDA(cudaMemsetAsync(net->err, 0, sizeof(int), s->stream));
                mlp_forward(net, X, n, y, s->stream);
                k_precond<<<g, 256, 0, s->stream>>>(n, y, P);
                MAPPG_CUDA(cudaGetLastError());
                int e = 0;
                MAPPG_CUDA(cudaMemcpyAsync(&e, net->err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
                MAPPG_CUDA(cudaStreamSynchronize(s->stream));
                if (e) throw Error{MAPPG_ERR_TIMEOUT, "tensor-core MMA did not complete"};
            };
            predict();
            struct Refresh {
                mappg_sys* s;
                ~Refresh() {
                    s->precond_refresh = nullptr;
                    s->precond_every = 0;
                }
            } refresh{s};
            s->precond_refresh = predict;
            s->precond_every = net->refresh_every;
            if (batch) {
                batch_lbfgs_run(s, m, e_tol, max_dx, f_tol, c, rho, min_alpha, nsteps, P, stats);
            } else {
                long long nfb = 0;
                double st6[6];
                LsParams ls;
                ls.c = c;
                ls.rho = rho;
                ls.min_alpha = min_alpha;
                lbfgs_run(s, m, e_tol, max_dx, f_tol, ls, nsteps, st6, P, &nfb);
                if (stats) {
                    for (int k = 0; k < 6; k++) stats[k] = st6[k];
                    stats[6] = (double)nfb;
                }
            }
        } catch (...) {
            release();
            throw;
        }
        release();
}

}  // extern "C"

namespace mappg {
void sys_upload(mappg_sys* s, const double* host, double* dev);  // system.cu
}  // namespace mappg

// P = 1/d, d the caller's Hessian diagonal (bin order, SoA)
__global__ void k_inv_diag(int n3, double* __restrict__ P, int* __restrict__ bad) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += gridDim.x * blockDim.x) {
        const double d = P[q];
        if (!(d > 0.0) || !isfinite(d)) {
            *bad = 1;
            P[q] = 1.0;
        } else {
            P[q] = 1.0 / d;
        }
    }
}

extern "C" {

int mappg_lbfgs_run_diag(mappg_sys* s, const double* hdiag, int m, double e_tol, double max_dx, double f_tol,
                         double c, double rho, double min_alpha, int nsteps, double* stats) {
    return guarded([&] {
        if (!s || !hdiag) throw Error{MAPPG_ERR_ARG, "null argument"};
        const int n = s->n;
        double* P = nullptr;
        int* bad = nullptr;
        struct Release {
            double*& P;
            int*& bad;
            ~Release() {
                if (P) cudaFree(P);
                if (bad) cudaFree(bad);
            }
        } release{P, bad};
        MAPPG_CUDA(cudaMalloc(&P, sizeof(double) * 3 * (size_t)n));
        MAPPG_CUDA(cudaMalloc(&bad, sizeof(int)));
        MAPPG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s->stream));
        sys_upload(s, hdiag, P);
        const int g = std::max(1, std::min(1024, (3 * n + 255) / 256));
        k_inv_diag<<<g, 256, 0, s->stream>>>(3 * n, P, bad);
        MAPPG_CUDA(cudaGetLastError());
        int hb = 0;
        MAPPG_CUDA(cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        MAPPG_CUDA(cudaStreamSynchronize(s->stream));
        if (hb) throw Error{MAPPG_ERR_ARG, "the Hessian diagonal must be positive and finite"};
        sys_build(s);
        if (s->ncell > 1) {
            batch_lbfgs_run(s, m, e_tol, max_dx, f_tol, c, rho, min_alpha, nsteps, P, stats);
        } else {
            long long nfb = 0;
            double st6[6];
            LsParams ls;
            ls.c = c;
            ls.rho = rho;
            ls.min_alpha = min_alpha;
            lbfgs_run(s, m, e_tol, max_dx, f_tol, ls, nsteps, st6, P, &nfb);
            if (stats) {
                for (int k = 0; k < 6; k++) stats[k] = st6[k];
                stats[6] = (double)nfb;
            }
        }
    });
}

int mappg_mlp_set_refresh(mappg_mlp* net, int every) {
    return guarded([&] {
        if (!net || every < 0) throw Error{MAPPG_ERR_ARG, "bad argument"};
        net->refresh_every = every;
    });
}

int mappg_lbfgs_run_precond(mappg_sys* s, mappg_mlp* net, int m, double e_tol, double max_dx, double f_tol,
                            double c, double rho, double min_alpha, int nsteps, double* stats) {
    return guarded([&] {
        if (!s || !net) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell > 1) throw Error{MAPPG_ERR_UNSUPP, "a batch of cells runs with mappg_batch_lbfgs_run_precond"};
        run_precond(s, net, m, e_tol, max_dx, f_tol, c, rho, min_alpha, nsteps, stats, false);
    });
}

int mappg_batch_lbfgs_run_precond(mappg_sys* s, mappg_mlp* net, int m, double e_tol, double max_dx, double f_tol,
                                  double c, double rho, double min_alpha, int nsteps, double* stats) {
    return guarded([&] {
        if (!s || !net) throw Error{MAPPG_ERR_ARG, "null handle"};
        if (s->ncell < 2) throw Error{MAPPG_ERR_ARG, "not a batch of cells"};
        run_precond(s, net, m, e_tol, max_dx, f_tol, c, rho, min_alpha, nsteps, stats, true);
    });
}

}  // extern "C"
