// Reduction helpers shared by the EAM kernels: block partials written to a
// per-block slot row, and a fixed-order final sum by the last block to
// finish (deterministic, no floating-point atomics).
#pragma once

#include "system.h"

namespace mappg {

// 32-byte read-only loads (one sector per lane, one instruction): the spline
// records are 32 bytes and 32-byte aligned, so a lane fetches a whole record
// with one L1 request instead of two
__device__ __forceinline__ Dbl4 ldg4(const Dbl4* p) {
    Dbl4 r;
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];" : "=d"(r.x), "=d"(r.y), "=d"(r.z), "=d"(r.w) : "l"(p));
    return r;
}

__device__ __forceinline__ void ldg8(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// block-wide sum of K doubles into partials[blockIdx.x*kRedSlots + slot0 + k];
// returns true in the block that finished last (its threads then see all
// partials)
template <int K>
__device__ bool block_partials(double (&v)[K], double* partials, int slot0, unsigned* counter) {
    __shared__ double red[32][K];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[w][k] = t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int q = 0; q < nw; q++) t += red[q][threadIdx.x];
        partials[blockIdx.x * kRedSlots + slot0 + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

// block sums of K floats (FP32 within each warp, FP64 across warps and
// blocks): for per-atom quantities whose warp sums need no more than FP32,
// as kinetic tensors and displacement sums; FP64 work is scarce on this GPU
template <int K>
__device__ bool block_partials_f32(const float (&v)[K], double* partials, int slot0, unsigned* counter) {
    __shared__ double red[32][K];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        float t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[w][k] = (double)t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int q = 0; q < nw; q++) t += red[q][threadIdx.x];
        partials[blockIdx.x * kRedSlots + slot0 + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

// the same with the K values produced on demand by get(k): only one of them
// is live at a time, which keeps the register count of kernels with many
// sums down
template <int K, class Get>
__device__ bool block_partials_fn(Get get, double* partials, int slot0, unsigned* counter) {
    __shared__ double red[32][K];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll 1
    for (int k = 0; k < K; k++) {
        double t = get(k);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[w][k] = t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int q = 0; q < nw; q++) t += red[q][threadIdx.x];
        partials[blockIdx.x * kRedSlots + slot0 + threadIdx.x] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

// final_sums into shared memory (out[k], written by lane 0 of the calling
// warp; the warp synchronises before returning)
template <int K>
__device__ void final_sums_smem(const double* partials, int nblk, double* out) {
    const int lane = threadIdx.x & 31;
#pragma unroll 1
    for (int k = 0; k < K; k++) {
        double t = 0.0;
        for (int b = lane; b < nblk; b += 32) t += partials[b * kRedSlots + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) out[k] = t;
    }
    __syncwarp();
}

// block sums of K values from get(k) into out[0..K-1] (one batch chunk)
template <int K, class Get>
__device__ __forceinline__ void chunk_store(Get get, double* out) {
    __shared__ double red[8][K];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll 1
    for (int k = 0; k < K; k++) {
        double t = get(k);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[w][k] = t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int q = 0; q < nw; q++) t += red[q][threadIdx.x];
        out[threadIdx.x] = t;
    }
    __syncthreads();
}

// chunk_store for FP32 per-thread values (streaming MD sums): FP32 warp
// sums (a warp holds a few dozen terms), FP64 across the block's warps; the
// FP64 shuffle tree of chunk_store costs more than the chunk's atoms here
template <int K>
__device__ __forceinline__ void chunk_store_f32(const float (&v)[K], double* out) {
    __shared__ double red[8][K];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        float t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[w][k] = (double)t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int q = 0; q < nw; q++) t += red[q][threadIdx.x];
        out[threadIdx.x] = t;
    }
    __syncthreads();
}

// sums of the first K partial slots over nblk blocks by one warp, in a fixed
// order (lane-strided, then a shuffle tree): every lane gets the totals
template <int K>
__device__ void final_sums(const double* partials, int nblk, double (&tot)[K]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double t = 0.0;
        for (int b = lane; b < nblk; b += 32) t += partials[b * kRedSlots + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        tot[k] = t;
    }
}

}  // namespace mappg
