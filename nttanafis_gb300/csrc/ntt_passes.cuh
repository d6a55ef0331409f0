// In-shared-memory NTT passes: radix-2^RB register blocks over a padded layout.
//
// The reference runs radix-2/4/8/16 stages over remainder trees with 16-point
// register leaves (src/transform/forward.rs:200-298, src/transform/stage.rs:34-175,
// src/arch/schedule/leaf.rs:28-82). Here one CTA transforms one or more vectors of
// n = 2^log_n points held in shared memory. Each thread loads 2^RB points spaced
// `hq` apart into registers, runs RB butterfly levels there, and stores them back,
// so shared memory is touched twice per RB levels. Roots come from level-major
// tables (entry h + j holds w_{2h}^{+-j}), read through the read-only cache.
//
// Forward: decimation in frequency, natural order in, bit-reversed order out.
// Inverse: decimation in time, bit-reversed order in, natural order out.
#pragma once
#include "ntt_arith.cuh"

// Shared-memory slot of logical index i: one pad word per 32 words.
__device__ __forceinline__ int pad_index(int i) { return i + (i >> 5); }

// Padded words that hold one vector of n points.
__host__ __device__ inline int padded_len(int n) { return n + (n >> 5); }

template <class A, int RB>
__device__ __forceinline__ void dif_pass(u32* __restrict__ s, int log_n, int level, int nvec,
                                         int vstride, const uint2* __restrict__ tw, u32 p) {
    constexpr int E = 1 << RB;
    const int log_hq = log_n - level - RB;
    const int hq = 1 << log_hq;
    const int log_gpv = log_n - RB;
    const int total = nvec << log_gpv;
    for (int g = threadIdx.x; g < total; g += blockDim.x) {
        const int v = g >> log_gpv;
        const int gg = g & ((1 << log_gpv) - 1);
        const int j0 = gg & (hq - 1);
        const int i0 = ((gg >> log_hq) << (log_hq + RB)) + j0;
        u32* base = s + v * vstride;
        u32 x[E];
#pragma unroll
        for (int m = 0; m < E; ++m) x[m] = base[pad_index(i0 + m * hq)];
#pragma unroll
        for (int t = 0; t < RB; ++t) {
            const int half = E >> (t + 1);
            const int hl = hq * half;
#pragma unroll
            for (int m = 0; m < E; ++m) {
                if ((m & half) == 0) {
                    const int j = j0 + (m & (half - 1)) * hq;
                    const uint2 w = __ldg(tw + hl + j);
                    A::dif(x[m], x[m + half], w, p);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < E; ++m) base[pad_index(i0 + m * hq)] = x[m];
    }
}

template <class A, int RB>
__device__ __forceinline__ void dit_pass(u32* __restrict__ s, int log_n, int level, int nvec,
                                         int vstride, const uint2* __restrict__ tw, u32 p) {
    constexpr int E = 1 << RB;
    const int hs = 1 << level;
    const int log_gpv = log_n - RB;
    const int total = nvec << log_gpv;
    for (int g = threadIdx.x; g < total; g += blockDim.x) {
        const int v = g >> log_gpv;
        const int gg = g & ((1 << log_gpv) - 1);
        const int j0 = gg & (hs - 1);
        const int i0 = ((gg >> level) << (level + RB)) + j0;
        u32* base = s + v * vstride;
        u32 x[E];
#pragma unroll
        for (int m = 0; m < E; ++m) x[m] = base[pad_index(i0 + m * hs)];
#pragma unroll
        for (int t = 0; t < RB; ++t) {
            const int dist = 1 << t;
            const int h = hs << t;
#pragma unroll
            for (int m = 0; m < E; ++m) {
                if ((m & dist) == 0) {
                    const int j = j0 + (m & (dist - 1)) * hs;
                    const uint2 w = __ldg(tw + h + j);
                    A::dit(x[m], x[m + dist], w, p);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < E; ++m) base[pad_index(i0 + m * hs)] = x[m];
    }
}

// Full forward transform of nvec vectors; ends with a barrier.
template <class A>
__device__ __forceinline__ void dif_full(u32* s, int log_n, int nvec, int vstride,
                                         const uint2* tw, u32 p) {
    int level = 0;
    while (log_n - level >= 4) {
        dif_pass<A, 4>(s, log_n, level, nvec, vstride, tw, p);
        level += 4;
        __syncthreads();
    }
    switch (log_n - level) {
        case 1: dif_pass<A, 1>(s, log_n, level, nvec, vstride, tw, p); break;
        case 2: dif_pass<A, 2>(s, log_n, level, nvec, vstride, tw, p); break;
        case 3: dif_pass<A, 3>(s, log_n, level, nvec, vstride, tw, p); break;
        default: break;
    }
    __syncthreads();
}

// Full inverse transform (unscaled) of nvec vectors; ends with a barrier.
template <class A>
__device__ __forceinline__ void dit_full(u32* s, int log_n, int nvec, int vstride,
                                         const uint2* tw, u32 p) {
    int level = 0;
    switch (log_n & 3) {
        case 1: dit_pass<A, 1>(s, log_n, 0, nvec, vstride, tw, p); level = 1; break;
        case 2: dit_pass<A, 2>(s, log_n, 0, nvec, vstride, tw, p); level = 2; break;
        case 3: dit_pass<A, 3>(s, log_n, 0, nvec, vstride, tw, p); level = 3; break;
        default: break;
    }
    if (level) __syncthreads();
    while (level < log_n) {
        dit_pass<A, 4>(s, log_n, level, nvec, vstride, tw, p);
        level += 4;
        __syncthreads();
    }
}
