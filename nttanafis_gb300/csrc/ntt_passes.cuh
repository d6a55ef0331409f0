// In-shared-memory NTT passes: radix-2^RB register blocks over a padded layout.
//
// The reference runs radix-2/4/8/16 stages over remainder trees with 16-point
// register leaves (src/transform/forward.rs:200-298, src/transform/stage.rs:34-175,
// src/arch/schedule/leaf.rs:28-82). Here one CTA transforms one or more vectors of
// n = 2^LOG_N points held in shared memory. Each thread loads 2^RB points spaced
// HQ apart into registers, runs RB butterfly levels there, and stores them back,
// so shared memory is touched twice per RB levels. Roots come from level-major
// tables (entry h + j holds w_{2h}^{+-j}), in shared memory or global memory.
//
// Every size is a template parameter, so the slot of point m of a register block
// is the block's base plus a compile-time offset and each twiddle load has an
// immediate offset from one per-block base: the only per-point instructions left
// are the loads, the stores and the butterflies themselves.
//
// Forward: decimation in frequency, natural order in, bit-reversed order out.
// Inverse: decimation in time, bit-reversed order in, natural order out.
#pragma once
#include "ntt_arith.cuh"

// Butterflies whose twiddle is 1 (the first of every group when a register block
// holds consecutive points) run without a product.
#ifndef NTT_UNIT_C0
#define NTT_UNIT_C0 1
#endif

// Shared-memory slot of logical index i: one pad word per 32 words.
__host__ __device__ constexpr int pad_index(int i) { return i + (i >> 5); }

// log2 of a power of two.
__host__ __device__ constexpr int ilog2(int n) { return n > 1 ? 1 + ilog2(n >> 1) : 0; }

// Padded words that hold one vector of n points.
__host__ __device__ constexpr int padded_len(int n) { return n + (n >> 5); }

// For a register block of 2^RB points spaced S apart whose first point i0 satisfies
// i0 mod 32 + (2^RB - 1) * S < 32 whenever 2^RB * S <= 32 (blocks are aligned), the
// slot of point m is pad_index(i0) + m*S + ((m*S) >> 5).
template <int S>
__device__ __forceinline__ constexpr int slot_offset(int m) {
    return m * S + ((m * S) >> 5);
}

// Vectors a thread transforms together: register blocks at the same position of
// two vectors share their twiddles, so each twiddle load serves both and the two
// butterfly chains interleave. Pairs are taken only while every thread still gets
// a block (2^LOG_GPV blocks per vector, NT threads).
template <int NV, int LOG_GPV, int NT>
__host__ __device__ constexpr int vectors_per_block() {
    return NV % 2 == 0 && ((NV / 2) << LOG_GPV) >= NT ? 2 : 1;
}

// RB forward levels on VP register blocks of 2^RB points spaced H apart; the
// twiddle of butterfly c at the level of half-size h = 2^(RB-1-t) * H is
// twb[h + c * H], twb = table + (first point mod H). With HZ the upper half of
// every block is zero, so the first level only multiplies: (x, 0) -> (x, x*w).
//
// With OPEN (blocks of consecutive points, H = 1) the last level, whose twiddle is
// 1, is left open: its pairs come out as (x + y, x - y + 2p) unreduced (A::dif_open)
// for a caller that multiplies them next.
template <class A, int RB, int H, int VP, bool HZ = false, bool OPEN = false>
__device__ __forceinline__ void dif_levels(u32 (&x)[VP][1 << RB], const uint2* __restrict__ twb, u32 p) {
    constexpr int E = 1 << RB;
    static_assert(!OPEN || H == 1, "an open last level has twiddle 1 only for consecutive points");
#pragma unroll
    for (int t = 0; t < RB; ++t) {
        if (OPEN && t == RB - 1) {
#pragma unroll
            for (int q = 0; q < VP; ++q)
#pragma unroll
                for (int b = 0; b < E; b += 2) A::dif_open(x[q][b], x[q][b + 1], p);
            break;
        }
        const int half = E >> (t + 1);
#pragma unroll
        for (int c = 0; c < half; ++c) {
            if (NTT_UNIT_C0 && H == 1 && c == 0) {
                // consecutive points: the first butterfly of every group has twiddle 1
#pragma unroll
                for (int q = 0; q < VP; ++q)
#pragma unroll
                    for (int b = 0; b < E; b += 2 * half) {
                        if (HZ && t == 0) x[q][b + half] = x[q][b];
                        else A::dif_unit(x[q][b], x[q][b + half], p);
                    }
                continue;
            }
            // butterflies (m, m + half) with m = blk*2*half + c share twiddle c
            const uint2 w = twb[H * half + c * H];
#pragma unroll
            for (int q = 0; q < VP; ++q)
#pragma unroll
                for (int b = 0; b < E; b += 2 * half) {
                    if (HZ && t == 0) x[q][b + c + half] = A::mulc(x[q][b + c], w, p);
                    else A::dif(x[q][b + c], x[q][b + c + half], w, p);
                }
        }
    }
}

// RB inverse levels on VP register blocks of 2^RB points spaced H apart. UNIT
// (H = 1: the first level's twiddle is 1) runs that level without products:
// 1 for inputs in [0, 4p) (A::dit_unit), 2 for inputs in [0, 2p) (A::dit_unit_2p).
template <class A, int RB, int H, int VP, int UNIT = 0>
__device__ __forceinline__ void dit_levels(u32 (&x)[VP][1 << RB], const uint2* __restrict__ twb, u32 p) {
    constexpr int E = 1 << RB;
    static_assert(UNIT == 0 || H == 1, "a product-free first level needs consecutive points");
#pragma unroll
    for (int t = 0; t < RB; ++t) {
        const int dist = 1 << t;
        if (UNIT && t == 0) {
#pragma unroll
            for (int q = 0; q < VP; ++q)
#pragma unroll
                for (int b = 0; b < E; b += 2) {
                    if (UNIT == 2) A::dit_unit_2p(x[q][b], x[q][b + 1], p);
                    else A::dit_unit(x[q][b], x[q][b + 1], p);
                }
            continue;
        }
#pragma unroll
        for (int c = 0; c < dist; ++c) {
            if (NTT_UNIT_C0 && H == 1 && c == 0) {  // twiddle 1: no product
#pragma unroll
                for (int q = 0; q < VP; ++q)
#pragma unroll
                    for (int b = 0; b < E; b += 2 * dist) A::dit_unit(x[q][b], x[q][b + dist], p);
                continue;
            }
            const uint2 w = twb[(H << t) + c * H];
#pragma unroll
            for (int q = 0; q < VP; ++q)
#pragma unroll
                for (int b = 0; b < E; b += 2 * dist) A::dit(x[q][b + c], x[q][b + c + dist], w, p);
        }
    }
}

// Start of register block gg of a pass whose blocks span 2^RB points H apart:
// i0 = a * H * 2^RB + j with j < H. With the plain order (j = gg mod H), a warp
// whose 32 blocks have 2 <= H <= 16 covers 32 / H values of a, whose starts are H/2
// banks apart in the padded layout: two-way conflicts. Taking H/2 values of j and
// 64/H values of a per warp instead spreads the 32 starts over distinct banks (the
// other half of j goes to the next warp).
template <int LOG_H, int RB, int LOG_GPV>
__device__ __forceinline__ int block_start(int gg, int& j) {
    constexpr int H = 1 << LOG_H;
    if constexpr (LOG_H >= 1 && LOG_H <= 4 && LOG_GPV >= 6) {
        constexpr int LOG_HH = LOG_H - 1;  // log2(H / 2)
        const int l = gg & 31, hi = gg >> 5;
        j = ((hi & 1) << LOG_HH) + (l & ((1 << LOG_HH) - 1));
        const int a = ((hi >> 1) << (6 - LOG_H)) + (l >> LOG_HH);
        return (a << (LOG_H + RB)) + j;
    } else {
        j = gg & (H - 1);
        return ((gg >> LOG_H) << (LOG_H + RB)) + j;
    }
}

// One pass of RB forward levels starting at LEVEL over NV vectors of 2^LOG_N points,
// VS words apart. Register block gg of a vector starts at block_start(gg) and spans
// 2^RB points HQ apart.
template <class A, int LOG_N, int LEVEL, int RB, int NT, int NV, int VS>
__device__ __forceinline__ void dif_pass(u32* __restrict__ s, const uint2* __restrict__ tw, u32 p) {
    constexpr int E = 1 << RB;
    constexpr int LOG_HQ = LOG_N - LEVEL - RB;
    constexpr int HQ = 1 << LOG_HQ;
    constexpr int LOG_GPV = LOG_N - RB;
    constexpr int VP = vectors_per_block<NV, LOG_GPV, NT>();
    constexpr int ITEMS = (NV / VP) << LOG_GPV;
#pragma unroll 1
    for (int it = threadIdx.x; it < ITEMS; it += NT) {
        const int v = (it >> LOG_GPV) * VP;
        const int gg = it & ((1 << LOG_GPV) - 1);
        int j0;
        const int i0 = block_start<LOG_HQ, RB, LOG_GPV>(gg, j0);
        u32* base = s + v * VS + pad_index(i0);
        u32 x[VP][E];
#pragma unroll
        for (int q = 0; q < VP; ++q)
#pragma unroll
            for (int m = 0; m < E; ++m) x[q][m] = base[q * VS + slot_offset<HQ>(m)];
        dif_levels<A, RB, HQ, VP>(x, tw + j0, p);
#pragma unroll
        for (int q = 0; q < VP; ++q)
#pragma unroll
            for (int m = 0; m < E; ++m) base[q * VS + slot_offset<HQ>(m)] = x[q][m];
    }
}

// One pass of RB inverse levels starting at LEVEL; block gg starts at
// block_start(gg) and spans 2^RB points HS = 2^LEVEL apart.
template <class A, int LOG_N, int LEVEL, int RB, int NT, int NV, int VS>
__device__ __forceinline__ void dit_pass(u32* __restrict__ s, const uint2* __restrict__ tw, u32 p) {
    constexpr int E = 1 << RB;
    constexpr int HS = 1 << LEVEL;
    constexpr int LOG_GPV = LOG_N - RB;
    constexpr int VP = vectors_per_block<NV, LOG_GPV, NT>();
    constexpr int ITEMS = (NV / VP) << LOG_GPV;
#pragma unroll 1
    for (int it = threadIdx.x; it < ITEMS; it += NT) {
        const int v = (it >> LOG_GPV) * VP;
        const int gg = it & ((1 << LOG_GPV) - 1);
        int j0;
        const int i0 = block_start<LEVEL, RB, LOG_GPV>(gg, j0);
        u32* base = s + v * VS + pad_index(i0);
        u32 x[VP][E];
#pragma unroll
        for (int q = 0; q < VP; ++q)
#pragma unroll
            for (int m = 0; m < E; ++m) x[q][m] = base[q * VS + slot_offset<HS>(m)];
        dit_levels<A, RB, HS, VP>(x, tw + j0, p);
#pragma unroll
        for (int q = 0; q < VP; ++q)
#pragma unroll
            for (int m = 0; m < E; ++m) base[q * VS + slot_offset<HS>(m)] = x[q][m];
    }
}

// Levels per register block (2^RB points per thread and pass).
#ifndef NTT_MAX_RB
#define NTT_MAX_RB 4
#endif
constexpr int kMaxRB = NTT_MAX_RB;

// Full forward transform of NV vectors of 2^LOG_N points, VS words apart; ends
// with a barrier.
template <class A, int LOG_N, int NT, int NV, int VS, int LEVEL = 0>
__device__ __forceinline__ void dif_full(u32* s, const uint2* tw, u32 p) {
    if constexpr (LOG_N - LEVEL >= kMaxRB) {
        dif_pass<A, LOG_N, LEVEL, kMaxRB, NT, NV, VS>(s, tw, p);
        __syncthreads();
        dif_full<A, LOG_N, NT, NV, VS, LEVEL + kMaxRB>(s, tw, p);
    } else if constexpr (LOG_N - LEVEL > 0) {
        dif_pass<A, LOG_N, LEVEL, LOG_N - LEVEL, NT, NV, VS>(s, tw, p);
        __syncthreads();
    }
}

// Forward passes of kMaxRB levels from LEVEL up to END (exclusive), each followed by
// a barrier.
template <class A, int LOG_N, int NT, int NV, int VS, int LEVEL, int END>
__device__ __forceinline__ void dif_range(u32* s, const uint2* tw, u32 p) {
    if constexpr (LEVEL < END) {
        dif_pass<A, LOG_N, LEVEL, kMaxRB, NT, NV, VS>(s, tw, p);
        __syncthreads();
        dif_range<A, LOG_N, NT, NV, VS, LEVEL + kMaxRB, END>(s, tw, p);
    }
}

// Inverse passes of kMaxRB levels from LEVEL up to END (exclusive), each followed by
// a barrier.
template <class A, int LOG_N, int NT, int NV, int VS, int LEVEL, int END>
__device__ __forceinline__ void dit_range(u32* s, const uint2* tw, u32 p) {
    if constexpr (LEVEL < END) {
        dit_pass<A, LOG_N, LEVEL, kMaxRB, NT, NV, VS>(s, tw, p);
        __syncthreads();
        dit_range<A, LOG_N, NT, NV, VS, LEVEL + kMaxRB, END>(s, tw, p);
    }
}

// Full inverse transform (unscaled); the short pass runs first. Ends with a barrier.
template <class A, int LOG_N, int NT, int NV, int VS, int LEVEL = -1>
__device__ __forceinline__ void dit_full(u32* s, const uint2* tw, u32 p) {
    if constexpr (LEVEL < 0) {
        constexpr int R0 = LOG_N % kMaxRB;
        if constexpr (R0 > 0) {
            dit_pass<A, LOG_N, 0, R0, NT, NV, VS>(s, tw, p);
            __syncthreads();
        }
        dit_full<A, LOG_N, NT, NV, VS, R0>(s, tw, p);
    } else if constexpr (LEVEL < LOG_N) {
        dit_pass<A, LOG_N, LEVEL, kMaxRB, NT, NV, VS>(s, tw, p);
        __syncthreads();
        dit_full<A, LOG_N, NT, NV, VS, LEVEL + kMaxRB>(s, tw, p);
    }
}
