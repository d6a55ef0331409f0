// CRT pieces shared by the CRT kernels: reconstruction of a coefficient from its
// residues, the limb sums of a tile held four limbs per thread, and the carry scan
// inside a tile. See crt.cu for the algorithm and its reference.
#pragma once
#include "crt_chains.cuh"
#include "launch.h"

namespace ntt {

constexpr int kCrtThreads = kCrtTile / 4;

// The multiples q * P (q = 0..np) of a prime set, staged in shared memory by the
// CRT kernels: every thread calls it, a barrier of the caller publishes it.
__device__ __forceinline__ void stage_multiples(const CrtParams& cp, u32 (*qp)[kQpStride]) {
    for (int i = threadIdx.x; i < (kMaxPrimes + 1) * kQpStride; i += blockDim.x)
        qp[i / kQpStride][i % kQpStride] = cp.qP[i / kQpStride][i % kQpStride];
}

// Reconstructs X from its residues y_i = r_i*(P/p_i)^-1 mod p_i (canonical; the
// transforms fold the cofactor inverse into their scale): returns the NP + 1 u32
// words (two's complement) of X = S - q*P, S = sum_i y_i*(P/p_i), q rounded from
// sum_i y_i/p_i and q*P read from the staged multiples. Unsigned: 0 <= X < P/2.
// Signed: |X| <= P/4.
template <int NP>
__device__ __forceinline__ void crt_words(const u32 (&y)[NP], const CrtParams& cp, const u32 (*qp)[kQpStride],
                                          u32 (&x)[NP + 1]) {
    float f = 0.0f;
#pragma unroll
    for (int i = 0; i < NP; ++i) f = fmaf((float)y[i], cp.pinv[i], f);
    // S = sum_i y_i * M_i in NP + 1 words (the top word stays zero), by carry
    // chains: the low halves of y_i * M_i[w] into word w, the high halves into w+1.
    u32 S[NP + 1];
#pragma unroll
    for (int w = 0; w <= NP; ++w) S[w] = 0;
#pragma unroll
    for (int i = 0; i < NP; ++i) CrtChains<NP>::accumulate(S, y[i], cp.M[i]);
    // X = S - q*P in NP + 1 words; the top word is the sign (0 or all ones).
    const u32 q = min((u32)(f + cp.bias), (u32)NP);
    u32 U[NP + 1];
#pragma unroll
    for (int w = 0; w <= NP; ++w) U[w] = qp[q][w];
    CrtChains<NP>::subtract(x, S, U);
}

// The first W u64 words of X (sign-filled above its NP + 1 u32 words).
template <int NP, int W>
__device__ __forceinline__ void pack_words(const u32 (&x)[NP + 1], u64 (&out)[W]) {
    const u64 fill = x[NP] ? ~0ull : 0ull;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int lo = 2 * w, hi = 2 * w + 1;
        const u64 l = lo <= NP ? (u64)x[lo] : fill & 0xffffffffull;
        const u64 h = hi <= NP ? (u64)x[hi] : fill & 0xffffffffull;
        out[w] = l | (h << 32);
    }
}

// u64 words of a reconstructed coefficient for NP primes below 2^31 (X < 2^(31 NP - 1)).
__host__ __device__ constexpr int crt_limb_words(int np) {
    return (31 * np - 1 + 63) / 64 < 4 ? (31 * np - 1 + 63) / 64 : 4;
}

__device__ __forceinline__ void compose(u32& g, u32& p, u32 g_earlier, u32 p_earlier) {
    g = g | (p & g_earlier);
    p = p & p_earlier;
}

// Inclusive warp scan of (generate, propagate) pairs over the lanes.
__device__ __forceinline__ void warp_scan_gp(u32& g, u32& p) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const u32 og = __shfl_up_sync(0xffffffffu, g, d);
        const u32 op = __shfl_up_sync(0xffffffffu, p, d);
        if (lane >= d) compose(g, p, og, op);
    }
}

constexpr int kCrtPer = 4;
static_assert(kCrtThreads * kCrtPer == kCrtTile, "four limbs per thread");

// Inside a tile held kCrtPer limbs per thread, with (generate, propagate) bits per
// limb: (xg, xp) composes the limbs of the earlier threads of the tile (the carry
// into this thread's first limb is xg | (xp & carry into the tile)); (tg, tp) is
// the tile's own pair. Holds one barrier.
__device__ __forceinline__ void tile_scan(const u32 (&gb)[kCrtPer], const u32 (&pb)[kCrtPer], u32& xg, u32& xp,
                                          u32& tg, u32& tp) {
    constexpr int NW = kCrtThreads / 32;
    __shared__ u32 s_wg[NW], s_wp[NW];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u32 G = gb[0], P = pb[0];
#pragma unroll
    for (int c = 1; c < kCrtPer; ++c) {
        G = gb[c] | (pb[c] & G);
        P = pb[c] & P;
    }
    u32 ig = G, ip = P;
    warp_scan_gp(ig, ip);
    u32 eg = __shfl_up_sync(0xffffffffu, ig, 1), ep = __shfl_up_sync(0xffffffffu, ip, 1);
    if (lane == 0) { eg = 0; ep = 1; }
    if (lane == 31) { s_wg[warp] = ig; s_wp[warp] = ip; }
    __syncthreads();
    u32 wg = 0, wp = 1;  // the earlier warps of the tile
    for (int w = 0; w < warp; ++w) {
        wg = s_wg[w] | (s_wp[w] & wg);
        wp = s_wp[w] & wp;
    }
    xg = eg | (ep & wg);
    xp = ep & wp;
    tg = 0;
    tp = 1;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        tg = s_wg[w] | (s_wp[w] & tg);
        tp = s_wp[w] & tp;
    }
}

// The limbs of a thread's four positions of a tile before the carries: limb c
// sums word w of coefficient c - w (w < L), the thread's own coefficient words cw
// where c - w >= 0, else the previous thread's (warp shuffle, or shared memory
// across warps; the first thread of the tile takes the words of the L coefficients
// before the tile from pre, which threads 0..L-1 filled before the call). A limb's
// sum is a low word plus an overflow count that joins the next limb; returns the
// values sv and their (generate, propagate) bits. Holds one barrier.
template <int L>
__device__ __forceinline__ void tile_limbs(const u64 (&cw)[kCrtPer][L], const u64 (*pre)[L], u64 (&sv)[kCrtPer],
                                           u32 (&gb)[kCrtPer], u32 (&pb)[kCrtPer]) {
    constexpr int NW = kCrtThreads / 32;
    constexpr int NE = L * (L - 1) / 2;  // words a thread takes from its predecessor
    __shared__ u64 s_edge[NW][NE > 0 ? NE : 1];
    __shared__ u32 s_edge_h[NW];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto limb = [&](int c, const u64 (&prev)[NE > 0 ? NE : 1], u32& h) -> u64 {
        u64 lo = 0;
        h = 0;
#pragma unroll
        for (int w = 0; w < L; ++w) {
            // pair (w, c) with c < w comes from the predecessor: index w(w-1)/2 + c
            const u64 v = c - w >= 0 ? cw[c - w >= 0 ? c - w : 0][w] : prev[w * (w - 1) / 2 + c];
            lo += v;
            h += lo < v ? 1u : 0u;
        }
        return lo;
    };
    // What the successor needs: words w of coefficients 4 + c - w (c < w) and the
    // overflow count of limb 3 (own words only).
    u64 mine[NE > 0 ? NE : 1];
#pragma unroll
    for (int w = 1; w < L; ++w)
#pragma unroll
        for (int c = 0; c < w; ++c) mine[w * (w - 1) / 2 + c] = cw[kCrtPer + c - w][w];
    u32 h3;
    {
        const u64 dummy[NE > 0 ? NE : 1] = {};
        limb(kCrtPer - 1, dummy, h3);  // limb 3 uses own words only (L <= 4)
    }
    if (lane == 31) {
#pragma unroll
        for (int e = 0; e < NE; ++e) s_edge[warp][e] = mine[e];
        s_edge_h[warp] = h3;
    }
    __syncthreads();
    u64 prev[NE > 0 ? NE : 1];
    u32 hprev;
#pragma unroll
    for (int e = 0; e < NE; ++e) prev[e] = __shfl_up_sync(0xffffffffu, mine[e], 1);
    hprev = __shfl_up_sync(0xffffffffu, h3, 1);
    if (lane == 0) {
        if (warp > 0) {
#pragma unroll
            for (int e = 0; e < NE; ++e) prev[e] = s_edge[warp - 1][e];
            hprev = s_edge_h[warp - 1];
        } else {
            // predecessor = the coefficients before the tile: pre[i] plays the
            // predecessor's coefficient 4 - L + i
#pragma unroll
            for (int w = 1; w < L; ++w)
#pragma unroll
                for (int c = 0; c < w; ++c) prev[w * (w - 1) / 2 + c] = pre[L + c - w][w];
            // overflow count of the limb before the tile
            u64 lo = 0;
            hprev = 0;
#pragma unroll
            for (int w = 0; w < L; ++w) {
                const u64 v = pre[L - 1 - w][w];
                lo += v;
                hprev += lo < v ? 1u : 0u;
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kCrtPer; ++c) {
        u32 h;
        const u64 lo = limb(c, prev, h);
        const u64 s2 = lo + hprev;
        sv[c] = s2;
        gb[c] = s2 < lo ? 1u : 0u;
        pb[c] = s2 == ~0ull ? 1u : 0u;
        hprev = h;
    }
}

// Adds the carries into a thread's four limbs and stores those below len.
__device__ __forceinline__ void store_limbs(u64* __restrict__ dst, u64 k0, u64 len, const u64 (&sv)[kCrtPer],
                                            const u32 (&gb)[kCrtPer], const u32 (&pb)[kCrtPer], u32 c) {
    u64 out[kCrtPer];
#pragma unroll
    for (int i = 0; i < kCrtPer; ++i) {
        out[i] = sv[i] + c;
        c = gb[i] | (pb[i] & c);
    }
    u64* d = dst + k0;
    if (k0 + kCrtPer <= len && (reinterpret_cast<uintptr_t>(d) & 15) == 0) {
        reinterpret_cast<uint4*>(d)[0] = make_uint4((u32)out[0], (u32)(out[0] >> 32), (u32)out[1], (u32)(out[1] >> 32));
        reinterpret_cast<uint4*>(d)[1] = make_uint4((u32)out[2], (u32)(out[2] >> 32), (u32)out[3], (u32)(out[3] >> 32));
    } else {
#pragma unroll
        for (int i = 0; i < kCrtPer; ++i)
            if (k0 + i < len) d[i] = out[i];
    }
}

}  // namespace ntt
