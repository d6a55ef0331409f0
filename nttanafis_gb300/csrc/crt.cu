// Exact CRT reconstruction fused with the windowed limb sum and the carry scan,
// the disjoint-block convolution output, and the short-operand column sums.
//
// Reference: cofactor CRT with one approximate quotient (src/limb/cofactor.rs:59-111),
// coefficients added at bit i*w with carries across ranges
// (src/limb/reconstruction.rs:77-483), signed offsets for convolutions
// (src/limb/reconstruction.rs:94-163), and direct column sums for short operands
// (src/convolve.rs:188-351).
//
// Here every product coefficient is a 64-bit-limb convolution value, so coefficient
// k lands at limb k and spans l64 limbs. One CTA owns 1024 output limbs: it
// reconstructs the coefficients that reach them, sums the overlapping windows,
// propagates carries inside the tile with a generate/propagate block scan and
// resolves the tile's carry-in with a decoupled look-back over the earlier tiles'
// published (generate, propagate) pairs, so the limbs are written once, final.
// Every look-back wait is bounded; a wait that gives up is counted and flagged.
#include "launch.h"

namespace ntt {

constexpr int kCrtThreads = 256;

// Reconstructs coefficient k from its residues: returns four u64 words of
// S - q*P, S = sum_i y_i*(P/p_i), y_i = x_i*(P/p_i)^-1 mod p_i, q rounded from
// sum_i y_i/p_i. Unsigned: 0 <= X < P/2. Signed: two's complement, |X| <= P/4.
template <int NP>
__device__ __forceinline__ void crt_coeff(const u32* __restrict__ resid, int log_t, u64 k,
                                          const CrtParams& cp, u64 out[4]) {
    u32 y[NP];
    float f = 0.0f;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        const u32 x = __ldg(resid + ((size_t)i << log_t) + k);
        const u32 p = cp.p[i];
        u32 v = shoup_mul(x, cp.inv[i].x, cp.inv[i].y, p);
        v = sub_if_ge(v, p);
        y[i] = v;
        f = fmaf((float)v, cp.pinv[i], f);
    }
    constexpr int MW = NP > 1 ? NP - 1 : 1;  // words of P/p_i
    // S = sum_i y_i * M_i in NP + 1 words (the top word stays zero), by carry
    // chains: the low halves of y_i * M_i[w] into word w, the high halves into w+1.
    u32 S[NP + 1];
#pragma unroll
    for (int w = 0; w <= NP; ++w) S[w] = 0;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        const u32 yi = y[i];
        asm volatile("mad.lo.cc.u32 %0, %1, %2, %0;" : "+r"(S[0]) : "r"(yi), "r"(cp.M[i][0]));
#pragma unroll
        for (int w = 1; w < MW; ++w)
            asm volatile("madc.lo.cc.u32 %0, %1, %2, %0;" : "+r"(S[w]) : "r"(yi), "r"(cp.M[i][w]));
#pragma unroll
        for (int w = MW; w <= NP; ++w) asm volatile("addc.cc.u32 %0, %0, 0;" : "+r"(S[w]));
        asm volatile("mad.hi.cc.u32 %0, %1, %2, %0;" : "+r"(S[1]) : "r"(yi), "r"(cp.M[i][0]));
#pragma unroll
        for (int w = 2; w <= MW; ++w)
            asm volatile("madc.hi.cc.u32 %0, %1, %2, %0;" : "+r"(S[w]) : "r"(yi), "r"(cp.M[i][w - 1]));
#pragma unroll
        for (int w = MW + 1; w <= NP; ++w) asm volatile("addc.cc.u32 %0, %0, 0;" : "+r"(S[w]));
    }
    // X = S - q*P in NP + 1 words; the top word is the sign (0 or all ones).
    const u32 q = (u32)(f + cp.bias);
    u32 U[NP + 1];
#pragma unroll
    for (int w = 0; w < NP; ++w) U[w] = q * cp.P[w];
    U[NP] = 0;
    asm volatile("mad.hi.cc.u32 %0, %1, %2, %0;" : "+r"(U[1]) : "r"(q), "r"(cp.P[0]));
#pragma unroll
    for (int w = 2; w <= NP; ++w)
        asm volatile("madc.hi.cc.u32 %0, %1, %2, %0;" : "+r"(U[w]) : "r"(q), "r"(cp.P[w - 1]));
    u32 x[NP + 1];
    asm volatile("sub.cc.u32 %0, %1, %2;" : "=r"(x[0]) : "r"(S[0]), "r"(U[0]));
#pragma unroll
    for (int w = 1; w <= NP; ++w) asm volatile("subc.cc.u32 %0, %1, %2;" : "=r"(x[w]) : "r"(S[w]), "r"(U[w]));
    const u64 fill = x[NP] ? ~0ull : 0ull;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const int lo = 2 * w, hi = 2 * w + 1;
        const u64 l = lo < NP ? (u64)x[lo] : (lo == NP ? (u64)x[NP] : fill & 0xffffffffull);
        const u64 h = hi < NP ? (u64)x[hi] : (hi == NP ? (u64)x[NP] : fill & 0xffffffffull);
        out[w] = l | (h << 32);
    }
}

__device__ __forceinline__ void compose(u32& g, u32& p, u32 g_earlier, u32 p_earlier) {
    g = g | (p & g_earlier);
    p = p & p_earlier;
}

// Block-wide exclusive scan of carry (generate, propagate) pairs; returns the
// exclusive pair in (g, p) and the inclusive total of the block in (tg, tp).
__device__ __forceinline__ void block_scan_gp(u32& g, u32& p, u32& tg, u32& tp) {
    __shared__ u32 wg[32], wp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    u32 ig = g, ip = p;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const u32 og = __shfl_up_sync(0xffffffffu, ig, d);
        const u32 op = __shfl_up_sync(0xffffffffu, ip, d);
        if (lane >= d) compose(ig, ip, og, op);
    }
    if (lane == 31) { wg[warp] = ig; wp[warp] = ip; }
    __syncthreads();
    if (warp == 0) {
        u32 a = lane < nwarps ? wg[lane] : 0u, b = lane < nwarps ? wp[lane] : 1u;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const u32 og = __shfl_up_sync(0xffffffffu, a, d);
            const u32 op = __shfl_up_sync(0xffffffffu, b, d);
            if (lane >= d) compose(a, b, og, op);
        }
        if (lane < nwarps) { wg[lane] = a; wp[lane] = b; }
    }
    __syncthreads();
    // exclusive inside the warp
    u32 eg = __shfl_up_sync(0xffffffffu, ig, 1), ep = __shfl_up_sync(0xffffffffu, ip, 1);
    if (lane == 0) { eg = 0; ep = 1; }
    if (warp > 0) compose(eg, ep, wg[warp - 1], wp[warp - 1]);
    g = eg;
    p = ep;
    tg = wg[nwarps - 1];
    tp = wp[nwarps - 1];
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

// Look-back state of a tile: bits 0-1 the state, bit 2 the generate bit (or, for
// an inclusive state, the carry out of every tile up to this one), bit 3 the
// propagate bit.
constexpr u32 kTileAggregate = 1, kTileInclusive = 2;
// Spins (about 64 ns each) before a look-back gives up: far above any real wait.
constexpr u32 kMaxSpins = 1u << 20;
// Look-back waits that gave up since the library was loaded (none expected).
__device__ u32 g_lookback_timeouts;

// The carry out of tiles 0..t-1: walks back from tile t-1, composing aggregates
// until it meets an inclusive state or the composite stops propagating (almost
// always at tile t-1). Tile 0 always publishes an inclusive state, so the walk
// ends. Returns false if a wait exceeded kMaxSpins.
__device__ __forceinline__ bool look_back(volatile u32* status, u32 t, u32& cin) {
    u32 ga = 0, pa = 1;  // composite of the tiles after the current one, up to t-1
    for (int j = (int)t - 1; j >= 0; --j) {
        u32 s, spins = 0;
        while (((s = status[j]) & 3u) == 0) {
            if (++spins > kMaxSpins) return false;
            __nanosleep(64);
        }
        const u32 gj = (s >> 2) & 1u, pj = (s >> 3) & 1u;
        if ((s & 3u) == kTileInclusive) {
            cin = ga | (pa & gj);
            return true;
        }
        ga = ga | (pa & gj);
        pa = pa & pj;
        if (!pa) {  // tiles j..t-1 do not propagate: their carry out is known
            cin = ga;
            return true;
        }
    }
    cin = ga;  // not reached: tile 0 is inclusive
    return true;
}

// Tile of kCrtTile output limbs. Coefficient words sit in shared memory as four
// word planes, so a warp reads consecutive 64-bit words. Warp w owns limbs
// [128w, 128w + 128) of the tile; lane l handles limbs 32c + l of them (c < 4),
// so every shared and global access of a warp is to consecutive words.
// flags: [0] tile counter, [1] error word, [2 + t] look-back state of tile t; all
// zero when the kernel starts (the preceding transform kernel clears them).
template <int NP>
__global__ void __launch_bounds__(kCrtThreads) k_crt_mul(const u32* __restrict__ resid, int log_t,
                                                          u64 conv_len, u64 out_len, u64* __restrict__ dst,
                                                          u32* __restrict__ flags,
                                                          const __grid_constant__ CrtParams cp,
                                                          const ProductDesc* __restrict__ batch) {
    if (batch) {  // member blockIdx.y of a batch: grid.x covers its largest member
        const ProductDesc& d = batch[blockIdx.y];
        resid = d.spec;
        conv_len = d.conv_len;
        out_len = d.out_len;
        dst = d.dst;
        flags = reinterpret_cast<u32*>(d.agg);
    }
    // Tiles are numbered in the order CTAs start, so a tile only ever waits for
    // tiles whose CTAs are already running.
    __shared__ u32 s_tile, s_cin;
    if (threadIdx.x == 0) s_tile = atomicAdd(&flags[0], 1u);
    __syncthreads();
    const u32 tile = s_tile;
    const u32 tiles = (u32)((out_len + kCrtTile - 1) / kCrtTile);
    if (tile >= tiles) return;
    constexpr int kBack = 4;  // coefficients before the tile that reach into it (l64 <= 4)
    constexpr int kWords = kCrtTile + kBack;
    constexpr int kChunks = kCrtTile / (32 * (kCrtThreads / 32));  // 4 chunks of 32 limbs per warp
    __shared__ u64 xs[4][kWords];
    __shared__ u32 wsum_g[32], wsum_p[32];
    const u64 j0 = (u64)tile * kCrtTile;
    for (int kk = threadIdx.x; kk < kWords; kk += kCrtThreads) {
        const int64_t k = (int64_t)j0 - kBack + kk;
        u64 w[4] = {0, 0, 0, 0};
        if (k >= 0 && (u64)k < conv_len) crt_coeff<NP>(resid, log_t, (u64)k, cp, w);
        xs[0][kk] = w[0];
        xs[1][kk] = w[1];
        xs[2][kk] = w[2];
        xs[3][kk] = w[3];
    }
    __syncthreads();
    const int L = cp.l64;
    // Window sum of limb j0 + rel: low word and the count of its overflows.
    auto limb_sum = [&](int rel, u32& hi) -> u64 {
        u64 lo = 0;
        hi = 0;
        for (int w = 0; w < L; ++w) {
            const u64 v = xs[w][rel - w + kBack];
            lo += v;
            hi += (lo < v) ? 1u : 0u;
        }
        return lo;
    };
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u64 r[kChunks];
    u32 eg[kChunks], ep[kChunks], cg[kChunks], cpp[kChunks];
    u32 WG = 0, WP = 1;  // composite of this warp's chunks so far
    u32 h_last = 0;      // overflow count of the previous chunk's last limb
    if (lane == 0) limb_sum(warp * 32 * kChunks - 1, h_last);
    h_last = __shfl_sync(0xffffffffu, h_last, 0);
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const int rel = warp * 32 * kChunks + c * 32 + lane;
        u32 h;
        const u64 lo = limb_sum(rel, h);
        u32 hprev = __shfl_up_sync(0xffffffffu, h, 1);
        if (lane == 0) hprev = h_last;
        h_last = __shfl_sync(0xffffffffu, h, 31);
        const u64 s = lo + hprev;
        r[c] = s;
        u32 g = s < lo ? 1u : 0u, p = s == ~0ull ? 1u : 0u;
        warp_scan_gp(g, p);
        cg[c] = __shfl_sync(0xffffffffu, g, 31);
        cpp[c] = __shfl_sync(0xffffffffu, p, 31);
        u32 xg = __shfl_up_sync(0xffffffffu, g, 1), xp = __shfl_up_sync(0xffffffffu, p, 1);
        if (lane == 0) { xg = 0; xp = 1; }
        eg[c] = xg;
        ep[c] = xp;
        u32 ng = cg[c], np = cpp[c];
        compose(ng, np, WG, WP);
        WG = ng;
        WP = np;
    }
    if (lane == 0) { wsum_g[warp] = WG; wsum_p[warp] = WP; }
    __syncthreads();
    if (threadIdx.x == 0) {
        u32 tg = 0, tp = 1;  // the tile's (generate, propagate) pair
        for (int w = 0; w < kCrtThreads / 32; ++w) {
            u32 g = wsum_g[w], p = wsum_p[w];
            compose(g, p, tg, tp);
            tg = g;
            tp = p;
        }
        u32* status = flags + 2;
        u32 cin = 0;
        if (tile > 0) {
            atomicExch(status + tile, kTileAggregate | (tg << 2) | (tp << 3));
            if (!look_back(status, tile, cin)) {
                atomicAdd(&g_lookback_timeouts, 1u);
                atomicOr(&flags[1], 1u);
                cin = 0;
            }
        }
        atomicExch(status + tile, kTileInclusive | ((tg | (tp & cin)) << 2));
        s_cin = cin;
    }
    __syncthreads();
    // carry into this warp's first limb: the tile's carry-in through earlier warps
    u32 cin = s_cin;
    for (int w = 0; w < warp; ++w) cin = wsum_g[w] | (wsum_p[w] & cin);
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const u64 j = j0 + (u64)(warp * 32 * kChunks + c * 32 + lane);
        const u32 carry = eg[c] | (ep[c] & cin);
        if (j < out_len) dst[j] = r[c] + carry;
        cin = cg[c] | (cpp[c] & cin);
    }
}

// Disjoint blocks: coefficient k fills limbs [k*stride, (k+1)*stride).
template <int NP>
__global__ void __launch_bounds__(kCrtThreads) k_crt_conv(const u32* __restrict__ resid, int log_t,
                                                           u64 conv_len, u64* __restrict__ dst,
                                                           const __grid_constant__ CrtParams cp,
                                                           const ProductDesc* __restrict__ batch) {
    int stride = cp.stride;
    if (batch) {  // member blockIdx.y of a batch
        const ProductDesc& d = batch[blockIdx.y];
        resid = d.spec;
        conv_len = d.conv_len;
        dst = d.dst;
        stride = (int)d.stride;
    }
    const u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= conv_len) return;
    u64 w[4];
    crt_coeff<NP>(resid, log_t, k, cp, w);
    const u64 fill = (w[3] >> 63) ? ~0ull : 0ull;
    u64* out = dst + k * (u64)stride;
    out[0] = w[0];
    if (stride > 1) out[1] = w[1];
    if (stride > 2) out[2] = w[2];
    if (stride > 3) out[3] = w[3];
    for (int s = 4; s < stride; ++s) out[s] = fill;
}

// Short operand (<= 24 terms): exact sums of 128-bit products in three limbs.
template <bool SIGNED>
__global__ void __launch_bounds__(kCrtThreads) k_conv_school(const u64* __restrict__ a, u64 la,
                                                              const u64* __restrict__ b, u64 lb,
                                                              u64* __restrict__ dst, int stride) {
    const u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (k + 1 >= la + lb) return;
    const u64 i_lo = k + 1 > lb ? k + 1 - lb : 0;
    const u64 i_hi = min(k, la - 1);
    u64 w0 = 0, w1 = 0, w2 = 0;
    for (u64 i = i_lo; i <= i_hi; ++i) {
        const u64 x = a[i], y = b[k - i];
        const u64 lo = x * y;
        const u64 hi = SIGNED ? (u64)__mul64hi((long long)x, (long long)y) : __umul64hi(x, y);
        w0 += lo;
        const u64 c0 = w0 < lo ? 1 : 0;
        const u64 t = w1 + hi;
        const u64 c1 = t < hi ? 1 : 0;
        w1 = t + c0;
        const u64 c2 = w1 < c0 ? 1 : 0;
        w2 += c1 + c2;
        if (SIGNED && (int64_t)hi < 0) w2 -= 1;
    }
    u64* out = dst + k * (u64)stride;
    const u64 fill = (SIGNED && (int64_t)w2 < 0) ? ~0ull : 0ull;
    for (int s = 0; s < stride; ++s) out[s] = s == 0 ? w0 : (s == 1 ? w1 : (s == 2 ? w2 : fill));
}

// ---------------------------------------------------------------------------------

template <int NP>
static void crt_mul_np(const u32* resid, int log_t, u64 conv_len, u64 out_len, u64* dst, uint8_t* agg,
                       const CrtParams& cp, cudaStream_t st, void (*mark)(cudaStream_t)) {
    const int tiles = (int)((out_len + kCrtTile - 1) / kCrtTile);
    k_crt_mul<NP><<<tiles, kCrtThreads, 0, st>>>(resid, log_t, conv_len, out_len, dst,
                                                  reinterpret_cast<u32*>(agg), cp, nullptr);
    if (mark) mark(st);
}

template <int NP>
static void crt_mul_batch_np(const ProductDesc* batch, int count, int max_tiles, int log_t, const CrtParams& cp,
                             cudaStream_t st) {
    k_crt_mul<NP><<<dim3(max_tiles, count), kCrtThreads, 0, st>>>(nullptr, log_t, 0, 0, nullptr, nullptr, cp,
                                                                   batch);
}

cudaError_t launch_crt_mul_batch(const ProductDesc* batch, int count, int max_tiles, int log_t,
                                 const CrtParams& cp, cudaStream_t st) {
    switch (cp.np) {
        case 1: crt_mul_batch_np<1>(batch, count, max_tiles, log_t, cp, st); break;
        case 2: crt_mul_batch_np<2>(batch, count, max_tiles, log_t, cp, st); break;
        case 3: crt_mul_batch_np<3>(batch, count, max_tiles, log_t, cp, st); break;
        case 4: crt_mul_batch_np<4>(batch, count, max_tiles, log_t, cp, st); break;
        case 5: crt_mul_batch_np<5>(batch, count, max_tiles, log_t, cp, st); break;
        case 6: crt_mul_batch_np<6>(batch, count, max_tiles, log_t, cp, st); break;
        case 7: crt_mul_batch_np<7>(batch, count, max_tiles, log_t, cp, st); break;
        case 8: crt_mul_batch_np<8>(batch, count, max_tiles, log_t, cp, st); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_crt_conv_batch(const ProductDesc* batch, int count, u64 max_conv_len, int log_t,
                                  const CrtParams& cp, cudaStream_t st) {
    const dim3 grid((unsigned)((max_conv_len + kCrtThreads - 1) / kCrtThreads), count);
    switch (cp.np) {
        case 1: k_crt_conv<1><<<grid, kCrtThreads, 0, st>>>(nullptr, log_t, 0, nullptr, cp, batch); break;
        case 2: k_crt_conv<2><<<grid, kCrtThreads, 0, st>>>(nullptr, log_t, 0, nullptr, cp, batch); break;
        case 3: k_crt_conv<3><<<grid, kCrtThreads, 0, st>>>(nullptr, log_t, 0, nullptr, cp, batch); break;
        case 4: k_crt_conv<4><<<grid, kCrtThreads, 0, st>>>(nullptr, log_t, 0, nullptr, cp, batch); break;
        case 5: k_crt_conv<5><<<grid, kCrtThreads, 0, st>>>(nullptr, log_t, 0, nullptr, cp, batch); break;
        case 6: k_crt_conv<6><<<grid, kCrtThreads, 0, st>>>(nullptr, log_t, 0, nullptr, cp, batch); break;
        case 7: k_crt_conv<7><<<grid, kCrtThreads, 0, st>>>(nullptr, log_t, 0, nullptr, cp, batch); break;
        case 8: k_crt_conv<8><<<grid, kCrtThreads, 0, st>>>(nullptr, log_t, 0, nullptr, cp, batch); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_crt_mul(const u32* resid, int log_t, u64 conv_len, u64 out_len, u64* dst, uint8_t* agg,
                           const CrtParams& cp, cudaStream_t st, void (*mark)(cudaStream_t)) {
    switch (cp.np) {
        case 1: crt_mul_np<1>(resid, log_t, conv_len, out_len, dst, agg, cp, st, mark); break;
        case 2: crt_mul_np<2>(resid, log_t, conv_len, out_len, dst, agg, cp, st, mark); break;
        case 3: crt_mul_np<3>(resid, log_t, conv_len, out_len, dst, agg, cp, st, mark); break;
        case 4: crt_mul_np<4>(resid, log_t, conv_len, out_len, dst, agg, cp, st, mark); break;
        case 5: crt_mul_np<5>(resid, log_t, conv_len, out_len, dst, agg, cp, st, mark); break;
        case 6: crt_mul_np<6>(resid, log_t, conv_len, out_len, dst, agg, cp, st, mark); break;
        case 7: crt_mul_np<7>(resid, log_t, conv_len, out_len, dst, agg, cp, st, mark); break;
        case 8: crt_mul_np<8>(resid, log_t, conv_len, out_len, dst, agg, cp, st, mark); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_crt_conv(const u32* resid, int log_t, u64 conv_len, u64* dst, bool sign,
                            const CrtParams& cp, cudaStream_t st) {
    (void)sign;  // the quotient bias in cp selects signed rounding
    const unsigned blocks = (unsigned)((conv_len + kCrtThreads - 1) / kCrtThreads);
    switch (cp.np) {
        case 1: k_crt_conv<1><<<blocks, kCrtThreads, 0, st>>>(resid, log_t, conv_len, dst, cp, nullptr); break;
        case 2: k_crt_conv<2><<<blocks, kCrtThreads, 0, st>>>(resid, log_t, conv_len, dst, cp, nullptr); break;
        case 3: k_crt_conv<3><<<blocks, kCrtThreads, 0, st>>>(resid, log_t, conv_len, dst, cp, nullptr); break;
        case 4: k_crt_conv<4><<<blocks, kCrtThreads, 0, st>>>(resid, log_t, conv_len, dst, cp, nullptr); break;
        case 5: k_crt_conv<5><<<blocks, kCrtThreads, 0, st>>>(resid, log_t, conv_len, dst, cp, nullptr); break;
        case 6: k_crt_conv<6><<<blocks, kCrtThreads, 0, st>>>(resid, log_t, conv_len, dst, cp, nullptr); break;
        case 7: k_crt_conv<7><<<blocks, kCrtThreads, 0, st>>>(resid, log_t, conv_len, dst, cp, nullptr); break;
        case 8: k_crt_conv<8><<<blocks, kCrtThreads, 0, st>>>(resid, log_t, conv_len, dst, cp, nullptr); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_conv_schoolbook(const u64* a, u64 la, const u64* b, u64 lb, u64* dst, int stride,
                                   bool sign, cudaStream_t st) {
    const u64 n = la + lb - 1;
    const unsigned blocks = (unsigned)((n + kCrtThreads - 1) / kCrtThreads);
    if (sign) k_conv_school<true><<<blocks, kCrtThreads, 0, st>>>(a, la, b, lb, dst, stride);
    else k_conv_school<false><<<blocks, kCrtThreads, 0, st>>>(a, la, b, lb, dst, stride);
    return cudaGetLastError();
}

cudaError_t init_crt_kernels() { return cudaSuccess; }

u32 lookback_timeouts() {
    u32 n = 0;
    if (cudaMemcpyFromSymbol(&n, g_lookback_timeouts, sizeof(n)) != cudaSuccess) return ~0u;
    return n;
}

}  // namespace ntt
