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
// propagates carries inside the tile with a generate/propagate scan (crt.cuh) and
// resolves the tile's carry-in with a decoupled look-back over the earlier tiles'
// published (generate, propagate) pairs, so the limbs are written once, final.
// Every look-back wait is bounded; a wait that gives up is counted and flagged.
// The same file holds the big-integer addition of the block split (k_add_limbs)
// and the descriptors of its blocks (k_split_descs).
#include "crt.cuh"
#include "launch.h"
#include "transform_common.cuh"

namespace ntt {

// Coefficient k of a residue array [prime][T] as four u64 words.
template <int NP>
__device__ __forceinline__ void crt_coeff(const u32* __restrict__ resid, int log_t, u64 k,
                                          const CrtParams& cp, const u32 (*qp)[kQpStride], u64 out[4]) {
    u32 r[NP], x[NP + 1];
#pragma unroll
    for (int i = 0; i < NP; ++i) r[i] = __ldg(resid + ((size_t)i << log_t) + k);
    crt_words<NP>(r, cp, qp, x);
    u64 w[4];
    pack_words<NP, 4>(x, w);
#pragma unroll
    for (int i = 0; i < 4; ++i) out[i] = w[i];
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

// Carries of a tile of kCrtTile limbs held four per thread, each limb with its
// (generate, propagate) bits: the thread's composite, an inclusive warp scan, the
// warps in order, and the tiles before this one by the decoupled look-back
// (flags: [0] tile counter, [1] error word, [2 + t] state of tile t). A wait that
// gives up is reported in the status bytes (launch.h) as well. Returns the carry
// into the thread's first limb. Every thread of the CTA calls it (two barriers).
__device__ __forceinline__ u32 tile_carry_in(const u32 (&gb)[kCrtPer], const u32 (&pb)[kCrtPer], u32 tile,
                                             u32* flags, u32* status) {
    __shared__ u32 s_cin;
    u32 xg, xp, tg, tp;
    tile_scan(gb, pb, xg, xp, tg, tp);
    if (threadIdx.x == 0) {
        u32* state = flags + 2;
        u32 cin = 0;
        if (tile > 0) {
            atomicExch(state + tile, kTileAggregate | (tg << 2) | (tp << 3));
            if (!look_back(state, tile, cin)) {
                // the product is wrong: counted, flagged in the call's error word
                // and in the caller's status, which fails the call
                atomicAdd(&g_lookback_timeouts, 1u);
                atomicOr(&flags[1], 1u);
                report_status(status, 0);
                cin = 0;
            }
        }
        atomicExch(state + tile, kTileInclusive | ((tg | (tp & cin)) << 2));
        s_cin = cin;
    }
    __syncthreads();
    return xg | (xp & s_cin);
}

// Tile of kCrtTile output limbs, four per thread: thread t reconstructs the
// coefficients j0 + 4t .. j0 + 4t + 3 (coefficient k lands at limb k and spans L
// limbs) and owns the limbs with the same indices. Limb j sums word w of coefficient
// j - w for w < L; the words that come from the previous thread's coefficients
// arrive by warp shuffle, or through shared memory across warps (the L coefficients
// before the tile are reconstructed by threads 0..L-1). A limb's sum is a low word
// plus an overflow count that joins the next limb; the carries that remain are
// single bits, resolved per thread, by a warp scan, across warps, and across tiles
// by the look-back.
// flags: [0] tile counter, [1] error word, [2 + t] look-back state of tile t; all
// zero when the kernel starts (the preceding transform kernel clears them).
template <int NP>
__global__ void __launch_bounds__(kCrtThreads, 5) k_crt_mul(const u32* __restrict__ resid, int log_t,
                                                          u64 conv_len, u64 out_len, u64* __restrict__ dst,
                                                          u32* __restrict__ flags,
                                                          const __grid_constant__ CrtParams cp,
                                                          const ProductDesc* __restrict__ batch,
                                                          u32* __restrict__ status) {
    constexpr int L = crt_limb_words(NP);
    if (batch) {  // member blockIdx.y of a batch: grid.x covers its largest member
        const ProductDesc& d = batch[blockIdx.y];
        resid = d.spec;
        conv_len = d.conv_len;
        out_len = d.out_len;
        dst = d.dst;
        flags = reinterpret_cast<u32*>(d.agg);
    }
    wait_prior_grid();  // the residues and cleared flags of the transform before it
    // Tiles are numbered in the order CTAs start, so a tile only ever waits for
    // tiles whose CTAs are already running.
    __shared__ u32 s_tile;
    __shared__ u64 s_pre[L][L];  // the L coefficients before the tile
    __shared__ u32 s_qp[kMaxPrimes + 1][kQpStride];
    if (threadIdx.x == 0) s_tile = atomicAdd(&flags[0], 1u);
    stage_multiples(cp, s_qp);
    __syncthreads();
    const u32 tile = s_tile;
    const u32 tiles = (u32)((out_len + kCrtTile - 1) / kCrtTile);
    if (tile >= tiles) return;
    const int t = threadIdx.x;
    const u64 j0 = (u64)tile * kCrtTile;
    const u64 k0 = j0 + (u64)t * kCrtPer;
    // Coefficients k0 .. k0 + 3 (zero past the convolution).
    u64 cw[kCrtPer][L];
    {
        u32 r[kCrtPer][NP];
        if (k0 + kCrtPer <= conv_len && (reinterpret_cast<uintptr_t>(resid) & 15) == 0) {
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const uint4 v = __ldg(reinterpret_cast<const uint4*>(resid + ((size_t)i << log_t) + k0));
                r[0][i] = v.x; r[1][i] = v.y; r[2][i] = v.z; r[3][i] = v.w;
            }
        } else {
#pragma unroll
            for (int c = 0; c < kCrtPer; ++c)
#pragma unroll
                for (int i = 0; i < NP; ++i)
                    r[c][i] = k0 + c < conv_len ? __ldg(resid + ((size_t)i << log_t) + k0 + c) : 0u;
        }
#pragma unroll
        for (int c = 0; c < kCrtPer; ++c) {
            u32 x[NP + 1];
            crt_words<NP>(r[c], cp, s_qp, x);
            pack_words<NP, L>(x, cw[c]);
        }
    }
    if (t < L) {  // coefficient j0 - L + t, before the tile
        u64 w[L];
#pragma unroll
        for (int i = 0; i < L; ++i) w[i] = 0;
        if (j0 >= (u64)(L - t)) {
            const u64 k = j0 - (u64)(L - t);
            u32 r[NP], x[NP + 1];
#pragma unroll
            for (int i = 0; i < NP; ++i) r[i] = __ldg(resid + ((size_t)i << log_t) + k);
            crt_words<NP>(r, cp, s_qp, x);
            pack_words<NP, L>(x, w);
        }
#pragma unroll
        for (int i = 0; i < L; ++i) s_pre[t][i] = w[i];
    }
    u64 sv[kCrtPer];
    u32 gb[kCrtPer], pb[kCrtPer];
    tile_limbs<L>(cw, s_pre, sv, gb, pb);
    store_limbs(dst, k0, out_len, sv, gb, pb, tile_carry_in(gb, pb, tile, flags, status));
}

// dst[j] += add[j] for j < len as one big-integer addition (the sum fits in len
// limbs): four limbs per thread, carries resolved like those of k_crt_mul.
__global__ void __launch_bounds__(kCrtThreads) k_add_limbs(u64* __restrict__ dst, const u64* __restrict__ add,
                                                            u64 len, u32* __restrict__ flags,
                                                            u32* __restrict__ status) {
    __shared__ u32 s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(&flags[0], 1u);
    __syncthreads();
    const u32 tile = s_tile;
    if ((u64)tile * kCrtTile >= len) return;
    const u64 k0 = (u64)tile * kCrtTile + (u64)threadIdx.x * kCrtPer;
    u64 sv[kCrtPer];
    u32 gb[kCrtPer], pb[kCrtPer];
#pragma unroll
    for (int i = 0; i < kCrtPer; ++i) {
        const u64 d = k0 + i < len ? dst[k0 + i] : 0, a = k0 + i < len ? __ldg(add + k0 + i) : 0;
        const u64 t = d + a;
        sv[i] = t;
        gb[i] = t < d ? 1u : 0u;
        pb[i] = t == ~0ull ? 1u : 0u;
    }
    store_limbs(dst, k0, len, sv, gb, pb, tile_carry_in(gb, pb, tile, flags, status));
}

// Descriptors of blocks first .. first + count - 1 of a split product: block m
// multiplies a[m*block, m*block + len) by b and lands at limb m*block of dst (m
// even) or of odd (m odd), so the products of each parity are disjoint.
__global__ void k_split_descs(ProductDesc* __restrict__ d, u64 first, u64 count, const u64* a, u64 la,
                              const u64* b, u64 lb, u64 block, u64* dst, u64* odd, uint8_t* arena,
                              u64 member_bytes, u64 spec_bytes) {
    const u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const u64 m = first + i, off = m * block;
    const u64 len = min(block, la - off);
    uint8_t* base = arena + i * member_bytes;
    ProductDesc x;
    x.a = a + off;
    x.b = b;
    x.la = len;
    x.lb = lb;
    x.spec = reinterpret_cast<u32*>(base);
    x.conv_len = len + lb - 1;
    x.dst = ((m & 1) ? odd : dst) + off;
    x.out_len = len + lb;
    x.agg = base + spec_bytes;
    x.square = 0;
    x.stride = 1;
    x.max_a = x.max_b = 0;
    x.votes = nullptr;
    d[i] = x;
}

// Whether a convolution may be written: false when any admission vote is set
// (votes: kAdmitSlots words, or null when the coefficients were admitted on the
// host). Every thread of the CTA calls it: it holds one barrier in either case.
__device__ __forceinline__ bool admitted(const u32* __restrict__ votes) {
    int bad = 0;
    if (votes)
        for (int i = threadIdx.x; i < kAdmitSlots; i += blockDim.x) bad |= __ldcg(votes + i) != 0u;
    return !__syncthreads_or(bad);
}

// Admission scan (src/convolve.rs:169-184) for the schoolbook convolutions, which
// have no transform to check the coefficients as it loads them: CTA s reads every
// (kAdmitSlots)-th stretch of a and b, compares each coefficient with its bound
// (the magnitude of a two's complement coefficient when signed) and writes vote s.
// Each thread keeps kAdmitUnroll loads in flight, so that the scan runs near the
// HBM rate. grid = kAdmitSlots.
constexpr int kAdmitThreads = 1024, kAdmitUnroll = 8;

template <bool SIGNED>
__device__ __forceinline__ int scan_over(const u64* __restrict__ v, u64 n, u64 mx) {
    int bad = 0;
    const u64 stride = (u64)kAdmitSlots * kAdmitThreads;
    u64 i = (u64)blockIdx.x * kAdmitThreads + threadIdx.x;
    for (; i + (kAdmitUnroll - 1) * stride < n; i += kAdmitUnroll * stride) {
        u64 x[kAdmitUnroll];
#pragma unroll
        for (int u = 0; u < kAdmitUnroll; ++u) x[u] = __ldcs(v + i + u * stride);
#pragma unroll
        for (int u = 0; u < kAdmitUnroll; ++u) bad |= coefficient_over<SIGNED>(x[u], mx);
    }
    for (; i < n; i += stride) bad |= coefficient_over<SIGNED>(__ldcs(v + i), mx);
    return bad;
}

template <bool SIGNED>
__global__ void __launch_bounds__(kAdmitThreads) k_conv_admit(const u64* __restrict__ a, u64 la,
                                                              const u64* __restrict__ b, u64 lb, u64 max_a,
                                                              u64 max_b, u32* __restrict__ votes) {
    int bad = scan_over<SIGNED>(a, la, max_a);
    if (b != a || lb != la || max_b != max_a) bad |= scan_over<SIGNED>(b, lb, max_b);
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) votes[blockIdx.x] = bad ? 1u : 0u;
}

// A convolution whose admission votes (launch.h) reject it is left unwritten and
// reported in the status bytes.
template <int NP>
__global__ void __launch_bounds__(kCrtThreads) k_crt_conv(const u32* __restrict__ resid, int log_t,
                                                           u64 conv_len, u64* __restrict__ dst,
                                                           const __grid_constant__ CrtParams cp,
                                                           const ProductDesc* __restrict__ batch,
                                                           const u32* __restrict__ votes, u32* __restrict__ status) {
    int stride = cp.stride;
    wait_prior_grid();  // the residues of the transform before it
    if (batch) {  // member blockIdx.y of a batch
        const ProductDesc& d = batch[blockIdx.y];
        resid = d.spec;
        conv_len = d.conv_len;
        dst = d.dst;
        stride = (int)d.stride;
        votes = d.votes;
    }
    if ((u64)blockIdx.x * blockDim.x >= conv_len) return;
    __shared__ u32 s_qp[kMaxPrimes + 1][kQpStride];
    stage_multiples(cp, s_qp);  // published by the barrier in admitted()
    if (!admitted(votes)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) report_status(status, 1);
        return;
    }
    const u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= conv_len) return;
    u64 w[4];
    crt_coeff<NP>(resid, log_t, k, cp, s_qp, w);
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
                                                              u64* __restrict__ dst, int stride,
                                                              const u32* __restrict__ votes,
                                                              u32* __restrict__ status) {
    if (!admitted(votes)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) report_status(status, 1);
        return;
    }
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

// Launches k_crt_mul<NP> for NP = cp.np (1..8).
template <class... Args>
static cudaError_t crt_mul_any(int np, dim3 grid, cudaStream_t st, Args... args) {
    switch (np) {
        case 1: return launch_dependent(k_crt_mul<1>, grid, dim3(kCrtThreads), 0, st, args...);
        case 2: return launch_dependent(k_crt_mul<2>, grid, dim3(kCrtThreads), 0, st, args...);
        case 3: return launch_dependent(k_crt_mul<3>, grid, dim3(kCrtThreads), 0, st, args...);
        case 4: return launch_dependent(k_crt_mul<4>, grid, dim3(kCrtThreads), 0, st, args...);
        case 5: return launch_dependent(k_crt_mul<5>, grid, dim3(kCrtThreads), 0, st, args...);
        case 6: return launch_dependent(k_crt_mul<6>, grid, dim3(kCrtThreads), 0, st, args...);
        case 7: return launch_dependent(k_crt_mul<7>, grid, dim3(kCrtThreads), 0, st, args...);
        case 8: return launch_dependent(k_crt_mul<8>, grid, dim3(kCrtThreads), 0, st, args...);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_crt_mul_batch(const ProductDesc* batch, int count, int max_tiles, int log_t,
                                 const CrtParams& cp, cudaStream_t st, u32* status) {
    return crt_mul_any(cp.np, dim3(max_tiles, count), st, (const u32*)nullptr, log_t, (u64)0, (u64)0,
                       (u64*)nullptr, (u32*)nullptr, cp, batch, status);
}

cudaError_t launch_crt_mul(const u32* resid, int log_t, u64 conv_len, u64 out_len, u64* dst, uint8_t* agg,
                           const CrtParams& cp, cudaStream_t st, void (*mark)(cudaStream_t), u32* status) {
    const int tiles = (int)((out_len + kCrtTile - 1) / kCrtTile);
    const cudaError_t e = crt_mul_any(cp.np, dim3(tiles), st, resid, log_t, conv_len, out_len, dst,
                                      reinterpret_cast<u32*>(agg), cp, (const ProductDesc*)nullptr, status);
    if (mark) mark(st);
    return e;
}

// Launches k_crt_conv<NP> for NP = cp.np (1..8).
static cudaError_t crt_conv_any(dim3 grid, cudaStream_t st, const u32* resid, int log_t, u64 conv_len, u64* dst,
                                const CrtParams& cp, const ProductDesc* batch, const u32* votes, u32* status) {
    switch (cp.np) {
#define NTT_CRT_CONV(NP)                                                                                     \
    case NP:                                                                                                 \
        return launch_dependent(k_crt_conv<NP>, grid, dim3(kCrtThreads), 0, st, resid, log_t, conv_len, dst, \
                                cp, batch, votes, status);
        NTT_CRT_CONV(1) NTT_CRT_CONV(2) NTT_CRT_CONV(3) NTT_CRT_CONV(4)
        NTT_CRT_CONV(5) NTT_CRT_CONV(6) NTT_CRT_CONV(7) NTT_CRT_CONV(8)
#undef NTT_CRT_CONV
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_crt_conv_batch(const ProductDesc* batch, int count, u64 max_conv_len, int log_t,
                                  const CrtParams& cp, cudaStream_t st, u32* status) {
    const dim3 grid((unsigned)((max_conv_len + kCrtThreads - 1) / kCrtThreads), count);
    return crt_conv_any(grid, st, nullptr, log_t, 0, nullptr, cp, batch, nullptr, status);
}

cudaError_t launch_crt_conv(const u32* resid, int log_t, u64 conv_len, u64* dst, bool sign,
                            const CrtParams& cp, cudaStream_t st, const u32* votes, u32* status) {
    (void)sign;  // the quotient bias in cp selects signed rounding
    const unsigned blocks = (unsigned)((conv_len + kCrtThreads - 1) / kCrtThreads);
    return crt_conv_any(dim3(blocks), st, resid, log_t, conv_len, dst, cp, nullptr, votes, status);
}

cudaError_t launch_conv_admit(const u64* a, u64 la, const u64* b, u64 lb, u64 max_a, u64 max_b, bool sign,
                              u32* votes, cudaStream_t st) {
    if (sign)
        k_conv_admit<true><<<kAdmitSlots, kAdmitThreads, 0, st>>>(a, la, b, lb, max_a, max_b, votes);
    else
        k_conv_admit<false><<<kAdmitSlots, kAdmitThreads, 0, st>>>(a, la, b, lb, max_a, max_b, votes);
    return cudaGetLastError();
}

// Zeroes the admission votes of every convolution member of a batch class, before
// a forward column pass that raises them. grid = members.
__global__ void __launch_bounds__(kAdmitSlots) k_clear_votes(const ProductDesc* __restrict__ batch) {
    u32* votes = batch[blockIdx.x].votes;
    if (votes) votes[threadIdx.x] = 0u;
}

cudaError_t launch_clear_votes_batch(const ProductDesc* batch, int count, cudaStream_t st) {
    k_clear_votes<<<count, kAdmitSlots, 0, st>>>(batch);
    return cudaGetLastError();
}

cudaError_t launch_conv_schoolbook(const u64* a, u64 la, const u64* b, u64 lb, u64* dst, int stride,
                                   bool sign, cudaStream_t st, const u32* votes, u32* status) {
    const u64 n = la + lb - 1;
    const unsigned blocks = (unsigned)((n + kCrtThreads - 1) / kCrtThreads);
    if (sign) k_conv_school<true><<<blocks, kCrtThreads, 0, st>>>(a, la, b, lb, dst, stride, votes, status);
    else k_conv_school<false><<<blocks, kCrtThreads, 0, st>>>(a, la, b, lb, dst, stride, votes, status);
    return cudaGetLastError();
}

cudaError_t launch_add_limbs(u64* dst, const u64* add, u64 len, u32* flags, cudaStream_t st, u32* status) {
    const u64 tiles = (len + kCrtTile - 1) / kCrtTile;
    k_add_limbs<<<(unsigned)tiles, kCrtThreads, 0, st>>>(dst, add, len, flags, status);
    return cudaGetLastError();
}

cudaError_t launch_split_descs(ProductDesc* d, u64 first, u64 count, const u64* a, u64 la, const u64* b, u64 lb,
                               u64 block, u64* dst, u64* odd, uint8_t* arena, u64 member_bytes, u64 spec_bytes,
                               cudaStream_t st) {
    k_split_descs<<<(unsigned)((count + 127) / 128), 128, 0, st>>>(d, first, count, a, la, b, lb, block, dst, odd,
                                                                    arena, member_bytes, spec_bytes);
    return cudaGetLastError();
}

cudaError_t init_crt_kernels() { return cudaSuccess; }

u32 lookback_timeouts() {
    u32 n = 0;
    if (cudaMemcpyFromSymbol(&n, g_lookback_timeouts, sizeof(n)) != cudaSuccess) return ~0u;
    return n;
}

}  // namespace ntt
