// Transforms held whole by one CTA per prime (T = 2^LOG_N <= 2^13 points).
//
// Reference path (per prime): pack a and b (src/limb/packing.rs:113-292), forward
// transform (src/transform/forward.rs:95-298), pointwise product and inverse with
// the N^-1 scale (src/transform/inverse.rs:52-218, src/multiply/schedule.rs:225-279),
// then for products the CRT and carries of src/multiply/crt.rs (see crt.cu).
//
//  * k_small: one CTA per prime writes canonical residues for the CRT kernels
//    (every convolution, and products that the fused kernel does not take);
//  * k_small_fused: a whole product in one launch, a cluster of one CTA per prime
//    that also reconstructs and carries the product through distributed shared
//    memory.
#include "transform_common.cuh"
#include "crt.cuh"

#include <cooperative_groups.h>

namespace ntt {

// One CTA transforms one prime: pack, forward a (and b), pointwise, inverse, scale.
// grid = (np, members). The prime-0 CTA of a member also clears its CRT flags.
// MODE (RowMode, launch.h): kRowMul a * b, kRowSqr a * a, kRowFwd the forward
// spectrum of a written to g.shared_spec, kRowPre a times the spectrum there.
template <class A, int MODE, bool SIGNED, int LOG_N>
__global__ void __launch_bounds__(kThreads) k_small(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    constexpr bool SQUARE = MODE != kRowMul;
    constexpr int N = 1 << LOG_N;
    constexpr int VS = padded_len(N);
    const PrimeParams& pp = g.ps.pr[blockIdx.x];
    const Member m = member_of(g, blockIdx.y, SQUARE);
    if (blockIdx.x == 0) clear_flags(g, blockIdx.y);
    // convolutions: the prime-0 CTA checks every coefficient's bound as it loads it
    u32* votes = g.votes;
    u64 max_a = g.max_a, max_b = g.max_b;
    if (g.batch) {
        const ProductDesc& d = g.batch[blockIdx.y];
        votes = g.admit ? d.votes : nullptr;
        max_a = d.max_a;
        max_b = d.max_b;
    }
    const bool check = votes && blockIdx.x == 0;
    int bad = 0;
    u32* sa = sm;
    u32* sb = sm + VS;
    for (int i = threadIdx.x; i < N; i += kThreads) {
        const u64 x = (u64)i < m.la ? __ldg(m.a + i) : 0;
        sa[pad_index(i)] = reduce_coefficient<A, SIGNED>(x, pp);
        if (check) bad |= coefficient_over<SIGNED>(x, max_a);
        if (!SQUARE) {
            const u64 y = (u64)i < m.lb ? __ldg(m.b + i) : 0;
            sb[pad_index(i)] = reduce_coefficient<A, SIGNED>(y, pp);
            if (check) bad |= coefficient_over<SIGNED>(y, max_b);
        }
    }
    bad = __syncthreads_or(bad);
    if (check)  // every vote is written: vote 0 carries the verdict
        for (int i = threadIdx.x; i < kAdmitSlots; i += kThreads) votes[i] = i == 0 && bad ? 1u : 0u;
    dif_full<A, LOG_N, kThreads, SQUARE ? 1 : 2, VS>(sm, pp.fwd, pp.p);
    u32* spectrum = g.shared_spec + ((size_t)blockIdx.x << LOG_N);
    if constexpr (MODE == kRowFwd) {
        for (int i = threadIdx.x; i < N; i += kThreads) spectrum[i] = sa[pad_index(i)];
        return;
    }
    for (int i = threadIdx.x; i < N; i += kThreads) {
        const int k = pad_index(i);
        const u32 x = sa[k];
        const u32 y = MODE == kRowMul ? sb[k] : MODE == kRowPre ? __ldg(spectrum + i) : x;
        sa[k] = A::mulc(A::pointwise(x, y, pp.p, pp.pni), pp.scale, pp.p);
    }
    __syncthreads();
    dit_full<A, LOG_N, kThreads, 1, VS>(sa, pp.inv, pp.p);
    u32* out = m.spec + ((size_t)blockIdx.x << LOG_N);
    for (int i = threadIdx.x; i < (int)m.conv_len; i += kThreads) out[i] = A::canonical(sa[pad_index(i)], pp.p);
}

// A whole product of T = 2^LOG_N <= 2^13 points in one kernel: a cluster of NP
// CTAs, one per prime, runs the one-CTA transform of k_small and keeps its
// canonical residues in shared memory; after a cluster barrier CTA r reconstructs
// output tiles r, r + NP, ... (kCrtTile limbs, four per thread) from every CTA's residues
// through distributed shared memory, publishes the tile's (generate, propagate)
// pair, and after a second barrier takes the carry of the earlier tiles from their
// pairs. No residue leaves the chip and the product costs one launch.
// grid = (NP, members), cluster = (NP, 1, 1).
template <bool SQUARE, int LOG_N, int NP>
__global__ void __launch_bounds__(kThreads) k_small_fused(const __grid_constant__ TransformArgs g,
                                                          const __grid_constant__ CrtParams cp) {
    using A = LazyArith;
    namespace cg = cooperative_groups;
    extern __shared__ u32 sm[];
    constexpr int N = 1 << LOG_N;
    constexpr int VS = padded_len(N);
    constexpr int L = crt_limb_words(NP);
    static_assert(kThreads == kCrtThreads, "one CRT tile per CTA of the transform's size");
    cg::cluster_group cluster = cg::this_cluster();
    const int prime = (int)cluster.block_rank();
    const PrimeParams& pp = g.ps.pr[prime];
    const Member m = member_of(g, blockIdx.y, SQUARE);
    u64* dst = g.dst;
    u64 out_len = g.out_len;
    if (g.batch) {
        dst = g.batch[blockIdx.y].dst;
        out_len = g.batch[blockIdx.y].out_len;
    }
    u32* sa = sm;
    u32* sb = sm + VS;
    for (int i = threadIdx.x; i < N; i += kThreads) {
        sa[pad_index(i)] = (u64)i < m.la ? reduce_coefficient<A, false>(__ldg(m.a + i), pp) : 0u;
        if (!SQUARE) sb[pad_index(i)] = (u64)i < m.lb ? reduce_coefficient<A, false>(__ldg(m.b + i), pp) : 0u;
    }
    __syncthreads();
    dif_full<A, LOG_N, kThreads, SQUARE ? 1 : 2, VS>(sm, pp.fwd, pp.p);
    for (int i = threadIdx.x; i < N; i += kThreads) {
        const int k = pad_index(i);
        const u32 x = sa[k];
        const u32 y = SQUARE ? x : sb[k];
        sa[k] = A::mulc(A::pointwise(x, y, pp.p, pp.pni), pp.scale, pp.p);
    }
    __syncthreads();
    dit_full<A, LOG_N, kThreads, 1, VS>(sa, pp.inv, pp.p);
    for (int i = threadIdx.x; i < N; i += kThreads) sa[pad_index(i)] = A::canonical(sa[pad_index(i)], pp.p);
    __shared__ u32 s_qp[kMaxPrimes + 1][kQpStride];
    stage_multiples(cp, s_qp);
    cluster.sync();  // every prime's residues (and this CTA's multiples) are in place
    // CTA r reconstructs output tiles r, r + NP, ... (at most MT of them).
    constexpr int MT = ((N + kCrtTile) / kCrtTile + NP - 1) / NP;
    __shared__ u64 s_pre[L][L];
    __shared__ u32 s_pair[MT];
    const u64 conv_len = m.conv_len;
    const u32 tiles = (u32)((out_len + kCrtTile - 1) / kCrtTile);
    const int t = threadIdx.x;
    const u32* res[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) res[i] = cluster.map_shared_rank(sa, i);
    auto coefficient = [&](u64 k, u64 (&w)[L]) {
        u32 r[NP], x[NP + 1];
#pragma unroll
        for (int i = 0; i < NP; ++i) r[i] = k < conv_len ? res[i][pad_index((int)k)] : 0u;
        crt_words<NP>(r, cp, s_qp, x);
        pack_words<NP, L>(x, w);
    };
    u64 sv[MT][kCrtPer];
    u32 gb[MT][kCrtPer], pb[MT][kCrtPer], xg[MT], xp[MT];
#pragma unroll
    for (int q = 0; q < MT; ++q) {
        const u32 tile = (u32)prime + (u32)q * NP;
        if (tile >= tiles) break;  // the same for the whole CTA
        const u64 j0 = (u64)tile * kCrtTile, k0 = j0 + (u64)t * kCrtPer;
        u64 cw[kCrtPer][L];
#pragma unroll
        for (int c = 0; c < kCrtPer; ++c) coefficient(k0 + c, cw[c]);
        if (t < L) {  // coefficient j0 - L + t, before the tile
            u64 w[L];
#pragma unroll
            for (int i = 0; i < L; ++i) w[i] = 0;
            if (j0 >= (u64)(L - t)) coefficient(j0 - (u64)(L - t), w);
#pragma unroll
            for (int i = 0; i < L; ++i) s_pre[t][i] = w[i];
        }
        tile_limbs<L>(cw, s_pre, sv[q], gb[q], pb[q]);
        u32 tg, tp;
        tile_scan(gb[q], pb[q], xg[q], xp[q], tg, tp);
        if (t == 0) s_pair[q] = tg | (tp << 1);
    }
    cluster.sync();  // every tile's pair is published
#pragma unroll
    for (int q = 0; q < MT; ++q) {
        const u32 tile = (u32)prime + (u32)q * NP;
        if (tile >= tiles) break;
        u32 cin = 0;  // carry out of tiles 0 .. tile-1 (tile j sits in CTA j mod NP)
        for (u32 j = 0; j < tile; ++j) {
            const u32 a = *cluster.map_shared_rank(&s_pair[j / NP], (int)(j % NP));
            cin = (a & 1u) | ((a >> 1) & cin);
        }
        store_limbs(dst, (u64)tile * kCrtTile + (u64)t * kCrtPer, out_len, sv[q], gb[q], pb[q], xg[q] | (xp[q] & cin));
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// ---------------------------------------------------------------------------------

template <class A, int L>
static cudaError_t small_at(const TransformArgs& g, int mode, bool sign, cudaStream_t st, bool init) {
    auto k = mode == kRowMul ? (sign ? k_small<A, kRowMul, true, L> : k_small<A, kRowMul, false, L>)
             : mode == kRowSqr ? (sign ? k_small<A, kRowSqr, true, L> : k_small<A, kRowSqr, false, L>)
             : mode == kRowFwd ? k_small<A, kRowFwd, false, L>
                               : k_small<A, kRowPre, false, L>;
    if (init) return opt_in(k);
    const size_t smem = (size_t)(mode == kRowMul ? 2 : 1) * padded_len(1 << L) * sizeof(u32);
    k<<<dim3(g.np, g.batch ? g.count : 1), kThreads, smem, st>>>(g);
    return cudaGetLastError();
}

template <int L>
static cudaError_t fused_at(const TransformArgs& g, const CrtParams* cp, bool square, cudaStream_t st, bool init) {
    auto k = square ? k_small_fused<true, L, kFusedPrimes> : k_small_fused<false, L, kFusedPrimes>;
    if (init) return opt_in(k);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kFusedPrimes, g.batch ? g.count : 1);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = (size_t)(square ? 1 : 2) * padded_len(1 << L) * sizeof(u32);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kFusedPrimes;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, g, *cp);
}

static cudaError_t fused_any(const TransformArgs& g, const CrtParams* cp, bool square, cudaStream_t st, bool init) {
    switch (g.log_t) {
        case 4: return fused_at<4>(g, cp, square, st, init);
        case 5: return fused_at<5>(g, cp, square, st, init);
        case 6: return fused_at<6>(g, cp, square, st, init);
        case 7: return fused_at<7>(g, cp, square, st, init);
        case 8: return fused_at<8>(g, cp, square, st, init);
        case 9: return fused_at<9>(g, cp, square, st, init);
        case 10: return fused_at<10>(g, cp, square, st, init);
        case 11: return fused_at<11>(g, cp, square, st, init);
        case 12: return fused_at<12>(g, cp, square, st, init);
        case 13: return fused_at<13>(g, cp, square, st, init);
        default: return cudaErrorNotSupported;
    }
}

static cudaError_t small_any(const TransformArgs& g, int mode, bool sign, cudaStream_t st, bool init) {
    switch (g.log_t) {
        case 4: return small_at<LazyArith, 4>(g, mode, sign, st, init);
        case 5: return small_at<LazyArith, 5>(g, mode, sign, st, init);
        case 6: return small_at<LazyArith, 6>(g, mode, sign, st, init);
        case 7: return small_at<LazyArith, 7>(g, mode, sign, st, init);
        case 8: return small_at<LazyArith, 8>(g, mode, sign, st, init);
        case 9: return small_at<LazyArith, 9>(g, mode, sign, st, init);
        case 10: return small_at<LazyArith, 10>(g, mode, sign, st, init);
        case 11: return small_at<LazyArith, 11>(g, mode, sign, st, init);
        case 12: return small_at<LazyArith, 12>(g, mode, sign, st, init);
        case 13: return small_at<LazyArith, 13>(g, mode, sign, st, init);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_small_fused(const TransformArgs& g, const CrtParams& cp, bool square, cudaStream_t st) {
    if (g.wide || g.np != kFusedPrimes || cp.np != kFusedPrimes || g.log_t > kFusedMaxLog || g.log_t < 4)
        return cudaErrorNotSupported;
    return fused_any(g, &cp, square, st, false);
}

cudaError_t launch_small(const TransformArgs& g, int mode, bool sign, cudaStream_t st) {
    return small_any(g, mode, sign, st, false);
}

// Raises the dynamic shared-memory limit of every one-CTA transform kernel.
cudaError_t init_small_kernels() {
    cudaError_t e = cudaSuccess;
    TransformArgs g{};
    for (int sq = 0; sq < 2; ++sq)
        for (int l = 4; l <= kMaxBlockLog && e == cudaSuccess; ++l) {
            g.log_t = l;
            e = small_any(g, sq ? kRowSqr : kRowMul, false, 0, true);
            if (e == cudaSuccess) e = small_any(g, sq ? kRowSqr : kRowMul, true, 0, true);
            if (e == cudaSuccess) e = small_any(g, sq ? kRowFwd : kRowPre, false, 0, true);
            if (e == cudaSuccess && l <= kFusedMaxLog) e = fused_any(g, nullptr, sq, 0, true);
        }
    return e;
}

}  // namespace ntt
