// Transform-domain kernels: limb packing fused into the first forward pass, the
// pointwise product fused between the last forward and first inverse pass, and the
// inverse scale folded into the last twiddle multiply.
//
// Reference path (per prime): pack a and b (src/limb/packing.rs:113-292), forward
// transforms (src/transform/forward.rs:95-298), pointwise product (fused into the
// inverse leaves for long rows, src/multiply/schedule.rs:259-279), inverse with the
// N^-1 scale (src/transform/inverse.rs:52-218, src/multiply/schedule.rs:225-252).
//
// Layouts:
//  * one CTA per prime holds the whole transform (T <= 2^13): k_small and
//    k_small_fused, in small.cu;
//  * four-step for T = R*C > 2^13: k_fwd_cols (pack + column DIF + twiddle; for
//    R = 2^10 k_fwd_cols2, two radix-32 passes), k_rows (row DIF of a and b,
//    pointwise, row DIT, inverse twiddle) and k_inv_cols (column DIT + canonical
//    residues; for R = 2^10 k_inv_cols2). The spectrum order between the passes is
//    the four-step's transposed, bit-reversed order; only the inverse reads it, so
//    no transpose is ever materialised.
//  * k_step_tables builds the four-step factor tables of a transform length.
// Every kernel is instantiated per transform size so all shared-memory strides are
// compile-time constants.
#include "transform_common.cuh"

#include <algorithm>
#include <atomic>

namespace ntt {

#ifndef NTT_ROW_THREADS
#define NTT_ROW_THREADS 128
#endif
// Minimum resident CTAs per SM requested from the register allocator (0: none).
#ifndef NTT_COLS_MINB
#define NTT_COLS_MINB 0
#endif
#if NTT_COLS_MINB > 0
#define NTT_COLS_BOUNDS __launch_bounds__(kThreads, NTT_COLS_MINB)
#else
#define NTT_COLS_BOUNDS __launch_bounds__(kThreads)
#endif
// Threads of a row-pass CTA: at least NTT_ROW_THREADS, and one per register block
// of the first pass (C / 16) up to 512, so that no pass loops twice over its
// blocks (two iterations made the compiler hold both in registers).
__host__ __device__ constexpr int row_threads(int log_c) {
    return (1 << (log_c - 4)) > NTT_ROW_THREADS ? ((1 << (log_c - 4)) < 512 ? (1 << (log_c - 4)) : 512)
                                                : NTT_ROW_THREADS;
}

// Padded words per column in shared memory: congruent to 32/G mod 32 (1 when G >=
// 32) so that a warp's G columns times 32/G rows fall in distinct banks.
__host__ __device__ constexpr int col_words_mod(int log_r) {
    return col_group_log(log_r) >= 5 ? 1 : 32 >> col_group_log(log_r);
}
__host__ __device__ constexpr int col_vstride(int log_r) {
    return padded_len(1 << log_r) + (((col_words_mod(log_r) - padded_len(1 << log_r)) % 32) + 32) % 32;
}

// Column pass of the forward four-step: G columns of R = 2^LOG_R points per CTA.
// grid = (C / G, np, operands). Coefficient n = n1*C + n2 sits at row n1, column n2.
// Column passes map thread t to column c = t mod G and rows r0 + k*RS (r0 = t / G,
// RS = 256 / G rows per sweep), so global addresses advance by a constant and the
// shared-memory slot of sweep k is a compile-time offset from the thread's first.
template <int LOG_R>
struct ColumnMap {
    static constexpr int LOG_G = col_group_log(LOG_R);
    static constexpr int G = 1 << LOG_G;
    static constexpr int VS = col_vstride(LOG_R);
    static constexpr int LOG_RS = col_log_rs(LOG_R);
    static constexpr int RS = kThreads / G;        // rows per sweep (power of two <= 32)
    static constexpr int SWEEPS = (1 << LOG_R) / RS;
    static constexpr int LOG_SW = LOG_R - (8 - LOG_G);
    __device__ static int col() { return threadIdx.x & (G - 1); }
    __device__ static int row0() { return threadIdx.x >> LOG_G; }
    __device__ static int slot0() { return col() * VS + pad_index(row0()); }
    // bit-reversed row index of sweep k, less that of row0 (the bits are disjoint)
    __device__ static constexpr u32 brev_sweep(int k) {
        u32 r = 0;
        for (int b = 0; b < LOG_SW; ++b) r |= ((u32)(k >> b) & 1u) << (LOG_SW - 1 - b);
        return r;
    }
};

// CHECK: a convolution's coefficients are checked against their bounds on the way
// in (column_votes); products are instantiated without the check.
template <class A, bool SIGNED, int LOG_R, bool CHECK = SIGNED>
__global__ void NTT_COLS_BOUNDS k_fwd_cols(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    using M = ColumnMap<LOG_R>;
    release_dependents();
    constexpr int B = M::SWEEPS < 8 ? M::SWEEPS : 8;  // sweeps per batch; B*RS is a multiple of 32
    static_assert(M::SWEEPS % B == 0 && (B * M::RS) % 32 == 0, "column batches");
    const int prime = (int)(blockIdx.x % (u32)g.np);  // prime fastest: see k_fwd_cols4
    const u32 group = blockIdx.x / (u32)g.np;
    // grid.z: operands (1 or 2) of one member, or per member in a batch (2, or 1
    // when the batch's other factor is a stored spectrum)
    const int op = g.batch ? (g.a_only ? 0 : blockIdx.z & 1) : blockIdx.z + g.op_base;
    const Member m = member_of(g, g.batch ? (g.a_only ? blockIdx.z : blockIdx.z >> 1) : 0, false);
    if (op && m.square) return;
    const PrimeParams& pp = g.ps.pr[prime];
    const u64* __restrict__ src = op ? m.b : m.a;
    const u64 len = op ? m.lb : m.la;
    u64 vmax = 0;
    u32* const votes =
        CHECK ? column_votes(g, g.batch ? (g.a_only ? blockIdx.z : blockIdx.z >> 1) : 0, op, prime, vmax) : nullptr;
    int bad = 0;
    const int log_c = g.log_c;
    const u32 col0 = group << M::LOG_G;
    const u32 col = col0 + M::col();
    const int r0 = M::row0();
    const u64 first = ((u64)r0 << log_c) + col;
    const u64 step = (u64)M::RS << log_c;
    u32* s = sm + M::slot0();
    uint2* tw = reinterpret_cast<uint2*>(sm + M::G * M::VS);
    load_table<LOG_R>(tw, pp.fwd);
    // Per-sweep four-step factors of the CTA's columns, rows padded to SW + 1 entries
    // so that the G columns of a warp read distinct banks.
    uint2* fb = tw + (1 << LOG_R);
    {
        const uint2* src = pp.f4_b + ((size_t)col0 << M::LOG_SW);
        for (int i = threadIdx.x; i < (M::G << M::LOG_SW); i += kThreads)
            fb[(i >> M::LOG_SW) * (M::SWEEPS + 1) + (i & (M::SWEEPS - 1))] = __ldg(src + i);
    }
    const uint2 fa = __ldg(pp.f4_a + ((size_t)col << M::LOG_RS) + (__brev((u32)r0) >> (32 - M::LOG_RS)));
    // First forward pass fused with the limb reduction (its roots come from global
    // memory: the shared table is published by the barrier after it). Item it takes
    // column c = it mod G and block gg = it / G (rows gg + k * HQ), so a warp loads
    // four rows of G consecutive limbs at a time and stores to distinct banks. When
    // len <= T/2 (every balanced product) rows R/2 and above hold no limb: their
    // loads and the first level's butterflies are skipped.
    {
        constexpr int RB = kMaxRB, LOG_HQ = LOG_R - RB, HQ = 1 << LOG_HQ, E = 1 << RB;
        const bool half = len <= ((u64)1 << (g.log_t - 1));
        const u64 kstep = (u64)HQ << log_c;
#pragma unroll 1
        for (int it = threadIdx.x; it < (M::G << LOG_HQ); it += kThreads) {
            const int c = it & (M::G - 1), gg = it >> M::LOG_G;
            const u64 n0 = ((u64)gg << log_c) + col0 + c;
            u32 x[1][E];
            if (half) {
#pragma unroll
                for (int k = 0; k < E / 2; ++k) {
                    const u64 n = n0 + k * kstep;
                    const u64 v = n < len ? __ldcs(src + n) : 0;
                    if (CHECK && votes) bad |= coefficient_over<SIGNED>(v, vmax);
                    x[0][k] = n < len ? reduce_coefficient<A, SIGNED>(v, pp) : 0u;
                }
                dif_levels<A, RB, HQ, 1, true>(x, pp.fwd + gg, pp.p);
            } else {
#pragma unroll
                for (int k = 0; k < E; ++k) {
                    const u64 n = n0 + k * kstep;
                    const u64 v = n < len ? __ldcs(src + n) : 0;
                    if (CHECK && votes) bad |= coefficient_over<SIGNED>(v, vmax);
                    x[0][k] = n < len ? reduce_coefficient<A, SIGNED>(v, pp) : 0u;
                }
                dif_levels<A, RB, HQ, 1>(x, pp.fwd + gg, pp.p);
            }
            u32* base = sm + c * M::VS + pad_index(gg);
#pragma unroll
            for (int k = 0; k < E; ++k) base[slot_offset<HQ>(k)] = x[0][k];
        }
    }
    if (CHECK && bad) votes[(blockIdx.x + threadIdx.x) % kAdmitSlots] = 1u;
    __syncthreads();
    dif_full<A, LOG_R, kThreads, M::G, M::VS, kMaxRB>(sm, tw, pp.p);
    // Four-step twiddle w_T^(col * brev(row)) = fa * fb[col][brev(k)], then the store.
    u32* dst = m.spec + ((size_t)(op * g.np + prime) << g.log_t) + first;
    const uint2* fbc = fb + M::col() * (M::SWEEPS + 1);
#pragma unroll 1
    for (int k0 = 0; k0 < M::SWEEPS; k0 += B) {
        const uint2* fk = fbc + (__brev((u32)k0) >> (32 - M::LOG_SW));
        const u32* sk = s + slot_offset<M::RS>(k0);
#pragma unroll
        for (int u = 0; u < B; ++u) {
            u32 x = sk[slot_offset<M::RS>(u)];
            x = A::mulc(x, fk[M::brev_sweep(u)], pp.p);
            x = A::mulc(x, fa, pp.p);
            dst[u * step] = x;
        }
        dst += B * step;
    }
}

// Column passes for R = 2^10 (every product with T = 2^20 or 2^21, the 1M x 1M
// bench shape among them) in two radix-32 passes: one barrier and one round trip
// through shared memory per element. A thread owns one register block per pass:
// column c = t mod 8 and either rows gg + 32k (block gg) or rows 32 g2 + k (block
// g2), k < 32. With the padded column stride (4 mod 32) both orders put a warp's
// 8 columns x 4 blocks on 32 distinct banks, and both read or write global memory
// as 4 rows x 8 consecutive columns. The forward four-step twiddle of row
// 32 g2 + k is w_T^(col * brev(row)) = f4_a[col][brev5(k)] * f4_b[col][brev5(g2)]
// (brev(row) = 32 brev5(k) + brev5(g2)). Four CTAs per SM (64 registers) measured
// best.
constexpr int kCol2LogR = 10;
static_assert(col_group_log(10) == 3 && col_log_rs(10) == 5, "two-pass columns assume 8 columns per CTA");
// Resident CTAs per SM the two-pass column kernels ask the register allocator for.
#ifndef NTT_COLS2_MINB
#define NTT_COLS2_MINB 4
#endif
#ifndef NTT_INV_COLS2_MINB
#define NTT_INV_COLS2_MINB 4
#endif

template <class A, bool SIGNED, bool CHECK = SIGNED>
__global__ void __launch_bounds__(kThreads, NTT_COLS2_MINB) k_fwd_cols2(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    release_dependents();
    constexpr int LOG_R = kCol2LogR, G = 8, VS = col_vstride(LOG_R), E = 32;
    const int prime = (int)(blockIdx.x % (u32)g.np);  // prime fastest: see k_fwd_cols4
    const u32 group = blockIdx.x / (u32)g.np;
    const int op = g.batch ? (g.a_only ? 0 : blockIdx.z & 1) : blockIdx.z + g.op_base;
    const Member m = member_of(g, g.batch ? (g.a_only ? blockIdx.z : blockIdx.z >> 1) : 0, false);
    if (op && m.square) return;
    const PrimeParams& pp = g.ps.pr[prime];
    const u64* __restrict__ src = op ? m.b : m.a;
    const u64 len = op ? m.lb : m.la;
    u64 vmax = 0;
    u32* const votes =
        CHECK ? column_votes(g, g.batch ? (g.a_only ? blockIdx.z : blockIdx.z >> 1) : 0, op, prime, vmax) : nullptr;
    int bad = 0;
    const int log_c = g.log_c;
    const u32 col0 = group * G;
    const int c = threadIdx.x & (G - 1), blk = threadIdx.x >> 3;
    const u32 col = col0 + c;
    // f4_a rows of the CTA's columns, padded to 33 entries per column.
    uint2* fa = reinterpret_cast<uint2*>(sm + G * VS);
    fa[c * (E + 1) + blk] = __ldg(pp.f4_a + ((size_t)col << 5) + blk);
    // Pass 1: levels 0-4 on rows blk + 32k, limbs reduced on the way in; rows R/2
    // and above hold no limb when len <= T/2.
    {
        const bool half = len <= ((u64)1 << (g.log_t - 1));
        const u64* p0 = src + ((u64)blk << log_c) + col;
        const u64 n0 = ((u64)blk << log_c) + col, kstep = (u64)E << log_c;
        u32 x[1][E];
        if (half) {
#pragma unroll
            for (int k = 0; k < E / 2; ++k) {
                const u64 v = n0 + k * kstep < len ? __ldcs(p0 + k * kstep) : 0;
                if (CHECK && votes) bad |= coefficient_over<SIGNED>(v, vmax);
                x[0][k] = n0 + k * kstep < len ? reduce_coefficient<A, SIGNED>(v, pp) : 0u;
            }
            dif_levels<A, 5, E, 1, true>(x, pp.fwd + blk, pp.p);
        } else {
#pragma unroll
            for (int k = 0; k < E; ++k) {
                const u64 v = n0 + k * kstep < len ? __ldcs(p0 + k * kstep) : 0;
                if (CHECK && votes) bad |= coefficient_over<SIGNED>(v, vmax);
                x[0][k] = n0 + k * kstep < len ? reduce_coefficient<A, SIGNED>(v, pp) : 0u;
            }
            dif_levels<A, 5, E, 1>(x, pp.fwd + blk, pp.p);
        }
        u32* base = sm + c * VS + blk;
#pragma unroll
        for (int k = 0; k < E; ++k) base[33 * k] = x[0][k];
    }
    if (CHECK && bad) votes[(blockIdx.x + threadIdx.x) % kAdmitSlots] = 1u;
    __syncthreads();
    // Pass 2: levels 5-9 on rows 32 blk + k, four-step twiddle, store.
    {
        const u32* base = sm + c * VS + 33 * blk;
        u32 x[1][E];
#pragma unroll
        for (int k = 0; k < E; ++k) x[0][k] = base[k];
        // the last level (twiddle 1) stays open: its outputs go straight into the
        // product by the four-step factor, which accepts them unreduced
        dif_levels<A, 5, 1, 1, false, true>(x, pp.small_fwd, pp.p);
        const uint2 fb = __ldg(pp.f4_b + ((size_t)col << 5) + (__brev((u32)blk) >> 27));
        const uint2* fac = fa + c * (E + 1);
        u32* dst = m.spec + ((size_t)(op * g.np + prime) << g.log_t) + ((u64)(blk * E) << log_c) + col;
#pragma unroll
        for (int k = 0; k < E; ++k) {
            const u32 y = A::mulc(A::mulc(x[0][k], fac[__brev((u32)k) >> 27], pp.p), fb, pp.p);
            dst[(u64)k << log_c] = y;
        }
    }
}

template <class A>
__global__ void __launch_bounds__(kThreads, NTT_INV_COLS2_MINB) k_inv_cols2(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    constexpr int LOG_R = kCol2LogR, G = 8, VS = col_vstride(LOG_R), E = 32;
    const int prime = blockIdx.y;
    const PrimeParams& pp = g.ps.pr[prime];
    const Member m = member_of(g, blockIdx.z, false);
    release_dependents();
    const int log_c = g.log_c;
    const int c = threadIdx.x & (G - 1), blk = threadIdx.x >> 3;
    wait_prior_grid();  // the row pass's output
    // the CRT look-back flags of this product, cleared once every kernel before
    // this one has completed
    if (blockIdx.x == 0 && prime == 0) clear_flags(g, blockIdx.z);
    u32* const spec = m.spec + ((size_t)prime << g.log_t) + blockIdx.x * G + c;
    // Pass 1: levels 0-4 on rows 32 blk + k (bit-reversed spectrum in).
    {
        const u32* q = spec + ((u64)(blk * E) << log_c);
        u32 x[1][E];
#pragma unroll
        for (int k = 0; k < E; ++k) x[0][k] = __ldcs(q + ((u64)k << log_c));
        dit_levels<A, 5, 1, 1, 2>(x, pp.small_inv, pp.p);  // the row pass wrote [0, 2p)
        u32* base = sm + c * VS + 33 * blk;
#pragma unroll
        for (int k = 0; k < E; ++k) base[k] = x[0][k];
    }
    __syncthreads();
    // Pass 2: levels 5-9 on rows blk + 32k, canonical residues out.
    {
        const u32* base = sm + c * VS + blk;
        u32 x[1][E];
#pragma unroll
        for (int k = 0; k < E; ++k) x[0][k] = base[33 * k];
        dit_levels<A, 5, E, 1>(x, pp.inv + blk, pp.p);
        u32* q = spec + ((u64)blk << log_c);
#pragma unroll
        for (int k = 0; k < E; ++k) q[(u64)(k * E) << log_c] = A::canonical(x[0][k], pp.p);
    }
}

// Column passes for R = 2^12 (the wide lengths T = 2^24 and 2^25) in two radix-64
// passes, the k_fwd_cols2 design at twice the block: G columns per CTA of 64 G
// threads, thread t owning column c = t mod G and either rows blk + 64k (pass 1)
// or rows 64 blk + k (pass 2), k < 64. Row r = 64a + b sits at slot 65a + b of its
// column, whose stride (32/G mod 32) puts a warp's G columns x 32/G blocks on 32
// distinct banks in both orders. The forward four-step twiddle of row 64 blk + k is
// w_T^(col * brev(row)) = f4_a[col][brev6(k)] * f4_b[col][brev6(blk)]. The level
// roots of the consecutive-point pass (entries 1..63) sit in shared memory.
// G = 8 (512 threads of 128 registers, 135 KB) fills an SM with one CTA. G = 4
// (two CTAs per SM, so that one CTA's loads overlap the other's butterflies)
// measured slower on GB300 at T = 2^25: 1.58 against 1.20 ms forward, 0.76 against
// 0.57 ms inverse (16-byte row segments instead of whole 32-byte sectors).
#ifndef NTT_COLS4_LOG_G
#define NTT_COLS4_LOG_G 3
#endif
constexpr int kCol4LogG = NTT_COLS4_LOG_G, kCol4G = 1 << kCol4LogG, kCol4Threads = 64 * kCol4G;
constexpr int kCol4Vs = 65 * 64 + 32 / kCol4G;
static_assert(kCol4Vs % 32 == 32 / kCol4G && step_log_u(kCol4LogR) == 6, "radix-64 column layout");
static_assert(kCol4Threads * 128 * (kCol4LogG == 2 ? 2 : 1) <= 65536, "register budget of the column CTAs");

// SMs of the current device (persistent kernels launch one CTA per SM).
static int sm_count() {
    static std::atomic<int> cached[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    int n = cached[dev].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    cached[dev].store(n, std::memory_order_relaxed);
    return n;
}

static size_t col4_smem(bool fwd) {
    return (size_t)kCol4G * kCol4Vs * sizeof(u32) + 64 * sizeof(uint2) + (fwd ? kCol4G * 65 * sizeof(uint2) : 0);
}

template <class A, bool SIGNED, bool CHECK = SIGNED>
__global__ void __launch_bounds__(kCol4Threads, kCol4LogG == 2 ? 2 : 1)
    k_fwd_cols4(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    release_dependents();
    constexpr int G = kCol4G, LOG_G = kCol4LogG, VS = kCol4Vs, E = 64;
    // grid.x runs over (column group, prime) with the prime fastest, so the np CTAs
    // that read the same limbs run together and all but the first read them from L2
    const int prime = (int)(blockIdx.x % (u32)g.np);
    const u32 group = blockIdx.x / (u32)g.np;
    const int op = g.batch ? (g.a_only ? 0 : blockIdx.z & 1) : blockIdx.z + g.op_base;
    const Member m = member_of(g, g.batch ? (g.a_only ? blockIdx.z : blockIdx.z >> 1) : 0, false);
    if (op && m.square) return;
    const PrimeParams& pp = g.ps.pr[prime];
    const u64* __restrict__ src = op ? m.b : m.a;
    const u64 len = op ? m.lb : m.la;
    u64 vmax = 0;
    u32* const votes =
        CHECK ? column_votes(g, g.batch ? (g.a_only ? blockIdx.z : blockIdx.z >> 1) : 0, op, prime, vmax) : nullptr;
    int bad = 0;
    const int log_c = g.log_c;
    const u32 col0 = group * G;
    const int c = threadIdx.x & (G - 1), blk = threadIdx.x >> LOG_G;
    const u32 col = col0 + c;
    uint2* tw = reinterpret_cast<uint2*>(sm + G * VS);
    uint2* fa = tw + 64;  // f4_a rows of the CTA's columns, 65 entries apart
    if (threadIdx.x < 64) tw[threadIdx.x] = __ldg(pp.fwd + threadIdx.x);
    fa[c * (E + 1) + blk] = __ldg(pp.f4_a + ((size_t)col << 6) + blk);
    // Pass 1: levels 0-5 on rows blk + 64k, limbs reduced on the way in; rows R/2
    // and above hold no limb when len <= T/2.
    {
        const bool half = len <= ((u64)1 << (g.log_t - 1));
        const u64* p0 = src + ((u64)blk << log_c) + col;
        const u64 n0 = ((u64)blk << log_c) + col, kstep = (u64)E << log_c;
        u32 x[1][E];
        if (half) {
#pragma unroll
            for (int k = 0; k < E / 2; ++k) {
                const u64 v = n0 + k * kstep < len ? __ldcs(p0 + k * kstep) : 0;
                if (CHECK && votes) bad |= coefficient_over<SIGNED>(v, vmax);
                x[0][k] = n0 + k * kstep < len ? reduce_coefficient<A, SIGNED>(v, pp) : 0u;
            }
            dif_levels<A, 6, E, 1, true>(x, pp.fwd + blk, pp.p);
        } else {
#pragma unroll
            for (int k = 0; k < E; ++k) {
                const u64 v = n0 + k * kstep < len ? __ldcs(p0 + k * kstep) : 0;
                if (CHECK && votes) bad |= coefficient_over<SIGNED>(v, vmax);
                x[0][k] = n0 + k * kstep < len ? reduce_coefficient<A, SIGNED>(v, pp) : 0u;
            }
            dif_levels<A, 6, E, 1>(x, pp.fwd + blk, pp.p);
        }
        u32* base = sm + c * VS + blk;
#pragma unroll
        for (int k = 0; k < E; ++k) base[65 * k] = x[0][k];
    }
    if (CHECK && bad) votes[(blockIdx.x + threadIdx.x) % kAdmitSlots] = 1u;
    __syncthreads();
    // Pass 2: levels 6-11 on rows 64 blk + k, four-step twiddle, store.
    {
        const u32* base = sm + c * VS + 65 * blk;
        u32 x[1][E];
#pragma unroll
        for (int k = 0; k < E; ++k) x[0][k] = base[k];
        // the last level (twiddle 1) stays open for the four-step product
        dif_levels<A, 6, 1, 1, false, true>(x, tw, pp.p);
        const uint2 fb = __ldg(pp.f4_b + ((size_t)col << 6) + (__brev((u32)blk) >> 26));
        const uint2* fac = fa + c * (E + 1);
        u32* dst = m.spec + ((size_t)(op * g.np + prime) << g.log_t) + ((u64)(blk * E) << log_c) + col;
#pragma unroll
        for (int k = 0; k < E; ++k) {
            const u32 y = A::mulc(A::mulc(x[0][k], fac[__brev((u32)k) >> 26], pp.p), fb, pp.p);
            dst[(u64)k << log_c] = y;
        }
    }
}

template <class A>
__global__ void __launch_bounds__(kCol4Threads, kCol4LogG == 2 ? 2 : 1)
    k_inv_cols4(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    constexpr int G = kCol4G, LOG_G = kCol4LogG, VS = kCol4Vs, E = 64;
    const int prime = blockIdx.y;
    const PrimeParams& pp = g.ps.pr[prime];
    const Member m = member_of(g, blockIdx.z, false);
    release_dependents();
    const int log_c = g.log_c;
    const int c = threadIdx.x & (G - 1), blk = threadIdx.x >> LOG_G;
    uint2* tw = reinterpret_cast<uint2*>(sm + G * VS);
    if (threadIdx.x < 64) tw[threadIdx.x] = __ldg(pp.inv + threadIdx.x);
    __syncthreads();
    wait_prior_grid();  // the row pass's output
    // the CRT look-back flags of this product, cleared once every kernel before
    // this one has completed
    if (blockIdx.x == 0 && prime == 0) clear_flags(g, blockIdx.z);
    u32* const spec = m.spec + ((size_t)prime << g.log_t) + blockIdx.x * G + c;
    // Pass 1: levels 0-5 on rows 64 blk + k (bit-reversed spectrum in).
    {
        const u32* q = spec + ((u64)(blk * E) << log_c);
        u32 x[1][E];
#pragma unroll
        for (int k = 0; k < E; ++k) x[0][k] = __ldcs(q + ((u64)k << log_c));
        dit_levels<A, 6, 1, 1, 2>(x, tw, pp.p);  // the row pass wrote [0, 2p) ([0, p) when wide)
        u32* base = sm + c * VS + 65 * blk;
#pragma unroll
        for (int k = 0; k < E; ++k) base[k] = x[0][k];
    }
    __syncthreads();
    // Pass 2: levels 6-11 on rows blk + 64k, canonical residues out.
    {
        const u32* base = sm + c * VS + blk;
        u32 x[1][E];
#pragma unroll
        for (int k = 0; k < E; ++k) x[0][k] = base[65 * k];
        dit_levels<A, 6, E, 1>(x, pp.inv + blk, pp.p);
        u32* q = spec + ((u64)blk << log_c);
#pragma unroll
        for (int k = 0; k < E; ++k) q[(u64)(k * E) << log_c] = A::canonical(x[0][k], pp.p);
    }
}

// Persistent form of k_inv_cols4 (NTT_INV_COLS4_PERSIST): one CTA per SM loops
// over the (column group, prime, member) items. Once an item's second pass holds
// its points in registers, the shared buffer is free, and 16-byte cp.async copies
// bring the next item's residues into it while that pass computes and stores, so
// that the loads of one item overlap the butterflies of the one before. The copies
// land in a raw layout, row 64b + k of the 8 columns at word 520b + 8k: the first
// pass (rows 64 blk + k) reads it without bank conflicts, and it fits the buffer
// (64 x 520 <= 8 x kCol4Vs words). The inverse roots of every prime sit after it.
#ifndef NTT_INV_COLS4_PERSIST
#define NTT_INV_COLS4_PERSIST 1
#endif
constexpr int kRawBlockWords = 520;
static_assert(kCol4G == 8 && 64 * kRawBlockWords <= kCol4G * kCol4Vs && kRawBlockWords % 32 == 8,
              "raw layout of the persistent inverse column pass");

static size_t col4p_smem(int np) { return (size_t)kCol4G * kCol4Vs * sizeof(u32) + (size_t)np * 64 * sizeof(uint2); }

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <class A>
__global__ void __launch_bounds__(kCol4Threads, 1) k_inv_cols4p(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    constexpr int G = kCol4G, LOG_G = kCol4LogG, VS = kCol4Vs, E = 64, RB = kRawBlockWords;
    release_dependents();
    const int log_c = g.log_c;
    const u32 groups = 1u << (log_c - LOG_G), np = (u32)g.np;
    const u32 items = groups * np * (u32)(g.batch ? g.count : 1);
    const int c = threadIdx.x & (G - 1), blk = threadIdx.x >> LOG_G;
    uint2* tw = reinterpret_cast<uint2*>(sm + G * VS);  // [prime][64] inverse roots
    for (int i = threadIdx.x; i < g.np * 64; i += kCol4Threads) tw[i] = __ldg(g.ps.pr[i >> 6].inv + (i & 63));
    wait_prior_grid();  // the row pass's output
    // residues of item it: [prime][T] of its member, from column group * G
    auto source = [&](u32 it) -> u32* {
        const u32 group = it % groups, rest = it / groups;
        const Member mm = member_of(g, (int)(rest / np), false);
        return mm.spec + ((size_t)(rest % np) << g.log_t) + (size_t)group * G;
    };
    auto prefetch = [&](u32 it) {
        const u32* src = source(it);
        for (int j = threadIdx.x; j < 2 * 4096; j += kCol4Threads) {
            const int r = j >> 1, h = j & 1;
            cp_async16(sm + RB * (r >> 6) + 8 * (r & 63) + 4 * h, src + ((u64)r << log_c) + 4 * h);
        }
        cp_async_commit();
    };
    if (blockIdx.x < items) prefetch(blockIdx.x);
    for (u32 it = blockIdx.x; it < items; it += gridDim.x) {
        const u32 group = it % groups, rest = it / groups;
        const int prime = (int)(rest % np), member = (int)(rest / np);
        const PrimeParams& pp = g.ps.pr[prime];
        // the CRT look-back flags of this product, cleared once every kernel before
        // this one has completed
        if (group == 0 && prime == 0) clear_flags(g, member);
        cp_async_wait_all();
        __syncthreads();
        // Pass 1: levels 0-5 on rows 64 blk + k (bit-reversed spectrum in).
        u32 x[1][E];
        {
            const u32* raw = sm + RB * blk + c;
#pragma unroll
            for (int k = 0; k < E; ++k) x[0][k] = raw[8 * k];
            dit_levels<A, 6, 1, 1, 2>(x, tw + 64 * prime, pp.p);  // [0, 2p) in ([0, p) when wide)
        }
        __syncthreads();  // every raw read is done before the padded layout overwrites it
        {
            u32* base = sm + c * VS + 65 * blk;
#pragma unroll
            for (int k = 0; k < E; ++k) base[k] = x[0][k];
        }
        __syncthreads();
        // Pass 2: levels 6-11 on rows blk + 64k, canonical residues out; the next
        // item's residues come in behind it.
        {
            const u32* base = sm + c * VS + blk;
#pragma unroll
            for (int k = 0; k < E; ++k) x[0][k] = base[65 * k];
        }
        __syncthreads();
        if (it + gridDim.x < items) prefetch(it + gridDim.x);
        dit_levels<A, 6, E, 1>(x, pp.inv + blk, pp.p);
        u32* q = source(it) + c + ((u64)blk << log_c);
#pragma unroll
        for (int k = 0; k < E; ++k) q[(u64)(k * E) << log_c] = A::canonical(x[0][k], pp.p);
    }
    cp_async_wait_all();
}

// Rows per CTA of the row pass: enough that every thread owns a register block of
// the first pass (2^(log_c - kMaxRB) blocks per row).
__host__ __device__ constexpr int row_log_rpc(int log_c) {
    return log_c - kMaxRB >= ilog2(row_threads(log_c)) ? 0 : ilog2(row_threads(log_c)) - (log_c - kMaxRB);
}

// Row pass: forward rows of a (and b), pointwise product, inverse rows, inverse
// four-step twiddle with the 2^32 / T scale. grid = (R / RPC, np); writes over a's
// rows. A CTA owns RPC consecutive rows; shared memory holds vectors [RPC][a, b].
//
// Shared memory is touched as little as the register blocks allow: the first
// forward pass reads the rows from global memory, the last forward pass, the
// pointwise product and the first inverse pass run on the same registers (both
// work on blocks of 2^RBL consecutive points), and the last inverse pass applies
// the twiddle and writes global memory.
template <class A, int MODE, int LOG_C>
__global__ void __launch_bounds__(row_threads(LOG_C)) k_rows(const __grid_constant__ TransformArgs g) {
    constexpr int kRowThreads = row_threads(LOG_C);
    extern __shared__ u32 sm[];
    constexpr int C = 1 << LOG_C;
    constexpr int VS = padded_len(C);
    constexpr int NV = MODE == kRowMul ? 2 : 1;  // a (and b), transformed together
    constexpr int LOG_RPC = row_log_rpc(LOG_C);
    constexpr int RPC = 1 << LOG_RPC;
    constexpr int RB = kMaxRB;
    constexpr int RBL = LOG_C % RB ? LOG_C % RB : RB;  // levels of the fused middle pass
    constexpr int LL = LOG_C - RBL;              // its first forward level
    constexpr int NL = 1 << kRowTwLoBits, NH = C >> kRowTwLoBits;
    static_assert(LOG_C > RB && LOG_C > kRowTwLoBits, "at least two passes each way");
    const int prime = blockIdx.y;
    const int row0 = blockIdx.x << LOG_RPC;
    const PrimeParams& pp = g.ps.pr[prime];
    const Member m = member_of(g, blockIdx.z, NV == 1);
    release_dependents();
    u32* ra = m.spec + ((size_t)prime << g.log_t) + ((size_t)row0 << LOG_C);
    const u32* rb = m.spec + ((size_t)(g.np + prime) << g.log_t) + ((size_t)row0 << LOG_C);
    // the stored spectrum of the rows (kRowFwd writes it, kRowPre multiplies by it)
    u32* rs = g.shared_spec + ((size_t)prime << g.log_t) + ((size_t)row0 << LOG_C);
    // The rows' inverse four-step factors: RPC x 64 low-digit entries, RPC x C/64 high.
    uint2* il = reinterpret_cast<uint2*>(sm + RPC * NV * VS);
    uint2* ih = il + RPC * NL;
    if constexpr (MODE != kRowFwd) {
        const uint2* lo = pp.i4_lo + (size_t)row0 * NL;
        const uint2* hi = pp.i4_hi + (size_t)row0 * NH;
        for (int i = threadIdx.x; i < RPC * (NL + NH); i += kRowThreads)
            il[i] = __ldg(i < RPC * NL ? lo + i : hi + (i - RPC * NL));
    }
    wait_prior_grid();  // the column pass's output
    // First forward pass: global -> shared. Block gg of a row holds points gg + k * HQ.
    {
        constexpr int LOG_HQ = LOG_C - RB;
        constexpr int HQ = 1 << LOG_HQ;
#pragma unroll 1
        for (int it = threadIdx.x; it < (RPC << LOG_HQ); it += kRowThreads) {
            const int r = it >> LOG_HQ, gg = it & (HQ - 1);
            const size_t off = ((size_t)r << LOG_C) + gg;
            u32 x[NV][1 << RB];
#pragma unroll
            for (int k = 0; k < (1 << RB); ++k) {
                x[0][k] = __ldcs(ra + off + k * HQ);
                if constexpr (NV == 2) x[NV - 1][k] = __ldcs(rb + off + k * HQ);
            }
            dif_levels<A, RB, HQ, NV>(x, pp.fwd + gg, pp.p);
            u32* base = sm + r * NV * VS + pad_index(gg);
#pragma unroll
            for (int q = 0; q < NV; ++q)
#pragma unroll
                for (int k = 0; k < (1 << RB); ++k) base[q * VS + slot_offset<HQ>(k)] = x[q][k];
        }
    }
    __syncthreads();
    dif_range<A, LOG_C, kRowThreads, RPC * NV, VS, RB, LL>(sm, pp.fwd, pp.p);
    // Last forward pass, pointwise product, first inverse pass: blocks of 2^RBL
    // consecutive points (twiddles of half-size below 2^RBL, shared by all blocks).
    {
        constexpr int E = 1 << RBL;
#pragma unroll 1
        for (int it = threadIdx.x; it < (RPC << (LOG_C - RBL)); it += kRowThreads) {
            const int r = it >> (LOG_C - RBL), gg = it & ((C >> RBL) - 1);
            u32* base = sm + r * NV * VS + pad_index(gg << RBL);
            u32 x[NV][E];
#pragma unroll
            for (int q = 0; q < NV; ++q)
#pragma unroll
                for (int k = 0; k < E; ++k) x[q][k] = base[q * VS + k];
            // a's last level stays open (the Montgomery product takes one factor
            // below 4p), the other factor's is reduced; the product is below 3p, so
            // the first inverse level (twiddle 1) needs no products either
            u32 y[E];
            if constexpr (MODE == kRowMul) {
                u32(&xa)[1][E] = *reinterpret_cast<u32(*)[1][E]>(&x[0]);
                u32(&xb)[1][E] = *reinterpret_cast<u32(*)[1][E]>(&x[1]);
                dif_levels<A, RBL, 1, 1, false, true>(xa, pp.small_fwd, pp.p);
                dif_levels<A, RBL, 1, 1>(xb, pp.small_fwd, pp.p);
#pragma unroll
                for (int k = 0; k < E; ++k) y[k] = x[1][k];
            } else if constexpr (MODE == kRowSqr || MODE == kRowFwd) {
                dif_levels<A, RBL, 1, 1>(x, pp.small_fwd, pp.p);
                if constexpr (MODE == kRowFwd) {  // the reduced spectrum, stored
                    u32* out = rs + ((size_t)r << LOG_C) + (gg << RBL);
#pragma unroll
                    for (int k = 0; k < E; ++k) out[k] = x[0][k];
                    continue;
                }
#pragma unroll
                for (int k = 0; k < E; ++k) y[k] = x[0][k];
            } else {  // kRowPre: the other factor is the stored spectrum
                const u32* in = rs + ((size_t)r << LOG_C) + (gg << RBL);
#pragma unroll
                for (int k = 0; k < E; ++k) y[k] = __ldg(in + k);
                dif_levels<A, RBL, 1, 1, false, true>(x, pp.small_fwd, pp.p);
            }
#pragma unroll
            for (int k = 0; k < E; ++k) x[0][k] = A::pointwise(x[0][k], y[k], pp.p, pp.pni);
            u32(&z)[1][E] = *reinterpret_cast<u32(*)[1][E]>(&x[0]);
            dit_levels<A, RBL, 1, 1, 1>(z, pp.small_inv, pp.p);
#pragma unroll
            for (int k = 0; k < E; ++k) base[k] = x[0][k];
        }
    }
    if constexpr (MODE == kRowFwd) return;
    __syncthreads();
    dit_range<A, LOG_C, kRowThreads, RPC, NV * VS, RBL, LOG_C - RB>(sm, pp.inv, pp.p);
    // Last inverse pass: shared -> global, times the inverse four-step twiddle of
    // n2 = 64 hi + lo (i4_lo of lo, i4_hi of hi with the scale folded in).
    {
        constexpr int LOG_HS = LOG_C - RB;
        constexpr int HS = 1 << LOG_HS;
#pragma unroll 1
        for (int it = threadIdx.x; it < (RPC << LOG_HS); it += kRowThreads) {
            const int r = it >> LOG_HS, gg = it & (HS - 1);
            const u32* base = sm + r * NV * VS + pad_index(gg);
            u32 x[1][1 << RB];
#pragma unroll
            for (int k = 0; k < (1 << RB); ++k) x[0][k] = base[slot_offset<HS>(k)];
            dit_levels<A, RB, HS, 1>(x, pp.inv + gg, pp.p);
            const uint2* lo = il + r * NL;
            const uint2* hi = ih + r * NH;
            u32* out = ra + ((size_t)r << LOG_C);
#pragma unroll
            for (int k = 0; k < (1 << RB); ++k) {
                const int n2 = gg + k * HS;
                out[n2] = A::mulc(A::mulc(x[0][k], lo[n2 & (NL - 1)], pp.p), hi[n2 >> kRowTwLoBits], pp.p);
            }
        }
    }
}

// Column pass of the inverse four-step: column DIT, canonical residues in place.
template <class A, int LOG_R>
__global__ void NTT_COLS_BOUNDS k_inv_cols(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    using M = ColumnMap<LOG_R>;
    constexpr int B = M::SWEEPS < 8 ? M::SWEEPS : 8;
    static_assert(M::SWEEPS % B == 0 && (B * M::RS) % 32 == 0, "column batches");
    const int prime = blockIdx.y;
    const PrimeParams& pp = g.ps.pr[prime];
    const Member m = member_of(g, blockIdx.z, false);
    release_dependents();
    const u64 step = (u64)M::RS << g.log_c;
    u32* const base = m.spec + ((size_t)prime << g.log_t) + ((u64)M::row0() << g.log_c) +
                      (blockIdx.x << M::LOG_G) + M::col();
    u32* s = sm + M::slot0();
    uint2* tw = reinterpret_cast<uint2*>(sm + M::G * M::VS);
    load_table<LOG_R>(tw, pp.inv);
    wait_prior_grid();  // the row pass's output
    if (blockIdx.x == 0 && prime == 0) clear_flags(g, blockIdx.z);  // after every earlier kernel
    u32* q = base;
#pragma unroll 1
    for (int k0 = 0; k0 < M::SWEEPS; k0 += B) {
        u32 x[B];
#pragma unroll
        for (int u = 0; u < B; ++u) x[u] = __ldcs(q + u * step);
        q += B * step;
        u32* sk = s + slot_offset<M::RS>(k0);
#pragma unroll
        for (int u = 0; u < B; ++u) sk[slot_offset<M::RS>(u)] = x[u];
    }
    __syncthreads();
    // Every inverse pass but the last in shared memory (the short one first) ...
    constexpr int RB = kMaxRB;
    constexpr int R0 = LOG_R % RB;
    if constexpr (R0 > 0) {
        dit_pass<A, LOG_R, 0, R0, kThreads, M::G, M::VS>(sm, tw, pp.p);
        __syncthreads();
    }
    dit_range<A, LOG_R, kThreads, M::G, M::VS, R0, LOG_R - RB>(sm, tw, pp.p);
    // ... and the last one straight to global memory as canonical residues. Item it
    // takes column c = it mod G and block gg = it / G (rows gg + k * HS), so a warp
    // reads distinct banks and writes four rows of G consecutive residues at a time.
    {
        constexpr int LOG_HS = LOG_R - RB, HS = 1 << LOG_HS;
        u32* const out0 = m.spec + ((size_t)prime << g.log_t) + (blockIdx.x << M::LOG_G);
        const u64 kstep = (u64)HS << g.log_c;
#pragma unroll 1
        for (int it = threadIdx.x; it < (M::G << LOG_HS); it += kThreads) {
            const int c = it & (M::G - 1), gg = it >> M::LOG_G;
            const u32* base = sm + c * M::VS + pad_index(gg);
            u32 x[1][1 << RB];
#pragma unroll
            for (int k = 0; k < (1 << RB); ++k) x[0][k] = base[slot_offset<HS>(k)];
            dit_levels<A, RB, HS, 1>(x, tw + gg, pp.p);
            u32* out = out0 + ((u64)gg << g.log_c) + c;
#pragma unroll
            for (int k = 0; k < (1 << RB); ++k) out[k * kstep] = A::canonical(x[0][k], pp.p);
        }
    }
}

// ---------------------------------------------------------------------------------
// Four-step factor tables (layouts in launch.h). One thread per entry: the exponent
// of the entry, then the power as a product of the tabulated squares (Shoup
// products by constants), then its companion floor(x * 2^32 / p).

__device__ __forceinline__ u32 power_of(const uint2* pow2, u64 e, int bits, u32 p) {
    u32 x = 1;
    for (int i = 0; i < bits; ++i)
        if ((e >> i) & 1) x = sub_if_ge(shoup_mul(x, pow2[i].x, pow2[i].y, p), p);
    return x;
}

__global__ void __launch_bounds__(256) k_step_tables(const __grid_constant__ StepTableBuild b) {
    u64 n[4];
    step_table_sizes(b.log_t, b.log_r, n);
    const u64 mask = ((u64)1 << b.log_t) - 1;
    const int log_rs = step_log_u(b.log_r), log_sw = b.log_r - log_rs, log_nh = b.log_c - kRowTwLoBits;
    const u64 total = n[0] + n[1] + n[2] + n[3];
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x) {
        u64 k = i;
        u32 x;
        uint2* out;
        if (k < n[0]) {  // w^(col * u * SW)
            const u64 col = k >> log_rs, u = k & ((1u << log_rs) - 1);
            x = power_of(b.fwd_pow, ((col * u) << log_sw) & mask, b.log_t, b.p);
            out = b.f4_a + k;
        } else if ((k -= n[0]) < n[1]) {  // w^(col * j)
            const u64 col = k >> log_sw, j = k & (((u64)1 << log_sw) - 1);
            x = power_of(b.fwd_pow, (col * j) & mask, b.log_t, b.p);
            out = b.f4_b + k;
        } else if ((k -= n[1]) < n[2]) {  // w^(-k1 * lo)
            const u64 row = k >> kRowTwLoBits, lo = k & ((1u << kRowTwLoBits) - 1);
            const u64 k1 = __brev((u32)row) >> (32 - b.log_r);
            x = power_of(b.inv_pow, (k1 * lo) & mask, b.log_t, b.p);
            out = b.i4_lo + k;
        } else {  // w^(-k1 * 64 * hi) * scale
            k -= n[2];
            const u64 row = k >> log_nh, hi = k & (((u64)1 << log_nh) - 1);
            const u64 k1 = __brev((u32)row) >> (32 - b.log_r);
            x = power_of(b.inv_pow, ((k1 * hi) << kRowTwLoBits) & mask, b.log_t, b.p);
            x = sub_if_ge(shoup_mul(x, b.scale.x, b.scale.y, b.p), b.p);
            out = b.i4_hi + k;
        }
        *out = make_uint2(x, (u32)(((u64)x << 32) / b.p));
    }
}

cudaError_t launch_step_tables(const StepTableBuild& b, cudaStream_t st) {
    u64 n[4];
    step_table_sizes(b.log_t, b.log_r, n);
    const u64 total = n[0] + n[1] + n[2] + n[3];
    const unsigned blocks = (unsigned)std::min<u64>((total + 255) / 256, 152 * 16);
    k_step_tables<<<blocks, 256, 0, st>>>(b);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Launchers: one instantiation per transform size. The lazy arithmetic covers
// T <= 2^23 (one-CTA sizes 2^4..2^13, columns 2^6..2^11, rows 2^7..2^13); the wide
// arithmetic covers T = 2^24, 2^25 (columns 2^12, rows 2^12..2^13) and T = 2^22,
// 2^23 when the wide primes save one (columns 2^10, rows 2^12..2^13).

// Column residues plus the level root table (8-byte entries, 16-byte aligned); the
// forward pass adds its per-sweep four-step factors (G rows of SW + 1 entries).
static size_t col_smem(int log_r, bool fwd) {
    const int log_g = col_group_log(log_r);
    const size_t words = (size_t)col_vstride(log_r) * (1 << log_g);
    const size_t sweeps = (size_t)1 << (log_r - col_log_rs(log_r));
    return ((words * sizeof(u32) + 15) & ~(size_t)15) + ((size_t)8 << log_r) +
           (fwd ? 8 * ((size_t)1 << log_g) * (sweeps + 1) : 0);
}

// Row residues (one or two vectors per row) plus the rows' inverse four-step factors.
static size_t row_smem(int log_c, int mode) {
    const size_t rpc = (size_t)1 << row_log_rpc(log_c);
    return rpc * ((size_t)(mode == kRowMul ? 2 : 1) * padded_len(1 << log_c) * sizeof(u32) +
                  8 * (((size_t)1 << kRowTwLoBits) + ((size_t)1 << (log_c - kRowTwLoBits))));
}

// Preferred shared-memory carveout (percent of the unified L1/shared capacity) of
// the row and column passes; -1 leaves the driver's choice.
#ifndef NTT_ROWS_CARVEOUT
#define NTT_ROWS_CARVEOUT -1
#endif
#ifndef NTT_COLS_CARVEOUT
#define NTT_COLS_CARVEOUT -1
#endif

// Column data plus the f4_a rows of the two-pass forward kernel.
static size_t col2_smem(bool fwd) {
    const size_t words = (size_t)col_vstride(kCol2LogR) * 8;
    return ((words * sizeof(u32) + 15) & ~(size_t)15) + (fwd ? 8 * 8 * 33 : 0);
}

template <class A, int L>
static cudaError_t fwd_cols_at(const TransformArgs& g, bool square, bool sign, cudaStream_t st, bool init) {
    const unsigned ops = g.op_count ? g.op_count : (square ? 1 : 2);
    const unsigned zdim = g.batch ? (g.a_only ? 1 : 2) * g.count : ops;
    const dim3 grid((1u << (g.log_c - col_group_log(L))) * (unsigned)g.np, 1, zdim);
    // unsigned convolutions take the checking instantiation when they carry votes;
    // signed ones always do (a product is never signed)
    const bool check = g.batch ? g.admit != 0 : g.votes != nullptr;
    if constexpr (L == kCol2LogR) {
        auto k = sign ? k_fwd_cols2<A, true> : check ? k_fwd_cols2<A, false, true> : k_fwd_cols2<A, false>;
        if (init) {
            cudaError_t e = opt_in(k_fwd_cols2<A, false, true>, NTT_COLS_CARVEOUT);
            return e == cudaSuccess ? opt_in(k, NTT_COLS_CARVEOUT) : e;
        }
        k<<<grid, kThreads, col2_smem(true), st>>>(g);
    } else if constexpr (L == kCol4LogR) {
        auto k = sign ? k_fwd_cols4<A, true> : check ? k_fwd_cols4<A, false, true> : k_fwd_cols4<A, false>;
        if (init) {
            cudaError_t e = opt_in(k_fwd_cols4<A, false, true>, NTT_COLS_CARVEOUT);
            return e == cudaSuccess ? opt_in(k, NTT_COLS_CARVEOUT) : e;
        }
        k<<<dim3((1u << (g.log_c - kCol4LogG)) * (unsigned)g.np, 1, zdim), kCol4Threads, col4_smem(true), st>>>(g);
    } else {
        auto k = sign ? k_fwd_cols<A, true, L> : check ? k_fwd_cols<A, false, L, true> : k_fwd_cols<A, false, L>;
        if (init) {
            cudaError_t e = opt_in(k_fwd_cols<A, false, L, true>, NTT_COLS_CARVEOUT);
            return e == cudaSuccess ? opt_in(k, NTT_COLS_CARVEOUT) : e;
        }
        k<<<grid, kThreads, col_smem(L, true), st>>>(g);
    }
    return cudaGetLastError();
}

template <class A, int L>
static cudaError_t rows_at(const TransformArgs& g, int mode, cudaStream_t st, bool init) {
    auto k = mode == kRowMul ? k_rows<A, kRowMul, L>
             : mode == kRowSqr ? k_rows<A, kRowSqr, L>
             : mode == kRowFwd ? k_rows<A, kRowFwd, L>
                               : k_rows<A, kRowPre, L>;
    if (init) return opt_in(k, NTT_ROWS_CARVEOUT);
    const dim3 grid(1u << (g.log_r - row_log_rpc(L)), g.np, g.batch ? g.count : 1);
    const size_t smem = row_smem(L, mode);
    return launch_dependent(k, grid, dim3(row_threads(L)), smem, st, g);
}

template <class A, int L>
static cudaError_t inv_cols_at(const TransformArgs& g, cudaStream_t st, bool init) {
    const int log_g = L == kCol4LogR ? kCol4LogG : col_group_log(L);
    const dim3 grid(1u << (g.log_c - log_g), g.np, g.batch ? g.count : 1);
    if constexpr (L == kCol2LogR) {
        auto k = k_inv_cols2<A>;
        if (init) return opt_in(k, NTT_COLS_CARVEOUT);
        return launch_dependent(k, grid, dim3(kThreads), col2_smem(false), st, g);
    } else if constexpr (L == kCol4LogR) {
        if constexpr (NTT_INV_COLS4_PERSIST) {
            auto k = k_inv_cols4p<A>;
            if (init) return opt_in(k, NTT_COLS_CARVEOUT);
            const unsigned items = grid.x * grid.y * grid.z;
            return launch_dependent(k, dim3(std::min(items, (unsigned)sm_count())), dim3(kCol4Threads),
                                    col4p_smem(g.np), st, g);
        }
        auto k = k_inv_cols4<A>;
        if (init) return opt_in(k, NTT_COLS_CARVEOUT);
        return launch_dependent(k, grid, dim3(kCol4Threads), col4_smem(false), st, g);
    } else {
        auto k = k_inv_cols<A, L>;
        if (init) return opt_in(k, NTT_COLS_CARVEOUT);
        return launch_dependent(k, grid, dim3(kThreads), col_smem(L, false), st, g);
    }
}

static cudaError_t fwd_cols_any(const TransformArgs& g, bool square, bool sign, cudaStream_t st, bool init) {
    if (g.wide) {
        if (g.log_r == 12) return fwd_cols_at<WideArith, 12>(g, square, sign, st, init);
        if (g.log_r == 10) return fwd_cols_at<WideArith, 10>(g, square, sign, st, init);
        return cudaErrorInvalidValue;
    }
    switch (g.log_r) {
        case 6: return fwd_cols_at<LazyArith, 6>(g, square, sign, st, init);
        case 7: return fwd_cols_at<LazyArith, 7>(g, square, sign, st, init);
        case 8: return fwd_cols_at<LazyArith, 8>(g, square, sign, st, init);
        case 9: return fwd_cols_at<LazyArith, 9>(g, square, sign, st, init);
        case 10: return fwd_cols_at<LazyArith, 10>(g, square, sign, st, init);
        case 11: return fwd_cols_at<LazyArith, 11>(g, square, sign, st, init);
        default: return cudaErrorInvalidValue;
    }
}

static cudaError_t rows_any(const TransformArgs& g, int mode, cudaStream_t st, bool init) {
    if (g.wide) {
        if (g.log_c == 12) return rows_at<WideArith, 12>(g, mode, st, init);
        if (g.log_c == 13) return rows_at<WideArith, 13>(g, mode, st, init);
        return cudaErrorInvalidValue;
    }
    switch (g.log_c) {
        case 7: return rows_at<LazyArith, 7>(g, mode, st, init);
        case 8: return rows_at<LazyArith, 8>(g, mode, st, init);
        case 9: return rows_at<LazyArith, 9>(g, mode, st, init);
        case 10: return rows_at<LazyArith, 10>(g, mode, st, init);
        case 11: return rows_at<LazyArith, 11>(g, mode, st, init);
        case 12: return rows_at<LazyArith, 12>(g, mode, st, init);
        case 13: return rows_at<LazyArith, 13>(g, mode, st, init);
        default: return cudaErrorInvalidValue;
    }
}

static cudaError_t inv_cols_any(const TransformArgs& g, cudaStream_t st, bool init) {
    if (g.wide) {
        if (g.log_r == 12) return inv_cols_at<WideArith, 12>(g, st, init);
        if (g.log_r == 10) return inv_cols_at<WideArith, 10>(g, st, init);
        return cudaErrorInvalidValue;
    }
    switch (g.log_r) {
        case 6: return inv_cols_at<LazyArith, 6>(g, st, init);
        case 7: return inv_cols_at<LazyArith, 7>(g, st, init);
        case 8: return inv_cols_at<LazyArith, 8>(g, st, init);
        case 9: return inv_cols_at<LazyArith, 9>(g, st, init);
        case 10: return inv_cols_at<LazyArith, 10>(g, st, init);
        case 11: return inv_cols_at<LazyArith, 11>(g, st, init);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_fwd_cols(const TransformArgs& g, bool square, bool sign, cudaStream_t st) {
    return fwd_cols_any(g, square, sign, st, false);
}
cudaError_t launch_rows(const TransformArgs& g, int mode, cudaStream_t st) { return rows_any(g, mode, st, false); }
cudaError_t launch_inv_cols(const TransformArgs& g, cudaStream_t st) { return inv_cols_any(g, st, false); }

// Raises the dynamic shared-memory limit of every instantiation (both operand
// modes) on the current device.
cudaError_t init_transform_kernels() {
    cudaError_t e = init_small_kernels();
    TransformArgs g{};
    for (int sq = 0; sq < 2; ++sq)
        for (int sg = 0; sg < 2; ++sg) {
            for (int w = 0; w < 2; ++w) {
                g.wide = w;
                for (int l = 6; l <= 13 && e == cudaSuccess; ++l) {
                    g.log_r = l;
                    g.log_c = l;
                    const bool col_ok = w ? l == 12 || l == 10 : l <= 11;
                    const bool row_ok = w ? l >= 12 : l >= 7;
                    if (col_ok) e = fwd_cols_any(g, sq, sg, 0, true);
                    for (int mode = 0; mode < 4 && e == cudaSuccess && row_ok && sg == 0 && sq == 0; ++mode)
                        e = rows_any(g, mode, 0, true);
                    if (e == cudaSuccess && col_ok) e = inv_cols_any(g, 0, true);
                }
            }
        }
    return e;
}

}  // namespace ntt
