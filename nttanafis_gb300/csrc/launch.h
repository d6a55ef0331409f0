// Host-side launch interface between the planner/workspaces and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "ntt_arith.cuh"

namespace ntt {

// Largest transform held by one CTA, and the longest in-CTA vector of the
// four-step passes (C = 2^13 u32 rows, R = 2^12 u32 columns).
constexpr int kMaxBlockLog = 13;
// Largest transform length handled at all (coefficients of a product or convolution).
constexpr int kMaxLogT = 25;
// Output limbs per CTA of the CRT + carry kernel (four per thread).
#ifndef NTT_CRT_TILE
#define NTT_CRT_TILE 1024
#endif
constexpr int kCrtTile = NTT_CRT_TILE;

// Column passes of the four-step: a CTA of kColThreads threads owns G = 2^log_g
// columns of R = 2^log_r points; thread t takes column t mod G and rows r0 + k * RS
// with r0 = t / G, RS = 256 / G rows per sweep, k < SW = R / RS. G is 2^kColLogG
// for R >= 2^9 (a row segment of G residues is one 32-byte sector) and
// 2^(12 - log_r) below, so that the first pass, which holds 16 points of one
// column per thread, still has a register block for every thread.
#ifndef NTT_COLS_LOG_G
#define NTT_COLS_LOG_G 3
#endif
constexpr int kColThreads = 256;
constexpr int kColLogG = NTT_COLS_LOG_G;
__host__ __device__ constexpr int col_group_log(int log_r) {
    return log_r + kColLogG >= 12 ? kColLogG : 12 - log_r;
}
__host__ __device__ constexpr int col_log_rs(int log_r) { return 8 - col_group_log(log_r); }
// Columns of 2^12 points (the wide lengths T = 2^24, 2^25) run as two radix-64
// passes (k_fwd_cols4, k_inv_cols4 in transform.cu), 64 points per thread and pass.
constexpr int kCol4LogR = 12;
// log2 of the f4_a entries per column: the first factor of the forward four-step
// twiddle of row r is indexed by the top log_u bits of brev(r), the second (f4_b)
// by the rest.
__host__ __device__ constexpr int step_log_u(int log_r) { return log_r == kCol4LogR ? 6 : col_log_rs(log_r); }
// Four-step twiddles, tabulated per prime and transform length T = R * C:
//  - forward, applied by the column pass: w_T^(col * brev(row)). Row r0 + RS*k has
//    the bit-reversed index brev(r0) * SW + brev(k), so the twiddle is
//    f4_a[col * RS + brev(r0)] = w_T^(col * brev(r0) * SW) (one per thread) times
//    f4_b[col * SW + brev(k)] = w_T^(col * brev(k)) (one per sweep);
//  - inverse, applied by the row pass: w_T^(-k1 * n2) times the inverse scale for
//    the row of frequency k1 = brev(row) and n2 = 64 * hi + lo, as
//    i4_lo[row * 64 + lo] = w_T^(-k1 * lo) times
//    i4_hi[row * C / 64 + hi] = w_T^(-k1 * 64 * hi) * scale.
constexpr int kRowTwLoBits = 6;

// One product or convolution of a batch, read by the kernels from device memory.
// All members of one launch share the transform length, the primes and the sign
// mode; everything else varies per member.
struct ProductDesc {
    const u64* a;
    const u64* b;      // == a for a square
    u64 la, lb;
    u32* spec;         // this member's residues ([2][np][T] u32)
    u64 conv_len;
    u64* dst;
    u64 out_len;       // limbs of a product
    uint8_t* agg;      // CRT look-back flags of a product (carry_flag_words u32), or null
    u32 square;
    u32 stride;        // convolution limbs per coefficient
    u64 max_a, max_b;  // convolution coefficient bounds (magnitudes when signed)
    u32* votes;        // admission votes of a convolution (kAdmitSlots u32), or null
};

// Operands and geometry of one transform-domain product. With `batch` set, the
// kernels run `count` members: the member index is the launch's last grid
// dimension and the member fields override a, b, la, lb, spec and conv_len.
struct TransformArgs {
    const ProductDesc* batch;
    int count;
    const u64* a;
    const u64* b;
    u64 la, lb;
    u32* spec;         // [2][np][T] residues; region 0 ends as the product residues
    u64 conv_len;      // coefficients of the product/convolution
    int np;            // primes
    int log_t;         // log2 transform length
    int log_r, log_c;  // four-step split T = R * C (unused on the one-CTA path)
    int wide;          // 1: primes up to 2^31 in canonical arithmetic; 0: lazy, p < 2^30
    int op_base;       // first operand of a single-member column pass (0: a, 1: b)
    int op_count;      // operands of that pass; 0 means every operand of the member
    u32* flags;        // CRT look-back flags to clear (products), or null
    u32 flag_words;
    u64* dst;          // product limbs of the fused one-kernel path (single member)
    u64 out_len;
    // Coefficient admission of a convolution by the transform that loads the
    // coefficients (prime 0's CTAs check them: the one-CTA transform writes every
    // vote, the forward column pass raises votes zeroed before it): votes (null: no
    // check) and bounds; batch members take theirs from the descriptors.
    u32* votes;
    u64 max_a, max_b;
    int admit;         // batch: check the members' coefficients (their votes)
    // A spectrum shared by the members (the shorter operand of a block-split
    // product): [np][T] u32, written by the row pass in kRowFwd mode, read in
    // kRowPre; a_only: the members' column passes transform operand a alone.
    u32* shared_spec;
    int a_only;
    PrimeSet ps;
};

// Transform modes of the row pass (k_rows) and the one-CTA transform (k_small).
enum RowMode : int {
    kRowMul = 0,  // a and b: forward both, pointwise a * b, inverse
    kRowSqr = 1,  // a alone: forward, pointwise a * a, inverse
    kRowFwd = 2,  // a alone: forward; its reduced spectrum written to shared_spec
    kRowPre = 3,  // a alone: forward, pointwise by the spectrum in shared_spec, inverse
};

// Exact-CRT constants of one prime set (words in radix 2^32). The transforms fold
// each prime's (P/p_i)^-1 into their inverse scale, so the residues the CRT reads
// are already y_i = r_i * (P/p_i)^-1 mod p_i.
constexpr int kQpStride = kMaxPrimes + 2;  // odd row stride: conflict-free rows
struct CrtParams {
    int np;
    int l64;                           // u64 words of one reconstructed coefficient
    int stride;                        // output limbs per coefficient (convolutions)
    float bias;                        // 0.25 unsigned, 0.5 signed quotient rounding
    u32 p[kMaxPrimes];
    float pinv[kMaxPrimes];            // 1/p_i in fp32
    u32 M[kMaxPrimes][kMaxPrimes];     // P/p_i
    u32 P[kMaxPrimes];                 // P
    u32 qP[kMaxPrimes + 1][kQpStride]; // q * P for q = 0..np (np + 1 words each)
};

// q * P of a prime set for q = 0..np into cp.qP (host side).
inline void fill_multiples(CrtParams& cp) {
    for (int q = 0; q <= cp.np; ++q) {
        u64 carry = 0;
        for (int w = 0; w <= cp.np; ++w) {
            const u64 t = (u64)q * (w < cp.np ? cp.P[w] : 0u) + carry;
            cp.qP[q][w] = (u32)t;
            carry = t >> 32;
        }
    }
}

// Launchers; each returns the launch status.
cudaError_t launch_small(const TransformArgs& g, int mode, bool sign, cudaStream_t st);
// Whole products of T <= 2^kFusedMaxLog points with kFusedPrimes primes in one
// kernel: a cluster of one CTA per prime transforms, then reconstructs and carries
// the product from the cluster's shared memory. Returns cudaErrorNotSupported for
// other shapes (the caller then takes launch_small and the CRT kernel).
constexpr int kFusedMaxLog = 13, kFusedPrimes = 5;
cudaError_t launch_small_fused(const TransformArgs& g, const CrtParams& cp, bool square, cudaStream_t st);
cudaError_t launch_fwd_cols(const TransformArgs& g, bool square, bool sign, cudaStream_t st);
cudaError_t launch_rows(const TransformArgs& g, int mode, cudaStream_t st);
cudaError_t launch_inv_cols(const TransformArgs& g, cudaStream_t st);

// Failure status of the calls of a workspace or batch: four bytes in page-locked
// host memory that the kernels reach through its device address (null: none). A
// kernel that fails sets its byte to 1; the host reads the bytes after the call's
// stream completes. Byte 0: a carry look-back wait gave up; byte 1: a convolution
// coefficient exceeded its bound (the result was not written).
constexpr u32 kStatusLookback = 1, kStatusBound = 2;
__device__ __forceinline__ void report_status(u32* status, int byte) {
    if (status) {
        reinterpret_cast<volatile uint8_t*>(status)[byte] = 1;
        __threadfence_system();
    }
}

// Device-side coefficient admission of a convolution (src/convolve.rs:169-184):
// kAdmitSlots CTAs scan the operands and each writes one vote (1: some coefficient
// it saw exceeds its bound, 0: none), so every vote is rewritten by every check and
// nothing needs clearing. The kernels that write the result skip the write when any
// vote is 1.
constexpr int kAdmitSlots = 128;
constexpr u64 kAdmitBytes = 4 * kAdmitSlots;

cudaError_t launch_crt_mul(const u32* resid, int log_t, u64 conv_len, u64 out_len, u64* dst,
                           uint8_t* agg, const CrtParams& cp, cudaStream_t st,
                           void (*mark)(cudaStream_t) = nullptr, u32* status = nullptr);
cudaError_t launch_crt_conv(const u32* resid, int log_t, u64 conv_len, u64* dst, bool sign,
                            const CrtParams& cp, cudaStream_t st, const u32* votes = nullptr,
                            u32* status = nullptr);
// Batched forms: every member of `batch` (device array of `count` descriptors)
// shares log_t and the prime set of `cp`. Convolution members with votes are
// written only when admitted.
cudaError_t launch_crt_mul_batch(const ProductDesc* batch, int count, int max_tiles, int log_t,
                                 const CrtParams& cp, cudaStream_t st, u32* status = nullptr);
cudaError_t launch_crt_conv_batch(const ProductDesc* batch, int count, u64 max_conv_len, int log_t,
                                  const CrtParams& cp, cudaStream_t st, u32* status = nullptr);
// Admission votes of one schoolbook convolution (votes: kAdmitSlots u32, every one
// written), and the zeroing of a batch class's member votes before a forward column
// pass that raises them.
cudaError_t launch_conv_admit(const u64* a, u64 la, const u64* b, u64 lb, u64 max_a, u64 max_b, bool sign,
                              u32* votes, cudaStream_t st);
cudaError_t launch_clear_votes_batch(const ProductDesc* batch, int count, cudaStream_t st);
// dst[0, len) += add[0, len) with carries (flags: carry_flag_words(len), zeroed).
cudaError_t launch_add_limbs(u64* dst, const u64* add, u64 len, u32* flags, cudaStream_t st,
                             u32* status = nullptr);
// Member descriptors of blocks first .. first + count - 1 of a split product
// (block m of a times b into dst or odd at limb m * block; member m's residues and
// flags at arena + (m - first) * member_bytes, flags spec_bytes in).
cudaError_t launch_split_descs(ProductDesc* d, u64 first, u64 count, const u64* a, u64 la, const u64* b, u64 lb,
                               u64 block, u64* dst, u64* odd, uint8_t* arena, u64 member_bytes, u64 spec_bytes,
                               cudaStream_t st);
// Short products by direct column sums in one thread-block cluster (school.cu): for
// products of at most kSchoolMaxOut limbs (one CRT tile); needs no scratch.
constexpr int kSchoolSmemMax = 200 * 1024;
// Default basecase threshold in limb products (a_len * b_len), from per-call timings
// on GB300: the basecase wins up to 96 x 96 (6.2 against 8.2 us), ties at 128 x 128
// (8.2 us each) and loses from 192 x 192 on (256 x 256: 10.3 against 8.2 us).
constexpr u64 kSchoolDefaultProducts = 12288;
constexpr u64 kSchoolMaxOut = kCrtTile;
bool school_fits(u64 la, u64 lb);
// Dynamic shared memory of the basecase with a cluster of cl CTAs.
size_t school_smem_cl(u64 la, u64 lb, int cl);
cudaError_t launch_school_mul(const u64* a, u64 la, const u64* b, u64 lb, u64* dst, cudaStream_t st);
cudaError_t init_school_kernels();
cudaError_t launch_conv_schoolbook(const u64* a, u64 la, const u64* b, u64 lb, u64* dst,
                                   int stride, bool sign, cudaStream_t st, const u32* votes = nullptr,
                                   u32* status = nullptr);
// Four-step factor tables of one prime and transform length, built on the GPU:
// every entry is a power of w (forward) or w^-1 (inverse) with its Shoup companion,
// computed from the squares w^(2^i) (with companions) given here.
struct StepTableBuild {
    u32 p;
    int log_t, log_r, log_c;
    uint2 fwd_pow[kMaxLogT + 1];  // w^(2^i), i <= log_t
    uint2 inv_pow[kMaxLogT + 1];  // w^(-2^i)
    uint2 scale;                  // inverse scale folded into i4_hi
    uint2 *f4_a, *f4_b, *i4_lo, *i4_hi;
};
// Entries of the four tables (in the order f4_a, f4_b, i4_lo, i4_hi) of the split
// T = 2^log_t = R * C, R = 2^log_r.
__host__ __device__ inline void step_table_sizes(int log_t, int log_r, u64 sizes[4]) {
    const int log_c = log_t - log_r;
    const u64 R = (u64)1 << log_r, C = (u64)1 << log_c;
    sizes[0] = C << step_log_u(log_r);             // f4_a: [col][u]
    sizes[1] = C * (R >> step_log_u(log_r));       // f4_b: [col][j]
    sizes[2] = R << kRowTwLoBits;                  // i4_lo: [row][lo]
    sizes[3] = R * (C >> kRowTwLoBits);            // i4_hi: [row][hi]
}
cudaError_t launch_step_tables(const StepTableBuild& b, cudaStream_t st);

// Scratch bytes of the CRT look-back flags for `out_len` output limbs: a tile
// counter, an error word and one state word per tile of kCrtTile limbs.
__host__ __device__ inline u64 carry_flag_words(u64 out_len) { return 2 + (out_len + kCrtTile - 1) / kCrtTile; }
inline u64 carry_scratch_bytes(u64 out_len) { return 4 * carry_flag_words(out_len); }
// Look-back waits that gave up since load (0 unless the GPU misbehaved).
u32 lookback_timeouts();

// Sets the message returned by ntt_last_error() on this thread.
void set_last_error(const std::string& message);

// Programmatic dependent launch between the kernels of the four-step sequence:
// the row pass, the inverse column pass and the CRT kernel are launched so that
// they may be scheduled while the kernel before them drains; each waits
// (wait_prior_grid) for that kernel's completion and memory before it reads its
// output, and each producer lets its dependent launch (release_dependents) once
// all of its own CTAs are running. The first kernel of a product launches
// normally, so it never overlaps the previous product. Both device calls are
// no-ops for a kernel launched without the attribute.
#ifndef NTT_PDL
#define NTT_PDL 1
#endif
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void release_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

template <class... KArgs, class... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                    Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = NTT_PDL;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// One-time kernel attribute setup (shared-memory opt-in) for the current device.
cudaError_t init_small_kernels();      // small.cu (called by init_transform_kernels)
cudaError_t init_transform_kernels();
cudaError_t init_crt_kernels();

}  // namespace ntt
