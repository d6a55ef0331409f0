// Transform-domain kernels: limb packing fused into the first forward pass, the
// pointwise product fused between the last forward and first inverse pass, and the
// inverse scale folded into the last twiddle multiply.
//
// Reference path (per prime): pack a and b (src/limb/packing.rs:113-292), forward
// transforms (src/transform/forward.rs:95-298), pointwise product (fused into the
// inverse leaves for long rows, src/multiply/schedule.rs:259-279), inverse with the
// N^-1 scale (src/transform/inverse.rs:52-218, src/multiply/schedule.rs:225-252).
//
// Two layouts:
//  * one CTA per prime holds the whole transform (T <= 2^13): k_small;
//  * four-step for T = R*C > 2^13: k_fwd_cols (pack + column DIF + twiddle),
//    k_rows (row DIF of a and b, pointwise, row DIT, inverse twiddle) and
//    k_inv_cols (column DIT + canonical residues). The spectrum order between the
//    passes is the four-step's transposed, bit-reversed order; only the inverse
//    reads it, so no transpose is ever materialised.
#include "launch.h"
#include "ntt_passes.cuh"

namespace ntt {

constexpr int kThreads = 256;

template <class A, bool SIGNED>
__device__ __forceinline__ u32 load_coefficient(const u64* __restrict__ src, u64 idx, u64 len,
                                                const PrimeParams& pp) {
    if (idx >= len) return 0;
    const u64 x = __ldg(src + idx);
    return SIGNED ? reduce_signed<A>(x, pp) : reduce_limb<A>(x, pp);
}

// One CTA transforms one prime: pack, forward a (and b), pointwise, inverse, scale.
template <class A, bool SQUARE, bool SIGNED>
__global__ void __launch_bounds__(kThreads) k_small(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    const PrimeParams& pp = g.ps.pr[blockIdx.x];
    const int n = 1 << g.log_t;
    const int vs = padded_len(n);
    u32* sa = sm;
    u32* sb = sm + vs;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        sa[pad_index(i)] = load_coefficient<A, SIGNED>(g.a, (u64)i, g.la, pp);
        if (!SQUARE) sb[pad_index(i)] = load_coefficient<A, SIGNED>(g.b, (u64)i, g.lb, pp);
    }
    __syncthreads();
    dif_full<A>(sm, g.log_t, SQUARE ? 1 : 2, vs, pp.fwd, pp.p);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int k = pad_index(i);
        const u32 x = sa[k];
        const u32 y = SQUARE ? x : sb[k];
        sa[k] = A::mulc(A::pointwise(x, y, pp.p, pp.pni), pp.scale, pp.p);
    }
    __syncthreads();
    dit_full<A>(sa, g.log_t, 1, vs, pp.inv, pp.p);
    u32* out = g.spec + ((size_t)blockIdx.x << g.log_t);
    for (int i = threadIdx.x; i < (int)g.conv_len; i += blockDim.x)
        out[i] = A::canonical(sa[pad_index(i)], pp.p);
}

// Column pass of the forward four-step: G columns of R points per CTA.
// grid = (C / G, np, operands). Coefficient n = n1*C + n2 sits at row n1, column n2.
template <class A, bool SIGNED>
__global__ void __launch_bounds__(kThreads) k_fwd_cols(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    const int prime = blockIdx.y;
    const int op = blockIdx.z;
    const PrimeParams& pp = g.ps.pr[prime];
    const u64* src = op ? g.b : g.a;
    const u64 len = op ? g.lb : g.la;
    const int G = 1 << g.log_g;
    const int col0 = blockIdx.x << g.log_g;
    const int count = 1 << (g.log_r + g.log_g);
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
        const int c = e & (G - 1);
        const int r = e >> g.log_g;
        const u64 idx = ((u64)r << g.log_c) + (u64)(col0 + c);
        sm[c * g.vstride_col + pad_index(r)] = load_coefficient<A, SIGNED>(src, idx, len, pp);
    }
    __syncthreads();
    dif_full<A>(sm, g.log_r, G, g.vstride_col, pp.fwd, pp.p);
    u32* dst = g.spec + ((size_t)(op * g.np + prime) << g.log_t);
    const u32 lo_mask = (1u << g.s_bits) - 1;
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
        const int c = e & (G - 1);
        const int j = e >> g.log_g;
        u32 x = sm[c * g.vstride_col + pad_index(j)];
        const u32 ex = (u32)(col0 + c) * (__brev((u32)j) >> (32 - g.log_r));
        x = A::mulc(x, __ldg(pp.f4_lo + (ex & lo_mask)), pp.p);
        x = A::mulc(x, __ldg(pp.f4_hi + (ex >> g.s_bits)), pp.p);
        dst[((size_t)j << g.log_c) + col0 + c] = x;
    }
}

// Row pass: forward rows of a (and b), pointwise product, inverse rows, inverse
// four-step twiddle with the 2^32 / T scale. grid = (R, np); writes over a's rows.
template <class A, bool SQUARE>
__global__ void __launch_bounds__(kThreads) k_rows(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    const int prime = blockIdx.y;
    const int row = blockIdx.x;
    const PrimeParams& pp = g.ps.pr[prime];
    const int C = 1 << g.log_c;
    const int vs = padded_len(C);
    uint4* ra = reinterpret_cast<uint4*>(g.spec + ((size_t)prime << g.log_t) + ((size_t)row << g.log_c));
    const uint4* rb = reinterpret_cast<const uint4*>(
        g.spec + ((size_t)(g.np + prime) << g.log_t) + ((size_t)row << g.log_c));
    u32* sa = sm;
    u32* sb = sm + vs;
    for (int q = threadIdx.x; q < (C >> 2); q += blockDim.x) {
        const int k = pad_index(q << 2);
        const uint4 v = ra[q];
        sa[k] = v.x; sa[k + 1] = v.y; sa[k + 2] = v.z; sa[k + 3] = v.w;
        if (!SQUARE) {
            const uint4 w = rb[q];
            sb[k] = w.x; sb[k + 1] = w.y; sb[k + 2] = w.z; sb[k + 3] = w.w;
        }
    }
    __syncthreads();
    dif_full<A>(sm, g.log_c, SQUARE ? 1 : 2, vs, pp.fwd, pp.p);
    for (int i = threadIdx.x; i < C; i += blockDim.x) {
        const int k = pad_index(i);
        const u32 x = sa[k];
        sa[k] = A::pointwise(x, SQUARE ? x : sb[k], pp.p, pp.pni);
    }
    __syncthreads();
    dit_full<A>(sa, g.log_c, 1, vs, pp.inv, pp.p);
    const u32 rowexp = __brev((u32)row) >> (32 - g.log_r);
    const u32 lo_mask = (1u << g.s_bits) - 1;
    for (int q = threadIdx.x; q < (C >> 2); q += blockDim.x) {
        const int k = pad_index(q << 2);
        u32 v[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const u32 ex = (u32)((q << 2) + t) * rowexp;
            u32 x = A::mulc(sa[k + t], __ldg(pp.i4_lo + (ex & lo_mask)), pp.p);
            v[t] = A::mulc(x, __ldg(pp.i4_hi + (ex >> g.s_bits)), pp.p);
        }
        ra[q] = make_uint4(v[0], v[1], v[2], v[3]);
    }
}

// Column pass of the inverse four-step: column DIT, canonical residues in place.
template <class A>
__global__ void __launch_bounds__(kThreads) k_inv_cols(const __grid_constant__ TransformArgs g) {
    extern __shared__ u32 sm[];
    const int prime = blockIdx.y;
    const PrimeParams& pp = g.ps.pr[prime];
    const int G = 1 << g.log_g;
    const int col0 = blockIdx.x << g.log_g;
    const int count = 1 << (g.log_r + g.log_g);
    u32* base = g.spec + ((size_t)prime << g.log_t);
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
        const int c = e & (G - 1);
        const int r = e >> g.log_g;
        sm[c * g.vstride_col + pad_index(r)] = base[((size_t)r << g.log_c) + col0 + c];
    }
    __syncthreads();
    dit_full<A>(sm, g.log_r, G, g.vstride_col, pp.inv, pp.p);
    for (int e = threadIdx.x; e < count; e += blockDim.x) {
        const int c = e & (G - 1);
        const int r = e >> g.log_g;
        base[((size_t)r << g.log_c) + col0 + c] = A::canonical(sm[c * g.vstride_col + pad_index(r)], pp.p);
    }
}

// ---------------------------------------------------------------------------------
// Launchers

static size_t small_smem(const TransformArgs& g, bool square) {
    return (size_t)(square ? 1 : 2) * padded_len(1 << g.log_t) * sizeof(u32);
}
static size_t col_smem(const TransformArgs& g) {
    return (size_t)g.vstride_col * (1u << g.log_g) * sizeof(u32);
}
static size_t row_smem(const TransformArgs& g, bool square) {
    return (size_t)(square ? 1 : 2) * padded_len(1 << g.log_c) * sizeof(u32);
}

template <class A>
static cudaError_t small_for(const TransformArgs& g, bool square, bool sign, cudaStream_t st) {
    const dim3 grid(g.np);
    const size_t sm = small_smem(g, square);
    if (square) {
        if (sign) k_small<A, true, true><<<grid, kThreads, sm, st>>>(g);
        else k_small<A, true, false><<<grid, kThreads, sm, st>>>(g);
    } else {
        if (sign) k_small<A, false, true><<<grid, kThreads, sm, st>>>(g);
        else k_small<A, false, false><<<grid, kThreads, sm, st>>>(g);
    }
    return cudaGetLastError();
}

cudaError_t launch_small(const TransformArgs& g, bool square, bool sign, cudaStream_t st) {
    return g.wide ? small_for<WideArith>(g, square, sign, st) : small_for<LazyArith>(g, square, sign, st);
}

template <class A>
static cudaError_t fwd_cols_for(const TransformArgs& g, bool square, bool sign, cudaStream_t st) {
    const dim3 grid(1u << (g.log_c - g.log_g), g.np, square ? 1 : 2);
    const size_t sm = col_smem(g);
    if (sign) k_fwd_cols<A, true><<<grid, kThreads, sm, st>>>(g);
    else k_fwd_cols<A, false><<<grid, kThreads, sm, st>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_fwd_cols(const TransformArgs& g, bool square, bool sign, cudaStream_t st) {
    return g.wide ? fwd_cols_for<WideArith>(g, square, sign, st)
                  : fwd_cols_for<LazyArith>(g, square, sign, st);
}

template <class A>
static cudaError_t rows_for(const TransformArgs& g, bool square, cudaStream_t st) {
    const dim3 grid(1u << g.log_r, g.np);
    const size_t sm = row_smem(g, square);
    if (square) k_rows<A, true><<<grid, kThreads, sm, st>>>(g);
    else k_rows<A, false><<<grid, kThreads, sm, st>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_rows(const TransformArgs& g, bool square, cudaStream_t st) {
    return g.wide ? rows_for<WideArith>(g, square, st) : rows_for<LazyArith>(g, square, st);
}

template <class A>
static cudaError_t inv_cols_for(const TransformArgs& g, cudaStream_t st) {
    const dim3 grid(1u << (g.log_c - g.log_g), g.np);
    k_inv_cols<A><<<grid, kThreads, col_smem(g), st>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_inv_cols(const TransformArgs& g, cudaStream_t st) {
    return g.wide ? inv_cols_for<WideArith>(g, st) : inv_cols_for<LazyArith>(g, st);
}

template <class K>
static cudaError_t opt_in(K kernel, int bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <class A>
static cudaError_t init_for() {
    const int big = 200 * 1024;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
    chk(opt_in(k_small<A, true, true>, big));
    chk(opt_in(k_small<A, true, false>, big));
    chk(opt_in(k_small<A, false, true>, big));
    chk(opt_in(k_small<A, false, false>, big));
    chk(opt_in(k_fwd_cols<A, true>, big));
    chk(opt_in(k_fwd_cols<A, false>, big));
    chk(opt_in(k_rows<A, true>, big));
    chk(opt_in(k_rows<A, false>, big));
    chk(opt_in(k_inv_cols<A>, big));
    return e;
}

cudaError_t init_transform_kernels() {
    cudaError_t e = init_for<LazyArith>();
    if (e != cudaSuccess) return e;
    return init_for<WideArith>();
}

}  // namespace ntt
