// Device helpers shared by the transform kernels (small.cu, transform.cu): the
// operand reduction into a prime field, the launch member a CTA works on, the CRT
// flag clearing, the root-table copy into shared memory, and the host-side
// shared-memory opt-in.
#pragma once
#include "launch.h"
#include "ntt_passes.cuh"

namespace ntt {

constexpr int kThreads = kColThreads;
// Dynamic shared memory a transform kernel may request (of the 227 KB a CTA can
// hold on sm_103a).
constexpr int kSmemOptIn = 200 * 1024;

template <class A, bool SIGNED>
__device__ __forceinline__ u32 reduce_coefficient(u64 x, const PrimeParams& pp) {
    return SIGNED ? reduce_signed<A>(x, pp) : reduce_limb<A>(x, pp);
}

// A convolution coefficient above its bound (its magnitude when signed).
template <bool SIGNED>
__device__ __forceinline__ int coefficient_over(u64 x, u64 mx) {
    if (SIGNED) return ((int64_t)x < 0 ? (u64)0 - x : x) > mx;
    return x > mx;
}

// Operands of the launch member a CTA works on (TransformArgs::batch).
struct Member {
    const u64* a;
    const u64* b;
    u64 la, lb;
    u32* spec;
    u64 conv_len;
    bool square;
};

__device__ __forceinline__ Member member_of(const TransformArgs& g, int idx, bool square) {
    if (g.batch) {
        const ProductDesc& d = g.batch[idx];
        return Member{d.a, d.b, d.la, d.lb, d.spec, d.conv_len, d.square != 0};
    }
    return Member{g.a, g.b, g.la, g.lb, g.spec, g.conv_len, square};
}

// Admission votes of a convolution (src/convolve.rs:169-184) checked by the forward
// column passes as they load the coefficients: the votes and bound of operand op
// of a member, or null when the CTA checks nothing. Only prime 0's CTAs check, as
// every prime reads the same coefficients. The votes were zeroed before the pass; a
// thread that loads a coefficient above its bound sets one (the CRT kernel then
// leaves the destination unwritten).
__device__ __forceinline__ u32* column_votes(const TransformArgs& g, int member, int op, int prime, u64& mx) {
    mx = 0;
    if (prime != 0) return nullptr;
    if (g.batch) {
        if (!g.admit) return nullptr;
        const ProductDesc& d = g.batch[member];
        mx = op ? d.max_b : d.max_a;
        return d.votes;
    }
    mx = op ? g.max_b : g.max_a;
    return g.votes;
}

// Clears the CRT look-back flags of a member (products only; see k_crt_mul).
__device__ __forceinline__ void clear_flags(const TransformArgs& g, int idx) {
    u32* f = g.flags;
    u32 n = g.flag_words;
    if (g.batch) {
        const ProductDesc& d = g.batch[idx];
        f = reinterpret_cast<u32*>(d.agg);
        n = f ? (u32)carry_flag_words(d.out_len) : 0u;
    }
    for (u32 i = threadIdx.x; i < n; i += blockDim.x) f[i] = 0;
}

// Copies the level-major root table of a 2^LOG_N-point transform (entries below
// 2^LOG_N) into shared memory; the caller's barrier publishes it.
template <int LOG_N>
__device__ __forceinline__ void load_table(uint2* dst, const uint2* __restrict__ src) {
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    for (int i = threadIdx.x; i < (1 << LOG_N) / 2; i += kThreads) d4[i] = __ldg(s4 + i);
}

// Raises a kernel's dynamic shared-memory limit to the opt-in maximum (and sets its
// carveout preference when one is given).
template <class K>
static cudaError_t opt_in(K kernel, int carveout = -1) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemOptIn);
    if (e == cudaSuccess && carveout >= 0)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, carveout);
    return e;
}

}  // namespace ntt
