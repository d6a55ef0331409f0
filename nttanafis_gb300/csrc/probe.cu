// Register-only arithmetic probes: the compute ceilings the transform kernels are
// measured against, and the per-butterfly cost of the candidate residue
// arithmetics. A measurement tool built into its own library (libntt_probe.so,
// include/ntt_probe.h); the product library does not contain it.
//
// Each butterfly probe keeps 16 residues and 8 twiddles per thread in registers and
// runs radix-16 forward passes (4 levels, 32 butterflies per pass) with no memory
// traffic, so its rate is bounded by instruction issue alone. Variants:
//   0  lazy 32-bit Shoup butterfly, p < 2^30 (LazyArith::dif, the transforms' own)
//   1  32-bit Montgomery butterfly by a constant (w and w * -p^-1 precomputed)
//   2  64-bit Shoup butterfly, p < 2^50 (the reference's prime size in integers)
//   3  the reference's f64 butterfly: exact remainder of the product by FMA
//      (src/arch/scalar/product.rs:95-109), residues in (-p, p) as doubles
// and instruction-throughput loops (8 independent chains per thread):
//   4  IMAD (32-bit multiply-add)   5  IMAD.HI (__umulhi)   6  IADD3-class adds
//   7  64-bit integer multiply (low word)   8  f64 FMA
//   9  IMAD.WIDE (32 x 32 -> 64-bit multiply-add)   10  I2F (u32 -> f32 conversion,
//      with one LOP3 each)
// and two more forms of variant 0's butterfly, whose Shoup quotient is the high
// word of a 32 x 32 -> 64-bit product: 11 PTX mul.wide, 12 a 64-bit product in C.
// The result is a checksum, so no work can be dropped, and the milliseconds of the
// timed launch (after one shorter warm-up launch).
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

#include "../../include/ntt_probe.h"
#include "ntt_arith.cuh"

namespace {

__device__ __forceinline__ void mont_dif(u32& x, u32& y, uint2 w, u32 p) {
    // w.x = w * 2^32 mod p, w.y = w.x * (-p^-1) mod 2^32: y' = (x - y + 2p) * w mod p
    const u32 p2 = p << 1;
    const u32 s = x + y;
    const u32 d = x - y + p2;
    x = min(s, s - p2);
    const u32 m = d * w.y;
    y = __umulhi(d, w.x) - __umulhi(m, p) + p;  // [0, 2p)
}

__device__ __forceinline__ void shoup64_dif(u64& x, u64& y, ulonglong2 w, u64 p) {
    const u64 p2 = p << 1;
    const u64 s = x + y;
    const u64 d = x - y + p2;
    x = s >= p2 ? s - p2 : s;
    const u64 q = __umul64hi(d, w.y);
    y = d * w.x - q * p;  // [0, 2p)
}

// The lazy Shoup butterfly with its quotient taken from the high word of a
// 32 x 32 -> 64-bit multiply (PTX mul.wide) instead of a multiply-high.
__device__ __forceinline__ void shoup_wide_dif(u32& x, u32& y, uint2 w, u32 p) {
    const u32 p2 = p << 1;
    const u32 s = x + y;
    const u32 d = x - y + p2;
    x = min(s, s - p2);
    u64 t;
    asm("mul.wide.u32 %0, %1, %2;" : "=l"(t) : "r"(d), "r"(w.y));
    const u32 q = (u32)(t >> 32);
    y = d * w.x - q * p;
}

// The same written as a 64-bit product in C, for the compiler's own choice.
__device__ __forceinline__ void shoup_c64_dif(u32& x, u32& y, uint2 w, u32 p) {
    const u32 p2 = p << 1;
    const u32 s = x + y;
    const u32 d = x - y + p2;
    x = min(s, s - p2);
    const u32 q = (u32)(((u64)d * w.y) >> 32);
    y = d * w.x - q * p;
}

// The reference's exact product: h + l = d * w exactly (FMA), quotient from h,
// remainder by FMA; residues stay in (-p, p).
__device__ __forceinline__ void f64_dif(double& x, double& y, double w, double p, double pinv) {
    const double s = x + y, d = x - y;
    x = s - p * rint(s * pinv);
    const double h = d * w;
    const double l = fma(d, w, -h);
    const double q = rint(h * pinv);
    y = fma(-q, p, h) + l;
}

template <int V>
__global__ void __launch_bounds__(256) k_probe(u64* __restrict__ out, u64 p, u64 w0, u64 wp0, int iters) {
    u64 acc = 0;
    if constexpr (V <= 3 || V >= 11) {
        // T: residue type of the variant
        using T = typename std::conditional<V == 2, u64, typename std::conditional<V == 3, double, u32>::type>::type;
        T x[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = (T)((threadIdx.x * 16 + i) % p);
        uint2 w32[8];
        ulonglong2 w64[8];
        double wf[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            w32[i] = make_uint2((u32)(w0 + i), (u32)(wp0 + i));
            w64[i] = make_ulonglong2(w0 + i, wp0 + i);
            wf[i] = (double)(w0 + i);
        }
        const double pf = (double)p, pinv = 1.0 / (double)p;
#pragma unroll 1
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int half = 8 >> t;
#pragma unroll
                for (int b = 0; b < 16; b += 2 * half)
#pragma unroll
                    for (int c = 0; c < half; ++c) {
                        if constexpr (V == 0) LazyArith::dif(x[b + c], x[b + c + half], w32[c], (u32)p);
                        if constexpr (V == 1) mont_dif(x[b + c], x[b + c + half], w32[c], (u32)p);
                        if constexpr (V == 2) shoup64_dif(x[b + c], x[b + c + half], w64[c], p);
                        if constexpr (V == 3) f64_dif(x[b + c], x[b + c + half], wf[c], pf, pinv);
                        if constexpr (V == 11) shoup_wide_dif(x[b + c], x[b + c + half], w32[c], (u32)p);
                        if constexpr (V == 12) shoup_c64_dif(x[b + c], x[b + c + half], w32[c], (u32)p);
                    }
            }
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) acc ^= (u64)x[i];
    } else {
        // eight independent chains of one instruction kind, 8 per chain per iteration
        u32 a[8];
        u64 b[8];
        double f[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            a[i] = threadIdx.x * 8 + i + 1;
            b[i] = ((u64)threadIdx.x << 32) + i + 3;
            f[i] = 1.0 + 1e-9 * (threadIdx.x * 8 + i);
        }
        const u32 m = (u32)w0 | 1u, c = (u32)wp0;
        const u64 m64 = w0 | 1ull;
        const double fm = 1.0 + 1e-12, fc = 1e-15;
#pragma unroll 1
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    // each one PTX instruction that the compiler may not fold
                    if constexpr (V == 4) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[i]) : "r"(m), "r"(c));
                    if constexpr (V == 5) asm volatile("mad.hi.u32 %0, %0, %1, %0;" : "+r"(a[i]) : "r"(m));
                    if constexpr (V == 6) asm volatile("add.u32 %0, %0, %1;" : "+r"(a[i]) : "r"(m));
                    if constexpr (V == 7) asm volatile("mul.lo.u64 %0, %0, %1;" : "+l"(b[i]) : "l"(m64));
                    if constexpr (V == 8) f[i] = fma(f[i], fm, fc);
                    if constexpr (V == 9) asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(b[i]) : "r"(a[i]), "r"(m));
                    if constexpr (V == 10) {
                        float t;
                        asm volatile("cvt.rn.f32.u32 %0, %1;" : "=f"(t) : "r"(a[i]));
                        a[i] ^= __float_as_uint(t);
                    }
                }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) acc ^= a[i] ^ b[i] ^ (u64)__double_as_longlong(f[i]);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

template <int V>
void launch(int blocks, u64* out, u64 p, u64 w0, u64 wp0, int iters) {
    k_probe<V><<<blocks, 256>>>(out, p, w0, wp0, iters);
}

using Launcher = void (*)(int, u64*, u64, u64, u64, int);
constexpr Launcher kLaunchers[] = {launch<0>, launch<1>, launch<2>,  launch<3>,  launch<4>,
                                   launch<5>, launch<6>, launch<7>,  launch<8>,  launch<9>,
                                   launch<10>, launch<11>, launch<12>};
constexpr int kVariants = sizeof(kLaunchers) / sizeof(kLaunchers[0]);

// Operations one thread performs per iteration of variant v.
double ops_per_iter(int v) { return v <= 3 || v >= 11 ? 32.0 : 64.0; }

}  // namespace

extern "C" {

int ntt_probe_variants(void) { return kVariants; }

uint8_t ntt_probe_arith(int variant, int blocks, int iters, float* ms, double* ops) {
    if (variant < 0 || variant >= kVariants || blocks <= 0 || iters <= 0 || !ms) return 0;
    // a 30-bit NTT prime for the 32-bit variants, a 50-bit one (the reference's
    // first catalog prime) for the 64-bit and f64 variants
    const u64 p = variant == 2 || variant == 3 ? 1108307720798209ull : 998244353ull;
    const u64 w0 = variant == 2 || variant == 3 ? 123456789012345ull : 12345u;
    const u64 wp0 = variant == 2 || variant == 3 ? 1234567ull : 678u;
    u64* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = cudaMalloc(&out, (size_t)blocks * 256 * sizeof(u64)) == cudaSuccess &&
              cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
    if (ok) {
        kLaunchers[variant](blocks, out, p, w0, wp0, iters / 8 + 1);
        cudaEventRecord(e0);
        kLaunchers[variant](blocks, out, p, w0, wp0, iters);
        cudaEventRecord(e1);
        ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(ms, e0, e1) == cudaSuccess;
    }
    if (ops) *ops = (double)blocks * 256 * iters * ops_per_iter(variant);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    return ok ? 1 : 0;
}

uint8_t ntt_probe_butterflies(int blocks, int iters, float* ms) {
    return ntt_probe_arith(0, blocks, iters, ms, nullptr);
}

}  // extern "C"
