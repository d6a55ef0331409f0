// Batched modular arithmetic in the reference's 50-bit prime fields, on device
// arrays: the PrimeField / CrtPair API of ntt_anafis (src/field/prime_field.rs),
// one element per thread.
//
// Two exact products are built and measured (ntt_field_mul_method selects one):
//  - FP64, the reference's own method (prime_field.rs:232-247): the quotient
//    q = rint(RN(RN(a*b) * RN(1/p))) lies within 3/8 of a*b/p, so a*b - q*p,
//    evaluated with wrapping 64-bit arithmetic, lies in (-p, p) and one masked
//    addition makes it canonical;
//  - Barrett on 64-bit integers with mu = floor(2^113 / p): for a*b < p^2 < 2^100
//    the estimate floor((a*b >> 49) * mu / 2^64) is at most two below the true
//    quotient, so the remainder taken modulo 2^64 lies in [0, 3p) and two
//    conditional subtractions make it canonical.
// Products by a fixed factor use Shoup's quotient floor(w * 2^64 / p) as the
// reference does. Every result is the unique canonical residue, so the outputs
// equal the reference's bit for bit whichever method runs.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "launch.h"
#include "ntt_gb300.h"

namespace ntt {
namespace {

typedef unsigned __int128 u128;

// Reference constants: the catalog (src/field/catalog.rs:67-76), the admitted
// modulus range 2^49 < p < 2^50 (catalog.rs:19-21) and the Miller-Rabin bases
// (catalog.rs:25), which decide primality below 3.8 * 10^18.
constexpr u64 kCatalog[8] = {1108307720798209ull, 1086317488242689ull, 910395627798529ull, 659706976665601ull,
                             699289395265537ull,  1022545813831681ull, 1013749720809473ull, 868614185943041ull};
constexpr u64 kMinModulus = (u64)1 << 49, kMaxModulus = (u64)1 << 50;
constexpr u64 kWitnesses[9] = {2, 3, 5, 7, 11, 13, 17, 19, 23};

struct Field {
    u64 p;
    u64 mu;       // floor(2^113 / p)
    double pinv;  // RN(1 / p)
    int fp64;     // products by the FP64 quotient estimate instead of Barrett
};

// Product method of the batched field calls (1: FP64, 0: Barrett). Barrett is the
// default: on GB300 an array product runs at the HBM bound with it (266G products/s
// over 64M residues, 94% of the measured copy bandwidth) and at the FP64 bound with
// the reference's method (112G/s). Both are tested bit-exact.
int g_field_fp64 = 0;

u64 host_mulmod(u64 a, u64 b, u64 p) { return (u64)((u128)a * b % p); }

u64 host_powmod(u64 a, u64 e, u64 p) {
    u64 r = 1 % p;
    a %= p;
    while (e) {
        if (e & 1) r = host_mulmod(r, a, p);
        a = host_mulmod(a, a, p);
        e >>= 1;
    }
    return r;
}

// Strong-probable-prime test to the reference's bases (odd p above 2^49).
bool is_prime(u64 p) {
    for (u64 w : kWitnesses)
        if (p % w == 0) return false;
    const int shift = __builtin_ctzll(p - 1);
    const u64 odd = (p - 1) >> shift;
    for (u64 w : kWitnesses) {
        u64 x = host_powmod(w, odd, p);
        if (x == 1 || x == p - 1) continue;
        bool ok = false;
        for (int i = 1; i < shift && !ok; ++i) {
            x = host_mulmod(x, x, p);
            ok = x == p - 1;
        }
        if (!ok) return false;
    }
    return true;
}

bool admitted(u64 p) { return p > kMinModulus && p < kMaxModulus && is_prime(p); }

Field field_of(u64 p) { return Field{p, (u64)((((u128)1) << 113) / p), 1.0 / (double)p, g_field_fp64}; }

// Shoup's quotient floor(w * 2^64 / p) of a fixed factor.
u64 shoup64(u64 w, u64 p) { return (u64)((((u128)w) << 64) / p); }

bool fail(const char* what) {
    set_last_error(what);
    return false;
}

// ---------------------------------------------------------------------------------
// Device arithmetic

__device__ __forceinline__ u64 f_add(u64 a, u64 b, u64 p) {
    const u64 s = a + b;
    return min(s, s - p);
}

__device__ __forceinline__ u64 f_sub(u64 a, u64 b, u64 p) {
    const u64 d = a - b;
    return min(d, d + p);
}

// r in [0, 3p) -> [0, p)
__device__ __forceinline__ u64 f_fix3(u64 r, u64 p) {
    r = min(r, r - p);
    return min(r, r - p);
}

// Barrett remainder of lo + 2^64 hi < 2^113.
__device__ __forceinline__ u64 f_barrett(u64 lo, u64 hi, const Field& f) {
    const u64 x = (hi << 15) | (lo >> 49);
    const u64 q = __umul64hi(x, f.mu);
    return f_fix3(lo - q * f.p, f.p);
}

// a*b - q*p with q the nearest integer to RN(RN(a*b) * RN(1/p)): in (-p, p).
__device__ __forceinline__ u64 f_mul_fp64(u64 a, u64 b, const Field& f) {
    const double est = __dmul_rn(__dmul_rn((double)a, (double)b), f.pinv);
    const u64 q = (u64)__double2ll_rn(est);
    const int64_t r = (int64_t)(a * b - q * f.p);
    return (u64)(r + ((r >> 63) & (int64_t)f.p));
}

__device__ __forceinline__ u64 f_mul(u64 a, u64 b, const Field& f) {
    return f.fp64 ? f_mul_fp64(a, b, f) : f_barrett(a * b, __umul64hi(a, b), f);
}

__device__ __forceinline__ u64 f_mul_shoup(u64 a, u64 w, u64 wq, u64 p) {
    const u64 r = a * w - __umul64hi(a, wq) * p;  // [0, 2p) for every 64-bit a
    return min(r, r - p);
}

__device__ __forceinline__ u64 f_pow(u64 base, u64 e, const Field& f) {
    u64 r = 1, x = base;
    while (e) {
        if (e & 1) r = f_mul(r, x, f);
        e >>= 1;
        if (e) x = f_mul(x, x, f);
    }
    return r;
}

__device__ __forceinline__ u64 f_reduce_u64(u64 v, const Field& f) { return f_barrett(v, 0, f); }

__device__ __forceinline__ u64 f_reduce_i64(int64_t v, const Field& f) {
    const u64 mag = v < 0 ? 0 - (u64)v : (u64)v;
    const u64 r = f_reduce_u64(mag, f);
    return v < 0 && r ? f.p - r : r;
}

enum BinaryOp { kAdd = 0, kSub = 1, kMul = 2 };
enum UnaryOp { kNeg = 0, kPow = 1, kInv = 2, kSigned = 3, kReduceSigned = 4, kReduceUnsigned = 5 };

__global__ void k_field_binary(u64* __restrict__ out, const u64* __restrict__ a, const u64* __restrict__ b, u64 n,
                               int op, Field f) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u64 x = a[i], y = b[i];
        out[i] = op == kAdd ? f_add(x, y, f.p) : op == kSub ? f_sub(x, y, f.p) : f_mul(x, y, f);
    }
}

__global__ void k_field_unary(u64* __restrict__ out, const u64* __restrict__ a, u64 n, int op, u64 exponent,
                              uint8_t* __restrict__ mask, Field f) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u64 x = a[i];
        u64 y;
        switch (op) {
            case kNeg: y = f_sub(0, x, f.p); break;
            case kPow: y = f_pow(x, exponent, f); break;
            case kInv:  // Fermat: x^(p-2); zero has no inverse
                y = x ? f_pow(x, f.p - 2, f) : 0;
                if (mask) mask[i] = x ? 1 : 0;
                break;
            case kSigned: y = x > (f.p >> 1) ? x - f.p : x; break;
            case kReduceSigned: y = f_reduce_i64((int64_t)x, f); break;
            default: y = f_reduce_u64(x, f); break;
        }
        out[i] = y;
    }
}

// target[i] = w * target[i], or target[i] - w * source[i] with a source.
__global__ void k_field_scale(u64* __restrict__ target, const u64* __restrict__ source, u64 n, u64 w, u64 wq,
                              u64 p) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        if (source) target[i] = f_sub(target[i], f_mul_shoup(source[i], w, wq, p), p);
        else target[i] = f_mul_shoup(target[i], w, wq, p);
    }
}

// out[j] = sum_i coeffs[i] * points[j]^i by Horner's rule; the coefficients pass
// through shared memory in chunks read by every thread of the CTA.
__global__ void k_field_evaluate(u64* __restrict__ out, const u64* __restrict__ coeffs, u64 nc,
                                 const u64* __restrict__ points, u64 np, Field f) {
    constexpr int kChunk = 1024;
    __shared__ u64 chunk[kChunk];
    const u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    const u64 x = j < np ? points[j] : 0;
    u64 v = 0;
    // Horner from the top coefficient down, chunk by chunk.
    for (u64 end = nc; end > 0;) {
        const u64 begin = end > kChunk ? end - kChunk : 0;
        __syncthreads();
        for (u64 i = begin + threadIdx.x; i < end; i += blockDim.x) chunk[i - begin] = coeffs[i];
        __syncthreads();
        for (u64 i = end; i-- > begin;) v = f_add(f_mul(v, x, f), chunk[i - begin], f.p);
        end = begin;
    }
    if (j < np) out[j] = v;
}

// Garner: x = r1 + p1 * ((r2 - r1) * p1^-1 mod p2) in [0, p1 p2), then centred.
__global__ void k_crt_combine(u64* __restrict__ out, const u64* __restrict__ r1, const u64* __restrict__ r2, u64 n,
                              u64 p1, Field f2, u64 inv, u64 invq) {
    const u128 m = (u128)p1 * f2.p;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u64 a = r1[i];
        const u64 digit = f_mul_shoup(f_sub(r2[i], f_reduce_u64(a, f2), f2.p), inv, invq, f2.p);
        u128 v = (u128)a + (u128)p1 * digit;
        if (v > (m >> 1)) v -= m;  // two's complement of the negative value
        out[2 * i] = (u64)v;
        out[2 * i + 1] = (u64)(v >> 64);
    }
}

unsigned blocks_for(u64 n) {
    const u64 b = (n + 255) / 256;
    return (unsigned)(b < 152 * 32 ? (b ? b : 1) : 152 * 32);
}

uint8_t launched(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail((std::string(what) + ": " + cudaGetErrorString(e)).c_str());
    return 1;
}

}  // namespace
}  // namespace ntt

using namespace ntt;

extern "C" {

int ntt_field_check(uint64_t modulus) { return admitted(modulus) ? 1 : 0; }

int ntt_field_mul_method(int method) {
    const int previous = g_field_fp64;
    if (method == 0 || method == 1) g_field_fp64 = method;
    return previous;
}

uint64_t ntt_field_below(uint64_t bound) {
    const u64 top = bound < kMaxModulus ? bound : kMaxModulus;
    if (top < 3) return 0;
    for (u64 c = (top - 2) | 1; c > kMinModulus; c -= 2)
        if (is_prime(c)) return c;
    return 0;
}

size_t ntt_field_catalog(uint64_t* out, size_t capacity) {
    const size_t n = sizeof(kCatalog) / sizeof(kCatalog[0]);
    for (size_t i = 0; i < n && i < capacity && out; ++i) out[i] = kCatalog[i];
    return n;
}

uint8_t ntt_field_binary_device(uint64_t modulus, int op, uint64_t* d_out, const uint64_t* d_a,
                                const uint64_t* d_b, size_t n, void* stream) {
    if (!admitted(modulus)) return fail("modulus is not a prime in (2^49, 2^50)");
    if (op < kAdd || op > kMul) return fail("unknown field operation");
    if (n && (!d_out || !d_a || !d_b)) return fail("null array");
    if (!n) return 1;
    k_field_binary<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(d_out, d_a, d_b, n, op, field_of(modulus));
    return launched("field launch");
}

uint8_t ntt_field_unary_device(uint64_t modulus, int op, uint64_t* d_out, const uint64_t* d_a, size_t n,
                               uint64_t exponent, uint8_t* d_mask, void* stream) {
    if (!admitted(modulus)) return fail("modulus is not a prime in (2^49, 2^50)");
    if (op < kNeg || op > kReduceUnsigned) return fail("unknown field operation");
    if (n && (!d_out || !d_a)) return fail("null array");
    if (!n) return 1;
    k_field_unary<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(d_out, d_a, n, op, exponent, d_mask,
                                                                    field_of(modulus));
    return launched("field launch");
}

uint8_t ntt_field_scale_device(uint64_t modulus, uint64_t* d_target, const uint64_t* d_source, size_t n,
                               uint64_t factor, void* stream) {
    if (!admitted(modulus)) return fail("modulus is not a prime in (2^49, 2^50)");
    if (factor >= modulus) return fail("factor is not a residue");
    if (n && !d_target) return fail("null array");
    if (!n) return 1;
    k_field_scale<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(d_target, d_source, n, factor,
                                                                    shoup64(factor, modulus), modulus);
    return launched("field launch");
}

uint8_t ntt_field_evaluate_device(uint64_t modulus, uint64_t* d_out, const uint64_t* d_coeffs, size_t n_coeffs,
                                  const uint64_t* d_points, size_t n_points, void* stream) {
    if (!admitted(modulus)) return fail("modulus is not a prime in (2^49, 2^50)");
    if (n_points && (!d_out || !d_points || (n_coeffs && !d_coeffs))) return fail("null array");
    if (!n_points) return 1;
    const unsigned blocks = (unsigned)((n_points + 255) / 256);
    k_field_evaluate<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_out, d_coeffs, n_coeffs, d_points, n_points,
                                                                field_of(modulus));
    return launched("field launch");
}

uint8_t ntt_crt_pair_combine_device(uint64_t first, uint64_t second, int64_t* d_out, const uint64_t* d_first,
                                    const uint64_t* d_second, size_t n, void* stream) {
    if (!admitted(first) || !admitted(second)) return fail("modulus is not a prime in (2^49, 2^50)");
    if (first == second) return fail("the two fields coincide");
    if (n && (!d_out || !d_first || !d_second)) return fail("null array");
    if (!n) return 1;
    const u64 inv = host_powmod(first % second, second - 2, second);
    k_crt_combine<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>((u64*)d_out, d_first, d_second, n, first,
                                                                    field_of(second), inv, shoup64(inv, second));
    return launched("field launch");
}

}  // extern "C"
