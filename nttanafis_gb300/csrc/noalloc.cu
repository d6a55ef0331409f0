// Exact products of short operands for callers that cannot allocate device memory.
//
// Some callers of this library are not allowed to call cudaMalloc: code that runs
// under a device-memory budget owned by another allocator (a serving loop that has
// already partitioned the GPU's memory among requests, a host framework that
// reserves all device memory up front), and latency-critical paths where the
// implicit device-wide synchronisation of cudaMalloc/cudaFree would stall work on
// other streams. ntt_mul_noalloc_device gives them the short-product path with no
// allocation at all: its scratch (the residues of both operands and the carry
// flags) and its root tables live in the file-scope device arrays below, which
// every GPU that loads the library holds until the process exits
// (NTT_NOALLOC_SCRATCH_BYTES + NTT_NOALLOC_TABLE_BYTES, about 480 KiB).
//
// Limits and rules of use:
//  * a_len + b_len - 1 <= NTT_NOALLOC_MAX_COEFFICIENTS (4096), so the product fits
//    one 4096-point transform held by one CTA per prime; larger shapes are
//    rejected with a message in ntt_last_error();
//  * the first call on a device does a one-time set-up with that device current:
//    it looks up the arrays' device addresses (cudaGetSymbolAddress) and copies
//    the root tables into them. Make that first call before any stream capture;
//  * all calls share the one scratch array, so calls that overlap on the GPU
//    (different streams, or different host threads without ordering) race and
//    corrupt each other's results. Serialise them on one stream;
//  * nothing in the scratch needs to start at zero: every call writes each
//    scratch word before it reads it, so the contents left by the previous call
//    do not matter.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <string>

#include "../../include/ntt_gb300.h"
#include "launch.h"
#include "ntt_passes.cuh"

namespace ntt {

namespace {

constexpr int kNaLogT = 12;
constexpr int kNaPoints = 1 << kNaLogT;
constexpr int kNaPrimes = 5;
// The five largest catalog primes below 2^30 whose 2-adic valuation reaches 2^21;
// their product holds every coefficient of a product whose shorter operand has at
// most 2^20 limbs, so it holds every product this path admits.
constexpr u32 kNaPrime[kNaPrimes] = {1012924417u, 1004535809u, 998244353u, 985661441u, 975175681u};
constexpr size_t kNaSpecWords = (size_t)2 * kNaPrimes * kNaPoints;
constexpr size_t kNaFlagWords = 64;  // CRT look-back flags: 2 + at most 5 output tiles
constexpr size_t kNaRootEntries = (size_t)2 * kNaPrimes * kNaPoints;

}  // namespace

// Residues of a and b ([operand][prime][4096] u32), then the carry flags.
static __device__ __align__(256) u32 g_noalloc_scratch[kNaSpecWords + kNaFlagWords];
// Level-major roots per prime: forward[4096] then inverse[4096], Shoup companions.
static __device__ __align__(256) uint2 g_noalloc_roots[kNaRootEntries];

namespace {

struct NoAllocDevice {
    std::atomic<bool> ready{false};  // set (release) once scratch and roots are valid
    u32* scratch = nullptr;
    uint2* roots = nullptr;
};

std::mutex g_na_mutex;
NoAllocDevice g_na_device[64];
PrimeParams g_na_params[kNaPrimes];  // pointers filled per device at call time
uint2 g_na_scale[kNaPrimes][kNaLogT + 1];
CrtParams g_na_crt;
bool g_na_constants = false;
uint2 g_na_host_roots[kNaRootEntries];  // staging for the one-time table copy


u32 na_mulmod(u32 a, u32 b, u32 p) { return (u32)((u64)a * b % p); }
u32 na_pow(u32 a, u64 e, u32 p) {
    u32 r = 1;
    a %= p;
    while (e) {
        if (e & 1) r = na_mulmod(r, a, p);
        a = na_mulmod(a, a, p);
        e >>= 1;
    }
    return r;
}
uint2 na_shoup(u32 w, u32 p) { return make_uint2(w, (u32)(((u64)w << 32) / p)); }

u32 na_generator(u32 p) {
    u32 m = p - 1, factors[16];
    int nf = 0;
    for (u32 q = 2; (u64)q * q <= m; ++q)
        if (m % q == 0) {
            factors[nf++] = q;
            while (m % q == 0) m /= q;
        }
    if (m > 1) factors[nf++] = m;
    for (u32 g = 2; g < p; ++g) {
        bool ok = true;
        for (int i = 0; i < nf && ok; ++i) ok = na_pow(g, (p - 1) / factors[i], p) != 1;
        if (ok) return g;
    }
    return 0;
}

// Host constants shared by every device: Shoup scales, CRT words, root tables.
void na_build_constants() {
    if (g_na_constants) return;
    // P and the cofactors M_i = P / p_i in radix 2^32.
    u32 P[kMaxPrimes + 1] = {1};
    int pw = 1;
    for (int i = 0; i < kNaPrimes; ++i) {
        u64 c = 0;
        for (int w = 0; w < pw; ++w) {
            const u64 t = (u64)P[w] * kNaPrime[i] + c;
            P[w] = (u32)t;
            c = t >> 32;
        }
        if (c) P[pw++] = (u32)c;
    }
    int bits = (pw - 1) * 32 + 32 - __builtin_clz(P[pw - 1]);
    g_na_crt = CrtParams{};
    g_na_crt.np = kNaPrimes;
    g_na_crt.l64 = (bits - 2 + 63) / 64;
    g_na_crt.stride = 1;
    g_na_crt.bias = 0.25f;
    for (int w = 0; w < pw && w < kMaxPrimes; ++w) g_na_crt.P[w] = P[w];
    for (int i = 0; i < kNaPrimes; ++i) {
        const u32 p = kNaPrime[i];
        u32 M[kMaxPrimes + 1] = {1};
        int mw = 1;
        for (int j = 0; j < kNaPrimes; ++j) {
            if (j == i) continue;
            u64 c = 0;
            for (int w = 0; w < mw; ++w) {
                const u64 t = (u64)M[w] * kNaPrime[j] + c;
                M[w] = (u32)t;
                c = t >> 32;
            }
            if (c) M[mw++] = (u32)c;
        }
        u64 mmod = 0;
        for (int w = mw - 1; w >= 0; --w) mmod = ((mmod << 32) | M[w]) % p;
        for (int w = 0; w < mw && w < kMaxPrimes; ++w) g_na_crt.M[i][w] = M[w];
        g_na_crt.p[i] = p;
        g_na_crt.pinv[i] = 1.0f / (float)p;
        const u32 cofactor = na_pow((u32)mmod, p - 2, p);  // (P/p_i)^-1, folded into the scale

        PrimeParams& pp = g_na_params[i];
        pp = PrimeParams{};
        pp.p = p;
        u32 pinv = 1;
        for (int k = 0; k < 5; ++k) pinv *= 2u - p * pinv;
        pp.pni = 0u - pinv;
        pp.inv2_32 = (u32)(((u64)1 << 32) / p);
        const u32 r32 = (u32)(((u64)1 << 32) % p);
        pp.neg64 = na_mulmod(r32, r32, p);
        pp.r32 = na_shoup(r32, p);
        for (int lt = 0; lt <= kNaLogT; ++lt) {
            const u32 tinv = na_pow((u32)(((u64)1 << lt) % p), p - 2, p);
            g_na_scale[i][lt] = na_shoup(na_mulmod(na_mulmod(tinv, r32, p), cofactor, p), p);
        }
        const u32 g = na_generator(p);
        uint2* fwd = g_na_host_roots + (size_t)(2 * i) * kNaPoints;
        uint2* inv = fwd + kNaPoints;
        fwd[0] = inv[0] = na_shoup(1, p);
        for (int h = 1; h < kNaPoints; h <<= 1) {
            const u32 root = na_pow(g, (p - 1) / (2 * (u64)h), p);
            const u32 iroot = na_pow(root, p - 2, p);
            u32 w = 1, iw = 1;
            for (int j = 0; j < h; ++j) {
                fwd[h + j] = na_shoup(w, p);
                inv[h + j] = na_shoup(iw, p);
                w = na_mulmod(w, root, p);
                iw = na_mulmod(iw, iroot, p);
            }
        }
    }
    fill_multiples(g_na_crt);
    g_na_constants = true;
}

bool na_fail(const char* msg) {
    set_last_error(msg);
    return false;
}

// One-time set-up of the current device: device addresses of the static arrays
// and the root tables copied into them. After it, a call only reads the ready flag
// (no lock).
bool na_setup(int dev, NoAllocDevice*& out) {
    if (dev < 0 || dev >= 64) return na_fail("device index out of range");
    NoAllocDevice& d = g_na_device[dev];
    if (d.ready.load(std::memory_order_acquire)) {
        out = &d;
        return true;
    }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!d.ready.load(std::memory_order_relaxed)) {
        na_build_constants();
        void* scratch = nullptr;
        void* roots = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_last_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
            return false;
        }
        e = cudaGetSymbolAddress(&roots, g_noalloc_roots);
        if (e != cudaSuccess) {
            set_last_error(std::string("cudaGetSymbolAddress(roots): ") + cudaGetErrorString(e));
            return false;
        }
        e = cudaMemcpy(roots, g_na_host_roots, sizeof(g_na_host_roots), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_last_error(std::string("root table copy: ") + cudaGetErrorString(e));
            return false;
        }
        d.scratch = (u32*)scratch;
        d.roots = (uint2*)roots;
        d.ready.store(true, std::memory_order_release);
    }
    out = &d;
    return true;
}

}  // namespace

}  // namespace ntt

using namespace ntt;

extern "C" uint8_t ntt_mul_noalloc_device(uint64_t* d_dst, size_t dst_len, const uint64_t* d_a, size_t a_len,
                                          const uint64_t* d_b, size_t b_len, void* stream) {
    set_last_error("");
    cudaStream_t st = (cudaStream_t)stream;
    const u64 out_len = (u64)a_len + b_len;
    if (dst_len < out_len) return na_fail("destination is shorter than the product");
    if (a_len == 0 || b_len == 0)
        return cudaMemsetAsync(d_dst, 0, out_len * sizeof(u64), st) == cudaSuccess ? 1
                                                                                   : na_fail("zero product");
    if (out_len - 1 > (u64)NTT_NOALLOC_MAX_COEFFICIENTS)
        return na_fail("product exceeds the 4096 coefficients of the no-allocation path (a_len + b_len - 1)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return na_fail("no current CUDA device");
    NoAllocDevice* d = nullptr;
    if (!na_setup(dev, d)) return 0;
    const u64 conv_len = out_len - 1;
    int log_t = 4;
    while (((u64)1 << log_t) < conv_len) ++log_t;
    const bool square = d_a == d_b && a_len == b_len;
    TransformArgs ta{};
    ta.a = d_a;
    ta.b = square ? d_a : d_b;
    ta.la = a_len;
    ta.lb = square ? a_len : b_len;
    ta.spec = d->scratch;
    ta.conv_len = conv_len;
    ta.np = kNaPrimes;
    ta.log_t = log_t;
    ta.wide = 0;
    ta.flags = d->scratch + kNaSpecWords;  // cleared by the transform kernel of this call
    ta.flag_words = (u32)carry_flag_words(out_len);
    for (int i = 0; i < kNaPrimes; ++i) {
        PrimeParams pp = g_na_params[i];
        pp.scale = g_na_scale[i][log_t];
        pp.fwd = d->roots + (size_t)(2 * i) * kNaPoints;
        pp.inv = pp.fwd + kNaPoints;
        ta.ps.pr[i] = pp;
    }
    cudaError_t e = launch_small(ta, square ? kRowSqr : kRowMul, false, st);
    if (e == cudaSuccess)
        e = launch_crt_mul(d->scratch, log_t, conv_len, out_len, d_dst, (uint8_t*)(d->scratch + kNaSpecWords),
                           g_na_crt, st);
    if (e != cudaSuccess) {
        set_last_error(std::string("launch: ") + cudaGetErrorString(e));
        return 0;
    }
    return 1;
}

