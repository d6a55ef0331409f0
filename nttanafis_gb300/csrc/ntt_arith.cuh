// Modular arithmetic over 32-bit NTT primes, shared by every kernel.
//
// The reference multiplies in eight 50-bit prime fields held as integer-valued
// f64 (src/field/catalog.rs:67-76, src/arch/scalar/product.rs:99-109). GB300's
// FP64 rate is a small fraction of its 32-bit integer rate, so this library keeps
// every residue in a u32 and reduces with Shoup's precomputed-quotient product
// (one IMAD.HI, one IMUL, one IMAD) and Montgomery's product where neither factor
// is a constant. The integer product is unique, so the choice of primes does not
// change any output limb.
//
// Two residue domains exist, chosen per transform length by the planner:
//   Lazy  (p < 2^30): Harvey's lazy butterflies. Forward values lie in [0, 2p),
//                     inverse values in [0, 4p); 4p < 2^32 keeps every sum in a u32.
//   Wide  (p < 2^31): canonical values in [0, p). Used where no prime below 2^30
//                     has the two-power roots of the transform (T >= 2^24), and
//                     at T = 2^22, 2^23 where five of them hold what six
//                     lazy primes would.
#pragma once
#include <stdint.h>

typedef uint32_t u32;
typedef uint64_t u64;

// Returns x*w mod p in [0, 2p) for any x < 2^32, with wp = floor(w * 2^32 / p).
__device__ __forceinline__ u32 shoup_mul(u32 x, u32 w, u32 wp, u32 p) {
    const u32 q = __umulhi(x, wp);
    return x * w - q * p;
}

// Returns x - m when x >= m, else x; valid when x < 2m and 2m <= 2^32.
__device__ __forceinline__ u32 sub_if_ge(u32 x, u32 m) { return min(x, x - m); }

// Montgomery product a*b*2^-32 mod p for a*b < 2^62 and p < 2^31; result in [0, 2p).
__device__ __forceinline__ u32 mont_mul(u32 a, u32 b, u32 p, u32 pneg_inv) {
    const u64 t = (u64)a * b;
    const u32 m = (u32)t * pneg_inv;
    const u64 u = t + (u64)m * p;
    return (u32)(u >> 32);
}

struct LazyArith {
    static constexpr bool kWide = false;
    // Forward (Gentleman-Sande) butterfly: x, y in [0, 2p) -> [0, 2p).
    static __device__ __forceinline__ void dif(u32& x, u32& y, uint2 w, u32 p) {
        const u32 p2 = p << 1;
        const u32 s = x + y;
        const u32 d = x - y + p2;
        x = sub_if_ge(s, p2);
        y = shoup_mul(d, w.x, w.y, p);
    }
    // Inverse (Cooley-Tukey) butterfly: x, y in [0, 4p) -> [0, 4p).
    static __device__ __forceinline__ void dit(u32& x, u32& y, uint2 w, u32 p) {
        const u32 p2 = p << 1;
        const u32 a = sub_if_ge(x, p2);
        const u32 t = shoup_mul(y, w.x, w.y, p);
        x = a + t;
        y = a - t + p2;
    }
    // Product by a constant with Shoup companion; any x < 2^32 -> [0, 2p).
    static __device__ __forceinline__ u32 mulc(u32 x, uint2 w, u32 p) {
        return shoup_mul(x, w.x, w.y, p);
    }
    // Forward butterfly with twiddle 1: x, y in [0, 2p) -> [0, 2p), no product.
    static __device__ __forceinline__ void dif_unit(u32& x, u32& y, u32 p) {
        const u32 p2 = p << 1;
        const u32 s = x + y;
        const u32 d = x - y + p2;
        x = sub_if_ge(s, p2);
        y = sub_if_ge(d, p2);
    }
    // Last forward level (twiddle 1) left open for a following product: x, y in
    // [0, 2p) -> [0, 4p), without the reductions.
    static __device__ __forceinline__ void dif_open(u32& x, u32& y, u32 p) {
        const u32 s = x + y;
        y = x - y + (p << 1);
        x = s;
    }
    // First inverse level (twiddle 1): x, y in [0, 4p) -> [0, 4p), no product.
    static __device__ __forceinline__ void dit_unit(u32& x, u32& y, u32 p) {
        const u32 p2 = p << 1;
        const u32 a = sub_if_ge(x, p2), t = sub_if_ge(y, p2);
        x = a + t;
        y = a - t + p2;
    }
    // The same for x, y already in [0, 2p) (the residues the row pass writes).
    static __device__ __forceinline__ void dit_unit_2p(u32& x, u32& y, u32 p) {
        const u32 s = x + y;
        y = x - y + (p << 1);
        x = s;
    }
    // Pointwise product of two forward-domain values -> inverse domain, times 2^-32.
    static __device__ __forceinline__ u32 pointwise(u32 a, u32 b, u32 p, u32 pni) {
        return mont_mul(a, b, p, pni);
    }
    // Inverse-domain value -> canonical [0, p).
    static __device__ __forceinline__ u32 canonical(u32 x, u32 p) {
        return sub_if_ge(sub_if_ge(x, p << 1), p);
    }
    // Sum of two values in [0, 2p) -> forward domain [0, 2p).
    static __device__ __forceinline__ u32 add_fwd(u32 a, u32 b, u32 p) {
        return sub_if_ge(a + b, p << 1);
    }
    // [0, 2p) -> forward domain (identity here).
    static __device__ __forceinline__ u32 fwd_from_2p(u32 x, u32 p) { return x; }
};

struct WideArith {
    static constexpr bool kWide = true;
    // x, y in [0, p) -> [0, p).
    static __device__ __forceinline__ void dif(u32& x, u32& y, uint2 w, u32 p) {
        const u32 s = x + y;
        const u32 d = x - y + p;
        x = sub_if_ge(s, p);
        y = sub_if_ge(shoup_mul(d, w.x, w.y, p), p);
    }
    static __device__ __forceinline__ void dit(u32& x, u32& y, uint2 w, u32 p) {
        const u32 t = sub_if_ge(shoup_mul(y, w.x, w.y, p), p);
        const u32 s = x + t;
        const u32 d = x - t + p;
        x = sub_if_ge(s, p);
        y = sub_if_ge(d, p);
    }
    static __device__ __forceinline__ u32 mulc(u32 x, uint2 w, u32 p) {
        return sub_if_ge(shoup_mul(x, w.x, w.y, p), p);
    }
    // x, y in [0, p) -> [0, 2p), without the reductions.
    static __device__ __forceinline__ void dif_open(u32& x, u32& y, u32 p) {
        const u32 s = x + y;
        y = x - y + p;
        x = s;
    }
    // Twiddle-1 butterfly on canonical values (forward and inverse alike).
    static __device__ __forceinline__ void dit_unit(u32& x, u32& y, u32 p) {
        const u32 s = x + y, d = x - y + p;
        x = sub_if_ge(s, p);
        y = sub_if_ge(d, p);
    }
    static __device__ __forceinline__ void dif_unit(u32& x, u32& y, u32 p) { dit_unit(x, y, p); }
    static __device__ __forceinline__ void dit_unit_2p(u32& x, u32& y, u32 p) { dit_unit(x, y, p); }
    static __device__ __forceinline__ u32 pointwise(u32 a, u32 b, u32 p, u32 pni) {
        return sub_if_ge(mont_mul(a, b, p, pni), p);
    }
    static __device__ __forceinline__ u32 canonical(u32 x, u32 p) { return x; }
    static __device__ __forceinline__ u32 add_fwd(u32 a, u32 b, u32 p) {
        // a, b in [0, 2p) with 2p < 2^32: reduce each first so the sum fits.
        return sub_if_ge(sub_if_ge(a, p) + sub_if_ge(b, p), p);
    }
    static __device__ __forceinline__ u32 fwd_from_2p(u32 x, u32 p) { return sub_if_ge(x, p); }
};

// Per-prime constants handed to every kernel.
struct PrimeParams {
    u32 p;
    u32 pni;         // -p^-1 mod 2^32 (Montgomery)
    u32 inv2_32;     // floor(2^32 / p): Shoup companion of w = 1
    u32 neg64;       // 2^64 mod p, subtracted for negative two's complement limbs
    uint2 r32;       // 2^32 mod p with its Shoup companion
    uint2 scale;     // small-path inverse scale T^-1 * (P/p)^-1 * 2^32 with companion
    const uint2* fwd;    // level-major forward roots: fwd[h + j] = w_{2h}^j
    const uint2* inv;    // level-major inverse roots: inv[h + j] = w_{2h}^-j
    const uint2* f4_a;   // forward four-step twiddles: per column-pass thread
    const uint2* f4_b;   //                              per column and sweep
    const uint2* i4_lo;  // inverse four-step twiddles: per row, low digit of n2
    const uint2* i4_hi;  //                             per row, high digit, times the scale
    // Entries 1..31 of the level-major roots (fwd[h + j], inv[h + j] for h < 32), held
    // in the kernel parameters: register blocks of consecutive points read these
    // uniform twiddles from the constant cache instead of memory.
    uint2 small_fwd[32];
    uint2 small_inv[32];
};

constexpr int kMaxPrimes = 8;

struct PrimeSet {
    PrimeParams pr[kMaxPrimes];
};

// Reduces a 64-bit limb into the forward domain of its arithmetic.
template <class A>
__device__ __forceinline__ u32 reduce_limb(u64 x, const PrimeParams& pp) {
    const u32 lo = (u32)x, hi = (u32)(x >> 32);
    const u32 h = shoup_mul(hi, pp.r32.x, pp.r32.y, pp.p);   // [0, 2p)
    const u32 l = lo - __umulhi(lo, pp.inv2_32) * pp.p;      // [0, 2p)
    return A::add_fwd(h, l, pp.p);
}

// Reduces a two's complement 64-bit coefficient into the forward domain.
template <class A>
__device__ __forceinline__ u32 reduce_signed(u64 x, const PrimeParams& pp) {
    u32 r = reduce_limb<A>(x, pp);
    if ((int64_t)x < 0) {
        // value = x - 2^64: subtract 2^64 mod p, i.e. add p - neg64 in (0, p].
        r = A::add_fwd(A::fwd_from_2p(r, pp.p), pp.p - pp.neg64, pp.p);
    }
    return r;
}
