// Planning and device tables of the GB300 multiplication path: the prime catalog,
// the plan geometry of products and convolutions, the root tables and four-step
// factor tables per device, and the kernel constants of a plan.
//
// Planning mirrors the reference's admission rules (src/plan.rs:53-69,
// src/convolve.rs:75-116, src/profile/planner.rs:120-322) with this library's own
// geometry: every 64-bit limb is one transform coefficient, the transform length
// is the power of two that holds the convolution, and the fewest 32-bit primes
// whose product holds every coefficient are taken from a catalog of primes with
// the needed two-power roots.
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "host.h"

namespace ntt {

// ---------------------------------------------------------------------------------
// Prime catalog

// Primes below 2^30 with 2-adic valuation of p-1 at least 21 (lazy arithmetic).
static const u32 kLazyPrimes[] = {
    1012924417u, 1004535809u, 998244353u, 985661441u, 975175681u, 962592769u, 950009857u,
    943718401u,  935329793u,  924844033u, 918552577u, 899678209u, 897581057u, 880803841u,
    824180737u,  799014913u,  786432001u, 754974721u, 740294657u, 715128833u, 710934529u,
    683671553u,  666894337u,  648019969u, 645922817u, 639631361u, 635437057u, 597688321u,
    595591169u,  576716801u,  469762049u, 463470593u, 459276289u, 415236097u, 387973121u,
    383778817u,  377487361u,
};
// Primes below 2^31 with valuation at least 24 (canonical arithmetic): T >= 2^24,
// and T = 2^22, 2^23 where they save a prime (choose_primes).
static const u32 kWidePrimes[] = {
    2130706433u, 2113929217u, 2013265921u, 1811939329u, 1711276033u,
    1224736769u, 1107296257u, 754974721u,  469762049u,  167772161u,
};

constexpr int kLazyMaxLog = 23;

static u32 mulmod(u32 a, u32 b, u32 p) { return (u32)((u64)a * b % p); }
static u32 powmod(u32 a, u64 e, u32 p) {
    u32 r = 1 % p;
    a %= p;
    while (e) {
        if (e & 1) r = mulmod(r, a, p);
        a = mulmod(a, a, p);
        e >>= 1;
    }
    return r;
}
static u32 invmod(u32 a, u32 p) { return powmod(a, p - 2, p); }
static int valuation(u32 p) { return __builtin_ctz(p - 1); }

static u32 generator(u32 p) {
    u32 m = p - 1;
    std::vector<u32> factors;
    for (u32 q = 2; (u64)q * q <= m; ++q) {
        if (m % q == 0) {
            factors.push_back(q);
            while (m % q == 0) m /= q;
        }
    }
    if (m > 1) factors.push_back(m);
    for (u32 g = 2; g < p; ++g) {
        bool ok = true;
        for (u32 q : factors)
            if (powmod(g, (p - 1) / q, p) == 1) { ok = false; break; }
        if (ok) return g;
    }
    return 0;
}

static std::vector<u32> primes_for(int log_t, bool wide) {
    std::vector<u32> out;
    if (!wide) {
        for (u32 p : kLazyPrimes) if (valuation(p) >= log_t) out.push_back(p);
    } else {
        for (u32 p : kWidePrimes) if (valuation(p) >= log_t) out.push_back(p);
    }
    std::sort(out.begin(), out.end(), [](u32 x, u32 y) { return x > y; });
    if (out.size() > (size_t)kMaxPrimes) out.resize(kMaxPrimes);
    return out;
}

// Multiword helpers in radix 2^32, least significant first.
typedef std::vector<u32> Words;
static Words words_mul_small(const Words& a, u32 m) {
    Words r(a.size() + 1, 0);
    u64 c = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        const u64 t = (u64)a[i] * m + c;
        r[i] = (u32)t;
        c = t >> 32;
    }
    r[a.size()] = (u32)c;
    while (r.size() > 1 && r.back() == 0) r.pop_back();
    return r;
}
static int words_bitlen(const Words& a) {
    for (int i = (int)a.size() - 1; i >= 0; --i)
        if (a[i]) return i * 32 + 32 - __builtin_clz(a[i]);
    return 0;
}
static u32 words_mod(const Words& a, u32 p) {
    u64 r = 0;
    for (int i = (int)a.size() - 1; i >= 0; --i) r = ((r << 32) | a[i]) % p;
    return (u32)r;
}

// Coefficient capacity of the first np primes: X < 2^cap satisfies X <= P/2.
static int capacity(const std::vector<u32>& primes, int np) {
    Words P{1};
    for (int i = 0; i < np; ++i) P = words_mul_small(P, primes[i]);
    return words_bitlen(P) - 2;
}

static int ceil_log2(u64 x) { return x <= 1 ? 0 : 64 - __builtin_clzll(x - 1); }

// ---------------------------------------------------------------------------------
// Plans


// Fewest primes of one class whose capacity holds need_bits (0: none does).
static int fewest_primes(const std::vector<u32>& cand, int need_bits, int& cap) {
    for (int np = 1; np <= (int)cand.size(); ++np) {
        cap = capacity(cand, np);
        if (cap >= need_bits) return np;
    }
    return 0;
}

// Lengths up to 2^23 take the lazy primes (p < 2^30), longer ones the wide primes
// (p < 2^31, canonical arithmetic). At 2^22 and 2^23 the wide primes are taken as
// well when they hold the coefficients with one prime fewer: five lazy primes hold
// 148 and 147 bits there, five wide ones 153, so a product whose shorter operand
// has more than 2^20 (2^19) limbs needs six lazy primes but five wide ones. The
// wide butterfly costs the same per point (one more ALU subtraction, off the
// multiplier pipe), so a prime fewer is a sixth less work. Those lengths run the
// two-pass 2^10-point column kernels and the 2^12- and 2^13-point rows.
constexpr int kWideFromLog = 22;

static bool choose_primes(Geom& g, int need_bits) {
    const bool lazy_ok = g.log_t <= kLazyMaxLog;
    const bool wide_ok = g.log_t >= kWideFromLog;
    std::vector<u32> cand;
    int cap = 0, np = 0;
    bool wide = false;
    if (lazy_ok) {
        cand = primes_for(g.log_t, false);
        np = fewest_primes(cand, need_bits, cap);
    }
    if (wide_ok) {
        int wcap = 0;
        const std::vector<u32> wcand = primes_for(g.log_t, true);
        const int wnp = fewest_primes(wcand, need_bits, wcap);
        if (wnp && (!np || wnp < np)) {
            cand = wcand;
            np = wnp;
            cap = wcap;
            wide = true;
        }
    }
    if (!np) return false;
    g.np = np;
    g.cap = cap;
    for (int i = 0; i < np; ++i) g.primes[i] = cand[i];
    g.wide = wide ? 1 : 0;
    return true;
}

// Longest operand of a split product (limbs).
constexpr u64 kMaxSplitLimbs = (u64)1 << 40;

// Block split of an unbalanced product (the reference's Geometry::cheapest_blocks,
// src/profile/planner.rs:291-393, restated for this library's transforms): the
// longer operand (L limbs) in blocks of B = 2^k - S + 1 limbs, each multiplied by
// the shorter one (S limbs) with 2^k-point transforms. The shorter operand's
// spectrum is computed once and shared by every block (the reference's shared
// short-operand spectrum, src/multiply/execute.rs:114-130). Cost in butterfly
// levels: two transforms per block and one for the shorter operand,
// (2n + 1) * 2^k * k, plus a fixed kSplitOverhead for the block sums, the final
// addition and about ten more launches and copies, against 3 * 2^K * K for one
// transform of the whole product. Returns the chosen k, or 0 when one transform is
// within the margin. Measured on GB300 (per call, split against one transform):
// 1,048,576 x 1,024 99 against 160 us, 4,194,304 x 524,288 477 against 797 us,
// 1,048,576 x 131,072 149 against 165 us; below, the fixed part dominates
// (20,000 x 300: 41 against 24 us; 16,384 x 4,096: 51 against 24 us).
#ifndef NTT_SPLIT_MARGIN
#define NTT_SPLIT_MARGIN 0.8
#endif
constexpr double kSplitOverhead = 16777216.0;  // butterfly levels, about 25 us on GB300
static int split_log(u64 L, u64 S, int full_log) {
    const double full = full_log <= kMaxLogT ? 3.0 * std::ldexp(1.0, full_log) * full_log : 1e300;
    int best_k = 0;
    double best = NTT_SPLIT_MARGIN * full;
    const int lo = std::max(kSmallSplitLog, ceil_log2(2 * S));
    for (int k = lo; k <= kMaxLogT && k < full_log; ++k) {
        const u64 B = ((u64)1 << k) - S + 1;
        const double n = (double)((L + B - 1) / B);
        const double cost = (2.0 * n + 1.0) * std::ldexp(1.0, k) * k + kSplitOverhead;
        if (cost < best) {
            best = cost;
            best_k = k;
        }
    }
    return best_k;
}

// allow_split: callers that run one product per call (workspaces, plans) may take
// the block split; batch members always use one transform.
static bool plan_mul_new(u64 la, u64 lb, Geom& g, bool allow_split) {
    if (!la || !lb) return fail("operand length is zero");
    const u64 L = std::max(la, lb), S = std::min(la, lb);
    const int full_log = std::max(4, ceil_log2(la + lb - 1));
    int k = allow_split && L <= kMaxSplitLimbs ? split_log(L, S, full_log) : 0;
    if (!k && full_log > kMaxLogT)
        return fail(allow_split ? "product exceeds 2^25 transform coefficients and admits no block split"
                                : "product exceeds 2^25 transform coefficients");
    g = Geom();
    g.la = la;
    g.lb = lb;
    g.conv_len = la + lb - 1;
    g.out_len = la + lb;
    g.log_t = k ? k : full_log;
    if (k) {
        g.block = ((u64)1 << k) - S + 1;
        g.blocks = (L + g.block - 1) / g.block;
    }
    const int need = 128 + ceil_log2(S);
    if (!choose_primes(g, need)) return fail("no prime set holds the coefficients");
    return true;
}

static int bitlen128(u128 x) {
    const u64 hi = (u64)(x >> 64), lo = (u64)x;
    if (hi) return 128 - __builtin_clzll(hi);
    if (lo) return 64 - __builtin_clzll(lo);
    return 0;
}

// Bit length of terms*max_a*max_b (src/convolve.rs:358-369).
static int bound_bits(u64 terms, u64 max_a, u64 max_b) {
    const u128 product = (u128)max_a * max_b;
    const u128 bound = product * terms;
    const bool overflow = terms != 0 && bound / terms != product;
    if (!overflow) return bitlen128(bound);
    return bitlen128(product) + (terms > 1 ? 64 - __builtin_clzll(terms - 1) : 0);
}

static bool plan_conv_new(u64 la, u64 lb, u64 max_a, u64 max_b, int sign, Geom& g) {
    if (!la || !lb) return fail("operand length is zero");
    g = Geom();
    g.conv = true;
    g.la = la;
    g.lb = lb;
    g.max_a = max_a;
    g.max_b = max_b;
    g.sign = sign ? 1 : 0;
    const u64 shorter = std::min(la, lb);
    auto value_bits = [&](u64 m) { return (m ? 64 - __builtin_clzll(m) : 0) + g.sign; };
    if (value_bits(max_a) > 64 || value_bits(max_b) > 64)
        return fail("signed coefficient bound must lie below 2^63");
    g.bound_bits = bound_bits(shorter, max_a, max_b) + g.sign;
    g.stride = std::max<u64>(1, ((u64)g.bound_bits + 63) / 64);
    if (la > ((u64)1 << 40) || lb > ((u64)1 << 40)) return fail("convolution length out of range");
    g.conv_len = la + lb - 1;
    g.out_len = g.conv_len * g.stride;
    g.schoolbook = shorter <= 24;
    if (!g.schoolbook) {
        if (g.conv_len > ((u64)1 << kMaxLogT)) return fail("convolution exceeds 2^25 transform coefficients");
        g.log_t = std::max(4, ceil_log2(g.conv_len));
        if (!choose_primes(g, std::max(1, g.bound_bits))) return fail("no prime set holds the coefficients");
    }
    return true;
}

// Plans are pure functions of their arguments and batches repeat shapes, so each
// thread keeps the admitted plans it made (failures are recomputed, to set their
// message again). The caches are dropped whole when they grow past kPlanCache.
constexpr size_t kPlanCache = 1 << 13;

bool plan_mul(u64 la, u64 lb, Geom& g, bool allow_split) {
    thread_local std::map<std::tuple<u64, u64, bool>, Geom> cache;
    const auto key = std::make_tuple(la, lb, allow_split);
    auto it = cache.find(key);
    if (it != cache.end()) {
        g = it->second;
        return true;
    }
    if (!plan_mul_new(la, lb, g, allow_split)) return false;
    if (cache.size() >= kPlanCache) cache.clear();
    cache.emplace(key, g);
    return true;
}

bool plan_conv(u64 la, u64 lb, u64 max_a, u64 max_b, int sign, Geom& g) {
    thread_local std::map<std::tuple<u64, u64, u64, u64, int>, Geom> cache;
    const auto key = std::make_tuple(la, lb, max_a, max_b, sign);
    auto it = cache.find(key);
    if (it != cache.end()) {
        g = it->second;
        return true;
    }
    if (!plan_conv_new(la, lb, max_a, max_b, sign, g)) return false;
    if (cache.size() >= kPlanCache) cache.clear();
    cache.emplace(key, g);
    return true;
}

// ---------------------------------------------------------------------------------
// Device root tables (immutable once built; shared by all workspaces of a device)

struct PrimeTables {
    uint2* fwd = nullptr;
    uint2* inv = nullptr;
};
struct StepTables {
    uint2* f_a = nullptr;
    uint2* f_b = nullptr;
    uint2* i_lo = nullptr;
    uint2* i_hi = nullptr;
    uint2 scale{0, 0};
};

static std::mutex g_table_mutex;
static std::map<std::pair<int, u32>, PrimeTables> g_prime_tables;
static std::map<std::tuple<int, u32, int, int, u32>, StepTables> g_step_tables;
static std::map<int, bool> g_device_ready;

static uint2 shoup_pair(u32 w, u32 p) { return make_uint2(w, (u32)(((u64)w << 32) / p)); }

static bool upload(uint2** dst, const std::vector<uint2>& host) {
    if (!cuda_ok(cudaMalloc((void**)dst, host.size() * sizeof(uint2)), "cudaMalloc(table)")) return false;
    return cuda_ok(cudaMemcpy(*dst, host.data(), host.size() * sizeof(uint2), cudaMemcpyHostToDevice),
                   "cudaMemcpy(table)");
}

// Kernel attributes of every kernel on device `dev` (caller holds g_table_mutex).
static std::atomic<bool> g_kernels_ready[64];
static bool device_ready(int dev) {
    if (g_device_ready[dev]) return true;
    if (!cuda_ok(init_transform_kernels(), "kernel attributes")) return false;
    if (!cuda_ok(init_crt_kernels(), "kernel attributes")) return false;
    if (!cuda_ok(init_school_kernels(), "kernel attributes")) return false;
    g_device_ready[dev] = true;
    if (dev >= 0 && dev < 64) g_kernels_ready[dev].store(true, std::memory_order_release);
    return true;
}

bool kernels_ready() {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return false;
    if (dev >= 0 && dev < 64 && g_kernels_ready[dev].load(std::memory_order_acquire)) return true;
    std::lock_guard<std::mutex> lock(g_table_mutex);
    return device_ready(dev);
}

static bool prime_tables(int dev, u32 p, PrimeTables& out) {
    auto key = std::make_pair(dev, p);
    auto it = g_prime_tables.find(key);
    if (it != g_prime_tables.end()) { out = it->second; return true; }
    const u32 g = generator(p);
    const int n = 1 << kMaxBlockLog;
    std::vector<uint2> fwd(n), inv(n);
    fwd[0] = inv[0] = shoup_pair(1, p);
    for (int h = 1; h < n; h <<= 1) {
        const u32 root = powmod(g, (p - 1) / (2 * (u64)h), p);
        const u32 iroot = invmod(root, p);
        u32 w = 1, iw = 1;
        for (int j = 0; j < h; ++j) {
            fwd[h + j] = shoup_pair(w, p);
            inv[h + j] = shoup_pair(iw, p);
            w = mulmod(w, root, p);
            iw = mulmod(iw, iroot, p);
        }
    }
    PrimeTables t;
    if (!upload(&t.fwd, fwd) || !upload(&t.inv, inv)) return false;
    g_prime_tables[key] = t;
    out = t;
    return true;
}

// Stream of the one-time table builds of each device (non-blocking, so a build
// never waits for other work on the device).
static std::map<int, cudaStream_t> g_table_streams;

static cudaStream_t table_stream(int dev) {
    auto it = g_table_streams.find(dev);
    if (it != g_table_streams.end()) return it->second;
    cudaStream_t st = nullptr;
    if (!cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate")) return nullptr;
    g_table_streams[dev] = st;
    return st;
}

// Root tables of one transform length: the inverse scale and, for the four-step
// sizes, the forward and inverse twiddle factors in the layouts the column and row
// passes read (launch.h describes them), built by a kernel from the squares of w.
// `cofactor` is the prime's CRT factor (P/p)^-1 mod p of the prime set, folded into
// the scale.
static bool step_tables(int dev, u32 p, int log_t, int log_r, u32 cofactor, StepTables& out) {
    auto key = std::make_tuple(dev, p, log_t, log_r, cofactor);
    auto it = g_step_tables.find(key);
    if (it != g_step_tables.end()) { out = it->second; return true; }
    const u32 g = generator(p);
    const u32 w = powmod(g, (p - 1) >> log_t, p);
    const u32 iw = invmod(w, p);
    // Inverse scale: T^-1 times 2^32 (undoes the Montgomery pointwise product) times
    // the CRT cofactor inverse.
    const u32 scale = mulmod(mulmod(invmod((u32)(((u64)1 << log_t) % p), p), (u32)(((u64)1 << 32) % p), p),
                             cofactor, p);
    StepTables t;
    t.scale = shoup_pair(scale, p);
    if (log_r > 0) {
        StepTableBuild b;
        memset(&b, 0, sizeof(b));
        b.p = p;
        b.log_t = log_t;
        b.log_r = log_r;
        b.log_c = log_t - log_r;
        u32 x = w, ix = iw;
        for (int i = 0; i <= log_t; ++i) {
            b.fwd_pow[i] = shoup_pair(x, p);
            b.inv_pow[i] = shoup_pair(ix, p);
            x = mulmod(x, x, p);
            ix = mulmod(ix, ix, p);
        }
        b.scale = t.scale;
        u64 n[4];
        step_table_sizes(log_t, log_r, n);
        uint2** dst[4] = {&t.f_a, &t.f_b, &t.i_lo, &t.i_hi};
        for (int i = 0; i < 4; ++i)
            if (!cuda_ok(cudaMalloc((void**)dst[i], n[i] * sizeof(uint2)), "cudaMalloc(table)")) return false;
        b.f4_a = t.f_a;
        b.f4_b = t.f_b;
        b.i4_lo = t.i_lo;
        b.i4_hi = t.i_hi;
        cudaStream_t st = table_stream(dev);
        if (!st || !cuda_ok(launch_step_tables(b, st), "table build launch") ||
            !cuda_ok(cudaStreamSynchronize(st), "table build"))
            return false;
    }
    g_step_tables[key] = t;
    out = t;
    return true;
}

// Four-step split of the lazy transforms: log2 R for each length 2^log_t, 0 for
// the default floor(log_t / 2). Set by ntt_split_set, e.g. from ntt_tune_splits.
std::atomic<int> g_split[kMaxLogT + 1];

// Range of log2 R with column and row kernels for a lazy transform of 2^log_t
// points (columns 2^7..2^11, rows 2^7..2^13); false when the length has no
// four-step form or is one of the wide lengths.
bool split_range(int log_t, int& lo, int& hi) {
    if (log_t <= kMaxBlockLog || log_t > 23) return false;
    lo = std::max(6, log_t - 13);
    hi = std::min(11, log_t - 7);
    return lo <= hi;
}

int four_step_log_r(const Geom& g) {
    if (g.log_t <= kMaxBlockLog) return 0;
    // wide: 2^12-point columns from 2^24 on, 2^10-point ones at 2^22 and 2^23
    if (g.wide) return g.log_t >= 24 ? 12 : 10;
    const int o = g_split[g.log_t].load(std::memory_order_relaxed);
    return o ? o : g.log_t / 2;
}

int single_log_r(const Geom& g) {
    if (g.log_t == kMaxBlockLog && !g.wide) return 6;  // 2^6-point columns, 2^7-point rows
    return four_step_log_r(g);
}

// Fills the kernel constants of a plan whose four-step split is R = 2^log_r (0 for
// the one-CTA lengths); builds missing tables on the current device.
static std::map<std::tuple<int, int, int, int, int>, std::pair<PrimeSet, CrtParams>> g_param_cache;

bool prepare_params(const Geom& g, int log_r, PrimeSet& ps, CrtParams& cp) {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return false;
    std::lock_guard<std::mutex> lock(g_table_mutex);
    // the prime set is fixed by the length, the prime count and the class
    const auto key = std::make_tuple(dev, g.log_t, g.np, log_r, g.wide);
    auto hit = g_param_cache.find(key);
    if (hit != g_param_cache.end()) {
        ps = hit->second.first;
        cp = hit->second.second;
        cp.stride = (int)g.stride;
        cp.bias = g.sign ? 0.5f : 0.25f;
        return true;
    }
    if (!device_ready(dev)) return false;
    memset(&ps, 0, sizeof(ps));
    memset(&cp, 0, sizeof(cp));
    Words P{1};
    for (int i = 0; i < g.np; ++i) P = words_mul_small(P, g.primes[i]);
    cp.np = g.np;
    cp.l64 = std::min(4, (g.cap + 63) / 64);
    cp.stride = (int)g.stride;
    cp.bias = g.sign ? 0.5f : 0.25f;
    for (int w = 0; w < (int)P.size() && w < kMaxPrimes; ++w) cp.P[w] = P[w];
    for (int i = 0; i < g.np; ++i) {
        const u32 p = g.primes[i];
        // CRT cofactor M_i = P / p_i and its inverse, which the inverse scale absorbs
        Words M{1};
        for (int j = 0; j < g.np; ++j) if (j != i) M = words_mul_small(M, g.primes[j]);
        const u32 cofactor = invmod(words_mod(M, p), p);
        PrimeTables pt;
        StepTables st;
        if (!prime_tables(dev, p, pt) || !step_tables(dev, p, g.log_t, log_r, cofactor, st)) return false;
        PrimeParams& pp = ps.pr[i];
        pp.p = p;
        u32 pinv = 1;  // p^-1 mod 2^32 by Newton's iteration (bits double each step)
        for (int k = 0; k < 5; ++k) pinv *= 2u - p * pinv;
        pp.pni = 0u - pinv;
        pp.inv2_32 = (u32)(((u64)1 << 32) / p);
        const u32 r32 = (u32)(((u64)1 << 32) % p);
        pp.neg64 = mulmod(r32, r32, p);
        pp.r32 = shoup_pair(r32, p);
        pp.scale = st.scale;
        pp.fwd = pt.fwd;
        pp.inv = pt.inv;
        {
            const u32 gen = generator(p);
            pp.small_fwd[0] = pp.small_inv[0] = shoup_pair(1, p);
            for (int h = 1; h < 32; h <<= 1) {
                const u32 root = powmod(gen, (p - 1) / (2 * (u64)h), p), iroot = invmod(root, p);
                u32 w = 1, iw = 1;
                for (int j = 0; j < h; ++j) {
                    pp.small_fwd[h + j] = shoup_pair(w, p);
                    pp.small_inv[h + j] = shoup_pair(iw, p);
                    w = mulmod(w, root, p);
                    iw = mulmod(iw, iroot, p);
                }
            }
        }
        pp.f4_a = st.f_a;
        pp.f4_b = st.f_b;
        pp.i4_lo = st.i_lo;
        pp.i4_hi = st.i_hi;
        for (int w = 0; w < (int)M.size() && w < kMaxPrimes; ++w) cp.M[i][w] = M[w];
        cp.p[i] = p;
        cp.pinv[i] = 1.0f / (float)p;
    }
    fill_multiples(cp);
    g_param_cache[key] = std::make_pair(ps, cp);
    return true;
}

bool prepare_params(const Geom& g, PrimeSet& ps, CrtParams& cp) {
    return prepare_params(g, four_step_log_r(g), ps, cp);
}

}  // namespace ntt
