// Host side of the GB300 multiplication path: prime catalog, planner, device root
// tables, workspaces and the C ABI declared in include/ntt_gb300.h.
//
// Planning mirrors the reference's admission rules (src/plan.rs:53-69,
// src/convolve.rs:75-116, src/profile/planner.rs:120-322) with this library's own
// geometry: every 64-bit limb is one transform coefficient, the transform length
// is the power of two that holds the convolution, and the fewest 32-bit primes
// whose product holds every coefficient are taken from a catalog of primes with
// the needed two-power roots.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/ntt_gb300.h"
#include "launch.h"

namespace ntt {

typedef unsigned __int128 u128;

static thread_local std::string g_error;
static std::atomic<uint64_t> g_launches{0};
// Set while this thread captures a batch into a CUDA graph: the captured launches
// are counted when the graph runs, not when it is recorded.
static thread_local bool t_capturing = false;

static void note_launches(uint64_t n) {
    if (!t_capturing) g_launches += n;
}

// Optional per-kernel timing: when set, an event is recorded on the launching
// stream before the first kernel of a call and after every kernel.
static std::vector<cudaEvent_t> g_events;
static bool g_timing = false;
static int g_marks_n = 0;
static int g_marks_i = 0;

void mark(cudaStream_t st) {
    if (t_capturing) return;
    if (g_timing && g_marks_i < g_marks_n && cudaEventRecord(g_events[g_marks_i], st) == cudaSuccess) ++g_marks_i;
}

void set_last_error(const std::string& message) { g_error = message; }

static bool fail(const char* msg) {
    g_error = msg;
    return false;
}
static bool cuda_ok(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return true;
    g_error = std::string(where) + ": " + cudaGetErrorString(e);
    return false;
}

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
// Primes below 2^31 with valuation at least 24 (canonical arithmetic, T >= 2^24).
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

static std::vector<u32> primes_for(int log_t) {
    std::vector<u32> out;
    if (log_t <= kLazyMaxLog) {
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

// Smallest block transform of a split product (2^10 points).
constexpr int kSmallSplitLog = 10;

// ---------------------------------------------------------------------------------
// Plans

struct Geom {
    bool conv = false;
    u64 la = 0, lb = 0, conv_len = 0, out_len = 0;
    int log_t = 0, np = 0, wide = 0, cap = 0;
    u32 primes[kMaxPrimes] = {};
    // convolutions
    u64 max_a = 0, max_b = 0;
    int sign = 0, bound_bits = 0, schoolbook = 0;
    u64 stride = 1;
    // block split of an unbalanced product: the longer operand in blocks of `block`
    // limbs, each multiplied by the shorter one with transforms of 2^log_t points
    u64 block = 0, blocks = 0;

    bool matches(u64 a, u64 b) const { return a == la && b == lb; }
    bool split() const { return block != 0; }
    u64 spec_words(bool square) const { return (u64)(square ? 1 : 2) * np * ((u64)1 << log_t); }
    // residues and carry flags of one product of this geometry (one block if split)
    u64 member_bytes(bool square) const {
        const u64 spec = (spec_words(square) * 4 + 255) & ~(u64)255;
        const u64 out = split() ? block + std::min(la, lb) : out_len;
        return spec + ((conv ? 0 : carry_scratch_bytes(out)) + 255 & ~(u64)255);
    }
    // blocks per enqueue of a split product: bounded launch grids and arena
    u64 split_chunk() const {
        const u64 by_bytes = std::max<u64>(1, ((u64)512 << 20) / member_bytes(false));
        return std::min<u64>({blocks, 16384, by_bytes});
    }
    // split: [descriptors][odd-block sums (out_len limbs)][add flags][member arenas]
    u64 split_desc_bytes() const { return (split_chunk() * sizeof(ProductDesc) + 255) & ~(u64)255; }
    u64 split_odd_bytes() const { return (out_len * 8 + 255) & ~(u64)255; }
    u64 split_flag_bytes() const { return (carry_scratch_bytes(out_len) + 255) & ~(u64)255; }
    u64 scratch_bytes(bool square) const {
        if (conv && schoolbook) return 0;
        if (split())
            return split_desc_bytes() + split_odd_bytes() + split_flag_bytes() + split_chunk() * member_bytes(false);
        const u64 spec = (spec_words(square) * 4 + 255) & ~(u64)255;
        return spec + (conv ? 0 : carry_scratch_bytes(out_len));
    }
};

static bool choose_primes(Geom& g, int need_bits) {
    const std::vector<u32> cand = primes_for(g.log_t);
    for (int np = 1; np <= (int)cand.size(); ++np) {
        const int cap = capacity(cand, np);
        if (cap >= need_bits) {
            g.np = np;
            g.cap = cap;
            for (int i = 0; i < np; ++i) g.primes[i] = cand[i];
            g.wide = g.log_t > kLazyMaxLog;
            return true;
        }
    }
    return false;
}

// Longest operand of a split product (limbs).
constexpr u64 kMaxSplitLimbs = (u64)1 << 40;

// Block split of an unbalanced product (the reference's Geometry::cheapest_blocks,
// src/profile/planner.rs:291-393, restated for this library's transforms): the
// longer operand (L limbs) in blocks of B = 2^k - S + 1 limbs, each multiplied by
// the shorter one (S limbs) with 2^k-point transforms. Cost in butterfly levels:
// three transforms per block, n * 3 * 2^k * k, against 3 * 2^K * K for one
// transform of the whole product. Returns the chosen k, or 0 when one transform
// is cheaper (by the margin that pays for the block sums and the final addition).
static int split_log(u64 L, u64 S, int full_log) {
    const double full = full_log <= kMaxLogT ? 3.0 * std::ldexp(1.0, full_log) * full_log : 1e300;
    int best_k = 0;
    double best = 0.8 * full;
    const int lo = std::max(kSmallSplitLog, ceil_log2(2 * S));
    for (int k = lo; k <= kMaxLogT && k < full_log; ++k) {
        const u64 B = ((u64)1 << k) - S + 1;
        const double n = (double)((L + B - 1) / B);
        const double cost = n * 3.0 * std::ldexp(1.0, k) * k;
        if (cost < best) {
            best = cost;
            best_k = k;
        }
    }
    return best_k;
}

// allow_split: callers that run one product per call (workspaces, plans) may take
// the block split; batch members always use one transform.
static bool plan_mul(u64 la, u64 lb, Geom& g, bool allow_split = true) {
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

static bool plan_conv(u64 la, u64 lb, u64 max_a, u64 max_b, int sign, Geom& g) {
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
static std::map<std::tuple<int, u32, int, int>, StepTables> g_step_tables;
static std::map<int, bool> g_device_ready;

static uint2 shoup_pair(u32 w, u32 p) { return make_uint2(w, (u32)(((u64)w << 32) / p)); }

static bool upload(uint2** dst, const std::vector<uint2>& host) {
    if (!cuda_ok(cudaMalloc((void**)dst, host.size() * sizeof(uint2)), "cudaMalloc(table)")) return false;
    return cuda_ok(cudaMemcpy(*dst, host.data(), host.size() * sizeof(uint2), cudaMemcpyHostToDevice),
                   "cudaMemcpy(table)");
}

static bool device_ready(int dev) {
    if (g_device_ready[dev]) return true;
    if (!cuda_ok(init_transform_kernels(), "kernel attributes")) return false;
    if (!cuda_ok(init_crt_kernels(), "kernel attributes")) return false;
    g_device_ready[dev] = true;
    return true;
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
static bool step_tables(int dev, u32 p, int log_t, int log_r, StepTables& out) {
    auto key = std::make_tuple(dev, p, log_t, log_r);
    auto it = g_step_tables.find(key);
    if (it != g_step_tables.end()) { out = it->second; return true; }
    const u32 g = generator(p);
    const u32 w = powmod(g, (p - 1) >> log_t, p);
    const u32 iw = invmod(w, p);
    // Inverse scale: T^-1 times 2^32 (undoes the Montgomery pointwise product).
    const u32 scale = mulmod(invmod((u32)(((u64)1 << log_t) % p), p), (u32)(((u64)1 << 32) % p), p);
    StepTables t;
    t.scale = shoup_pair(scale, p);
    if (log_t > kMaxBlockLog) {
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
static std::atomic<int> g_split[kMaxLogT + 1];

// Range of log2 R with column and row kernels for a lazy transform of 2^log_t
// points (columns 2^7..2^11, rows 2^7..2^13); false when the length has no
// four-step form or is one of the wide lengths.
static bool split_range(int log_t, int& lo, int& hi) {
    if (log_t <= kMaxBlockLog || log_t > 23) return false;
    lo = std::max(7, log_t - 13);
    hi = std::min(11, log_t - 7);
    return lo <= hi;
}

static int four_step_log_r(const Geom& g) {
    if (g.log_t <= kMaxBlockLog) return 0;
    const int o = g.wide ? 0 : g_split[g.log_t].load(std::memory_order_relaxed);
    return o ? o : g.log_t / 2;
}

// Fills the kernel constants of a plan whose four-step split is R = 2^log_r (0 for
// the one-CTA lengths); builds missing tables on the current device.
static std::map<std::tuple<int, int, int, int>, std::pair<PrimeSet, CrtParams>> g_param_cache;

static bool prepare_params(const Geom& g, int log_r, PrimeSet& ps, CrtParams& cp) {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return false;
    std::lock_guard<std::mutex> lock(g_table_mutex);
    const auto key = std::make_tuple(dev, g.log_t, g.np, log_r);
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
        PrimeTables pt;
        StepTables st;
        if (!prime_tables(dev, p, pt) || !step_tables(dev, p, g.log_t, log_r, st)) return false;
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
        // CRT cofactors M_i = P / p_i and their inverses.
        Words M{1};
        for (int j = 0; j < g.np; ++j) if (j != i) M = words_mul_small(M, g.primes[j]);
        for (int w = 0; w < (int)M.size() && w < kMaxPrimes; ++w) cp.M[i][w] = M[w];
        cp.p[i] = p;
        cp.inv[i] = shoup_pair(invmod(words_mod(M, p), p), p);
        cp.pinv[i] = 1.0f / (float)p;
    }
    g_param_cache[key] = std::make_pair(ps, cp);
    return true;
}

static bool prepare_params(const Geom& g, PrimeSet& ps, CrtParams& cp) {
    return prepare_params(g, four_step_log_r(g), ps, cp);
}

// ---------------------------------------------------------------------------------
// Execution on device pointers

// Enqueues the kernels of `n` members of one transform class (same kind, length,
// primes, sign and square) whose descriptors sit in device memory; max_len is the
// longest member output (limbs of a product, coefficients of a convolution).
static bool run_members(const ProductDesc* descs, int n, const Geom& g0, bool sq, u64 max_len, cudaStream_t st) {
    TransformArgs ta;
    memset(&ta, 0, sizeof(ta));
    CrtParams cp;
    const int log_r = four_step_log_r(g0);
    if (!prepare_params(g0, log_r, ta.ps, cp)) return false;
    ta.batch = descs;
    ta.count = n;
    ta.np = g0.np;
    ta.log_t = g0.log_t;
    ta.wide = g0.wide;
    const bool sign = g0.sign != 0;
    mark(st);
    if (!g0.conv && g0.log_t <= kFusedMaxLog && g0.np == kFusedPrimes && !g0.wide) {
        note_launches(1);
        const bool ok = cuda_ok(launch_small_fused(ta, cp, sq, st), "batched fused product launch");
        mark(st);
        return ok;
    }
    if (g0.log_t <= kMaxBlockLog) {
        note_launches(1);
        if (!cuda_ok(launch_small(ta, sq, sign, st), "batched transform launch")) return false;
        mark(st);
    } else {
        ta.log_r = log_r;
        ta.log_c = g0.log_t - ta.log_r;
        note_launches(3);
        if (!cuda_ok(launch_fwd_cols(ta, sq, sign, st), "batched column pass launch")) return false;
        mark(st);
        if (!cuda_ok(launch_rows(ta, sq, st), "batched row pass launch")) return false;
        mark(st);
        if (!cuda_ok(launch_inv_cols(ta, st), "batched inverse column pass launch")) return false;
        mark(st);
    }
    note_launches(1);
    const bool ok =
        g0.conv ? cuda_ok(launch_crt_conv_batch(descs, n, max_len, g0.log_t, cp, st), "batched CRT launch")
                : cuda_ok(launch_crt_mul_batch(descs, n, (int)((max_len + kCrtTile - 1) / kCrtTile), g0.log_t, cp, st),
                          "batched CRT launch");
    mark(st);
    return ok;
}

// Enqueues a split product: the blocks of the longer operand times the shorter one
// as batch members in chunks (the even blocks' products straight into dst, the odd
// ones' into a second number), then dst += odd with carries.
static bool execute_split(const Geom& g, const u64* d_a, const u64* d_b, u64* d_dst, void* scratch, cudaStream_t st) {
    const bool swap = g.la < g.lb;
    const u64* lng = swap ? d_b : d_a;
    const u64* sht = swap ? d_a : d_b;
    const u64 L = std::max(g.la, g.lb), S = std::min(g.la, g.lb);
    uint8_t* base = (uint8_t*)scratch;
    ProductDesc* descs = (ProductDesc*)base;
    u64* odd = (u64*)(base + g.split_desc_bytes());
    u32* flags = (u32*)((uint8_t*)odd + g.split_odd_bytes());
    uint8_t* arena = (uint8_t*)flags + g.split_flag_bytes();
    const u64 member = g.member_bytes(false), spec = (g.spec_words(false) * 4 + 255) & ~(u64)255;
    if (!cuda_ok(cudaMemsetAsync(d_dst, 0, g.out_len * 8, st), "zero product") ||
        !cuda_ok(cudaMemsetAsync(odd, 0, g.out_len * 8, st), "zero odd blocks") ||
        !cuda_ok(cudaMemsetAsync(flags, 0, carry_scratch_bytes(g.out_len), st), "zero carry flags"))
        return false;
    const u64 chunk = g.split_chunk();
    for (u64 first = 0; first < g.blocks; first += chunk) {
        const u64 count = std::min(chunk, g.blocks - first);
        note_launches(1);
        if (!cuda_ok(launch_split_descs(descs, first, count, lng, L, sht, S, g.block, d_dst, odd, arena, member, spec,
                                        st),
                     "split descriptors") ||
            !run_members(descs, (int)count, g, false, g.block + S, st))
            return false;
    }
    note_launches(1);
    return cuda_ok(launch_add_limbs(d_dst, odd, g.out_len, flags, st), "block sum");
}

// Enqueues one product or convolution on `st`. With `b_ready` set (an event that
// completes when operand b is in place), the column pass of a runs first and the
// one of b waits for that event, so b's upload overlaps a's pass.
static bool execute(const Geom& g, bool square, const u64* d_a, const u64* d_b, u64* d_dst,
                    void* scratch, cudaStream_t st, cudaEvent_t b_ready = nullptr) {
    mark(st);
    if (g.split()) {
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        const bool ok = execute_split(g, d_a, square ? d_a : d_b, d_dst, scratch, st);
        mark(st);
        return ok;
    }
    if (g.conv && g.schoolbook) {
        note_launches(1);
        const bool ok = cuda_ok(launch_conv_schoolbook(d_a, g.la, square ? d_a : d_b, square ? g.la : g.lb, d_dst,
                                                       (int)g.stride, g.sign != 0, st),
                                "conv schoolbook launch");
        mark(st);
        return ok;
    }
    TransformArgs ta;
    memset(&ta, 0, sizeof(ta));
    CrtParams cp;
    const int log_r = four_step_log_r(g);
    if (!prepare_params(g, log_r, ta.ps, cp)) return false;
    ta.a = d_a;
    ta.b = square ? d_a : d_b;
    ta.la = g.la;
    ta.lb = square ? g.la : g.lb;
    ta.spec = (u32*)scratch;
    ta.conv_len = g.conv_len;
    ta.np = g.np;
    ta.log_t = g.log_t;
    ta.wide = g.wide;
    const u64 spec_bytes = (g.spec_words(square) * 4 + 255) & ~(u64)255;
    if (!g.conv) {
        ta.flags = (u32*)((uint8_t*)scratch + spec_bytes);
        ta.flag_words = (u32)carry_flag_words(g.out_len);
    }
    const bool sign = g.sign != 0;
    if (!g.conv && g.log_t <= kFusedMaxLog && g.np == kFusedPrimes && !g.wide) {
        // the whole product in one cluster launch
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        ta.dst = d_dst;
        ta.out_len = g.out_len;
        note_launches(1);
        const bool ok = cuda_ok(launch_small_fused(ta, cp, square, st), "fused product launch");
        mark(st);
        return ok;
    }
    if (g.log_t <= kMaxBlockLog) {
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        note_launches(1);
        if (!cuda_ok(launch_small(ta, square, sign, st), "transform launch")) return false;
        mark(st);
    } else {
        ta.log_r = log_r;
        ta.log_c = g.log_t - ta.log_r;
        if (b_ready && !square) {
            note_launches(1);
            ta.op_count = 1;
            if (!cuda_ok(launch_fwd_cols(ta, square, sign, st), "column pass launch")) return false;
            if (!cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
            ta.op_base = 1;
            if (!cuda_ok(launch_fwd_cols(ta, square, sign, st), "column pass launch")) return false;
            ta.op_base = 0;
            ta.op_count = 0;
        } else if (!cuda_ok(launch_fwd_cols(ta, square, sign, st), "column pass launch")) {
            return false;
        }
        note_launches(3);
        mark(st);
        if (!cuda_ok(launch_rows(ta, square, st), "row pass launch")) return false;
        mark(st);
        if (!cuda_ok(launch_inv_cols(ta, st), "inverse column pass launch")) return false;
        mark(st);
    }
    if (g.conv) {
        note_launches(1);
        const bool ok = cuda_ok(launch_crt_conv(ta.spec, g.log_t, g.conv_len, d_dst, sign, cp, st), "CRT launch");
        mark(st);
        return ok;
    }
    note_launches(1);
    return cuda_ok(launch_crt_mul(ta.spec, g.log_t, g.conv_len, g.out_len, d_dst,
                                  (uint8_t*)scratch + spec_bytes, cp, st, mark),
                   "CRT launch");
}

// Grow-only device buffer.
struct DeviceBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    bool ensure(size_t need) {
        if (need <= bytes) return true;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        if (!cuda_ok(cudaMalloc(&ptr, std::max<size_t>(need, 256)), "cudaMalloc(arena)")) return false;
        bytes = std::max<size_t>(need, 256);
        return true;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

static bool coefficients_admitted(const Geom& g, const u64* v, u64 n, u64 max) {
    if (g.sign) {
        for (u64 i = 0; i < n; ++i) {
            const int64_t s = (int64_t)v[i];
            const u64 mag = s < 0 ? (u64)0 - (u64)s : (u64)s;
            if (mag > max) return false;
        }
        return true;
    }
    u64 acc = 0;
    for (u64 i = 0; i < n; ++i) acc |= v[i];
    if (acc <= max) return true;
    for (u64 i = 0; i < n; ++i) if (v[i] > max) return false;
    return true;
}

}  // namespace ntt

using namespace ntt;

// ---------------------------------------------------------------------------------
// Workspaces

struct ntt_mul_workspace {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t upload = nullptr;    // copies operand b while a's column pass runs
    cudaEvent_t b_ready = nullptr;
    bool has_plan = false;
    Geom plan;
    DeviceBuf a, b, out, scratch;
};

struct ntt_conv_workspace {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t upload = nullptr;
    cudaEvent_t b_ready = nullptr;
    bool has_plan = false;
    Geom plan;
    DeviceBuf a, b, out, scratch;
};

template <class W>
static W* workspace_new() {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
    W* ws = new W();
    ws->device = dev;
    if (!cuda_ok(cudaStreamCreateWithFlags(&ws->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaStreamCreateWithFlags(&ws->upload, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaEventCreateWithFlags(&ws->b_ready, cudaEventDisableTiming), "cudaEventCreate")) {
        if (ws->stream) cudaStreamDestroy(ws->stream);
        if (ws->upload) cudaStreamDestroy(ws->upload);
        delete ws;
        return nullptr;
    }
    return ws;
}

template <class W>
static void workspace_free(W* ws) {
    if (!ws) return;
    cudaSetDevice(ws->device);
    cudaStreamSynchronize(ws->stream);
    ws->a.release();
    ws->b.release();
    ws->out.release();
    ws->scratch.release();
    cudaEventDestroy(ws->b_ready);
    cudaStreamDestroy(ws->upload);
    cudaStreamDestroy(ws->stream);
    delete ws;
}

// Device address of page-locked host memory, or null for other memory.
static void* mapped_host_pointer(void* p) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return attr.type == cudaMemoryTypeHost ? attr.devicePointer : nullptr;
}

// Host-pointer calls in flight in this process.
static std::atomic<int> g_host_calls{0};

// Runs a host-pointer call. The operands are copied in (b on a second stream,
// overlapping a's column pass); the result is written straight into dst when dst
// is page-locked host memory the GPU can address and no other host-pointer call is
// in flight, and copied out otherwise. One
// synchronisation at the end: every check runs before the first write, and a
// failed kernel stops the stream before the copy-out.
template <class W>
static bool run_host(W* ws, const Geom& g, bool square, u64* dst, const u64* a, const u64* b) {
    const size_t out_bytes = g.out_len * sizeof(u64);
    // The CRT kernel writes straight into page-locked dst when this is the only
    // host-pointer call in flight (lowest latency). With others in flight the copy
    // engine moves the result instead, so the SMs stay free for their kernels while
    // the bytes cross the host link. A split product adds into its destination:
    // that stays in device memory.
    struct InFlight {
        InFlight() { ++g_host_calls; }
        ~InFlight() { --g_host_calls; }
    } in_flight;
    const bool alone = g_host_calls.load() == 1;
    u64* direct = g.split() || !alone ? nullptr : (u64*)mapped_host_pointer(dst);
    if (!ws->a.ensure(g.la * 8) || (!square && !ws->b.ensure(g.lb * 8)) || (!direct && !ws->out.ensure(out_bytes)) ||
        !ws->scratch.ensure(g.scratch_bytes(square)))
        return false;
    cudaStream_t st = ws->stream;
    if (!cuda_ok(cudaMemcpyAsync(ws->a.ptr, a, g.la * 8, cudaMemcpyHostToDevice, st), "copy a")) return false;
    cudaEvent_t b_ready = nullptr;
    if (!square) {
        if (!cuda_ok(cudaMemcpyAsync(ws->b.ptr, b, g.lb * 8, cudaMemcpyHostToDevice, ws->upload), "copy b") ||
            !cuda_ok(cudaEventRecord(ws->b_ready, ws->upload), "cudaEventRecord"))
            return false;
        b_ready = ws->b_ready;
    }
    u64* out = direct ? direct : (u64*)ws->out.ptr;
    if (!execute(g, square, (const u64*)ws->a.ptr, (const u64*)ws->b.ptr, out, ws->scratch.ptr, st, b_ready))
        return false;
    if (!direct && !cuda_ok(cudaMemcpyAsync(dst, out, out_bytes, cudaMemcpyDeviceToHost, st), "copy dst"))
        return false;
    return cuda_ok(cudaStreamSynchronize(st), "kernels");
}

extern "C" {

int ntt_mul_plan_new(uint64_t len_a, uint64_t len_b, ntt_mul_plan* out) {
    Geom g;
    if (!out || !plan_mul(len_a, len_b, g)) return 0;
    out->len_a = len_a;
    out->len_b = len_b;
    out->primes = (uint32_t)g.np;
    out->log_transform = (uint32_t)g.log_t;
    out->scratch_len = (g.scratch_bytes(false) + 7) / 8;
    out->sqr_scratch_len = (g.scratch_bytes(true) + 7) / 8;
    out->block_len = g.block;
    out->blocks = g.blocks;
    return 1;
}

static uint8_t plan_run_device(const ntt_mul_plan* plan, bool square, uint64_t* d_dst, size_t dst_len,
                               const uint64_t* d_a, size_t a_len, const uint64_t* d_b, size_t b_len,
                               uint64_t* d_scratch, size_t scratch_len, void* stream) {
    Geom g;
    if (!plan || !plan_mul(plan->len_a, plan->len_b, g)) return 0;
    if (!g.matches(a_len, b_len)) return fail("operand lengths differ from the plan");
    if (square && a_len != b_len) return fail("a square needs a square plan");
    if (dst_len < g.out_len) return fail("destination is shorter than the product");
    if ((u64)scratch_len * 8 < g.scratch_bytes(square)) return fail("scratch is too short");
    return execute(g, square, d_a, square ? d_a : d_b, d_dst, d_scratch, (cudaStream_t)stream);
}

uint8_t ntt_mul_plan_mul_device(const ntt_mul_plan* plan, uint64_t* d_dst, size_t dst_len, const uint64_t* d_a,
                                size_t a_len, const uint64_t* d_b, size_t b_len, uint64_t* d_scratch,
                                size_t scratch_len, void* stream) {
    const bool alias = d_a == d_b && a_len == b_len;
    return plan_run_device(plan, alias, d_dst, dst_len, d_a, a_len, d_b, b_len, d_scratch, scratch_len, stream);
}

uint8_t ntt_mul_plan_sqr_device(const ntt_mul_plan* plan, uint64_t* d_dst, size_t dst_len, const uint64_t* d_a,
                                size_t a_len, uint64_t* d_scratch, size_t scratch_len, void* stream) {
    return plan_run_device(plan, true, d_dst, dst_len, d_a, a_len, d_a, a_len, d_scratch, scratch_len, stream);
}

ntt_mul_workspace* ntt_mul_workspace_new(void) { return workspace_new<ntt_mul_workspace>(); }
void ntt_mul_workspace_free(ntt_mul_workspace* ws) { workspace_free(ws); }

static bool mul_reserve(ntt_mul_workspace* ws, const Geom& g, bool host) {
    if (host && (!ws->a.ensure(g.la * 8) || !ws->b.ensure(g.lb * 8) || !ws->out.ensure(g.out_len * 8)))
        return false;
    if (!ws->scratch.ensure(g.scratch_bytes(false))) return false;
    PrimeSet ps;
    CrtParams cp;
    return prepare_params(g, ps, cp);
}

uint8_t ntt_mul_workspace_prepare(ntt_mul_workspace* ws, const ntt_mul_plan* plan) {
    if (!ws || !plan) return fail("null argument");
    Geom g;
    if (!plan_mul(plan->len_a, plan->len_b, g)) return 0;
    cudaSetDevice(ws->device);
    if (!mul_reserve(ws, g, true)) return 0;
    ws->plan = g;
    ws->has_plan = true;
    return 1;
}

// Empty operands, plan retention and the destination check of MulWorkspace::run
// (src/plan.rs:182-205).
static int mul_admit(ntt_mul_workspace* ws, size_t dst_len, size_t a_len, size_t b_len, Geom& g) {
    if (a_len == 0 || b_len == 0) {
        if ((u64)a_len + b_len > dst_len) {
            fail("destination is shorter than the product");
            return -1;
        }
        return 0;  // zero product
    }
    if (ws->has_plan && ws->plan.matches(a_len, b_len)) {
        g = ws->plan;
    } else {
        if (!plan_mul(a_len, b_len, g)) return -1;
        ws->plan = g;
        ws->has_plan = true;
    }
    if (dst_len < g.out_len) {
        fail("destination is shorter than the product");
        return -1;
    }
    return 1;
}

static uint8_t ws_mul_host(ntt_mul_workspace* ws, uint64_t* dst, size_t dst_len, const uint64_t* a, size_t a_len,
                           const uint64_t* b, size_t b_len, bool square) {
    if (!ws) return fail("null workspace");
    Geom g;
    const int adm = mul_admit(ws, dst_len, a_len, b_len, g);
    if (adm < 0) return 0;
    if (adm == 0) {
        memset(dst, 0, ((size_t)a_len + b_len) * 8);
        return 1;
    }
    if (!cuda_ok(cudaSetDevice(ws->device), "cudaSetDevice")) return 0;
    return run_host(ws, g, square, dst, a, b) ? 1 : 0;
}

uint8_t ntt_mul_workspace_mul(ntt_mul_workspace* ws, uint64_t* dst, size_t dst_len, const uint64_t* a,
                              size_t a_len, const uint64_t* b, size_t b_len) {
    const bool alias = a == b && a_len == b_len;
    return ws_mul_host(ws, dst, dst_len, a, a_len, b, b_len, alias);
}

uint8_t ntt_mul_workspace_sqr(ntt_mul_workspace* ws, uint64_t* dst, size_t dst_len, const uint64_t* a,
                              size_t a_len) {
    return ws_mul_host(ws, dst, dst_len, a, a_len, a, a_len, true);
}

static uint8_t ws_mul_device(ntt_mul_workspace* ws, uint64_t* d_dst, size_t dst_len, const uint64_t* d_a,
                             size_t a_len, const uint64_t* d_b, size_t b_len, bool square, void* stream) {
    if (!ws) return fail("null workspace");
    Geom g;
    const int adm = mul_admit(ws, dst_len, a_len, b_len, g);
    if (adm < 0) return 0;
    if (!cuda_ok(cudaSetDevice(ws->device), "cudaSetDevice")) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    if (adm == 0)
        return cuda_ok(cudaMemsetAsync(d_dst, 0, ((size_t)a_len + b_len) * 8, st), "zero product") ? 1 : 0;
    if (!ws->scratch.ensure(g.scratch_bytes(square))) return 0;
    return execute(g, square, d_a, d_b, d_dst, ws->scratch.ptr, st) ? 1 : 0;
}

uint8_t ntt_mul_workspace_mul_device(ntt_mul_workspace* ws, uint64_t* d_dst, size_t dst_len, const uint64_t* d_a,
                                     size_t a_len, const uint64_t* d_b, size_t b_len, void* stream) {
    const bool alias = d_a == d_b && a_len == b_len;
    return ws_mul_device(ws, d_dst, dst_len, d_a, a_len, d_b, b_len, alias, stream);
}

uint8_t ntt_mul_workspace_sqr_device(ntt_mul_workspace* ws, uint64_t* d_dst, size_t dst_len, const uint64_t* d_a,
                                     size_t a_len, void* stream) {
    return ws_mul_device(ws, d_dst, dst_len, d_a, a_len, d_a, a_len, true, stream);
}

// ---------------------------------------------------------------------------------
// Convolutions

int ntt_conv_plan_new(uint64_t len_a, uint64_t len_b, uint64_t max_a, uint64_t max_b, int is_signed,
                      ntt_conv_plan* out) {
    Geom g;
    if (!out || !plan_conv(len_a, len_b, max_a, max_b, is_signed, g)) return 0;
    out->len_a = len_a;
    out->len_b = len_b;
    out->max_a = max_a;
    out->max_b = max_b;
    out->is_signed = (uint32_t)g.sign;
    out->primes = g.schoolbook ? 0 : (uint32_t)g.np;
    out->log_transform = g.schoolbook ? 0 : (uint32_t)g.log_t;
    out->schoolbook = (uint32_t)g.schoolbook;
    out->stride = g.stride;
    out->output_len = g.out_len;
    out->scratch_len = (g.scratch_bytes(false) + 7) / 8;
    return 1;
}

static bool conv_geom(const ntt_conv_plan* plan, Geom& g) {
    return plan && plan_conv(plan->len_a, plan->len_b, plan->max_a, plan->max_b, (int)plan->is_signed, g);
}

uint8_t ntt_conv_plan_convolve_device(const ntt_conv_plan* plan, uint64_t* d_dst, size_t dst_len,
                                      const uint64_t* d_a, size_t a_len, const uint64_t* d_b, size_t b_len,
                                      uint64_t* d_scratch, size_t scratch_len, void* stream) {
    Geom g;
    if (!conv_geom(plan, g)) return 0;
    if (!g.matches(a_len, b_len)) return fail("operand lengths differ from the plan");
    if (dst_len < g.out_len) return fail("destination is shorter than the convolution");
    const bool square = d_a == d_b && a_len == b_len;
    if ((u64)scratch_len * 8 < g.scratch_bytes(square)) return fail("scratch is too short");
    return execute(g, square, d_a, d_b, d_dst, d_scratch, (cudaStream_t)stream) ? 1 : 0;
}

ntt_conv_workspace* ntt_conv_workspace_new(void) { return workspace_new<ntt_conv_workspace>(); }
void ntt_conv_workspace_free(ntt_conv_workspace* ws) { workspace_free(ws); }

uint8_t ntt_conv_workspace_prepare(ntt_conv_workspace* ws, const ntt_conv_plan* plan) {
    if (!ws) return fail("null workspace");
    Geom g;
    if (!conv_geom(plan, g)) return 0;
    if (!cuda_ok(cudaSetDevice(ws->device), "cudaSetDevice")) return 0;
    if (!ws->a.ensure(g.la * 8) || !ws->b.ensure(g.lb * 8) || !ws->out.ensure(g.out_len * 8) ||
        !ws->scratch.ensure(g.scratch_bytes(false)))
        return 0;
    if (!g.schoolbook) {
        PrimeSet ps;
        CrtParams cp;
        if (!prepare_params(g, ps, cp)) return 0;
    }
    ws->plan = g;
    ws->has_plan = true;
    return 1;
}

uint8_t ntt_conv_workspace_convolve(ntt_conv_workspace* ws, uint64_t* dst, size_t dst_len, const uint64_t* a,
                                    size_t a_len, const uint64_t* b, size_t b_len) {
    if (!ws) return fail("null workspace");
    if (!ws->has_plan) return fail("no prepared plan");
    const Geom& g = ws->plan;
    if (!g.matches(a_len, b_len)) return fail("operand lengths differ from the plan");
    if (!coefficients_admitted(g, a, a_len, g.max_a) || !coefficients_admitted(g, b, b_len, g.max_b))
        return fail("a coefficient exceeds its bound");
    if (dst_len < g.out_len) return fail("destination is shorter than the convolution");
    if (!cuda_ok(cudaSetDevice(ws->device), "cudaSetDevice")) return 0;
    const bool square = a == b && a_len == b_len;
    return run_host(ws, g, square, dst, a, b) ? 1 : 0;
}

uint8_t ntt_conv_workspace_convolve_device(ntt_conv_workspace* ws, uint64_t* d_dst, size_t dst_len,
                                           const uint64_t* d_a, size_t a_len, const uint64_t* d_b, size_t b_len,
                                           void* stream) {
    if (!ws) return fail("null workspace");
    if (!ws->has_plan) return fail("no prepared plan");
    const Geom& g = ws->plan;
    if (!g.matches(a_len, b_len)) return fail("operand lengths differ from the plan");
    if (dst_len < g.out_len) return fail("destination is shorter than the convolution");
    if (!cuda_ok(cudaSetDevice(ws->device), "cudaSetDevice")) return 0;
    const bool square = d_a == d_b && a_len == b_len;
    if (!ws->scratch.ensure(g.scratch_bytes(square))) return 0;
    return execute(g, square, d_a, d_b, d_dst, ws->scratch.ptr, (cudaStream_t)stream) ? 1 : 0;
}

int ntt_timing_start(int count) {
    if (count < 2) return 0;
    while ((int)g_events.size() < count) {
        cudaEvent_t e;
        if (!cuda_ok(cudaEventCreate(&e), "cudaEventCreate")) return 0;
        g_events.push_back(e);
    }
    g_marks_n = count;
    g_marks_i = 0;
    g_timing = true;
    return 1;
}

int ntt_timing_stop(float* ms, int capacity) {
    const int n = g_marks_i;
    g_timing = false;
    g_marks_i = 0;
    if (n < 2) return 0;
    if (!cuda_ok(cudaEventSynchronize(g_events[n - 1]), "cudaEventSynchronize")) return -1;
    int out = 0;
    for (int i = 0; i + 1 < n && out < capacity; ++i) {
        float t = 0.0f;
        if (!cuda_ok(cudaEventElapsedTime(&t, g_events[i], g_events[i + 1]), "cudaEventElapsedTime")) return -1;
        ms[out++] = t;
    }
    return out;
}

// ---------------------------------------------------------------------------------
// Batches: many products and convolutions in one enqueue. Members are grouped by
// transform class (kind, length, primes, sign, square); each class runs as one launch of
// every kernel of its path, with the member index in the last grid dimension.

// Scheduling of a batch run. Classes are independent: they run on 1, 2 or 4
// streams of the batch object (lanes, forked from and joined back into the
// caller's stream), so that one class's kernel tails overlap the next class's
// kernels. Which lane count is fastest depends on the composition (the sequence
// of classes with their member counts and longest results): many small classes
// gain from concurrency, a few large ones fill the GPU alone and lose L2 locality
// when they share it. So a composition that repeats is tuned on its own runs: its
// second to seventh runs try each lane count twice, timed by CUDA events on the
// caller's stream, and the fastest is captured into a CUDA graph that serves every
// later run (the members' pointers and lengths live in the device descriptors,
// uploaded before every run, so one graph serves every batch of the composition).
// A composition seen once runs with lanes picked from its size.
constexpr int kBatchLanes = 4;
constexpr size_t kBatchCompositions = 32;  // remembered per batch object
constexpr int kLaneChoices[3] = {4, 2, 1};
constexpr int kTrials = 6;                 // each lane count twice

struct Composition {
    uint64_t seen = 0;
    uint64_t used = 0;  // last use, for eviction
    int trials = 0;     // tuning runs enqueued
    cudaEvent_t t0[kTrials] = {}, t1[kTrials] = {};
    int lanes = 0;      // chosen lane count (0: not tuned yet)
    bool no_graph = false;  // its capture failed once: enqueued directly from then on
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;  // kernel nodes, counted at every replay
};

static void release_composition(Composition& c) {
    for (int i = 0; i < kTrials; ++i) {
        if (c.t0[i]) cudaEventDestroy(c.t0[i]);
        if (c.t1[i]) cudaEventDestroy(c.t1[i]);
        c.t0[i] = c.t1[i] = nullptr;
    }
    if (c.exec) cudaGraphExecDestroy(c.exec);
    c.exec = nullptr;
}

struct ntt_batch {
    int device = 0;
    DeviceBuf arena;  // residues and carry flags of every member
    DeviceBuf desc;   // member descriptors
    ProductDesc* host_desc = nullptr;
    size_t host_cap = 0;
    cudaEvent_t staged = nullptr;  // the last descriptor upload has been read
    bool pending = false;
    cudaStream_t lane[kBatchLanes] = {};
    cudaEvent_t lane_done[kBatchLanes] = {};
    cudaEvent_t fork = nullptr;
    bool graphs = true;
    int fixed_lanes = 0;  // 1..4 set by the caller, 0: tuned per composition
    int last_lanes = 0;
    uint64_t clock = 0;
    uint64_t replays = 0;
    uint64_t tuned = 0;
    std::map<std::vector<uint64_t>, Composition> comps;
};

static void destroy_batch_events(ntt_batch* b) {
    for (int i = 0; i < kBatchLanes; ++i) {
        if (b->lane[i]) cudaStreamDestroy(b->lane[i]);
        if (b->lane_done[i]) cudaEventDestroy(b->lane_done[i]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->staged) cudaEventDestroy(b->staged);
    for (auto& kv : b->comps) release_composition(kv.second);
    b->comps.clear();
}

ntt_batch* ntt_batch_new(void) {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
    ntt_batch* b = new ntt_batch();
    b->device = dev;
    bool ok = cuda_ok(cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming), "cudaEventCreate") &&
              cuda_ok(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate");
    for (int i = 0; ok && i < kBatchLanes; ++i)
        ok = cuda_ok(cudaStreamCreateWithFlags(&b->lane[i], cudaStreamNonBlocking), "cudaStreamCreate") &&
             cuda_ok(cudaEventCreateWithFlags(&b->lane_done[i], cudaEventDisableTiming), "cudaEventCreate");
    if (!ok) {
        destroy_batch_events(b);
        delete b;
        return nullptr;
    }
    return b;
}

void ntt_batch_free(ntt_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->pending) cudaEventSynchronize(b->staged);
    cudaDeviceSynchronize();
    b->arena.release();
    b->desc.release();
    if (b->host_desc) cudaFreeHost(b->host_desc);
    destroy_batch_events(b);
    delete b;
}

int ntt_batch_set_graphs(ntt_batch* b, int on) {
    if (!b) return -1;
    const int prev = b->graphs ? 1 : 0;
    if (on == 0 || on == 1) b->graphs = on == 1;
    return prev;
}

int ntt_batch_set_lanes(ntt_batch* b, int lanes) {
    if (!b) return -1;
    const int prev = b->fixed_lanes;
    if (lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4) b->fixed_lanes = lanes;
    return prev;
}

void ntt_batch_stats(const ntt_batch* b, uint64_t* out) {
    if (!out) return;
    out[0] = b ? b->replays : 0;
    out[1] = b ? b->tuned : 0;
    out[2] = b ? (uint64_t)b->last_lanes : 0;
    out[3] = b ? b->comps.size() : 0;
}

namespace {
struct Member {
    size_t index;
    Geom g;
    bool square;
    u64 offset;  // bytes into the arena
};

// Members [k, end) of one transform class, in descriptor order.
struct BatchClass {
    size_t k, end;
    Geom g;
    bool square;
    u64 max_len;
    double work;  // butterfly levels of the class
};
}  // namespace

// Lanes of a composition that is not tuned: concurrency for small batches (the
// lane count that the tuner picks for 64 to 1,024 mixed products of 256..65,536
// limbs), one stream for large ones.
static int default_lanes(const std::vector<BatchClass>& cls) {
    double work = 0;
    for (const BatchClass& c : cls) work += c.work;
    // about 1.5 ms of transforms on one GB300
    return work < 2.0e9 ? (work < 2.5e8 ? 4 : 2) : 1;
}

// Enqueues every class on `st`, spread over `lanes` streams. Returns false on a
// launch failure.
static bool enqueue_classes(ntt_batch* b, const std::vector<BatchClass>& cls, const ProductDesc* dev_desc,
                            cudaStream_t st, int lanes) {
    lanes = (int)std::min<size_t>(cls.size(), (size_t)lanes);
    b->last_lanes = lanes;
    if (lanes <= 1) {
        for (const BatchClass& c : cls)
            if (!run_members(dev_desc + c.k, (int)(c.end - c.k), c.g, c.square, c.max_len, st)) return false;
        return true;
    }
    if (!cuda_ok(cudaEventRecord(b->fork, st), "cudaEventRecord")) return false;
    for (int i = 0; i < lanes; ++i)
        if (!cuda_ok(cudaStreamWaitEvent(b->lane[i], b->fork, 0), "cudaStreamWaitEvent")) return false;
    // Largest classes first, each to the lane with the least work so far.
    std::vector<size_t> order(cls.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return cls[x].work > cls[y].work; });
    double load[kBatchLanes] = {};
    for (size_t i : order) {
        int lane = 0;
        for (int l = 1; l < lanes; ++l)
            if (load[l] < load[lane]) lane = l;
        load[lane] += cls[i].work;
        const BatchClass& c = cls[i];
        if (!run_members(dev_desc + c.k, (int)(c.end - c.k), c.g, c.square, c.max_len, b->lane[lane])) return false;
    }
    for (int i = 0; i < lanes; ++i)
        if (!cuda_ok(cudaEventRecord(b->lane_done[i], b->lane[i]), "cudaEventRecord") ||
            !cuda_ok(cudaStreamWaitEvent(st, b->lane_done[i], 0), "cudaStreamWaitEvent"))
            return false;
    return true;
}

// Kernel nodes of a captured graph.
static uint64_t graph_kernels(cudaGraph_t graph) {
    size_t n = 0;
    if (cudaGraphGetNodes(graph, nullptr, &n) != cudaSuccess || n == 0) return 0;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(graph, nodes.data(), &n) != cudaSuccess) return 0;
    uint64_t k = 0;
    for (size_t i = 0; i < n; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

// Captures the classes with `lanes` into the composition's graph and runs it.
static bool capture_and_run(ntt_batch* b, Composition& e, const std::vector<BatchClass>& cls,
                            const ProductDesc* dev_desc, cudaStream_t st, int lanes) {
    // Every table and constant the classes need exists by now (the first run built
    // them), so the capture records launches only.
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        e.no_graph = true;
        return enqueue_classes(b, cls, dev_desc, st, lanes);
    }
    t_capturing = true;
    const bool recorded = enqueue_classes(b, cls, dev_desc, st, lanes);
    t_capturing = false;
    cudaGraph_t graph = nullptr;
    const cudaError_t end = cudaStreamEndCapture(st, &graph);
    bool ok = recorded && cuda_ok(end, "cudaStreamEndCapture");
    if (ok) {
        e.kernels = graph_kernels(graph);
        ok = cuda_ok(cudaGraphInstantiate(&e.exec, graph, 0), "cudaGraphInstantiate");
    }
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {  // the capture recorded nothing that runs: enqueue directly instead
        if (e.exec) cudaGraphExecDestroy(e.exec);
        e.exec = nullptr;
        e.no_graph = true;
        cudaGetLastError();
        return enqueue_classes(b, cls, dev_desc, st, lanes);
    }
    if (!cuda_ok(cudaGraphLaunch(e.exec, st), "cudaGraphLaunch")) return false;
    note_launches(e.kernels);
    ++b->replays;
    return true;
}

// Runs the classes of one batch run (see the scheduling note above). Streams that
// cannot be captured (the legacy default stream) and batches with graphs off run
// directly, tuned lanes still applying when graphs are off.
static bool run_classes(ntt_batch* b, const std::vector<BatchClass>& cls, const ProductDesc* dev_desc,
                        cudaStream_t st) {
    const bool capturable = st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
    std::vector<uint64_t> sig;
    sig.reserve(4 * cls.size() + 2);
    sig.push_back((uint64_t)(uintptr_t)dev_desc);
    sig.push_back((uint64_t)b->fixed_lanes);
    for (const BatchClass& c : cls) {
        sig.push_back(c.end - c.k);
        sig.push_back(c.max_len);
        sig.push_back(((uint64_t)c.g.log_t << 32) | ((uint64_t)c.g.np << 16) | ((uint64_t)c.g.conv << 3) |
                      ((uint64_t)c.g.wide << 2) | ((uint64_t)(c.g.sign != 0) << 1) | (c.square ? 1u : 0u));
        sig.push_back(c.g.stride);
    }
    auto found = b->comps.find(sig);
    if (found == b->comps.end()) {
        if (b->comps.size() >= kBatchCompositions) {  // forget the least recently used composition
            auto old = b->comps.begin();
            for (auto it = b->comps.begin(); it != b->comps.end(); ++it)
                if (it->second.used < old->second.used) old = it;
            if (!cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return false;
            release_composition(old->second);
            b->comps.erase(old);
        }
        found = b->comps.emplace(sig, Composition()).first;
    }
    Composition& e = found->second;
    e.used = ++b->clock;
    ++e.seen;
    const int fixed = b->fixed_lanes;
    const bool graphs = b->graphs && capturable && !e.no_graph;
    if (!capturable) {
        const int lanes = fixed ? fixed : (e.lanes ? e.lanes : default_lanes(cls));
        return enqueue_classes(b, cls, dev_desc, st, lanes);
    }
    if (e.exec && graphs) {
        if (!cuda_ok(cudaGraphLaunch(e.exec, st), "cudaGraphLaunch")) return false;
        note_launches(e.kernels);
        ++b->replays;
        return true;
    }
    if (fixed) {  // the caller's lane count: no tuning, a graph from the second run
        if (e.seen >= 2 && graphs) return capture_and_run(b, e, cls, dev_desc, st, fixed);
        return enqueue_classes(b, cls, dev_desc, st, fixed);
    }
    if (e.seen < 2) return enqueue_classes(b, cls, dev_desc, st, e.lanes ? e.lanes : default_lanes(cls));
    if (e.lanes == 0 && e.trials < kTrials) {  // a timed tuning run
        const int i = e.trials++;
        if (!e.t0[i] && (!cuda_ok(cudaEventCreate(&e.t0[i]), "cudaEventCreate") ||
                         !cuda_ok(cudaEventCreate(&e.t1[i]), "cudaEventCreate")))
            return false;
        return cuda_ok(cudaEventRecord(e.t0[i], st), "cudaEventRecord") &&
               enqueue_classes(b, cls, dev_desc, st, kLaneChoices[i % 3]) &&
               cuda_ok(cudaEventRecord(e.t1[i], st), "cudaEventRecord");
    }
    if (e.lanes == 0) {  // every trial is enqueued: pick the fastest lane count
        float best[3] = {1e30f, 1e30f, 1e30f};
        if (!cuda_ok(cudaEventSynchronize(e.t1[kTrials - 1]), "cudaEventSynchronize")) return false;
        for (int i = 0; i < kTrials; ++i) {
            float ms = 0;
            if (cudaEventElapsedTime(&ms, e.t0[i], e.t1[i]) == cudaSuccess) best[i % 3] = std::min(best[i % 3], ms);
        }
        int pick = 0;
        for (int j = 1; j < 3; ++j)
            if (best[j] < best[pick]) pick = j;
        e.lanes = kLaneChoices[pick];
        ++b->tuned;
    }
    if (!graphs) return enqueue_classes(b, cls, dev_desc, st, e.lanes);
    return capture_and_run(b, e, cls, dev_desc, st, e.lanes);
}

uint8_t ntt_batch_run_device(ntt_batch* b, const ntt_request* reqs, size_t count, void* stream) {
    if (!b || (!reqs && count)) return fail("null argument");
    if (!cuda_ok(cudaSetDevice(b->device), "cudaSetDevice")) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (st && st != cudaStreamLegacy && st != cudaStreamPerThread &&
        (!cuda_ok(cudaStreamIsCapturing(st, &cap), "cudaStreamIsCapturing") || cap != cudaStreamCaptureStatusNone))
        return fail("the stream is being captured: a batch stages its descriptors from the host on every run "
                    "and captures its own graphs");
    // Plan every member first: a batch with an inadmissible member launches nothing.
    std::vector<Member> members;
    members.reserve(count);
    std::vector<size_t> empties;
    u64 arena_bytes = 0;
    for (size_t i = 0; i < count; ++i) {
        const ntt_request& r = reqs[i];
        Member m;
        m.index = i;
        if (r.kind == 0) {
            if (r.a_len == 0 || r.b_len == 0) {
                if ((u64)r.a_len + r.b_len > r.dst_len) return fail("destination is shorter than the product");
                empties.push_back(i);
                continue;
            }
            if (!plan_mul(r.a_len, r.b_len, m.g, false)) return 0;
        } else if (r.kind == 1) {
            if (!plan_conv(r.a_len, r.b_len, r.max_a, r.max_b, (int)r.is_signed, m.g)) return 0;
        } else {
            return fail("unknown request kind");
        }
        if (r.dst_len < m.g.out_len) return fail("destination is shorter than the result");
        m.square = r.a == r.b && r.a_len == r.b_len;
        m.offset = arena_bytes;
        arena_bytes += (m.g.scratch_bytes(m.square) + 255) & ~(u64)255;
        members.push_back(m);
    }
    for (size_t i : empties)
        if (!cuda_ok(cudaMemsetAsync(reqs[i].dst, 0, ((size_t)reqs[i].a_len + reqs[i].b_len) * 8, st), "zero product"))
            return 0;
    if (members.empty()) return 1;
    // Group by class: kind, schoolbook, transform length, primes, sign, square.
    std::sort(members.begin(), members.end(), [](const Member& x, const Member& y) {
        return std::make_tuple(x.g.conv, x.g.schoolbook, x.g.log_t, x.g.np, x.g.sign, x.square, x.index) <
               std::make_tuple(y.g.conv, y.g.schoolbook, y.g.log_t, y.g.np, y.g.sign, y.square, y.index);
    });
    if (!b->arena.ensure(std::max<u64>(arena_bytes, 256)) || !b->desc.ensure(members.size() * sizeof(ProductDesc)))
        return 0;
    if (b->pending && !cuda_ok(cudaEventSynchronize(b->staged), "descriptor staging")) return 0;
    b->pending = false;
    if (b->host_cap < members.size()) {
        if (b->host_desc) cudaFreeHost(b->host_desc);
        b->host_desc = nullptr;
        b->host_cap = 0;
        if (!cuda_ok(cudaHostAlloc((void**)&b->host_desc, members.size() * sizeof(ProductDesc), cudaHostAllocDefault),
                     "cudaHostAlloc"))
            return 0;
        b->host_cap = members.size();
    }
    uint8_t* arena = (uint8_t*)b->arena.ptr;
    for (size_t k = 0; k < members.size(); ++k) {
        const Member& m = members[k];
        const ntt_request& r = reqs[m.index];
        ProductDesc& d = b->host_desc[k];
        d.a = r.a;
        d.b = m.square ? r.a : r.b;
        d.la = r.a_len;
        d.lb = m.square ? r.a_len : r.b_len;
        d.spec = (u32*)(arena + m.offset);
        d.conv_len = m.g.conv_len;
        d.dst = r.dst;
        d.out_len = m.g.out_len;
        d.agg = m.g.conv ? nullptr : arena + m.offset + ((m.g.spec_words(m.square) * 4 + 255) & ~(u64)255);
        d.square = m.square ? 1u : 0u;
        d.stride = (u32)m.g.stride;
    }
    if (!cuda_ok(cudaMemcpyAsync(b->desc.ptr, b->host_desc, members.size() * sizeof(ProductDesc),
                                 cudaMemcpyHostToDevice, st),
                 "descriptor upload") ||
        !cuda_ok(cudaEventRecord(b->staged, st), "cudaEventRecord"))
        return 0;
    b->pending = true;
    const ProductDesc* dev_desc = (const ProductDesc*)b->desc.ptr;
    // Schoolbook convolutions take their operands as launch arguments: they run
    // directly. Every other class goes through the descriptors.
    constexpr size_t kMaxLaunchMembers = 16384;  // 2 * members fits gridDim.z
    std::vector<BatchClass> classes;
    size_t k = 0;
    while (k < members.size()) {
        const Geom& g0 = members[k].g;
        size_t end = k + 1;
        while (end < members.size() && end - k < kMaxLaunchMembers && members[end].g.conv == g0.conv &&
               members[end].g.schoolbook == g0.schoolbook && members[end].g.log_t == g0.log_t &&
               members[end].g.np == g0.np && members[end].g.sign == g0.sign &&
               members[end].square == members[k].square)
            ++end;
        if (g0.conv && g0.schoolbook) {
            for (size_t i = k; i < end; ++i) {
                const ProductDesc& d = b->host_desc[i];
                note_launches(1);
                if (!cuda_ok(launch_conv_schoolbook(d.a, d.la, d.b, d.lb, d.dst, (int)d.stride, g0.sign != 0, st),
                             "conv schoolbook launch"))
                    return 0;
            }
            k = end;
            continue;
        }
        BatchClass c;
        c.k = k;
        c.end = end;
        c.g = g0;
        c.square = members[k].square;
        c.max_len = 0;
        for (size_t i = k; i < end; ++i)
            c.max_len = std::max(c.max_len, g0.conv ? members[i].g.conv_len : members[i].g.out_len);
        c.work = (double)(end - k) * g0.np * (double)((u64)1 << g0.log_t) * g0.log_t;
        classes.push_back(c);
        k = end;
    }
    if (classes.empty()) return 1;
    // Tables and constants of every class before any capture.
    for (const BatchClass& c : classes) {
        PrimeSet ps;
        CrtParams cp;
        if (!prepare_params(c.g, ps, cp)) return 0;
    }
    return run_classes(b, classes, dev_desc, st) ? 1 : 0;
}

int ntt_split_set(int log_t, int log_r) {
    int lo = 0, hi = 0;
    if (!split_range(log_t, lo, hi) || (log_r != 0 && (log_r < lo || log_r > hi))) return -1;
    const int prev = g_split[log_t].exchange(log_r == log_t / 2 ? 0 : log_r);
    return prev ? prev : log_t / 2;
}

int ntt_split_get(int log_t) {
    int lo = 0, hi = 0;
    if (!split_range(log_t, lo, hi)) return 0;
    const int o = g_split[log_t].load();
    return o ? o : log_t / 2;
}

int ntt_split_range(int log_t, int* lo, int* hi) {
    int l = 0, h = 0;
    if (!split_range(log_t, l, h)) return 0;
    if (lo) *lo = l;
    if (hi) *hi = h;
    return 1;
}

uint8_t ntt_tune_splits(int min_log_t, int max_log_t, int reps, void* stream) {
    min_log_t = std::max(min_log_t, kMaxBlockLog + 1);
    max_log_t = std::min(max_log_t, 23);
    if (min_log_t > max_log_t) return 1;
    reps = std::max(1, reps);
    cudaStream_t st = (cudaStream_t)stream;
    const u64 half = (u64)1 << (max_log_t - 1);
    u64 *a = nullptr, *b = nullptr, *dst = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ntt_mul_workspace* ws = ntt_mul_workspace_new();
    bool ok = ws && cuda_ok(cudaMalloc(&a, half * 8), "cudaMalloc") && cuda_ok(cudaMalloc(&b, half * 8), "cudaMalloc") &&
              cuda_ok(cudaMalloc(&dst, 2 * half * 8), "cudaMalloc") &&
              cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") && cuda_ok(cudaEventCreate(&e1), "cudaEventCreate") &&
              cuda_ok(cudaMemsetAsync(a, 0xA5, half * 8, st), "cudaMemset") &&
              cuda_ok(cudaMemsetAsync(b, 0x3C, half * 8, st), "cudaMemset");
    for (int log_t = min_log_t; ok && log_t <= max_log_t; ++log_t) {
        int lo = 0, hi = 0;
        if (!split_range(log_t, lo, hi) || lo == hi) continue;
        // operands of 2^(log_t - 1) limbs: the product fills the transform
        const u64 n = (u64)1 << (log_t - 1);
        const int before = g_split[log_t].load();
        float best = 1e30f, standard = 1e30f;
        int pick = log_t / 2;
        for (int r = lo; ok && r <= hi; ++r) {
            g_split[log_t].store(r == log_t / 2 ? 0 : r);
            ok = ntt_mul_workspace_mul_device(ws, dst, 2 * n, a, n, b, n, st) == 1;  // tables, warm-up
            float ms = 1e30f;
            for (int round = 0; ok && round < 2; ++round) {
                ok = cuda_ok(cudaEventRecord(e0, st), "cudaEventRecord");
                for (int i = 0; ok && i < reps; ++i) ok = ntt_mul_workspace_mul_device(ws, dst, 2 * n, a, n, b, n, st) == 1;
                float t = 0;
                ok = ok && cuda_ok(cudaEventRecord(e1, st), "cudaEventRecord") &&
                     cuda_ok(cudaEventSynchronize(e1), "cudaEventSynchronize") &&
                     cuda_ok(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime");
                ms = std::min(ms, t / reps);
            }
            if (r == log_t / 2) standard = ms;
            if (ms < best) {
                best = ms;
                pick = r;
            }
        }
        if (!ok) {  // a failed trial leaves the split as it was
            g_split[log_t].store(before);
            break;
        }
        // another split only when it is at least 2% faster than the default
        if (!(best < 0.98f * standard)) pick = log_t / 2;
        g_split[log_t].store(pick == log_t / 2 ? 0 : pick);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (ws) ntt_mul_workspace_free(ws);
    if (a) cudaFree(a);
    if (b) cudaFree(b);
    if (dst) cudaFree(dst);
    return ok ? 1 : 0;
}

uint32_t ntt_lookback_timeouts(void) { return lookback_timeouts(); }

const char* ntt_last_error(void) { return g_error.c_str(); }
uint64_t ntt_kernel_launches(void) { return g_launches.load(); }
const char* ntt_version(void) { return "nttanafis_gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
