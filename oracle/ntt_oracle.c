/*
 * CPU restatement of ntt_anafis's multiplication path. TEST INFRASTRUCTURE ONLY:
 * the parity checker and the timed CPU baseline. Nothing in the product links it.
 *
 * It follows the reference crate's algorithm (paths relative to its root):
 *   - prime catalog and generators        src/field/catalog.rs:67-76
 *   - exact f64 remainder a*b - q*p      src/arch/scalar/product.rs:95-109
 *   - planner (profiles, widest chunk, row shape, cost 3*transform + crt)
 *                                          src/profile/planner.rs:120-322,401-422,558-591,
 *                                          src/profile/catalog.rs:20-45
 *   - packing into chunk_bits coefficients split in 49-bit parts
 *                                          src/limb/packing.rs:113-301,
 *                                          src/arch/schedule/expression/packing.rs:14-108
 *   - cyclic NTT per prime, pointwise product, inverse scaled by N^-1 (P/p_i)^-1
 *                                          src/transform/forward.rs:95-298,
 *                                          src/transform/inverse.rs:52-218,
 *                                          src/multiply/schedule.rs:160-279
 *   - cofactor CRT with one top-word quotient
 *                                          src/limb/cofactor.rs:59-301
 *   - reconstruction at bit i*w with carries, signed offset 2^s
 *                                          src/limb/reconstruction.rs:77-483
 *   - convolution plans, bounds, direct column sums
 *                                          src/convolve.rs:75-369
 * Simplifications that change no output value: the transform length is the power
 * of two >= the convolution length (the reference's 5N/4, 3N/2, 7N/4 rows are
 * remainder-tree tails of the same cyclic product), no block split of unbalanced
 * operands (src/profile/planner.rs:291-393 only reorders work), radix-2 stages
 * with canonical residues instead of lazy radix-4/16 leaves, and a pthread pool
 * over primes, operands and coefficient ranges in place of rayon.
 */
#include "ntt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;
typedef uint64_t u64;

#define MAX_PRIMES 8
#define MODULUS_BITS 50
#define PART_BITS 49
#define MAX_PARTS 4
#define MAX_CHUNK_BITS (PART_BITS * MAX_PARTS)
#define MIN_TRANSFORM_LEN 32
#define COLUMN_ALIGN 8
#define WORDS 7 /* ceil(8*50/64) */
#define LIMB_BITS 64
#define SCHOOLBOOK_MAX_TERMS 24

static const u64 CAT_P[MAX_PRIMES] = {
    1108307720798209ull, 1086317488242689ull, 910395627798529ull, 659706976665601ull,
    699289395265537ull,  1022545813831681ull, 1013749720809473ull, 868614185943041ull,
};
static const u64 CAT_G[MAX_PRIMES] = {11, 3, 7, 11, 5, 7, 3, 3};

static u64 mulmod_int(u64 a, u64 b, u64 p) { return (u64)((u128)a * b % p); }
static u64 powmod_int(u64 a, u64 e, u64 p) {
    u64 r = 1 % p;
    a %= p;
    while (e) {
        if (e & 1) r = mulmod_int(r, a, p);
        a = mulmod_int(a, a, p);
        e >>= 1;
    }
    return r;
}
static int max_root_order(void) {
    int order = 64;
    for (int i = 0; i < MAX_PRIMES; ++i) {
        const int v = __builtin_ctzll(CAT_P[i] - 1);
        if (v < order) order = v;
    }
    return order;
}

/* ------------------------------------------------------------------------------
 * Cofactor tables, src/limb/cofactor.rs:136-301 */
typedef struct {
    u64 inverses[MAX_PRIMES];
    u64 factors[MAX_PRIMES][WORDS];
    u64 multiples[MAX_PRIMES][WORDS];
    int capacity;
    u64 quotient_factor;
} Cofactors;

static Cofactors COF[MAX_PRIMES];
static pthread_once_t COF_ONCE = PTHREAD_ONCE_INIT;

static int capacity_of(const u64* product, int words) {
    const u64 top = product[words - 1];
    const int bits = (words - 1) * 64 + (64 - __builtin_clzll(top));
    const int second = bits - 2;
    return ((product[second >> 6] >> (second % 64)) & 1) ? bits - 1 : second;
}

static void cofactor_tables(void) {
    u64 product[WORDS] = {1, 0, 0, 0, 0, 0, 0};
    int words = 1;
    for (int count = 0; count < MAX_PRIMES; ++count) {
        const u64 p = CAT_P[count];
        u128 carry = 0;
        for (int i = 0; i < words; ++i) {
            const u128 full = (u128)product[i] * p + carry;
            product[i] = (u64)full;
            carry = full >> 64;
        }
        if (carry) product[words++] = (u64)carry;
        Cofactors* t = &COF[count];
        memset(t, 0, sizeof(*t));
        for (int row = 0; row <= count; ++row) {
            const u64 q = CAT_P[row];
            u128 rem = 0;
            for (int i = words - 1; i >= 0; --i) {
                const u128 dividend = (rem << 64) | product[i];
                t->factors[row][i] = (u64)(dividend / q);
                rem = dividend % q;
            }
            rem = 0;
            for (int i = words - 1; i >= 0; --i) rem = ((rem << 64) | t->factors[row][i]) % q;
            t->inverses[row] = powmod_int((u64)rem, q - 2, q);
        }
        u64 multiple[WORDS] = {0};
        for (int quotient = 0; quotient <= count; ++quotient) {
            memcpy(t->multiples[quotient], multiple, sizeof(multiple));
            int overflow = 0;
            for (int w = 0; w < WORDS; ++w) {
                const u128 s = (u128)multiple[w] + product[w] + (u64)overflow;
                multiple[w] = (u64)s;
                overflow = (int)(s >> 64);
            }
        }
        t->capacity = capacity_of(product, words);
        const int cw = (t->capacity + 63) / 64;
        const int top = cw - 1;
        const u64 low = top == 0 ? 0 : product[top - 1];
        const u128 leading = ((u128)product[top] << 64) | low;
        t->quotient_factor = (u64)(~(u128)0 / (leading + 1));
    }
}
static const Cofactors* cof_of(int count) {
    pthread_once(&COF_ONCE, cofactor_tables);
    return &COF[count - 1];
}

int oracle_capacity(int count) { return count >= 1 && count <= MAX_PRIMES ? cof_of(count)->capacity : -1; }

/* Cofactors::bounded (src/limb/cofactor.rs:59-111): residues already weighted by
 * the inverses; writes ceil(capacity/64) words of X. Instantiated per prime count
 * (cof_bounded below) so that the word loops unroll. */
static inline __attribute__((always_inline)) void cof_bounded_n(const Cofactors* t, const int count,
                                                                const u64* residue, u64* value) {
    const int words = (t->capacity + 63) / 64;
    const int factor_words = count == 1 ? 1 : (MODULUS_BITS * (count - 1) + 63) / 64;
    u128 carry = 0;
    for (int w = 0; w < words; ++w) {
        u128 sum = carry;
        if (w < factor_words)
            for (int row = 0; row < count; ++row) sum += (u128)t->factors[row][w] * residue[row];
        carry = sum >> 64;
        value[w] = (u64)sum;
    }
    const u64 top = value[words - 1];
    const u128 estimate = (u128)top * t->quotient_factor + ((u128)1 << 62);
    const u64* multiple = t->multiples[(int)(estimate >> 64)];
    u64 borrow = 0;
    for (int w = 0; w < words; ++w) {
        const u64 m = multiple[w];
        const u64 v = value[w];
        const u64 d = v - m - borrow;
        borrow = (v < m) || (v - m < borrow);
        value[w] = d;
    }
}
static void cof_bounded(const Cofactors* t, int count, const u64* residue, u64* value) {
    switch (count) {
#define COUNT_CASE(c) \
    case c: cof_bounded_n(t, c, residue, value); break;
        COUNT_CASE(1) COUNT_CASE(2) COUNT_CASE(3) COUNT_CASE(4) COUNT_CASE(5) COUNT_CASE(6) COUNT_CASE(7)
        COUNT_CASE(8)
#undef COUNT_CASE
    }
}

/* ------------------------------------------------------------------------------
 * Planner, src/profile/planner.rs */
typedef struct {
    int count;
    int chunk_bits;
    u64 digits_a, digits_b;
    int value_bits_a, value_bits_b;
    u64 conv_len;
    u64 transform_len, cyclic_len, table_len;
    u64 output_stride; /* bits */
    int disjoint;
    int sign_bit; /* -1: unsigned */
} Geometry;

static int clz_u64(u64 x) { return x ? __builtin_clzll(x) : 64; }
static int log_terms(u64 terms) { return 64 - clz_u64(terms - 1); }
static u64 div_ceil(u64 a, u64 b) { return (a + b - 1) / b; }
static u64 next_pow2(u64 x) {
    u64 p = 1;
    while (p < x) p <<= 1;
    return p;
}

/* product_bits, src/profile/planner.rs:558 */
static int product_bits(u64 width, u64 terms) { return (int)(2 * width) + log_terms(terms); }

/* row_shape, src/profile/planner.rs:573-591 */
static void row_shape(u64 conv_len, u64 longest, u64* t, u64* c, u64* tab) {
    u64 power = next_pow2(conv_len);
    if (power < MIN_TRANSFORM_LEN) power = MIN_TRANSFORM_LEN;
    const u64 cyclic = power >> 1, half = power >> 2, quarter = power >> 3;
    if (longest <= cyclic) {
        if (quarter >= MIN_TRANSFORM_LEN && conv_len <= cyclic + quarter) {
            *t = cyclic + quarter; *c = cyclic; *tab = cyclic; return;
        }
        if (half >= MIN_TRANSFORM_LEN && conv_len <= cyclic + half) {
            *t = cyclic + half; *c = cyclic; *tab = cyclic; return;
        }
        if (quarter >= MIN_TRANSFORM_LEN && conv_len <= cyclic + half + quarter) {
            *t = cyclic + half + quarter; *c = cyclic; *tab = cyclic; return;
        }
    }
    *t = power; *c = power; *tab = cyclic;
}

int oracle_row_shape(uint64_t conv_len, uint64_t longest, uint64_t* out3) {
    row_shape(conv_len, longest, &out3[0], &out3[1], &out3[2]);
    return 1;
}

/* Geometry::admit, src/profile/planner.rs:211-287 (blocks: -1 none, 0/1 unsigned/signed) */
static int admit(int count, int chunk, u64 da, int vba, u64 db, int vbb, int coefficient_bits,
                 u64 output_stride, int blocks, Geometry* g) {
    const int disjoint = blocks >= 0;
    int sign_bit = -1;
    if (blocks == 1) {
        if (coefficient_bits < 1) return 0;
        sign_bit = coefficient_bits - 1;
    }
    const u64 longest = da > db ? da : db;
    if (chunk > MAX_CHUNK_BITS || vba > chunk || vbb > chunk) return 0;
    if (coefficient_bits > cof_of(count)->capacity) return 0;
    if (disjoint && !(output_stride % LIMB_BITS == 0 && output_stride >= (u64)coefficient_bits)) return 0;
    if (longest > (~(u64)0) / (u64)chunk) return 0;
    const u64 conv_len = da + db - 1;
    u64 t, c, tab;
    row_shape(conv_len, longest, &t, &c, &tab);
    if (__builtin_ctzll(tab * 2) > max_root_order()) return 0;
    g->count = count;
    g->chunk_bits = chunk;
    g->digits_a = da;
    g->digits_b = db;
    g->value_bits_a = vba;
    g->value_bits_b = vbb;
    g->conv_len = conv_len;
    g->transform_len = t;
    g->cyclic_len = c;
    g->table_len = tab;
    g->output_stride = output_stride;
    g->disjoint = disjoint;
    g->sign_bit = sign_bit;
    return 1;
}

/* Geometry::under, src/profile/planner.rs:190-208 */
static int under(u64 bits_a, u64 bits_b, int count, int chunk, Geometry* g) {
    const u64 da = div_ceil(bits_a, chunk), db = div_ceil(bits_b, chunk);
    return admit(count, chunk, da, chunk, db, chunk, product_bits(chunk, da < db ? da : db), chunk, -1, g);
}

/* start chunks of PROFILES, src/profile/catalog.rs:26-45 */
static int profile_chunk(int count) {
    const int half = cof_of(count)->capacity >> 1;
    return half < MAX_CHUNK_BITS ? half : MAX_CHUNK_BITS;
}

/* Geometry::widest_under, src/profile/planner.rs:168-183 */
static int widest_under(u64 bits_a, u64 bits_b, int count, Geometry* g) {
    int width = profile_chunk(count);
    for (;;) {
        const u64 ta = div_ceil(bits_a, width), tb = div_ceil(bits_b, width);
        const int pb = product_bits(width, ta < tb ? ta : tb);
        const int cap = cof_of(count)->capacity;
        const int excess = pb > cap ? pb - cap : 0;
        if (excess == 0) return under(bits_a, bits_b, count, width, g);
        width -= (excess + 1) / 2;
        if (width <= 0) return 0;
    }
}

/* Geometry::work, src/profile/planner.rs:401-422 */
static void work(const Geometry* g, int crt_cost, u128* transform, u128* crt) {
    const u128 overhead = 4;
    const u64 tail = g->transform_len - g->cyclic_len;
    const u64 low_tail = tail & (0 - tail);
    const u64 high_tail = tail - low_tail;
#define PART(n) ((u128)(n) * (u128)((n) ? __builtin_ctzll(n) : 64))
    const u128 w = PART(g->cyclic_len) + PART(high_tail) + PART(low_tail) + (u128)tail * overhead;
#undef PART
    *transform = (u128)g->count * w;
    *crt = (u128)crt_cost * g->count * (g->count - 1) * g->conv_len;
}

/* Geometry::select, src/profile/planner.rs:147-161 */
static int select_geometry(u64 la, u64 lb, int crt_cost, Geometry* out) {
    if (!la || !lb || la > (~(u64)0) / 64 || lb > (~(u64)0) / 64) return 0;
    const u64 bits_a = la * 64, bits_b = lb * 64;
    int found = 0;
    u128 best = 0;
    for (int count = 1; count <= MAX_PRIMES; ++count) {
        Geometry g;
        if (!widest_under(bits_a, bits_b, count, &g)) continue;
        u128 tr, crt;
        work(&g, crt_cost, &tr, &crt);
        const u128 score = tr * 3 + crt;
        if (!found || score < best) {
            best = score;
            *out = g;
            found = 1;
        }
    }
    return found;
}

/* Geometry::for_residues, src/profile/planner.rs:120-139 */
static int for_residues(u64 la, u64 lb, int vba, int vbb, int bound_bits, u64 stride_bits, int is_signed,
                        Geometry* g) {
    for (int count = 1; count <= MAX_PRIMES; ++count)
        if (cof_of(count)->capacity >= bound_bits)
            return admit(count, LIMB_BITS, la, vba, lb, vbb, bound_bits, stride_bits, is_signed ? 1 : 0, g);
    return 0;
}

int oracle_mul_plan(uint64_t la, uint64_t lb, int crt_cost, int64_t* out) {
    Geometry g;
    if (!select_geometry(la, lb, crt_cost, &g)) return 0;
    out[0] = g.count;
    out[1] = g.chunk_bits;
    out[2] = (int64_t)g.digits_a;
    out[3] = (int64_t)g.digits_b;
    out[4] = (int64_t)g.conv_len;
    out[5] = (int64_t)g.transform_len;
    out[6] = (int64_t)g.cyclic_len;
    out[7] = (int64_t)g.table_len;
    return 1;
}

/* bound_bits, src/convolve.rs:358-369 */
static int bound_bits_of(u64 terms, u64 max_a, u64 max_b) {
    const u128 product = (u128)max_a * max_b;
    const u128 bound = product * terms;
    if (terms == 0 || bound / terms == product) {
        const u64 hi = (u64)(bound >> 64), lo = (u64)bound;
        return hi ? 128 - __builtin_clzll(hi) : (lo ? 64 - __builtin_clzll(lo) : 0);
    }
    const u64 hi = (u64)(product >> 64), lo = (u64)product;
    const int pb = hi ? 128 - __builtin_clzll(hi) : (lo ? 64 - __builtin_clzll(lo) : 0);
    return pb + log_terms(terms);
}

typedef struct {
    Geometry g;
    u64 stride; /* limbs */
    int bound_bits;
    int schoolbook;
    int is_signed;
    u64 max_a, max_b;
    u64 output_len;
} ConvPlan;

/* ConvPlan::new, src/convolve.rs:75-116 (without the block split) */
static int conv_plan(u64 la, u64 lb, u64 max_a, u64 max_b, int is_signed, ConvPlan* cp) {
    if (!la || !lb) return 0;
    const u64 shorter = la < lb ? la : lb;
    const int sign = is_signed ? 1 : 0;
    const int bb = bound_bits_of(shorter, max_a, max_b) + sign;
    const u64 stride = bb ? div_ceil((u64)bb, LIMB_BITS) : 1;
    int vb[2];
    const u64 maxes[2] = {max_a, max_b};
    for (int i = 0; i < 2; ++i) {
        int bits = (64 - clz_u64(maxes[i])) + sign;
        if (bits == 0) bits = 1;
        if (bits > LIMB_BITS) return 0;
        vb[i] = bits;
    }
    memset(cp, 0, sizeof(*cp));
    if (!for_residues(la, lb, vb[0], vb[1], bb, stride * LIMB_BITS, is_signed, &cp->g)) return 0;
    cp->stride = stride;
    cp->bound_bits = bb;
    cp->schoolbook = shorter <= SCHOOLBOOK_MAX_TERMS;
    cp->is_signed = sign;
    cp->max_a = max_a;
    cp->max_b = max_b;
    cp->output_len = (la + lb - 1) * stride;
    return 1;
}

int oracle_conv_plan(uint64_t la, uint64_t lb, uint64_t max_a, uint64_t max_b, int is_signed, int64_t* out) {
    ConvPlan cp;
    if (!conv_plan(la, lb, max_a, max_b, is_signed, &cp)) return 0;
    out[0] = cp.g.count;
    out[1] = (int64_t)cp.stride;
    out[2] = cp.bound_bits;
    out[3] = cp.schoolbook;
    out[4] = (int64_t)cp.g.transform_len;
    out[5] = (int64_t)cp.g.cyclic_len;
    out[6] = (int64_t)cp.g.table_len;
    out[7] = (int64_t)cp.output_len;
    return 1;
}

/* ------------------------------------------------------------------------------
 * Exact f64 residue arithmetic, src/arch/scalar/product.rs:95-109 */
static const double ROUND_BIAS = 6755399441055744.0; /* 1.5 * 2^52 */

static inline double nearest(double x) { return (x + ROUND_BIAS) - ROUND_BIAS; }

/* a*b mod p for canonical a, b; the remainder a*b - q*p is exact (FMA). */
static inline double fmulmod(double a, double b, double p, double pinv) {
    const double h = a * b;
    const double l = fma(a, b, -h);
    const double q = nearest(h * pinv);
    double r = fma(-q, p, h) + l;
    r = r < 0.0 ? r + p : r;
    r = r >= p ? r - p : r;
    return r;
}
static inline double addmod(double a, double b, double p) {
    const double s = a + b;
    return s >= p ? s - p : s;
}
static inline double submod(double a, double b, double p) {
    const double d = a - b;
    return d < 0.0 ? d + p : d;
}

typedef struct {
    double p, pinv;
    u64 pi;
    double* tw;  /* w^j, j < n/2, forward (radix-2 transforms only) */
    double* itw; /* w^-j */
    u64 n;
    int prime;
} Field;

/* tables: also build the radix-2 transforms' twiddles (the cache-blocked ones keep
 * their own, retained across calls). */
static int field_init(Field* f, int prime, u64 n, int tables) {
    f->pi = CAT_P[prime];
    f->p = (double)f->pi;
    f->pinv = 1.0 / f->p;
    f->n = n;
    f->prime = prime;
    f->tw = f->itw = NULL;
    if (!tables) return 1;
    const u64 half = n / 2 ? n / 2 : 1;
    f->tw = (double*)malloc(half * sizeof(double));
    f->itw = (double*)malloc(half * sizeof(double));
    if (!f->tw || !f->itw) return 0;
    const u64 w = powmod_int(CAT_G[prime], (f->pi - 1) / n, f->pi);
    const u64 iw = powmod_int(w, f->pi - 2, f->pi);
    u64 x = 1, ix = 1;
    for (u64 j = 0; j < half; ++j) {
        f->tw[j] = (double)x;
        f->itw[j] = (double)ix;
        x = mulmod_int(x, w, f->pi);
        ix = mulmod_int(ix, iw, f->pi);
    }
    return 1;
}
static void field_free(Field* f) {
    free(f->tw);
    free(f->itw);
}

/* Decimation-in-frequency cyclic NTT: natural order in, bit-reversed out. */
static void ntt_forward(double* a, const Field* f) {
    const u64 n = f->n;
    const double p = f->p, pinv = f->pinv;
    for (u64 h = n / 2, stride = 1; h >= 1; h >>= 1, stride <<= 1) {
        for (u64 blk = 0; blk < n; blk += 2 * h) {
            double* x = a + blk;
            double* y = x + h;
            for (u64 j = 0; j < h; ++j) {
                const double u = x[j], v = y[j];
                x[j] = addmod(u, v, p);
                y[j] = fmulmod(submod(u, v, p), f->tw[j * stride], p, pinv);
            }
        }
    }
}

/* Decimation-in-time inverse: bit-reversed in, natural out, unscaled. */
static void ntt_inverse(double* a, const Field* f) {
    const u64 n = f->n;
    const double p = f->p, pinv = f->pinv;
    for (u64 h = 1, stride = n / 2; h < n; h <<= 1, stride >>= 1) {
        for (u64 blk = 0; blk < n; blk += 2 * h) {
            double* x = a + blk;
            double* y = x + h;
            for (u64 j = 0; j < h; ++j) {
                const double t = fmulmod(y[j], f->itw[j * stride], p, pinv);
                const double u = x[j];
                x[j] = addmod(u, t, p);
                y[j] = submod(u, t, p);
            }
        }
    }
}

/* ------------------------------------------------------------------------------
 * Cache-blocked transforms (the timed CPU path; src/transform/forward.rs:95-298,
 * src/transform/inverse.rs:52-218 restated): the same cyclic DIF / DIT as
 * ntt_forward / ntt_inverse above, depth first so that every sub-transform of up
 * to 2^BLOCK_LOG points runs in cache, two levels per pass over memory above that,
 * twiddles from per-level contiguous tables retained across calls (the reference's
 * workspaces retain theirs, src/transform/twiddle.rs:50), and branch-free centred
 * residues: every stored value lies in (-1.5p, 1.5p); sums are reduced by the
 * nearest multiple of p, products by the exact FMA remainder without the final
 * corrections (src/arch/scalar/product.rs:95-109). The output is canonicalised, so
 * it equals the radix-2 transforms' bit for bit (oracle_transform_check). */
#define BLOCK_LOG 12

static inline double reduce_c(double v, double p, double pinv) { return fma(-nearest(v * pinv), p, v); }
static inline double mul_c(double a, double b, double p, double pinv) {
    const double h = a * b;
    const double l = fma(a, b, -h);
    const double q = nearest(h * pinv);
    return fma(-q, p, h) + l;
}
static inline double canon_c(double v, double p) {
    v = v < 0.0 ? v + p : v;
    v = v < 0.0 ? v + p : v;
    v = v >= p ? v - p : v;
    return v >= p ? v - p : v;
}

/* Level-major centred roots of one prime and transform length, retained: L[h + j]
 * = w_{2h}^j and IL[h + j] = w_{2h}^-j for h = 1, 2, ..., n/2 and j < h. Up to
 * TABLE_BUDGET bytes are kept across calls; beyond that a call builds private
 * tables and frees them (level_tables_release). */
typedef struct {
    u64 pi;
    int log_n;
    int cached;
    double* fwd;
    double* inv;
} LevelTables;

#define MAX_TABLES 64
#define TABLE_BUDGET ((u64)1 << 31)
static LevelTables TABLES[MAX_TABLES];
static int TABLE_COUNT = 0;
static u64 TABLE_BYTES = 0;
static pthread_mutex_t TABLE_LOCK = PTHREAD_MUTEX_INITIALIZER;

static int build_tables(LevelTables* t, int prime, int log_n) {
    const u64 pi = CAT_P[prime], n = 1ull << log_n;
    t->pi = pi;
    t->log_n = log_n;
    t->fwd = (double*)malloc(n * sizeof(double));
    t->inv = (double*)malloc(n * sizeof(double));
    u64* top = (u64*)malloc((n / 2 + 1) * sizeof(u64));
    u64* itop = (u64*)malloc((n / 2 + 1) * sizeof(u64));
    const int ok = t->fwd && t->inv && top && itop;
    if (ok) {
        const u64 w = powmod_int(CAT_G[prime], (pi - 1) / n, pi);
        const u64 iw = powmod_int(w, pi - 2, pi);
        u64 x = 1, ix = 1;
        for (u64 j = 0; j < n / 2; ++j) {
            top[j] = x;
            itop[j] = ix;
            x = mulmod_int(x, w, pi);
            ix = mulmod_int(ix, iw, pi);
        }
        const double pd = (double)pi;
        t->fwd[0] = t->inv[0] = 1.0;
        for (u64 h = 1; h < n; h <<= 1)
            for (u64 j = 0; j < h; ++j) {
                const u64 a = top[j * (n / (2 * h))], b = itop[j * (n / (2 * h))];
                t->fwd[h + j] = a > pi / 2 ? (double)a - pd : (double)a;
                t->inv[h + j] = b > pi / 2 ? (double)b - pd : (double)b;
            }
    } else {
        free(t->fwd);
        free(t->inv);
        t->fwd = t->inv = NULL;
    }
    free(top);
    free(itop);
    return ok;
}

/* Tables of (prime, 2^log_n) in *out: the retained copy, or private ones. */
static int level_tables(int prime, int log_n, LevelTables* out) {
    const u64 pi = CAT_P[prime], bytes = (2ull << log_n) * sizeof(double);
    pthread_mutex_lock(&TABLE_LOCK);
    for (int i = 0; i < TABLE_COUNT; ++i)
        if (TABLES[i].pi == pi && TABLES[i].log_n == log_n) {
            *out = TABLES[i];
            pthread_mutex_unlock(&TABLE_LOCK);
            return 1;
        }
    int ok;
    if (TABLE_COUNT < MAX_TABLES && TABLE_BYTES + bytes <= TABLE_BUDGET) {
        ok = build_tables(&TABLES[TABLE_COUNT], prime, log_n);
        if (ok) {
            TABLES[TABLE_COUNT].cached = 1;
            TABLE_BYTES += bytes;
            *out = TABLES[TABLE_COUNT++];
        }
        pthread_mutex_unlock(&TABLE_LOCK);
        return ok;
    }
    pthread_mutex_unlock(&TABLE_LOCK);
    ok = build_tables(out, prime, log_n);
    out->cached = 0;
    return ok;
}

static void level_tables_release(LevelTables* t) {
    if (t->cached) return;
    free(t->fwd);
    free(t->inv);
}

/* One radix-4 DIF step, half-sizes 2q then q, on x[j], x[j+q], x[j+2q], x[j+3q]
 * for j < count: w1 = roots of half-size 2q at j, w1h at j + q, w2 = roots of
 * half-size q at j. */
static void dif4_q(double* restrict x0, double* restrict x1, double* restrict x2, double* restrict x3, u64 count,
                   const double* restrict w1, const double* restrict w1h, const double* restrict w2, double p,
                   double pinv) {
    for (u64 j = 0; j < count; ++j) {
        const double a0 = x0[j], a1 = x1[j], a2 = x2[j], a3 = x3[j];
        const double b0 = reduce_c(a0 + a2, p, pinv), b2 = mul_c(a0 - a2, w1[j], p, pinv);
        const double b1 = reduce_c(a1 + a3, p, pinv), b3 = mul_c(a1 - a3, w1h[j], p, pinv);
        x0[j] = reduce_c(b0 + b1, p, pinv);
        x1[j] = mul_c(b0 - b1, w2[j], p, pinv);
        x2[j] = reduce_c(b2 + b3, p, pinv);
        x3[j] = mul_c(b2 - b3, w2[j], p, pinv);
    }
}

/* One radix-4 DIT step, half-sizes q then 2q (the inverse of dif4's shape). */
static void dit4_q(double* restrict x0, double* restrict x1, double* restrict x2, double* restrict x3, u64 count,
                   const double* restrict w2, const double* restrict w1, const double* restrict w1h, double p,
                   double pinv) {
    for (u64 j = 0; j < count; ++j) {
        const double a0 = x0[j], a1 = x1[j], a2 = x2[j], a3 = x3[j];
        const double t1 = mul_c(a1, w2[j], p, pinv), t3 = mul_c(a3, w2[j], p, pinv);
        const double b0 = reduce_c(a0 + t1, p, pinv), b1 = reduce_c(a0 - t1, p, pinv);
        const double b2 = reduce_c(a2 + t3, p, pinv), b3 = reduce_c(a2 - t3, p, pinv);
        const double u = mul_c(b2, w1[j], p, pinv), v = mul_c(b3, w1h[j], p, pinv);
        x0[j] = reduce_c(b0 + u, p, pinv);
        x2[j] = reduce_c(b0 - u, p, pinv);
        x1[j] = reduce_c(b1 + v, p, pinv);
        x3[j] = reduce_c(b1 - v, p, pinv);
    }
}

/* The quarters of x as separate restrict-qualified arrays (count <= q). */
static void dif4(double* x, u64 q, u64 count, const double* w1, const double* w1h, const double* w2, double p,
                 double pinv) {
    dif4_q(x, x + q, x + 2 * q, x + 3 * q, count, w1, w1h, w2, p, pinv);
}
static void dit4(double* x, u64 q, u64 count, const double* w2, const double* w1, const double* w1h, double p,
                 double pinv) {
    dit4_q(x, x + q, x + 2 * q, x + 3 * q, count, w2, w1, w1h, p, pinv);
}

/* The last two DIF levels (half-sizes 2 and 1) of every group of four, vectorised
 * across groups (stride-4 loads and stores). */
static void dif4_leaf(double* restrict a, u64 m, const double* L, double p, double pinv) {
    const double c1 = L[1], c2 = L[2], c3 = L[3];
    for (u64 i = 0; i < m; i += 4) {
        const double a0 = a[i], a1 = a[i + 1], a2 = a[i + 2], a3 = a[i + 3];
        const double b0 = reduce_c(a0 + a2, p, pinv), b2 = mul_c(a0 - a2, c2, p, pinv);
        const double b1 = reduce_c(a1 + a3, p, pinv), b3 = mul_c(a1 - a3, c3, p, pinv);
        a[i] = reduce_c(b0 + b1, p, pinv);
        a[i + 1] = mul_c(b0 - b1, c1, p, pinv);
        a[i + 2] = reduce_c(b2 + b3, p, pinv);
        a[i + 3] = mul_c(b2 - b3, c1, p, pinv);
    }
}
static void dit4_leaf(double* restrict a, u64 m, const double* IL, double p, double pinv) {
    const double c1 = IL[1], c2 = IL[2], c3 = IL[3];
    for (u64 i = 0; i < m; i += 4) {
        const double a0 = a[i], a1 = a[i + 1], a2 = a[i + 2], a3 = a[i + 3];
        const double t1 = mul_c(a1, c1, p, pinv), t3 = mul_c(a3, c1, p, pinv);
        const double b0 = reduce_c(a0 + t1, p, pinv), b1 = reduce_c(a0 - t1, p, pinv);
        const double b2 = reduce_c(a2 + t3, p, pinv), b3 = reduce_c(a2 - t3, p, pinv);
        const double u = mul_c(b2, c2, p, pinv), v = mul_c(b3, c3, p, pinv);
        a[i] = reduce_c(b0 + u, p, pinv);
        a[i + 2] = reduce_c(b0 - u, p, pinv);
        a[i + 1] = reduce_c(b1 + v, p, pinv);
        a[i + 3] = reduce_c(b1 - v, p, pinv);
    }
}

static int log2_u64(u64 m) { return 63 - clz_u64(m); }

/* One radix-2 level of half-size h over a[0, m). */
static void dif2(double* a, u64 m, u64 h, const double* L, double p, double pinv) {
    for (u64 blk = 0; blk < m; blk += 2 * h) {
        double* restrict x = a + blk;
        double* restrict y = x + h;
        const double* w = L + h;
        for (u64 j = 0; j < h; ++j) {
            const double u = x[j], v = y[j];
            x[j] = reduce_c(u + v, p, pinv);
            y[j] = mul_c(u - v, w[j], p, pinv);
        }
    }
}
static void dit2(double* a, u64 m, u64 h, const double* IL, double p, double pinv) {
    for (u64 blk = 0; blk < m; blk += 2 * h) {
        double* restrict x = a + blk;
        double* restrict y = x + h;
        const double* w = IL + h;
        for (u64 j = 0; j < h; ++j) {
            const double t = mul_c(y[j], w[j], p, pinv);
            const double u = x[j];
            x[j] = reduce_c(u + t, p, pinv);
            y[j] = reduce_c(u - t, p, pinv);
        }
    }
}

/* All DIF levels (half-sizes m/2 down to 1) of a[0, m) in cache: one radix-2
 * level first when log2 m is odd, then radix-4 steps, the last across groups. */
static void dif_block(double* a, u64 m, const double* L, double p, double pinv) {
    if (m < 2) return;
    u64 s = m;
    if (log2_u64(m) & 1) {
        dif2(a, m, m / 2, L, p, pinv);
        s = m / 2;
    }
    for (; s >= 16; s /= 4)
        for (u64 blk = 0; blk < m; blk += s) {
            const u64 q = s / 4;
            dif4(a + blk, q, q, L + 2 * q, L + 3 * q, L + q, p, pinv);
        }
    if (s == 4) dif4_leaf(a, m, L, p, pinv);
}

/* All DIT levels (half-sizes 1 up to m/2) of a[0, m) in cache (unscaled). */
static void dit_block(double* a, u64 m, const double* IL, double p, double pinv) {
    if (m < 2) return;
    const int lg = log2_u64(m);
    if (lg >= 2) {
        dit4_leaf(a, m, IL, p, pinv);
        for (u64 s = 16; s <= (1ull << (lg & ~1)); s *= 4)
            for (u64 blk = 0; blk < m; blk += s) {
                const u64 q = s / 4;
                dit4(a + blk, q, q, IL + q, IL + 2 * q, IL + 3 * q, p, pinv);
            }
    }
    if (lg & 1) dit2(a, m, m / 2, IL, p, pinv);
}

/* Cyclic DIF of a[0, m), natural order in, bit-reversed order out (centred). */
static void dif_rec(double* a, u64 m, const double* L, double p, double pinv) {
    if (m <= (1ull << BLOCK_LOG)) {
        dif_block(a, m, L, p, pinv);
        return;
    }
    const u64 q = m / 4;
    dif4(a, q, q, L + 2 * q, L + 3 * q, L + q, p, pinv);
    for (int k = 0; k < 4; ++k) dif_rec(a + k * q, q, L, p, pinv);
}

/* Cyclic DIT of a[0, m), bit-reversed order in, natural order out (unscaled). */
static void dit_rec(double* a, u64 m, const double* IL, double p, double pinv) {
    if (m <= (1ull << BLOCK_LOG)) {
        dit_block(a, m, IL, p, pinv);
        return;
    }
    const u64 q = m / 4;
    for (int k = 0; k < 4; ++k) dit_rec(a + k * q, q, IL, p, pinv);
    dit4(a, q, q, IL + q, IL + 2 * q, IL + 3 * q, p, pinv);
}

/* One prime's cyclic product in the spectrum (src/multiply/schedule.rs:18 and the
 * fused leaf schedules of src/arch/schedule/ restated): below the cache block each
 * sub-transform of a and of b is finished, multiplied pointwise with the folded
 * factor and inverted while it is in cache. */
typedef struct {
    const double *L, *IL;
    double p, pinv, factor;
    int square;
} Ring;

static void pointwise(double* restrict x, const double* y, u64 m, double factor, double p, double pinv) {
    for (u64 i = 0; i < m; ++i) {
        const double u = reduce_c(x[i], p, pinv), v = reduce_c(y[i], p, pinv);
        x[i] = mul_c(mul_c(u, v, p, pinv), factor, p, pinv);
    }
}

static void fused_rec(double* a, double* b, u64 m, const Ring* r) {
    if (m <= (1ull << BLOCK_LOG)) {
        dif_block(a, m, r->L, r->p, r->pinv);
        if (!r->square) dif_block(b, m, r->L, r->p, r->pinv);
        pointwise(a, r->square ? a : b, m, r->factor, r->p, r->pinv);
        dit_block(a, m, r->IL, r->p, r->pinv);
        return;
    }
    const u64 q = m / 4;
    dif4(a, q, q, r->L + 2 * q, r->L + 3 * q, r->L + q, r->p, r->pinv);
    if (!r->square) dif4(b, q, q, r->L + 2 * q, r->L + 3 * q, r->L + q, r->p, r->pinv);
    for (int k = 0; k < 4; ++k) fused_rec(a + k * q, b + k * q, q, r);
    dit4(a, q, q, r->IL + q, r->IL + 2 * q, r->IL + 3 * q, r->p, r->pinv);
}

/* The fast transforms on canonical input, canonical output. */
static int ntt_forward_fast(double* a, const Field* f) {
    int log_n = 0;
    while ((1ull << log_n) < f->n) ++log_n;
    LevelTables t;
    if (!level_tables(f->prime, log_n, &t)) return 0;
    dif_rec(a, f->n, t.fwd, f->p, f->pinv);
    for (u64 i = 0; i < f->n; ++i) a[i] = canon_c(a[i], f->p);
    level_tables_release(&t);
    return 1;
}
static int ntt_inverse_fast(double* a, const Field* f) {
    int log_n = 0;
    while ((1ull << log_n) < f->n) ++log_n;
    LevelTables t;
    if (!level_tables(f->prime, log_n, &t)) return 0;
    dit_rec(a, f->n, t.inv, f->p, f->pinv);
    for (u64 i = 0; i < f->n; ++i) a[i] = canon_c(a[i], f->p);
    level_tables_release(&t);
    return 1;
}

/* Bits [pos, pos+len) of a limb vector (len <= 64); zero past the end. */
static inline u64 get_bits(const u64* limbs, u64 count, u64 pos, int len) {
    const u64 li = pos >> 6;
    const int off = (int)(pos & 63);
    if (li >= count) return 0;
    u64 v = limbs[li] >> off;
    if (off && li + 1 < count) v |= limbs[li + 1] << (64 - off);
    return len == 64 ? v : v & ((1ull << len) - 1);
}

/* ------------------------------------------------------------------------------
 * Work pool (the rayon join analogue) */
typedef struct {
    void (*fn)(void* ctx, int task);
    void* ctx;
    int tasks;
    int next;
    pthread_mutex_t lock;
} Pool;

static void* pool_worker(void* arg) {
    Pool* pool = (Pool*)arg;
    for (;;) {
        pthread_mutex_lock(&pool->lock);
        const int t = pool->next++;
        pthread_mutex_unlock(&pool->lock);
        if (t >= pool->tasks) return NULL;
        pool->fn(pool->ctx, t);
    }
}

static void run_tasks(void (*fn)(void*, int), void* ctx, int tasks, int threads) {
    if (threads <= 1 || tasks <= 1) {
        for (int t = 0; t < tasks; ++t) fn(ctx, t);
        return;
    }
    Pool pool = {fn, ctx, tasks, 0, PTHREAD_MUTEX_INITIALIZER};
    const int n = threads < tasks ? threads : tasks;
    pthread_t* ids = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n);
    for (int i = 1; i < n; ++i) pthread_create(&ids[i], NULL, pool_worker, &pool);
    pool_worker(&pool);
    for (int i = 1; i < n; ++i) pthread_join(ids[i], NULL);
    free(ids);
}

/* ------------------------------------------------------------------------------
 * One multiplication under a geometry, in phases that each split into independent
 * tasks for the pool (the rayon joins of src/transform/forward.rs and
 * src/multiply/schedule.rs): digit parts of each operand, per-prime rows, the top
 * TOP_PASSES radix-4 steps of every forward transform, the fused leaf products of
 * the 4^TOP_PASSES sub-transforms, the top inverse steps, reconstruction. */
#define TOP_PASSES 2
#define TASK_SPAN 16384 /* elements per task of a streaming phase */

typedef struct {
    const Geometry* g;
    const u64 *a, *b;
    u64 la, lb;
    int square;
    int is_signed;
    u64 n;
    int ops; /* 1 for a square */
    Field* fields;
    LevelTables tab[MAX_PRIMES];
    double factor[MAX_PRIMES];
    double* parts[2]; /* [part][digit] of each operand */
    int nparts;
    double** spec_a;
    double** spec_b;
    int top;  /* radix-4 steps above the fused leaves */
    int pass; /* the top step in progress: sub-transforms of n >> 2*pass */
    /* reconstruction */
    const Cofactors* cof;
    u64 off[MAX_PRIMES]; /* residues of 2^sign_bit (P/p_i)^-1 */
    u64* out;
    u64 out_len;
    u64 range;  /* coefficients per reconstruction task */
    u64** part; /* per task partial windows */
    u64* part_start;
    u64* part_len;
    int tasks;
} Job;

static u64 spans(u64 len) { return len > TASK_SPAN ? div_ceil(len, TASK_SPAN) : 1; }

/* Digit parts (Packing::pack's 49-bit parts, src/limb/packing.rs:113-301). */
static void task_parts(void* ctx, int t) {
    Job* j = (Job*)ctx;
    const u64 per = spans(j->n);
    const int op = (int)(t / per);
    const u64 digits = op ? j->g->digits_b : j->g->digits_a;
    const u64* limbs = op ? j->b : j->a;
    const u64 count = op ? j->lb : j->la;
    const int w = j->g->chunk_bits;
    const u64 i0 = (t % per) * TASK_SPAN;
    const u64 i1 = i0 + TASK_SPAN < digits ? i0 + TASK_SPAN : digits;
    for (int part = 0; part < j->nparts; ++part) {
        const int len = (w - part * PART_BITS) < PART_BITS ? (w - part * PART_BITS) : PART_BITS;
        double* dst = j->parts[op] + (u64)part * j->n;
        for (u64 i = i0; i < i1; ++i)
            dst[i] = (double)get_bits(limbs, count, i * (u64)w + (u64)part * PART_BITS, len);
    }
}

/* A prime's row: sum_k part_k * (2^(49k) mod p), centred; signed geometries read
 * each limb as two's complement. */
static void task_rows(void* ctx, int t) {
    Job* j = (Job*)ctx;
    const u64 per = spans(j->n);
    const int row = (int)(t / per);
    const int prime = row / j->ops, op = row % j->ops;
    const Field* f = &j->fields[prime];
    const double p = f->p, pinv = f->pinv;
    const u64 digits = op ? j->g->digits_b : j->g->digits_a;
    const u64* limbs = op ? j->b : j->a;
    double* dst = op ? j->spec_b[prime] : j->spec_a[prime];
    double pw[MAX_PARTS];
    for (int k = 0; k < MAX_PARTS; ++k) {
        const u64 c = powmod_int(2, (u64)PART_BITS * k, f->pi);
        pw[k] = c > f->pi / 2 ? (double)c - p : (double)c;
    }
    const u64 c64 = powmod_int(2, 64, f->pi);
    const double two64 = c64 > f->pi / 2 ? (double)c64 - p : (double)c64;
    const u64 i0 = (t % per) * TASK_SPAN;
    const u64 i1 = i0 + TASK_SPAN < j->n ? i0 + TASK_SPAN : j->n;
    const u64 d1 = digits < i1 ? (digits > i0 ? digits : i0) : i1;
    /* part 0 is below 2^49 < p/2, already centred; each further term lies in
     * (-0.75p, 0.75p), so the sum stays below 2.75p before the reduction */
    const double* src = j->parts[op];
    for (u64 i = i0; i < d1; ++i) dst[i] = src[i];
    for (int k = 1; k < j->nparts; ++k) {
        const double* restrict part = src + (u64)k * j->n;
        double* restrict out = dst;
        const double c = pw[k];
        for (u64 i = i0; i < d1; ++i) out[i] += mul_c(part[i], c, p, pinv);
    }
    for (u64 i = i0; i < d1; ++i) dst[i] = reduce_c(dst[i], p, pinv);
    if (j->is_signed)
        for (u64 i = i0; i < d1; ++i)
            if ((int64_t)limbs[i] < 0) dst[i] = reduce_c(dst[i] - two64, p, pinv);
    for (u64 i = d1; i < i1; ++i) dst[i] = 0.0;
}

/* Task t of the top step `pass`: (prime, operand, sub-transform, span of j). */
static void task_forward_top(void* ctx, int t) {
    Job* j = (Job*)ctx;
    const u64 m = j->n >> (2 * j->pass), q = m / 4, per = spans(q), blocks = 1ull << (2 * j->pass);
    const u64 span = (u64)t % per, blk = ((u64)t / per) % blocks;
    const int row = (int)((u64)t / per / blocks);
    const int prime = row / j->ops, op = row % j->ops;
    const Field* f = &j->fields[prime];
    const double* L = j->tab[prime].fwd;
    const u64 j0 = span * TASK_SPAN, cnt = j0 + TASK_SPAN < q ? TASK_SPAN : q - j0;
    double* x = (op ? j->spec_b[prime] : j->spec_a[prime]) + blk * m + j0;
    dif4(x, q, cnt, L + 2 * q + j0, L + 3 * q + j0, L + q + j0, f->p, f->pinv);
}

static void task_leaves(void* ctx, int t) {
    Job* j = (Job*)ctx;
    const u64 blocks = 1ull << (2 * j->top), m = j->n >> (2 * j->top);
    const int prime = (int)((u64)t / blocks);
    const u64 blk = (u64)t % blocks;
    const Field* f = &j->fields[prime];
    const Ring r = {j->tab[prime].fwd, j->tab[prime].inv, f->p, f->pinv, j->factor[prime], j->square};
    fused_rec(j->spec_a[prime] + blk * m, j->square ? NULL : j->spec_b[prime] + blk * m, m, &r);
}

static void task_inverse_top(void* ctx, int t) {
    Job* j = (Job*)ctx;
    const u64 m = j->n >> (2 * j->pass), q = m / 4, per = spans(q), blocks = 1ull << (2 * j->pass);
    const u64 span = (u64)t % per, blk = ((u64)t / per) % blocks;
    const int prime = (int)((u64)t / per / blocks);
    const Field* f = &j->fields[prime];
    const double* IL = j->tab[prime].inv;
    const u64 j0 = span * TASK_SPAN, cnt = j0 + TASK_SPAN < q ? TASK_SPAN : q - j0;
    double* x = j->spec_a[prime] + blk * m + j0;
    dit4(x, q, cnt, IL + q + j0, IL + 2 * q + j0, IL + 3 * q + j0, f->p, f->pinv);
}

/* Adds `words` words of v shifted left by `shift` bits at limb `at` of dst[0..len). */
static void add_shifted(u64* dst, u64 len, u64 at, int shift, const u64* v, int words) {
    u64 carry = 0;
    u64 prev = 0;
    u64 i = 0;
    for (int w = 0; w <= words && at + i < len; ++w, ++i) {
        const u64 cur = w < words ? v[w] : 0;
        const u64 word = shift ? (cur << shift) | (prev >> (64 - shift)) : cur;
        prev = cur;
        const u128 s = (u128)dst[at + i] + word + carry;
        dst[at + i] = (u64)s;
        carry = (u64)(s >> 64);
    }
    while (carry && at + i < len) {
        const u128 s = (u128)dst[at + i] + carry;
        dst[at + i] = (u64)s;
        carry = (u64)(s >> 64);
        ++i;
    }
}

static void reconstruct_coefficient(const Job* j, u64 k, u64* value) {
    const int count = j->g->count;
    u64 r[MAX_PRIMES];
    for (int i = 0; i < count; ++i) {
        r[i] = (u64)canon_c(j->spec_a[i][k], j->fields[i].p);
        /* residue of 2^s times the inverse, src/limb/reconstruction.rs:94-113 */
        if (j->g->sign_bit >= 0) r[i] = (r[i] + j->off[i]) % CAT_P[i];
    }
    cof_bounded(j->cof, count, r, value);
}

static void task_reconstruct(void* ctx, int t) {
    Job* j = (Job*)ctx;
    const Geometry* g = j->g;
    const u64 k0 = (u64)t * j->range;
    u64 k1 = k0 + j->range;
    if (k1 > g->conv_len) k1 = g->conv_len;
    if (k0 >= k1) return;
    const int words = (j->cof->capacity + 63) / 64;
    u64 value[WORDS + 1];
    if (g->disjoint) {
        const u64 stride = g->output_stride / 64;
        for (u64 k = k0; k < k1; ++k) {
            memset(value, 0, sizeof(value));
            reconstruct_coefficient(j, k, value);
            u64* block = j->out + k * stride;
            for (u64 s = 0; s < stride; ++s) block[s] = s < (u64)words ? value[s] : 0;
            if (g->sign_bit >= 0) {
                /* subtract 2^s inside the block: two's complement result */
                const int sb = g->sign_bit;
                u64 borrow = 1ull << (sb & 63);
                for (u64 s = (u64)(sb >> 6); s < stride; ++s) {
                    const u64 v = block[s];
                    block[s] = v - borrow;
                    borrow = v < borrow ? 1 : 0;
                }
            }
        }
        return;
    }
    /* Coefficients at bit k*w: a private window, added to the output afterwards. */
    const u64 w = (u64)g->chunk_bits;
    const u64 start = (k0 * w) / 64;
    u64 end = ((k1 - 1) * w + (u64)j->cof->capacity) / 64 + 2;
    if (end > j->out_len) end = j->out_len;
    const u64 len = end - start;
    u64* win = (u64*)calloc(len, sizeof(u64));
    for (u64 k = k0; k < k1; ++k) {
        memset(value, 0, sizeof(value));
        reconstruct_coefficient(j, k, value);
        const u64 bit = k * w;
        add_shifted(win, len, bit / 64 - start, (int)(bit % 64), value, words);
    }
    j->part[t] = win;
    j->part_start[t] = start;
    j->part_len[t] = len;
}

static int multiply_under(const Geometry* g, u64* out, u64 out_len, const u64* a, u64 la, const u64* b, u64 lb,
                          int square, int is_signed, int threads) {
    Job j;
    memset(&j, 0, sizeof(j));
    j.g = g;
    j.a = a;
    j.b = b;
    j.la = la;
    j.lb = lb;
    j.square = square;
    j.ops = square ? 1 : 2;
    j.is_signed = is_signed;
    u64 n = next_pow2(g->conv_len);
    if (n < MIN_TRANSFORM_LEN) n = MIN_TRANSFORM_LEN;
    j.n = n;
    j.cof = cof_of(g->count);
    j.nparts = (g->chunk_bits + PART_BITS - 1) / PART_BITS;
    const int count = g->count;
    const int log_n = log2_u64(n);
    Field fields[MAX_PRIMES];
    double* sa[MAX_PRIMES] = {0};
    double* sb[MAX_PRIMES] = {0};
    int ok = 1, have[MAX_PRIMES] = {0};
    for (int op = 0; op < j.ops; ++op) {
        j.parts[op] = (double*)malloc((size_t)j.nparts * n * sizeof(double));
        ok &= j.parts[op] != NULL;
    }
    for (int i = 0; i < count; ++i) {
        ok &= field_init(&fields[i], i, n, 0);
        have[i] = level_tables(i, log_n, &j.tab[i]);
        ok &= have[i];
        sa[i] = (double*)malloc(n * sizeof(double));
        sb[i] = square ? NULL : (double*)malloc(n * sizeof(double));
        ok &= sa[i] != NULL && (square || sb[i] != NULL);
        /* N^-1 (P/p_i)^-1 folds into the pointwise product (src/multiply/schedule.rs:236-252) */
        const u64 pi = CAT_P[i];
        const u64 ninv = powmod_int(n % pi, pi - 2, pi);
        const u64 fac = mulmod_int(ninv, j.cof->inverses[i], pi);
        j.factor[i] = fac > pi / 2 ? (double)fac - (double)pi : (double)fac;
        if (g->sign_bit >= 0)
            j.off[i] = mulmod_int(powmod_int(2, (u64)g->sign_bit, pi), j.cof->inverses[i], pi);
    }
    if (ok) {
        j.fields = fields;
        j.spec_a = sa;
        j.spec_b = sb;
        for (u64 m = n; j.top < TOP_PASSES && m > (1ull << BLOCK_LOG); m /= 4) ++j.top;
        run_tasks(task_parts, &j, (int)(j.ops * spans(n)), threads);
        run_tasks(task_rows, &j, (int)(count * j.ops * spans(n)), threads);
        for (j.pass = 0; j.pass < j.top; ++j.pass) {
            const u64 q = (n >> (2 * j.pass)) / 4;
            run_tasks(task_forward_top, &j, (int)(count * j.ops * (1ull << (2 * j.pass)) * spans(q)), threads);
        }
        run_tasks(task_leaves, &j, (int)(count * (1ull << (2 * j.top))), threads);
        for (j.pass = j.top - 1; j.pass >= 0; --j.pass) {
            const u64 q = (n >> (2 * j.pass)) / 4;
            run_tasks(task_inverse_top, &j, (int)(count * (1ull << (2 * j.pass)) * spans(q)), threads);
        }
        j.out = out;
        j.out_len = out_len;
        const int tasks = threads > 1 ? 4 * threads : 1;
        j.range = div_ceil(g->conv_len, (u64)tasks);
        if (j.range < 256) j.range = 256;
        j.tasks = (int)div_ceil(g->conv_len, j.range);
        j.part = (u64**)calloc((size_t)j.tasks, sizeof(u64*));
        j.part_start = (u64*)calloc((size_t)j.tasks, sizeof(u64));
        j.part_len = (u64*)calloc((size_t)j.tasks, sizeof(u64));
        if (!g->disjoint) memset(out, 0, out_len * sizeof(u64));
        run_tasks(task_reconstruct, &j, j.tasks, threads);
        if (!g->disjoint) {
            /* carry fix-up across ranges, src/limb/reconstruction.rs:211-246 */
            for (int t = 0; t < j.tasks; ++t) {
                if (!j.part[t]) continue;
                add_shifted(out, out_len, j.part_start[t], 0, j.part[t], (int)j.part_len[t]);
                free(j.part[t]);
            }
        }
        free(j.part);
        free(j.part_start);
        free(j.part_len);
    }
    for (int op = 0; op < 2; ++op) free(j.parts[op]);
    for (int i = 0; i < count; ++i) {
        if (have[i]) level_tables_release(&j.tab[i]);
        field_free(&fields[i]);
        free(sa[i]);
        free(sb[i]);
    }
    return ok;
}

/* ------------------------------------------------------------------------------
 * Public entry points */

int oracle_mul(uint64_t* dst, const uint64_t* a, uint64_t la, const uint64_t* b, uint64_t lb, int threads) {
    if (!la || !lb) {
        memset(dst, 0, (la + lb) * sizeof(u64));
        return 1;
    }
    Geometry g;
    if (!select_geometry(la, lb, 1, &g)) return 0;
    const int square = a == b && la == lb;
    return multiply_under(&g, dst, la + lb, a, la, b, lb, square, 0, threads);
}

int oracle_sqr(uint64_t* dst, const uint64_t* a, uint64_t la, int threads) {
    return oracle_mul(dst, a, la, a, la, threads);
}

/* ConvPlan::admits, src/convolve.rs:169-184 */
static int admits(const ConvPlan* cp, const u64* v, u64 n, u64 max) {
    if (cp->is_signed) {
        for (u64 i = 0; i < n; ++i) {
            const int64_t s = (int64_t)v[i];
            const u64 mag = s < 0 ? (u64)0 - (u64)s : (u64)s;
            if (mag > max) return 0;
        }
        return 1;
    }
    u64 acc = 0;
    for (u64 i = 0; i < n; ++i) acc |= v[i];
    if (acc <= max) return 1;
    for (u64 i = 0; i < n; ++i)
        if (v[i] > max) return 0;
    return 1;
}

/* columns::<WORDS, SIGNED>, src/convolve.rs:284-351 */
static void sum_columns(u64* out, const u64* a, u64 la, const u64* b, u64 lb, u64 stride, int is_signed) {
    const u64 blocks = la + lb - 1;
    for (u64 k = 0; k < blocks; ++k) {
        const u64 first = k + 1 > lb ? k + 1 - lb : 0;
        const u64 last = k < la - 1 ? k : la - 1;
        u128 low = 0;
        u64 high = 0;
        for (u64 i = first; i <= last; ++i) {
            const u64 x = a[i], y = b[k - i];
            u128 prod;
            if (is_signed)
                prod = (u128)((__int128)(int64_t)x * (__int128)(int64_t)y);
            else
                prod = (u128)x * y;
            const u128 s = low + prod;
            high += s < low ? 1 : 0;
            low = s;
            if (is_signed && (int64_t)(u64)(prod >> 64) < 0) high -= 1;
        }
        u64* blk = out + k * stride;
        const u64 words[3] = {(u64)low, (u64)(low >> 64), high};
        for (u64 s = 0; s < stride && s < 3; ++s) blk[s] = words[s];
    }
}

int oracle_conv(uint64_t* dst, const uint64_t* a, uint64_t la, const uint64_t* b, uint64_t lb, uint64_t max_a,
                uint64_t max_b, int is_signed, int threads) {
    ConvPlan cp;
    if (!conv_plan(la, lb, max_a, max_b, is_signed, &cp)) return 0;
    if (!admits(&cp, a, la, max_a) || !admits(&cp, b, lb, max_b)) return 0;
    if (cp.schoolbook) {
        sum_columns(dst, a, la, b, lb, cp.stride, cp.is_signed);
        return 1;
    }
    const int square = a == b && la == lb;
    return multiply_under(&cp.g, dst, cp.output_len, a, la, b, lb, square, cp.is_signed, threads);
}

/* Schoolbook limb product (src/tests/schoolbook.rs:13-45): the reference's own test oracle. */
void oracle_schoolbook(uint64_t* dst, const uint64_t* a, uint64_t la, const uint64_t* b, uint64_t lb) {
    memset(dst, 0, (la + lb) * sizeof(u64));
    for (u64 i = 0; i < la; ++i) {
        u64 carry = 0;
        for (u64 j = 0; j < lb; ++j) {
            const u128 v = (u128)a[i] * b[j] + dst[i + j] + carry;
            dst[i + j] = (u64)v;
            carry = (u64)(v >> 64);
        }
        dst[i + lb] = carry;
    }
}

/* SplitMix64 operand, bench/src/lib.rs:13-29 */
void oracle_operand(uint64_t* dst, uint64_t len, uint64_t seed) {
    u64 state = seed;
    for (u64 i = 0; i < len; ++i) {
        state += 0x9e3779b97f4a7c15ull;
        u64 z = state;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        dst[i] = z ^ (z >> 31);
    }
}

/* The cache-blocked transforms against the radix-2 ones on seeded canonical input:
 * 1 when forward and inverse agree bit for bit (test infrastructure). */
int oracle_transform_check(int prime, int log_n, uint64_t seed) {
    if (prime < 0 || prime >= MAX_PRIMES || log_n < 1 || log_n > 24) return -1;
    const u64 n = 1ull << log_n;
    Field f;
    if (!field_init(&f, prime, n, 1)) return -1;
    double* x = (double*)malloc(n * sizeof(double));
    double* y = (double*)malloc(n * sizeof(double));
    int same = x && y;
    u64 st = seed;
    for (u64 i = 0; same && i < n; ++i) {
        st += 0x9E3779B97F4A7C15ull;
        u64 z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        x[i] = y[i] = (double)((z ^ (z >> 31)) % f.pi);
    }
    if (same) {
        ntt_forward(x, &f);
        same = ntt_forward_fast(y, &f);
        for (u64 i = 0; same && i < n; ++i) same = x[i] == y[i];
        ntt_inverse(x, &f);
        same = same && ntt_inverse_fast(y, &f);
        for (u64 i = 0; same && i < n; ++i) same = x[i] == y[i];
    }
    free(x);
    free(y);
    field_free(&f);
    return same;
}
