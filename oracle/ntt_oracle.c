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
 * the inverses; writes ceil(capacity/64) words of X. */
static void cof_bounded(const Cofactors* t, int count, const u64* residue, u64* value) {
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
    double* tw;  /* w^j, j < n/2, forward */
    double* itw; /* w^-j */
    u64 n;
} Field;

static int field_init(Field* f, int prime, u64 n) {
    f->pi = CAT_P[prime];
    f->p = (double)f->pi;
    f->pinv = 1.0 / f->p;
    f->n = n;
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

/* Bits [pos, pos+len) of a limb vector (len <= 64); zero past the end. */
static inline u64 get_bits(const u64* limbs, u64 count, u64 pos, int len) {
    const u64 li = pos >> 6;
    const int off = (int)(pos & 63);
    if (li >= count) return 0;
    u64 v = limbs[li] >> off;
    if (off && li + 1 < count) v |= limbs[li + 1] << (64 - off);
    return len == 64 ? v : v & ((1ull << len) - 1);
}

/* Packing::pack, src/limb/packing.rs:113-301: coefficient k is bits
 * [k*w, k*w+w), reduced as sum_k part_k * (2^(49k) mod p). Signed geometries
 * read each limb as two's complement. */
static void pack_row(double* row, const u64* limbs, u64 count, u64 digits, const Geometry* g, const Field* f,
                     int prime, int is_signed) {
    const int w = g->chunk_bits;
    double pw[MAX_PARTS];
    for (int k = 0; k < MAX_PARTS; ++k) pw[k] = (double)powmod_int(2, (u64)PART_BITS * k, CAT_P[prime]);
    const double two64 = (double)powmod_int(2, 64, CAT_P[prime]);
    for (u64 i = 0; i < f->n; ++i) {
        if (i >= digits) {
            row[i] = 0.0;
            continue;
        }
        double r = 0.0;
        const u64 base = i * (u64)w;
        for (int part = 0; part * PART_BITS < w; ++part) {
            const int len = (w - part * PART_BITS) < PART_BITS ? (w - part * PART_BITS) : PART_BITS;
            const u64 bits = get_bits(limbs, count, base + (u64)part * PART_BITS, len);
            r = addmod(r, fmulmod((double)bits, pw[part], f->p, f->pinv), f->p);
        }
        if (is_signed && (int64_t)limbs[i] < 0) r = submod(r, two64, f->p);
        row[i] = r;
    }
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
 * One multiplication under a geometry */
typedef struct {
    const Geometry* g;
    const u64 *a, *b;
    u64 la, lb;
    int square;
    int is_signed;
    u64 n;
    Field* fields;
    double** spec_a;
    double** spec_b;
    /* reconstruction */
    const Cofactors* cof;
    u64* out;
    u64 out_len;
    u64 range;  /* coefficients per reconstruction task */
    u64** part; /* per task partial windows */
    u64* part_start;
    u64* part_len;
    int tasks;
} Job;

static void task_forward(void* ctx, int t) {
    Job* j = (Job*)ctx;
    const int prime = t >> 1, op = t & 1;
    if (op && j->square) return;
    const Field* f = &j->fields[prime];
    if (op == 0)
        pack_row(j->spec_a[prime], j->a, j->la, j->g->digits_a, j->g, f, prime, j->is_signed);
    else
        pack_row(j->spec_b[prime], j->b, j->lb, j->g->digits_b, j->g, f, prime, j->is_signed);
    ntt_forward(op ? j->spec_b[prime] : j->spec_a[prime], f);
}

/* Pointwise product and inverse; the factor N^-1 (P/p_i)^-1 folds into the
 * pointwise product as src/multiply/schedule.rs:236-252 folds it. */
static void task_inverse(void* ctx, int prime) {
    Job* j = (Job*)ctx;
    const Field* f = &j->fields[prime];
    double* x = j->spec_a[prime];
    const double* y = j->square ? x : j->spec_b[prime];
    const u64 ninv = powmod_int(j->n % f->pi, f->pi - 2, f->pi);
    const double factor = (double)mulmod_int(ninv, j->cof->inverses[prime], f->pi);
    for (u64 i = 0; i < j->n; ++i) x[i] = fmulmod(fmulmod(x[i], y[i], f->p, f->pinv), factor, f->p, f->pinv);
    ntt_inverse(x, f);
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
        r[i] = (u64)j->spec_a[i][k];
        if (j->g->sign_bit >= 0) {
            /* residue of 2^s times the inverse, src/limb/reconstruction.rs:94-113 */
            const u64 p = CAT_P[i];
            const u64 off = mulmod_int(powmod_int(2, (u64)j->g->sign_bit, p), j->cof->inverses[i], p);
            r[i] = (r[i] + off) % p;
        }
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
    j.is_signed = is_signed;
    u64 n = next_pow2(g->conv_len);
    if (n < MIN_TRANSFORM_LEN) n = MIN_TRANSFORM_LEN;
    j.n = n;
    j.cof = cof_of(g->count);
    const int count = g->count;
    Field fields[MAX_PRIMES];
    double* sa[MAX_PRIMES] = {0};
    double* sb[MAX_PRIMES] = {0};
    int ok = 1;
    for (int i = 0; i < count; ++i) {
        ok &= field_init(&fields[i], i, n);
        sa[i] = (double*)malloc(n * sizeof(double));
        sb[i] = square ? NULL : (double*)malloc(n * sizeof(double));
        ok &= sa[i] != NULL && (square || sb[i] != NULL);
    }
    if (ok) {
        j.fields = fields;
        j.spec_a = sa;
        j.spec_b = sb;
        run_tasks(task_forward, &j, 2 * count, threads);
        run_tasks(task_inverse, &j, count, threads);
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
    for (int i = 0; i < count; ++i) {
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
