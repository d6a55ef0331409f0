/*
 * C ABI of the GB300 multiplication hot path: exact products, squares and dense
 * convolutions of 64-bit limb vectors on one GPU.
 *
 * Each entry point replaces one call of the reference crate `ntt_anafis` (paths are
 * relative to that crate's root):
 *
 *   ntt_mul_plan_new            MulPlan::new                 src/plan.rs:53
 *   ntt_mul_plan_mul_device     MulPlan::mul                 src/plan.rs:94
 *   ntt_mul_plan_sqr_device     MulPlan::sqr                 src/plan.rs:112
 *   ntt_mul_workspace_new/free  MulWorkspace::new            src/plan.rs:143
 *   ntt_mul_workspace_prepare   MulWorkspace::prepare        src/plan.rs:151
 *   ntt_mul_workspace_mul       MulWorkspace::mul            src/plan.rs:164
 *   ntt_mul_workspace_sqr       MulWorkspace::sqr            src/plan.rs:177
 *   ntt_conv_plan_new           ConvPlan::new                src/convolve.rs:75
 *   ntt_conv_plan_convolve_device ConvPlan::convolve         src/convolve.rs:148
 *   ntt_conv_workspace_new/free ConvWorkspace::new           src/convolve.rs:237
 *   ntt_conv_workspace_prepare  ConvWorkspace::prepare       src/convolve.rs:246
 *   ntt_conv_workspace_convolve ConvWorkspace::convolve      src/convolve.rs:264
 *
 * Conventions (as in the reference, src/lib.rs:1-24):
 *  - limbs are uint64_t, least significant first;
 *  - a product writes exactly a_len + b_len limbs, a square 2 * a_len limbs, a
 *    convolution (a_len + b_len - 1) * stride limbs; limbs past that are preserved;
 *  - every failure returns 0 and leaves dst unmodified; success returns 1;
 *  - a == b with a_len == b_len (the same slice twice) runs the square path;
 *  - dst must not overlap a or b (the reference's &mut dst cannot alias them).
 *
 * Host-pointer calls (`*_mul`, `*_sqr`, `*_convolve`) copy the operands to the GPU,
 * run, and copy the result back before returning. Pinned (page-locked) host buffers
 * copy fastest. `*_device` calls take device pointers and a cudaStream_t (as
 * void*), enqueue the work and return without synchronizing; the device buffers must
 * stay valid until the stream reaches that point.
 *
 * Failures found by the kernels themselves: every wait of the CRT carry scan is
 * bounded, and a wait that gives up (which a working GPU never causes: it means a
 * CTA that had started was not scheduled for about 70 ms) leaves a wrong product; a
 * device-pointer convolution whose coefficient exceeds its bound is not written.
 * Host-pointer calls return 0 for either. By then a page-locked dst may already
 * hold the wrong product (the kernels write it directly when a call runs alone);
 * other dst memory is untouched. Device-pointer calls report them afterwards in the
 * status of their workspace or batch (ntt_*_status, NTT_STATUS_* bits); plan calls
 * through ntt_lookback_timeouts() and ntt_conv_plan_status().
 *
 * A workspace owns device arenas that only grow and must not be used by two threads
 * at once. Plans are plain values. The root tables are shared by all workspaces of a
 * process and built once per device.
 */
#ifndef NTT_GB300_H
#define NTT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Admitted product geometry (MulPlan). Fields are outputs of ntt_mul_plan_new. */
typedef struct ntt_mul_plan {
    uint64_t len_a;
    uint64_t len_b;
    uint32_t primes;          /* NTT primes used */
    uint32_t log_transform;   /* log2 of the transform length */
    uint64_t scratch_len;     /* device scratch limbs of ntt_mul_plan_mul_device */
    uint64_t sqr_scratch_len; /* device scratch limbs of ntt_mul_plan_sqr_device */
    uint64_t block_len;       /* block split: limbs per block of the longer operand (0: none) */
    uint64_t blocks;          /* block split: blocks of the longer operand */
} ntt_mul_plan;

/* Admitted convolution geometry (ConvPlan). */
typedef struct ntt_conv_plan {
    uint64_t len_a;
    uint64_t len_b;
    uint64_t max_a;
    uint64_t max_b;
    uint32_t is_signed;
    uint32_t primes;          /* 0 when the short operand is summed directly */
    uint32_t log_transform;
    uint32_t schoolbook;      /* 1 when min(len_a, len_b) <= 24 */
    uint64_t stride;          /* limbs per output coefficient */
    uint64_t output_len;      /* (len_a + len_b - 1) * stride */
    uint64_t scratch_len;     /* device scratch limbs of ntt_conv_plan_convolve_device */
} ntt_conv_plan;

typedef struct ntt_mul_workspace ntt_mul_workspace;
typedef struct ntt_conv_workspace ntt_conv_workspace;

/* Plans positive lengths; returns 0 (no plan) for a zero length or a shape beyond
 * the GPU transform catalog: a_len + b_len - 1 > 2^25 coefficients unless the
 * product takes the block split (the longer operand in blocks, each multiplied by
 * the shorter one; shorter operand up to 2^24 limbs, longer up to 2^40). A very
 * unbalanced product takes the split whenever it is cheaper (log_transform is then
 * the block transform). MulPlan::new, src/plan.rs:53; the split follows
 * Geometry::cheapest_blocks, src/profile/planner.rs:291. */
int ntt_mul_plan_new(uint64_t len_a, uint64_t len_b, ntt_mul_plan* out);

/* a*b into d_dst with caller-owned device scratch (MulPlan::mul, src/plan.rs:94). */
uint8_t ntt_mul_plan_mul_device(const ntt_mul_plan* plan, uint64_t* d_dst, size_t dst_len,
                                const uint64_t* d_a, size_t a_len, const uint64_t* d_b,
                                size_t b_len, uint64_t* d_scratch, size_t scratch_len,
                                void* stream);
/* a*a (MulPlan::sqr, src/plan.rs:112). */
uint8_t ntt_mul_plan_sqr_device(const ntt_mul_plan* plan, uint64_t* d_dst, size_t dst_len,
                                const uint64_t* d_a, size_t a_len, uint64_t* d_scratch,
                                size_t scratch_len, void* stream);

/* Workspace bound to the current CUDA device (MulWorkspace::new, src/plan.rs:143);
 * NULL when no device is available. */
ntt_mul_workspace* ntt_mul_workspace_new(void);
void ntt_mul_workspace_free(ntt_mul_workspace* ws);
/* Retains the plan and grows the arenas (MulWorkspace::prepare, src/plan.rs:151).
 * Returns 0 when device memory cannot be allocated. */
uint8_t ntt_mul_workspace_prepare(ntt_mul_workspace* ws, const ntt_mul_plan* plan);
/* MulWorkspace::mul (src/plan.rs:164): empty operands write zeros; a shape other
 * than the retained plan is planned and retained. Host pointers. */
uint8_t ntt_mul_workspace_mul(ntt_mul_workspace* ws, uint64_t* dst, size_t dst_len,
                              const uint64_t* a, size_t a_len, const uint64_t* b, size_t b_len);
/* MulWorkspace::sqr (src/plan.rs:177). Host pointers. */
uint8_t ntt_mul_workspace_sqr(ntt_mul_workspace* ws, uint64_t* dst, size_t dst_len,
                              const uint64_t* a, size_t a_len);
/* Device-pointer forms of the two calls above, enqueued on `stream`. */
uint8_t ntt_mul_workspace_mul_device(ntt_mul_workspace* ws, uint64_t* d_dst, size_t dst_len,
                                     const uint64_t* d_a, size_t a_len, const uint64_t* d_b,
                                     size_t b_len, void* stream);
uint8_t ntt_mul_workspace_sqr_device(ntt_mul_workspace* ws, uint64_t* d_dst, size_t dst_len,
                                     const uint64_t* d_a, size_t a_len, void* stream);

/* ConvPlan::new (src/convolve.rs:75): bounds the magnitude of every coefficient;
 * signed bounds must lie below 2^63. */
int ntt_conv_plan_new(uint64_t len_a, uint64_t len_b, uint64_t max_a, uint64_t max_b,
                      int is_signed, ntt_conv_plan* out);
/* ConvPlan::convolve (src/convolve.rs:148) on device pointers with caller scratch
 * (plan->scratch_len limbs; its first 512 bytes hold the admission votes, so a
 * schoolbook plan needs them too). Lengths and buffer sizes are checked here (0,
 * nothing enqueued); the coefficient bounds (src/convolve.rs:169-184) are checked on
 * the GPU before anything is written: a coefficient above its bound leaves d_dst
 * untouched, which ntt_conv_plan_status reports. */
uint8_t ntt_conv_plan_convolve_device(const ntt_conv_plan* plan, uint64_t* d_dst,
                                      size_t dst_len, const uint64_t* d_a, size_t a_len,
                                      const uint64_t* d_b, size_t b_len, uint64_t* d_scratch,
                                      size_t scratch_len, void* stream);
/* Outcome of the last ntt_conv_plan_convolve_device that used this scratch: waits
 * for `stream`, then returns 1 (admitted and written), 0 (a coefficient exceeded its
 * bound: d_dst untouched) or -1 (CUDA error or short scratch). No reference
 * counterpart: the reference's convolve returns this as its bool. */
int ntt_conv_plan_status(const ntt_conv_plan* plan, const uint64_t* d_scratch, size_t scratch_len,
                         void* stream);

ntt_conv_workspace* ntt_conv_workspace_new(void);
void ntt_conv_workspace_free(ntt_conv_workspace* ws);
/* ConvWorkspace::prepare (src/convolve.rs:246). */
uint8_t ntt_conv_workspace_prepare(ntt_conv_workspace* ws, const ntt_conv_plan* plan);
/* ConvWorkspace::convolve (src/convolve.rs:264): fails without a prepared plan, for
 * mismatched lengths, a coefficient above its bound, or a short dst. Host pointers. */
uint8_t ntt_conv_workspace_convolve(ntt_conv_workspace* ws, uint64_t* dst, size_t dst_len,
                                    const uint64_t* a, size_t a_len, const uint64_t* b,
                                    size_t b_len);
/* Device-pointer form. Lengths and sizes are checked here; the coefficient bounds
 * on the GPU before anything is written (a coefficient above its bound leaves d_dst
 * untouched and sets NTT_STATUS_BOUND in ntt_conv_workspace_status). */
uint8_t ntt_conv_workspace_convolve_device(ntt_conv_workspace* ws, uint64_t* d_dst,
                                           size_t dst_len, const uint64_t* d_a, size_t a_len,
                                           const uint64_t* d_b, size_t b_len, void* stream);

/* Status bits of the device-pointer calls of a workspace or batch. */
#define NTT_STATUS_LOOKBACK 1u /* a carry look-back wait gave up: that product is wrong */
#define NTT_STATUS_BOUND 2u    /* a convolution coefficient exceeded its bound: not written */
/* The NTT_STATUS_* bits set by the workspace's device-pointer calls since the last
 * query (0: every one succeeded), cleared by reading. Call it after the calls'
 * streams have completed. No reference counterpart: the reference's calls return
 * these failures as their bool, which an enqueued GPU call cannot. */
uint32_t ntt_mul_workspace_status(ntt_mul_workspace* ws);
uint32_t ntt_conv_workspace_status(ntt_conv_workspace* ws);

/* One member of a batch (device pointers). kind 0: product a*b (a square when
 * a == b and a_len == b_len; empty operands write zeros); kind 1: convolution under
 * the bounds max_a, max_b, two's complement when is_signed (ConvPlan rules). dst
 * must hold dst_len >= the result's limbs. */
typedef struct ntt_request {
    uint64_t* dst;
    uint64_t dst_len;
    const uint64_t* a;
    const uint64_t* b;
    uint64_t a_len;
    uint64_t b_len;
    uint32_t kind;
    uint32_t is_signed;
    uint64_t max_a;
    uint64_t max_b;
} ntt_request;

typedef struct ntt_batch ntt_batch;

/* Batch executor bound to the current device. It owns a grow-only arena for the
 * members' residues and a descriptor buffer; calls on one batch object must be
 * ordered on one stream (use one object per concurrent stream). No counterpart in
 * the reference crate: it is the batched layer over MulPlan::mul / ConvPlan::convolve. */
ntt_batch* ntt_batch_new(void);
void ntt_batch_free(ntt_batch* batch);
/* Enqueues every request on `stream`: members are grouped by transform class and
 * each class runs as one launch per kernel; the classes run concurrently on 1, 2
 * or 4 streams of the batch (forked from and joined back into `stream`). A
 * composition (the sequence of classes with their member counts and longest
 * results) seen once runs with a lane count picked from its size; one that
 * repeats is tuned on its own runs (runs 2 to 7 time each lane count twice with
 * CUDA events on `stream`), then captured with the fastest lane count into a CUDA
 * graph that serves every later run (not on the legacy default stream). Returns 0
 * and launches nothing when a request has no plan or a short dst, or while
 * `stream` is being captured by the caller (message in ntt_last_error()). */
uint8_t ntt_batch_run_device(ntt_batch* batch, const ntt_request* requests, size_t count,
                             void* stream);
/* Graph replay on (1) or off (0) for this batch (default on); other values only
 * report. Returns the previous setting, -1 for a null batch. */
int ntt_batch_set_graphs(ntt_batch* batch, int on);
/* Lane count of every run: 1, 2 or 4 fixes it (no tuning), 0 returns to tuning
 * per composition (the default); other values only report. Returns the previous
 * setting, -1 for a null batch. */
int ntt_batch_set_lanes(ntt_batch* batch, int lanes);
/* out[0] runs served from a captured graph, out[1] compositions tuned, out[2]
 * lanes of the last run enqueued directly or captured, out[3] compositions held. */
void ntt_batch_stats(const ntt_batch* batch, uint64_t* out);
/* Products of the batch's runs that ran as block splits (an operand many times
 * longer than the other: the shorter operand's spectrum once per run, the longer
 * operand's blocks multiplied by it, as MulPlan's split products do). */
uint64_t ntt_batch_split_members(const ntt_batch* batch);
/* NTT_STATUS_* bits of the batch's runs since the last query, cleared by reading;
 * call it after the runs' stream has completed. A convolution member with a
 * coefficient above its bound is left unwritten (the other members complete). */
uint32_t ntt_batch_status(ntt_batch* batch);

/* Largest product (a_len + b_len - 1 coefficients) of ntt_mul_noalloc_device, and
 * the device memory its static arrays hold on every GPU that loads the library. */
#define NTT_NOALLOC_MAX_COEFFICIENTS 4096
#define NTT_NOALLOC_SCRATCH_BYTES 164096
#define NTT_NOALLOC_TABLE_BYTES 327680

/* Exact product a*b (a*a when d_a == d_b and a_len == b_len) on device pointers for
 * callers that must not allocate device memory: code running under a device-memory
 * budget owned by another allocator, or on a latency-critical path where the
 * device-wide synchronisation of cudaMalloc/cudaFree would stall other streams.
 * It calls no allocating routine: its scratch and root tables are static device
 * arrays that every GPU loading the library holds until exit. Limits:
 * a_len + b_len - 1 <= NTT_NOALLOC_MAX_COEFFICIENTS (larger shapes return 0 with a
 * message in ntt_last_error(), dst untouched); the first call on a device performs
 * a one-time set-up with that device current, so make it before any stream capture;
 * all calls share one scratch array, so calls that overlap on the GPU race - keep
 * them ordered on one stream. Empty operands write zeros. Enqueues on `stream` and
 * returns without synchronizing. This entry point has no counterpart in the
 * reference crate. */
uint8_t ntt_mul_noalloc_device(uint64_t* d_dst, size_t dst_len, const uint64_t* d_a, size_t a_len,
                               const uint64_t* d_b, size_t b_len, void* stream);

/* Per-kernel timing for measurement tools (not thread-safe). After
 * ntt_timing_start(count), each call records a CUDA event on its launching stream
 * before its first kernel and after every kernel, until `count` events are used.
 * ntt_timing_stop waits for the last event, writes the milliseconds between
 * consecutive events into ms[0..capacity) and returns how many it wrote (-1 on a
 * CUDA error), and switches timing off. */
int ntt_timing_start(int count);
int ntt_timing_stop(float* ms, int capacity);

/* ---------------------------------------------------------------------------
 * Batched modular arithmetic in 50-bit prime fields (the reference's PrimeField
 * and CrtPair, src/field/prime_field.rs), on device arrays of residues (uint64_t,
 * canonical 0 <= r < p; residues of another field give unspecified values). A
 * field is named by its modulus, a prime 2^49 < p < 2^50; every call checks it
 * (returns 0 otherwise). Calls enqueue on `stream` and return without waiting.
 */

/* 1 when `modulus` is a prime in (2^49, 2^50): PrimeField::new, prime_field.rs:99. */
int ntt_field_check(uint64_t modulus);
/* Selects how the calls below multiply two residues (process-wide; returns the
 * previous choice): 1 the reference's FP64 quotient estimate (prime_field.rs:232),
 * 0 Barrett on 64-bit integers; any other value only reports. Both are exact. No
 * reference counterpart: it exists to measure and test the two methods. */
int ntt_field_mul_method(int method);
/* Largest admitted prime below min(bound, 2^50), or 0: PrimeField::below, :118. */
uint64_t ntt_field_below(uint64_t bound);
/* The transform's catalog moduli in reconstruction order (writes at most
 * `capacity`, returns 8): PrimeField::catalog, :131. */
size_t ntt_field_catalog(uint64_t* out, size_t capacity);
/* out[i] = a[i] op b[i]; op 0 add (:205), 1 sub (:215), 2 mul (:232). */
uint8_t ntt_field_binary_device(uint64_t modulus, int op, uint64_t* d_out, const uint64_t* d_a,
                                const uint64_t* d_b, size_t n, void* stream);
/* out[i] = op(a[i]); op 0 neg (:225), 1 pow with `exponent` (:249, 0^0 = 1),
 * 2 inv (:271; zero gives 0 and, with d_mask, mask 0), 3 signed representative
 * as int64 bits (:193), 4 reduce of int64 bits (:158), 5 reduce of uint64 (:173). */
uint8_t ntt_field_unary_device(uint64_t modulus, int op, uint64_t* d_out, const uint64_t* d_a, size_t n,
                               uint64_t exponent, uint8_t* d_mask, void* stream);
/* target[i] = factor * target[i] (scale, :304), or with d_source
 * target[i] -= factor * source[i] (mul_sub, :296). factor < modulus. */
uint8_t ntt_field_scale_device(uint64_t modulus, uint64_t* d_target, const uint64_t* d_source, size_t n,
                               uint64_t factor, void* stream);
/* out[j] = sum_i coeffs[i] * points[j]^i for every point (evaluate, :313). */
uint8_t ntt_field_evaluate_device(uint64_t modulus, uint64_t* d_out, const uint64_t* d_coeffs, size_t n_coeffs,
                                  const uint64_t* d_points, size_t n_points, void* stream);
/* CrtPair::combine (:428) of two distinct fields: out[2i], out[2i+1] = low and
 * high words of the int128 in -(M-1)/2..(M-1)/2 congruent to first[i] and second[i]. */
uint8_t ntt_crt_pair_combine_device(uint64_t first, uint64_t second, int64_t* d_out, const uint64_t* d_first,
                                    const uint64_t* d_second, size_t n, void* stream);

/* Four-step split T = R * C of the lazy transform lengths 2^14..2^23, process-wide:
 * ntt_split_set makes R = 2^log_r for transforms of 2^log_t points (0 restores the
 * default floor(log_t / 2)) and returns the previous log_r, or -1 when log_t has no
 * choice of split or log_r is outside the range that ntt_split_range reports
 * (columns 2^6..2^11, rows 2^7..2^13). ntt_split_get returns the log_r in use (0
 * for lengths without a four-step split). The split changes speed, never results.
 * ntt_tune_splits times every split of each length in [min_log_t, max_log_t] on
 * products that fill the transform on the lazy primes (balanced up to 2^21 points,
 * a 2^19-limb shorter operand above; `reps` products per timing, best of two) on
 * `stream` and keeps the fastest when it beats the default by 2%; it
 * synchronizes `stream` and allocates its operands for the call. Calls made by other
 * threads meanwhile may run with a split under trial (their results stay exact). No
 * reference counterpart: the reference fixes its geometry in Geometry::select. */
/* Products of single calls (workspace and plan calls; batches keep the transforms)
 * with a_len * b_len <= max_products limb products and at most 1,024 result limbs
 * take the direct column-sum basecase: one thread-block cluster of 1 to 8 CTAs, no
 * scratch. 0 turns it off. Process-wide; returns the previous threshold. It changes
 * speed, never results. No reference counterpart: the reference's own basecase
 * crossover is inside its planner. */
uint64_t ntt_school_set(uint64_t max_products);
int ntt_split_set(int log_t, int log_r);
int ntt_split_get(int log_t);
int ntt_split_range(int log_t, int* lo, int* hi);
uint8_t ntt_tune_splits(int min_log_t, int max_log_t, int reps, void* stream);

/* Look-back waits of the CRT carry scan that gave up since the library was loaded
 * (each wait is bounded; a nonzero count means a result may be wrong). Synchronizes
 * the device. */
uint32_t ntt_lookback_timeouts(void);
/* Test hook for the failure path above: the next `count` products whose CRT uses
 * the carry look-back start that kernel with its tile counter at 1, so no CTA
 * takes tile 0 and the wait for it runs out (a bounded wait on a state that nothing
 * writes; the GPU stays usable). Returns the previous count. No reference
 * counterpart. */
int ntt_debug_stall_lookback(int count);

/* Message of the last failure on this thread ("" when none). */
const char* ntt_last_error(void);
/* Kernels launched by this process since load (counted per launch by the host). */
uint64_t ntt_kernel_launches(void);
/* Library version string. */
const char* ntt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NTT_GB300_H */
