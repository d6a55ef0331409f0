// Declarations shared by the host-side translation units of the library: the
// error and launch bookkeeping (api.cu), the plan geometry and planner, the device
// tables and kernel constants (plan.cu), the enqueue of one product or one class of
// batch members (exec.cu), and the grow-only device buffer. The C ABI itself is in
// include/ntt_gb300.h; api.cu and batch.cu define it.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <string>

#include "../../include/ntt_gb300.h"
#include "launch.h"

namespace ntt {

typedef unsigned __int128 u128;

// Message of the last failure on this thread (ntt_last_error), kernels launched so
// far (ntt_kernel_launches), and whether this thread is capturing a CUDA graph (its
// launches are counted when the graph runs).
extern thread_local std::string g_error;
extern std::atomic<uint64_t> g_launches;
extern thread_local bool t_capturing;
void note_launches(uint64_t n);
// Records a timing event on `st` when per-kernel timing is on (ntt_timing_start).
void mark(cudaStream_t st);
// Record a failure and return false.
bool fail(const char* msg);
bool cuda_ok(cudaError_t e, const char* where);

// Smallest block transform of a split product (2^10 points).
constexpr int kSmallSplitLog = 10;

// ---------------------------------------------------------------------------------
// Plans (plan.cu)

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
    u64 spec_words(bool square) const { return np ? (u64)(square ? 1 : 2) * np * ((u64)1 << log_t) : 0; }
    // Scratch of one product or convolution: [head][residues][tail]. The head holds
    // a convolution's admission votes (launch.h; at offset 0 whatever the shape), the
    // tail a product's carry flags.
    u64 head_bytes() const { return conv ? (kAdmitBytes + 255) & ~(u64)255 : 0; }
    // residues (0 for a schoolbook convolution)
    u64 spec_bytes(bool square) const { return (spec_words(square) * 4 + 255) & ~(u64)255; }
    u64 tail_bytes(u64 out) const { return conv ? 0 : (carry_scratch_bytes(out) + 255) & ~(u64)255; }
    // scratch of one product of this geometry; for a split product, of one block,
    // whose other factor is the stored spectrum of the shorter operand (one operand
    // of residues)
    u64 member_bytes(bool square) const {
        if (split()) return spec_bytes(true) + tail_bytes(block + std::min(la, lb));
        return head_bytes() + spec_bytes(square) + tail_bytes(out_len);
    }
    // blocks per enqueue of a split product: bounded launch grids and arena
    u64 split_chunk() const {
        const u64 by_bytes = std::max<u64>(1, ((u64)512 << 20) / member_bytes(false));
        return std::min<u64>({blocks, 16384, by_bytes});
    }
    // split: [descriptors][odd-block sums (out_len limbs)][add flags][spectrum of the
    // shorter operand][member arenas]
    u64 split_desc_bytes() const { return (split_chunk() * sizeof(ProductDesc) + 255) & ~(u64)255; }
    u64 split_odd_bytes() const { return (out_len * 8 + 255) & ~(u64)255; }
    u64 split_flag_bytes() const { return (carry_scratch_bytes(out_len) + 255) & ~(u64)255; }
    u64 scratch_bytes(bool square) const {
        if (split())
            return split_desc_bytes() + split_odd_bytes() + split_flag_bytes() + spec_bytes(true) +
                   split_chunk() * member_bytes(false);
        return member_bytes(square);
    }
};

bool plan_mul(u64 la, u64 lb, Geom& g, bool allow_split = true);
bool plan_conv(u64 la, u64 lb, u64 max_a, u64 max_b, int sign, Geom& g);

// Four-step split of the lazy transform lengths (log2 R, 0 for floor(log_t / 2)).
extern std::atomic<int> g_split[kMaxLogT + 1];
bool split_range(int log_t, int& lo, int& hi);
int four_step_log_r(const Geom& g);
// The split of a product or convolution enqueued alone (execute): as above, and
// four-step with 2^6-point columns for T = 2^13, where one CTA per prime would leave
// all but five SMs idle. Batch members of that length keep the one-CTA kernels.
int single_log_r(const Geom& g);
// Kernel constants of a plan with four-step split R = 2^log_r (tables built on
// first use), or with the split in use.
bool prepare_params(const Geom& g, int log_r, PrimeSet& ps, CrtParams& cp);
bool prepare_params(const Geom& g, PrimeSet& ps, CrtParams& cp);
// The kernel attributes (shared-memory opt-in, cluster sizes) are set on the current
// device; a lock-free check after the first call.
bool kernels_ready();

// ---------------------------------------------------------------------------------
// Enqueue (exec.cu)

// The kernels of n batch members of one transform class, descriptors in device
// memory; convolution members are admitted on the device (their votes).
// status: the failure bytes of launch.h, or null. shared_spec: the stored spectrum
// of a factor all members share (block-split products), or null.
bool run_members(const ProductDesc* descs, int n, const Geom& g0, bool sq, u64 max_len, cudaStream_t st,
                 u32* status = nullptr, u32* shared_spec = nullptr);
// Products of single calls with at most this many limb products (a_len * b_len)
// take the direct column-sum basecase (school.cu) when it holds them; 0 turns it
// off. Set by ntt_school_set.
extern std::atomic<uint64_t> g_school_max;
bool takes_basecase(const Geom& g);
// One product or convolution on `st`; b_ready (optional) completes when operand b
// is in place. status: the failure bytes of launch.h, or null. admit: check a
// convolution's coefficient bounds on the device first (device-pointer calls; the
// host-pointer calls check them on the host).
bool execute(const Geom& g, bool square, const u64* d_a, const u64* d_b, u64* d_dst, void* scratch,
             cudaStream_t st, cudaEvent_t b_ready = nullptr, u32* status = nullptr, bool admit = false);
// Test hook (ntt_debug_stall_lookback): true when the next look-back CRT launch
// should start with its tile counter at 1, so that tile 0 never publishes.
bool take_injected_stall();
// Every coefficient within the plan's bound (magnitude bound when signed).
bool coefficients_admitted(const Geom& g, const u64* v, u64 n, u64 max);

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

}  // namespace ntt
