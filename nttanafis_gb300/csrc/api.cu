// The C ABI of include/ntt_gb300.h outside the batch layer: error and launch
// bookkeeping, per-kernel timing, the MulPlan / ConvPlan entry points, the
// workspaces (device arenas, host staging and the host-pointer calls), the
// four-step split settings and their tuner, and diagnostics.
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "host.h"

namespace ntt {

thread_local std::string g_error;
std::atomic<uint64_t> g_launches{0};
// Set while this thread captures a batch into a CUDA graph: the captured launches
// are counted when the graph runs, not when it is recorded.
thread_local bool t_capturing = false;

void note_launches(uint64_t n) {
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

// Look-back CRT launches that still have to start with their tile counter at 1
// (ntt_debug_stall_lookback).
static std::atomic<int> g_injected_stalls{0};

bool take_injected_stall() {
    int n = g_injected_stalls.load();
    while (n > 0 && !g_injected_stalls.compare_exchange_weak(n, n - 1)) {
    }
    return n > 0;
}

// Failure status bytes (launch.h) in page-locked host memory that the kernels
// write through its device address.
struct StatusWord {
    u32* host = nullptr;
    u32* dev = nullptr;
    bool create() {
        if (!cuda_ok(cudaHostAlloc((void**)&host, sizeof(u32), cudaHostAllocMapped), "cudaHostAlloc(status)"))
            return false;
        *host = 0;
        return cuda_ok(cudaHostGetDevicePointer((void**)&dev, host, 0), "cudaHostGetDevicePointer(status)");
    }
    void destroy() {
        if (host) cudaFreeHost(host);
        host = dev = nullptr;
    }
    // the status bits (kStatusLookback, kStatusBound) since the last take, cleared
    u32 take() {
        volatile uint8_t* b = reinterpret_cast<volatile uint8_t*>(host);
        const u32 bits = (b[0] ? kStatusLookback : 0u) | (b[1] ? kStatusBound : 0u);
        if (bits) *reinterpret_cast<volatile u32*>(host) = 0;
        return bits;
    }
};

bool fail(const char* msg) {
    g_error = msg;
    return false;
}
bool cuda_ok(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return true;
    g_error = std::string(where) + ": " + cudaGetErrorString(e);
    return false;
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
    StatusWord status;                // failures of this workspace's calls
};

struct ntt_conv_workspace {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t upload = nullptr;
    cudaEvent_t b_ready = nullptr;
    bool has_plan = false;
    Geom plan;
    DeviceBuf a, b, out, scratch;
    StatusWord status;
};

template <class W>
static W* workspace_new() {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
    W* ws = new W();
    ws->device = dev;
    if (!cuda_ok(cudaStreamCreateWithFlags(&ws->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaStreamCreateWithFlags(&ws->upload, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaEventCreateWithFlags(&ws->b_ready, cudaEventDisableTiming), "cudaEventCreate") ||
        !ws->status.create()) {
        if (ws->stream) cudaStreamDestroy(ws->stream);
        if (ws->upload) cudaStreamDestroy(ws->upload);
        if (ws->b_ready) cudaEventDestroy(ws->b_ready);
        ws->status.destroy();
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
    ws->status.destroy();
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
// failed kernel stops the stream before the copy-out. A kernel-side failure (a
// carry look-back wait that gave up) fails the call after the synchronisation;
// by then the copy-out, or the direct write into page-locked dst, has happened.
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
    if (!execute(g, square, (const u64*)ws->a.ptr, (const u64*)ws->b.ptr, out, ws->scratch.ptr, st, b_ready,
                 ws->status.dev))
        return false;
    if (!direct && !cuda_ok(cudaMemcpyAsync(dst, out, out_bytes, cudaMemcpyDeviceToHost, st), "copy dst"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(st), "kernels")) return false;
    const u32 bits = ws->status.take();
    if (bits & kStatusLookback) return fail("a carry look-back wait gave up: the product is wrong");
    if (bits & kStatusBound) return fail("a coefficient exceeds its bound");
    return true;
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
    return execute(g, square, d_a, d_b, d_dst, ws->scratch.ptr, st, nullptr, ws->status.dev) ? 1 : 0;
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
    return execute(g, square, d_a, d_b, d_dst, d_scratch, (cudaStream_t)stream, nullptr, nullptr, true) ? 1 : 0;
}

int ntt_conv_plan_status(const ntt_conv_plan* plan, const uint64_t* d_scratch, size_t scratch_len, void* stream) {
    Geom g;
    if (!conv_geom(plan, g)) return -1;
    if (!d_scratch || (u64)scratch_len * 8 < g.head_bytes()) {
        fail("scratch is too short");
        return -1;
    }
    u32 votes[kAdmitSlots];
    cudaStream_t st = (cudaStream_t)stream;
    if (!cuda_ok(cudaMemcpyAsync(votes, d_scratch, kAdmitBytes, cudaMemcpyDeviceToHost, st), "copy votes") ||
        !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return -1;
    for (int i = 0; i < kAdmitSlots; ++i)
        if (votes[i]) return 0;
    return 1;
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
    return execute(g, square, d_a, d_b, d_dst, ws->scratch.ptr, (cudaStream_t)stream, nullptr, ws->status.dev, true)
               ? 1
               : 0;
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

int ntt_split_set(int log_t, int log_r) {
    int lo = 0, hi = 0;
    if (!split_range(log_t, lo, hi) || (log_r != 0 && (log_r < lo || log_r > hi))) return -1;
    const int prev = g_split[log_t].exchange(log_r == log_t / 2 ? 0 : log_r);
    return prev ? prev : log_t / 2;
}

uint64_t ntt_school_set(uint64_t max_products) { return g_school_max.exchange(max_products); }

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
    // The timed products fill the transform on the lazy primes, whose splits these
    // are: balanced up to 2^21 points; above, a shorter operand of 2^19 limbs (a
    // balanced product there takes the wide primes, whose split is fixed).
    constexpr int kLazyShortLog = 19;
    const u64 full = (u64)1 << max_log_t;
    u64 *a = nullptr, *b = nullptr, *dst = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ntt_mul_workspace* ws = ntt_mul_workspace_new();
    bool ok = ws && cuda_ok(cudaMalloc(&a, full * 8), "cudaMalloc") && cuda_ok(cudaMalloc(&b, full / 2 * 8), "cudaMalloc") &&
              cuda_ok(cudaMalloc(&dst, full * 8), "cudaMalloc") &&
              cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") && cuda_ok(cudaEventCreate(&e1), "cudaEventCreate") &&
              cuda_ok(cudaMemsetAsync(a, 0xA5, full * 8, st), "cudaMemset") &&
              cuda_ok(cudaMemsetAsync(b, 0x3C, full / 2 * 8, st), "cudaMemset");
    for (int log_t = min_log_t; ok && log_t <= max_log_t; ++log_t) {
        int lo = 0, hi = 0;
        if (!split_range(log_t, lo, hi) || lo == hi) continue;
        const u64 nb = (u64)1 << std::min(log_t - 1, log_t <= 21 ? log_t - 1 : kLazyShortLog);
        const u64 na = ((u64)1 << log_t) - nb;  // na + nb - 1 coefficients fill 2^log_t points
        const int before = g_split[log_t].load();
        float best = 1e30f, standard = 1e30f;
        int pick = log_t / 2;
        for (int r = lo; ok && r <= hi; ++r) {
            g_split[log_t].store(r == log_t / 2 ? 0 : r);
            ok = ntt_mul_workspace_mul_device(ws, dst, na + nb, a, na, b, nb, st) == 1;  // tables, warm-up
            float ms = 1e30f;
            for (int round = 0; ok && round < 2; ++round) {
                ok = cuda_ok(cudaEventRecord(e0, st), "cudaEventRecord");
                for (int i = 0; ok && i < reps; ++i)
                    ok = ntt_mul_workspace_mul_device(ws, dst, na + nb, a, na, b, nb, st) == 1;
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

uint32_t ntt_mul_workspace_status(ntt_mul_workspace* ws) { return ws ? ws->status.take() : 0; }
uint32_t ntt_conv_workspace_status(ntt_conv_workspace* ws) { return ws ? ws->status.take() : 0; }

int ntt_debug_stall_lookback(int count) { return g_injected_stalls.exchange(count < 0 ? 0 : count); }

const char* ntt_last_error(void) { return g_error.c_str(); }
uint64_t ntt_kernel_launches(void) { return g_launches.load(); }
const char* ntt_version(void) { return "nttanafis_gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
