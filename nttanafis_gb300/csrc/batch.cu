// The batch layer (ntt_batch_* in include/ntt_gb300.h): many products and
// convolutions per enqueue, grouped by transform class, with the class scheduling,
// its tuning per composition and the CUDA-graph replay.
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "host.h"

using namespace ntt;

extern "C" {

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
    // failure bytes of the batch's runs (launch.h) in page-locked host memory
    u32* status_host = nullptr;
    u32* status_dev = nullptr;
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
    uint64_t split_members = 0;  // products run as block splits
    std::map<std::vector<uint64_t>, Composition> comps;
};

static void destroy_batch_events(ntt_batch* b) {
    for (int i = 0; i < kBatchLanes; ++i) {
        if (b->lane[i]) cudaStreamDestroy(b->lane[i]);
        if (b->lane_done[i]) cudaEventDestroy(b->lane_done[i]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->staged) cudaEventDestroy(b->staged);
    if (b->status_host) cudaFreeHost(b->status_host);
    b->status_host = b->status_dev = nullptr;
    for (auto& kv : b->comps) release_composition(kv.second);
    b->comps.clear();
}

ntt_batch* ntt_batch_new(void) {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
    ntt_batch* b = new ntt_batch();
    b->device = dev;
    bool ok = cuda_ok(cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming), "cudaEventCreate") &&
              cuda_ok(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate") &&
              cuda_ok(cudaHostAlloc((void**)&b->status_host, sizeof(u32), cudaHostAllocMapped), "cudaHostAlloc") &&
              cuda_ok(cudaHostGetDevicePointer((void**)&b->status_dev, b->status_host, 0), "cudaHostGetDevicePointer");
    if (ok) *b->status_host = 0;
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

uint32_t ntt_batch_status(ntt_batch* b) {
    if (!b || !b->status_host) return 0;
    volatile uint8_t* v = reinterpret_cast<volatile uint8_t*>(b->status_host);
    const u32 bits = (v[0] ? kStatusLookback : 0u) | (v[1] ? kStatusBound : 0u);
    if (bits) *reinterpret_cast<volatile u32*>(b->status_host) = 0;
    return bits;
}

uint64_t ntt_batch_split_members(const ntt_batch* b) { return b ? b->split_members : 0; }

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
            if (!run_members(dev_desc + c.k, (int)(c.end - c.k), c.g, c.square, c.max_len, st, b->status_dev))
                return false;
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
        if (!run_members(dev_desc + c.k, (int)(c.end - c.k), c.g, c.square, c.max_len, b->lane[lane],
                         b->status_dev))
            return false;
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
    std::vector<Member> splits;  // unbalanced products: block splits, enqueued one by one
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
            if (!plan_mul(r.a_len, r.b_len, m.g, true)) return 0;
        } else if (r.kind == 1) {
            if (!plan_conv(r.a_len, r.b_len, r.max_a, r.max_b, (int)r.is_signed, m.g)) return 0;
        } else {
            return fail("unknown request kind");
        }
        if (r.dst_len < m.g.out_len) return fail("destination is shorter than the result");
        m.square = r.a == r.b && r.a_len == r.b_len;
        m.offset = arena_bytes;
        arena_bytes += (m.g.scratch_bytes(m.square) + 255) & ~(u64)255;
        (m.g.split() ? splits : members).push_back(m);
    }
    for (size_t i : empties)
        if (!cuda_ok(cudaMemsetAsync(reqs[i].dst, 0, ((size_t)reqs[i].a_len + reqs[i].b_len) * 8, st), "zero product"))
            return 0;
    if (members.empty() && splits.empty()) return 1;
    // Group by class: kind, schoolbook, transform length, primes, sign, square.
    std::sort(members.begin(), members.end(), [](const Member& x, const Member& y) {
        return std::make_tuple(x.g.conv, x.g.schoolbook, x.g.log_t, x.g.np, x.g.sign, x.square, x.index) <
               std::make_tuple(y.g.conv, y.g.schoolbook, y.g.log_t, y.g.np, y.g.sign, y.square, y.index);
    });
    if (!b->arena.ensure(std::max<u64>(arena_bytes, 256)) || !b->desc.ensure(members.size() * sizeof(ProductDesc)))
        return 0;
    if (b->pending && !cuda_ok(cudaEventSynchronize(b->staged), "descriptor staging")) return 0;
    b->pending = false;
    // A product that the planner splits (one operand many times longer than the
    // other) runs as its own block split: the shorter operand's spectrum once, the
    // longer operand's blocks as members of one class (exec.cu), in its arena slot.
    for (const Member& m : splits) {
        const ntt_request& r = reqs[m.index];
        if (!execute(m.g, false, r.a, r.b, r.dst, (uint8_t*)b->arena.ptr + m.offset, st, nullptr, b->status_dev,
                     false))
            return 0;
        ++b->split_members;
    }
    if (members.empty()) return 1;
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
        // the member's scratch: [admission votes][residues][carry flags] (host.h)
        d.spec = (u32*)(arena + m.offset + m.g.head_bytes());
        d.conv_len = m.g.conv_len;
        d.dst = r.dst;
        d.out_len = m.g.out_len;
        d.agg = m.g.conv ? nullptr : (uint8_t*)d.spec + m.g.spec_bytes(m.square);
        d.votes = m.g.conv ? (u32*)(arena + m.offset) : nullptr;
        d.square = m.square ? 1u : 0u;
        d.stride = (u32)m.g.stride;
        d.max_a = m.g.max_a;
        d.max_b = m.square ? m.g.max_a : m.g.max_b;
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
                note_launches(2);
                u32* votes = d.votes;
                if (!cuda_ok(launch_conv_admit(d.a, d.la, d.b, d.lb, d.max_a, d.max_b, g0.sign != 0, votes, st),
                             "admission launch") ||
                    !cuda_ok(launch_conv_schoolbook(d.a, d.la, d.b, d.lb, d.dst, (int)d.stride, g0.sign != 0, st,
                                                    votes, b->status_dev),
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

}  // extern "C"
