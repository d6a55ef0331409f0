// Enqueue of one product or convolution (single transforms, the four-step kernel
// sequence, the fused small products, block-split products) and of one transform
// class of batch members, on device pointers.
#include <cstring>

#include "host.h"

namespace ntt {

// ---------------------------------------------------------------------------------
// Execution on device pointers

// Enqueues the kernels of `n` members of one transform class (same kind, length,
// primes, sign and square) whose descriptors sit in device memory; max_len is the
// longest member output (limbs of a product, coefficients of a convolution).
bool run_members(const ProductDesc* descs, int n, const Geom& g0, bool sq, u64 max_len, cudaStream_t st,
                 u32* status, u32* shared_spec) {
    TransformArgs ta;
    memset(&ta, 0, sizeof(ta));
    CrtParams cp;
    const int log_r = four_step_log_r(g0);
    if (!prepare_params(g0, log_r, ta.ps, cp)) return false;
    ta.batch = descs;
    ta.count = n;
    ta.shared_spec = shared_spec;
    ta.a_only = shared_spec ? 1 : 0;
    ta.np = g0.np;
    ta.log_t = g0.log_t;
    ta.wide = g0.wide;
    const bool sign = g0.sign != 0;
    mark(st);
    // coefficient bounds of every convolution member (its votes): checked by the
    // one-CTA transform or the forward column pass as they load the coefficients;
    // the column pass only raises votes, so they are zeroed first
    ta.admit = g0.conv ? 1 : 0;
    if (g0.conv && g0.log_t > kMaxBlockLog) {
        note_launches(1);
        if (!cuda_ok(launch_clear_votes_batch(descs, n, st), "batched vote clearing launch")) return false;
        mark(st);
    }
    if (!shared_spec && !g0.conv && g0.log_t <= kFusedMaxLog && g0.np == kFusedPrimes && !g0.wide) {
        note_launches(1);
        const bool ok = cuda_ok(launch_small_fused(ta, cp, sq, st), "batched fused product launch");
        mark(st);
        return ok;
    }
    if (g0.log_t <= kMaxBlockLog) {
        note_launches(1);
        if (!cuda_ok(launch_small(ta, shared_spec ? kRowPre : sq ? kRowSqr : kRowMul, sign, st),
                     "batched transform launch"))
            return false;
        mark(st);
    } else {
        ta.log_r = log_r;
        ta.log_c = g0.log_t - ta.log_r;
        note_launches(3);
        if (!cuda_ok(launch_fwd_cols(ta, sq, sign, st), "batched column pass launch")) return false;
        mark(st);
        if (!cuda_ok(launch_rows(ta, shared_spec ? kRowPre : sq ? kRowSqr : kRowMul, st), "batched row pass launch"))
            return false;
        mark(st);
        if (!cuda_ok(launch_inv_cols(ta, st), "batched inverse column pass launch")) return false;
        mark(st);
    }
    note_launches(1);
    const bool ok =
        g0.conv ? cuda_ok(launch_crt_conv_batch(descs, n, max_len, g0.log_t, cp, st, status), "batched CRT launch")
                : cuda_ok(launch_crt_mul_batch(descs, n, (int)((max_len + kCrtTile - 1) / kCrtTile), g0.log_t, cp, st,
                                               status),
                          "batched CRT launch");
    mark(st);
    return ok;
}

// Enqueues a split product: the spectrum of the shorter operand once (its column
// pass, then the row pass in kRowFwd mode, or the one-CTA transform), then the
// blocks of the longer operand as batch members in chunks, each transforming its
// block alone and multiplying by that spectrum (the even blocks' products straight
// into dst, the odd ones' into a second number), then dst += odd with carries.
static bool execute_split(const Geom& g, const u64* d_a, const u64* d_b, u64* d_dst, void* scratch, cudaStream_t st,
                          u32* status) {
    const bool swap = g.la < g.lb;
    const u64* lng = swap ? d_b : d_a;
    const u64* sht = swap ? d_a : d_b;
    const u64 L = std::max(g.la, g.lb), S = std::min(g.la, g.lb);
    uint8_t* base = (uint8_t*)scratch;
    ProductDesc* descs = (ProductDesc*)base;
    u64* odd = (u64*)(base + g.split_desc_bytes());
    u32* flags = (u32*)((uint8_t*)odd + g.split_odd_bytes());
    u32* spectrum = (u32*)((uint8_t*)flags + g.split_flag_bytes());
    uint8_t* arena = (uint8_t*)spectrum + g.spec_bytes(true);
    const u64 member = g.member_bytes(false), spec = g.spec_bytes(true);
    if (!cuda_ok(cudaMemsetAsync(d_dst, 0, g.out_len * 8, st), "zero product") ||
        !cuda_ok(cudaMemsetAsync(odd, 0, g.out_len * 8, st), "zero odd blocks") ||
        !cuda_ok(cudaMemsetAsync(flags, 0, carry_scratch_bytes(g.out_len), st), "zero carry flags"))
        return false;
    // the shorter operand's spectrum, once for every block
    TransformArgs tb;
    memset(&tb, 0, sizeof(tb));
    CrtParams cp;
    const int log_r = four_step_log_r(g);
    if (!prepare_params(g, log_r, tb.ps, cp)) return false;
    tb.a = tb.b = sht;
    tb.la = tb.lb = S;
    tb.spec = spectrum;
    tb.conv_len = g.block + S - 1;
    tb.np = g.np;
    tb.log_t = g.log_t;
    tb.log_r = log_r;
    tb.log_c = g.log_t - log_r;
    tb.wide = g.wide;
    tb.op_count = 1;
    tb.shared_spec = spectrum;
    if (log_r == 0) {  // one CTA per prime holds the block transform
        note_launches(1);
        if (!cuda_ok(launch_small(tb, kRowFwd, false, st), "spectrum transform launch")) return false;
    } else {
        note_launches(2);
        if (!cuda_ok(launch_fwd_cols(tb, true, false, st), "spectrum column pass launch") ||
            !cuda_ok(launch_rows(tb, kRowFwd, st), "spectrum row pass launch"))
            return false;
    }
    mark(st);
    const u64 chunk = g.split_chunk();
    for (u64 first = 0; first < g.blocks; first += chunk) {
        const u64 count = std::min(chunk, g.blocks - first);
        note_launches(1);
        if (!cuda_ok(launch_split_descs(descs, first, count, lng, L, sht, S, g.block, d_dst, odd, arena, member, spec,
                                        st),
                     "split descriptors") ||
            !run_members(descs, (int)count, g, false, g.block + S, st, status, spectrum))
            return false;
    }
    note_launches(1);
    return cuda_ok(launch_add_limbs(d_dst, odd, g.out_len, flags, st, status), "block sum");
}

// Enqueues one product or convolution on `st`. With `b_ready` set (an event that
// completes when operand b is in place), the column pass of a runs first and the
// one of b waits for that event, so b's upload overlaps a's pass.
std::atomic<uint64_t> g_school_max{kSchoolDefaultProducts};

bool takes_basecase(const Geom& g) {
    return !g.conv && !g.split() && (double)g.la * (double)g.lb <= (double)g_school_max.load() &&
           school_fits(g.la, g.lb);
}

bool execute(const Geom& g, bool square, const u64* d_a, const u64* d_b, u64* d_dst,
             void* scratch, cudaStream_t st, cudaEvent_t b_ready, u32* status, bool admit) {
    mark(st);
    if (takes_basecase(g)) {  // one cluster of direct column sums, no scratch
        if (!kernels_ready()) return false;
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        note_launches(1);
        const bool ok = cuda_ok(launch_school_mul(d_a, g.la, square ? d_a : d_b, square ? g.la : g.lb, d_dst, st),
                                "basecase launch");
        mark(st);
        return ok;
    }
    if (g.split()) {
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        const bool ok = execute_split(g, d_a, square ? d_a : d_b, d_dst, scratch, st, status);
        mark(st);
        return ok;
    }
    // Device-side admission of a convolution's coefficients: votes at the start of
    // the scratch, written by the transform that loads the coefficients (the
    // one-CTA transform writes every vote; the forward column pass only raises
    // them, so they are zeroed first), or by a scan kernel before the schoolbook.
    u32* votes = g.conv && admit ? (u32*)scratch : nullptr;
    if (votes && !g.schoolbook && single_log_r(g) != 0 &&
        !cuda_ok(cudaMemsetAsync(votes, 0, kAdmitBytes, st), "zero admission votes"))
        return false;
    if (votes && g.schoolbook) {
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        b_ready = nullptr;
        note_launches(1);
        if (!cuda_ok(launch_conv_admit(d_a, g.la, square ? d_a : d_b, square ? g.la : g.lb, g.max_a,
                                       square ? g.max_a : g.max_b, g.sign != 0, votes, st),
                     "admission launch"))
            return false;
        mark(st);
    }
    if (g.conv && g.schoolbook) {
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        note_launches(1);
        const bool ok = cuda_ok(launch_conv_schoolbook(d_a, g.la, square ? d_a : d_b, square ? g.la : g.lb, d_dst,
                                                       (int)g.stride, g.sign != 0, st, votes, status),
                                "conv schoolbook launch");
        mark(st);
        return ok;
    }
    TransformArgs ta;
    memset(&ta, 0, sizeof(ta));
    CrtParams cp;
    const int log_r = single_log_r(g);
    if (!prepare_params(g, log_r, ta.ps, cp)) return false;
    ta.a = d_a;
    ta.b = square ? d_a : d_b;
    ta.la = g.la;
    ta.lb = square ? g.la : g.lb;
    ta.spec = (u32*)((uint8_t*)scratch + g.head_bytes());
    ta.conv_len = g.conv_len;
    ta.np = g.np;
    ta.log_t = g.log_t;
    ta.wide = g.wide;
    const u64 spec_bytes = g.spec_bytes(square);
    if (!g.conv) {
        ta.flags = (u32*)((uint8_t*)ta.spec + spec_bytes);
        ta.flag_words = (u32)carry_flag_words(g.out_len);
    }
    const bool sign = g.sign != 0;
    if (!g.conv && log_r == 0 && g.log_t <= kFusedMaxLog && g.np == kFusedPrimes && !g.wide) {
        // the whole product in one cluster launch
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        ta.dst = d_dst;
        ta.out_len = g.out_len;
        note_launches(1);
        const bool ok = cuda_ok(launch_small_fused(ta, cp, square, st), "fused product launch");
        mark(st);
        return ok;
    }
    if (log_r == 0) {
        if (b_ready && !cuda_ok(cudaStreamWaitEvent(st, b_ready, 0), "cudaStreamWaitEvent")) return false;
        ta.votes = votes;
        ta.max_a = g.max_a;
        ta.max_b = square ? g.max_a : g.max_b;
        note_launches(1);
        if (!cuda_ok(launch_small(ta, square ? kRowSqr : kRowMul, sign, st), "transform launch")) return false;
        mark(st);
    } else {
        ta.log_r = log_r;
        ta.log_c = g.log_t - ta.log_r;
        ta.votes = votes;
        ta.max_a = g.max_a;
        ta.max_b = square ? g.max_a : g.max_b;
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
        if (!cuda_ok(launch_rows(ta, square ? kRowSqr : kRowMul, st), "row pass launch")) return false;
        mark(st);
        if (!cuda_ok(launch_inv_cols(ta, st), "inverse column pass launch")) return false;
        mark(st);
    }
    if (g.conv) {
        note_launches(1);
        const bool ok =
            cuda_ok(launch_crt_conv(ta.spec, g.log_t, g.conv_len, d_dst, sign, cp, st, votes, status), "CRT launch");
        mark(st);
        return ok;
    }
    if (take_injected_stall() &&
        !cuda_ok(cudaMemsetAsync(ta.flags, 1, 1, st), "stall injection"))  // tile counter = 1
        return false;
    note_launches(1);
    return cuda_ok(launch_crt_mul(ta.spec, g.log_t, g.conv_len, g.out_len, d_dst, (uint8_t*)ta.flags, cp, st,
                                  mark, status),
                   "CRT launch");
}


bool coefficients_admitted(const Geom& g, const u64* v, u64 n, u64 max) {
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
