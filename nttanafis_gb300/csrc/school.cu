// Exact products of short operands by direct column sums (the basecase below the
// transform crossover; the reference's own crossover against schoolbook products
// sits near 192 limbs, README.md:39).
//
// One thread-block cluster of CL CTAs per product whose result fits one tile of
// kCrtTile limbs (a_len + b_len <= 1024). The longer operand x is cut into CL
// slices; CTA r multiplies its slice by the whole shorter operand y into column
// sums c_k = sum x_i y_(k-i) over the slice, each in three 64-bit words (a column
// of at most 1023 128-bit products stays below 2^138), and stores them straight
// into CTA 0's shared memory (distributed shared memory, plain stores). After one
// cluster barrier CTA 0 adds the partial sums of each column from its own shared
// memory, then forms the limbs and carries of the tile with the CRT kernels'
// window sums and scans (crt.cuh). No scratch memory, one launch, nothing
// round-trips through HBM. CL is chosen per shape (launch_school_mul): one CTA for
// the smallest products, up to 8 where the products' work pays for more SMs.
#include <cooperative_groups.h>

#include "crt.cuh"
#include "launch.h"

namespace ntt {

namespace {

constexpr int kThreadsS = kCrtThreads;  // 256: the tile of four limbs per thread

// acc (three words) += x * y, one carry chain in one PTX statement.
__device__ __forceinline__ void mac128(u64& a0, u64& a1, u64& a2, u64 x, u64 y) {
    asm("mad.lo.cc.u64 %0, %3, %4, %0;\n\t"
        "madc.hi.cc.u64 %1, %3, %4, %1;\n\t"
        "addc.u64 %2, %2, 0;"
        : "+l"(a0), "+l"(a1), "+l"(a2)
        : "l"(x), "l"(y));
}

// (a0, a1, a2) += (b0, b1, b2), one carry chain.
__device__ __forceinline__ void add192(u64& a0, u64& a1, u64& a2, u64 b0, u64 b1, u64 b2) {
    asm("add.cc.u64 %0, %0, %3;\n\t"
        "addc.cc.u64 %1, %1, %4;\n\t"
        "addc.u64 %2, %2, %5;"
        : "+l"(a0), "+l"(a1), "+l"(a2)
        : "l"(b0), "l"(b1), "l"(b2));
}

// Slice of the longer operand (lx limbs) held by cluster rank r of CL.
template <int CL>
__device__ __forceinline__ void slice_of(u64 lx, int r, u64& first, u64& count) {
    const u64 per = (lx + CL - 1) / CL;
    first = min((u64)r * per, lx);
    count = min(per, lx - first);
}

}  // namespace

// grid = cluster = (CL, 1, 1). Dynamic shared memory: the shorter operand, the
// CTA's slice, and (used in CTA 0) CL rows of three words per column.
template <int CL>
__global__ void __launch_bounds__(kThreadsS) k_school_mul(const u64* __restrict__ a, u64 la,
                                                          const u64* __restrict__ b, u64 lb,
                                                          u64* __restrict__ dst) {
    namespace cg = cooperative_groups;
    extern __shared__ u64 sm64[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const bool swap = la < lb;
    const u64* x = swap ? b : a;
    const u64* y = swap ? a : b;
    const u64 lx = swap ? lb : la, ly = swap ? la : lb;
    const u64 out_len = la + lb, conv_len = out_len - 1;
    const u64 per = (lx + CL - 1) / CL;
    u64 first, count;
    slice_of<CL>(lx, rank, first, count);
    u64* sy = sm64;        // y[0, ly)
    u64* sx = sy + ly;     // x[first, first + count)
    u64* acc = sx + per;   // [CL][conv_len][3] partial column sums, filled in CTA 0
    for (u64 i = threadIdx.x; i < ly; i += kThreadsS) sy[i] = __ldg(y + i);
    for (u64 i = threadIdx.x; i < count; i += kThreadsS) sx[i] = __ldg(x + first + i);
    __syncthreads();
    // Column first + c sums x_i y_(first + c - i) over the slice's i, in four
    // interleaved partial sums (independent carry chains), stored into CTA 0.
    u64* acc0 = cluster.map_shared_rank(acc, 0) + (size_t)rank * conv_len * 3;
    const u64 ncols = count ? count + ly - 1 : 0;
    for (u64 c = threadIdx.x; c < ncols; c += kThreadsS) {
        const u64 i_lo = c >= ly - 1 ? c - (ly - 1) : 0;  // slice-relative
        const u64 i_hi = min(c, count - 1);
        u64 s[4][3] = {};
        u64 i = i_lo;
        for (; i + 3 <= i_hi; i += 4) {
#pragma unroll
            for (int u = 0; u < 4; ++u) mac128(s[u][0], s[u][1], s[u][2], sx[i + u], sy[c - i - u]);
        }
        for (; i <= i_hi; ++i) mac128(s[0][0], s[0][1], s[0][2], sx[i], sy[c - i]);
#pragma unroll
        for (int u = 1; u < 4; ++u) add192(s[0][0], s[0][1], s[0][2], s[u][0], s[u][1], s[u][2]);
        u64* p = acc0 + 3 * (first + c);
        p[0] = s[0][0];
        p[1] = s[0][1];
        p[2] = s[0][2];
    }
    cluster.sync();  // every slice's column sums are in CTA 0
    if (rank != 0) return;

    // CTA 0: the column sums, then the tile's limbs and carries.
    constexpr int L = 3;
    __shared__ u64 s_pre[L][L];
    auto column = [&](u64 k, u64 (&w)[L]) {
        w[0] = w[1] = w[2] = 0;
        if (k >= conv_len) return;
#pragma unroll
        for (int r = 0; r < CL; ++r) {
            u64 f, n;
            slice_of<CL>(lx, r, f, n);
            if (!n || k < f || k >= f + n + ly - 1) continue;
            const u64* p = acc + ((size_t)r * conv_len + k) * 3;
            add192(w[0], w[1], w[2], p[0], p[1], p[2]);
        }
    };
    const int t = threadIdx.x;
    const u64 k0 = (u64)t * kCrtPer;
    u64 cw[kCrtPer][L];
#pragma unroll
    for (int c = 0; c < kCrtPer; ++c) column(k0 + c, cw[c]);
    if (t < L) {
#pragma unroll
        for (int i = 0; i < L; ++i) s_pre[t][i] = 0;  // nothing before the only tile
    }
    u64 sv[kCrtPer];
    u32 gb[kCrtPer], pb[kCrtPer], xg, xp, tg, tp;
    tile_limbs<L>(cw, s_pre, sv, gb, pb);
    tile_scan(gb, pb, xg, xp, tg, tp);
    store_limbs(dst, k0, out_len, sv, gb, pb, xg);  // carry into the tile: 0
}

namespace {

// Cluster size of a product by its limb products, from per-call timings on GB300
// (n x n, back to back on one stream): one CTA up to 1,024 (a cluster launch costs
// one more 2 us step: 8 x 8 took 4.6 us on one CTA, 6.1 us on two), two CTAs up to
// 4,096, four above (n = 96: 6.5 us on two, 6.2 on four). Within the shared-memory
// budget of CTA 0; NTT_SCHOOL_CL fixes it at build time.
#ifndef NTT_SCHOOL_CL
#define NTT_SCHOOL_CL 0
#endif
int school_cluster(u64 la, u64 lb) {
    const double work = (double)la * (double)lb;
    int cl = NTT_SCHOOL_CL ? NTT_SCHOOL_CL : work <= 1024 ? 1 : work <= 4096 ? 2 : work <= 16384 ? 4 : 8;
    while (cl > 1 && school_smem_cl(la, lb, cl) > (size_t)kSchoolSmemMax) cl >>= 1;
    return cl;
}

template <int CL>
cudaError_t launch_cl(const u64* a, u64 la, const u64* b, u64 lb, u64* dst, size_t smem, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CL);
    cfg.blockDim = dim3(kThreadsS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_school_mul<CL>, a, la, b, lb, dst);
}

}  // namespace

size_t school_smem_cl(u64 la, u64 lb, int cl) {
    const u64 lx = la > lb ? la : lb, ly = la > lb ? lb : la;
    const u64 per = (lx + cl - 1) / cl;
    return (size_t)(ly + per + (u64)cl * (la + lb - 1) * 3) * sizeof(u64);
}

bool school_fits(u64 la, u64 lb) {
    return la && lb && la + lb <= kSchoolMaxOut && school_smem_cl(la, lb, 1) <= (size_t)kSchoolSmemMax;
}

cudaError_t launch_school_mul(const u64* a, u64 la, const u64* b, u64 lb, u64* dst, cudaStream_t st) {
    const int cl = school_cluster(la, lb);
    const size_t smem = school_smem_cl(la, lb, cl);
    switch (cl) {
        case 1: return launch_cl<1>(a, la, b, lb, dst, smem, st);
        case 2: return launch_cl<2>(a, la, b, lb, dst, smem, st);
        case 4: return launch_cl<4>(a, la, b, lb, dst, smem, st);
        default: return launch_cl<8>(a, la, b, lb, dst, smem, st);
    }
}

cudaError_t init_school_kernels() {
    cudaError_t e = cudaFuncSetAttribute(k_school_mul<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSchoolSmemMax);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_school_mul<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSchoolSmemMax);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_school_mul<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSchoolSmemMax);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_school_mul<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSchoolSmemMax);
    return e;
}

}  // namespace ntt
