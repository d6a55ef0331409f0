// Integer-butterfly throughput probe: the compute ceiling the transform kernels
// are measured against. Each thread keeps 16 residues and 8 twiddles (with Shoup
// companions) in registers and runs radix-16 forward passes of the library's lazy
// butterfly (LazyArith::dif: 4 ALU-pipe and 3 FMA-pipe instructions) with no
// memory traffic, so the rate is bounded by instruction issue alone. The result is
// a checksum (so no work can be dropped) and the elapsed time of the timed launch.
#include <cuda_runtime.h>

#include "launch.h"

namespace ntt {
namespace {

__global__ void __launch_bounds__(256) k_probe_butterflies(u32* __restrict__ out, u32 p, u32 w0, u32 wp0,
                                                           int iters) {
    u32 x[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = (threadIdx.x * 16 + i) % p;
    uint2 w[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) w[i] = make_uint2(w0 + i, wp0 + i);
#pragma unroll 1
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int half = 8 >> t;
#pragma unroll
            for (int b = 0; b < 16; b += 2 * half)
#pragma unroll
                for (int c = 0; c < half; ++c) LazyArith::dif(x[b + c], x[b + c + half], w[c], p);
        }
    }
    u32 acc = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) acc ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace
}  // namespace ntt

using namespace ntt;

extern "C" {

// Runs `blocks` CTAs of 256 threads for `iters` radix-16 passes (32 butterflies
// per thread and pass) after one warm-up launch; writes the timed launch's
// milliseconds to *ms. Returns 0 on a CUDA failure.
uint8_t ntt_probe_butterflies(int blocks, int iters, float* ms) {
    if (blocks <= 0 || iters <= 0 || !ms) return 0;
    u32* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = cudaMalloc(&out, (size_t)blocks * 256 * sizeof(u32)) == cudaSuccess &&
              cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
    if (ok) {
        const u32 p = 998244353u;
        k_probe_butterflies<<<blocks, 256>>>(out, p, 12345u, 678u, iters / 8 + 1);
        cudaEventRecord(e0);
        k_probe_butterflies<<<blocks, 256>>>(out, p, 12345u, 678u, iters);
        cudaEventRecord(e1);
        ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(ms, e0, e1) == cudaSuccess;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    if (!ok) set_last_error("butterfly probe failed");
    return ok ? 1 : 0;
}

}  // extern "C"
