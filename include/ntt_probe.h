/*
 * C ABI of libntt_probe.so: register-only arithmetic probes for measurement tools
 * (the compute ceiling of the transform kernels, and the per-butterfly cost of
 * candidate residue arithmetics). Not part of the product library; no counterpart
 * in the reference crate.
 */
#ifndef NTT_PROBE_H
#define NTT_PROBE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Number of probe variants (see ntt_probe_arith). */
int ntt_probe_variants(void);

/* Runs `blocks` CTAs of 256 threads, each thread doing `iters` iterations of
 * variant `variant` with no memory traffic, after one shorter warm-up launch;
 * writes the timed launch's milliseconds to *ms and the operations it performed
 * to *ops (butterflies for variants 0-3 and 11-12, instructions for 4-10). Variants:
 * 0 lazy 32-bit Shoup butterfly (the transforms' own), 1 32-bit Montgomery
 * butterfly, 2 64-bit Shoup butterfly over a 50-bit prime, 3 the f64 FMA
 * exact-remainder butterfly over a 50-bit prime; 4 IMAD, 5 IMAD.HI, 6 integer
 * adds, 7 64-bit integer multiply, 8 f64 FMA, 9 IMAD.WIDE (32 x 32 -> 64-bit
 * multiply-add), 10 u32 -> f32 conversion; 11 and 12 variant 0 with its Shoup
 * quotient from a 64-bit product (11 PTX mul.wide, 12 C). Synchronizes the device; returns 0
 * on a CUDA failure or an unknown variant. */
uint8_t ntt_probe_arith(int variant, int blocks, int iters, float* ms, double* ops);

/* Variant 0 alone: 32 lazy butterflies per thread and iteration. */
uint8_t ntt_probe_butterflies(int blocks, int iters, float* ms);

#ifdef __cplusplus
}
#endif

#endif /* NTT_PROBE_H */
