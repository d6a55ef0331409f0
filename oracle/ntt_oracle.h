/* CPU restatement of ntt_anafis's multiplication path: test infrastructure (the
 * parity checker and the timed CPU baseline), never part of the product. */
#ifndef NTT_ORACLE_H
#define NTT_ORACLE_H
#include <stdint.h>

int oracle_mul(uint64_t* dst, const uint64_t* a, uint64_t la, const uint64_t* b, uint64_t lb, int threads);
int oracle_sqr(uint64_t* dst, const uint64_t* a, uint64_t la, int threads);
int oracle_conv(uint64_t* dst, const uint64_t* a, uint64_t la, const uint64_t* b, uint64_t lb, uint64_t max_a,
                uint64_t max_b, int is_signed, int threads);
/* [count, chunk_bits, digits_a, digits_b, conv_len, transform_len, cyclic_len, table_len] */
int oracle_mul_plan(uint64_t la, uint64_t lb, int crt_cost, int64_t* out);
/* [count, stride, bound_bits, schoolbook, transform_len, cyclic_len, table_len, output_len] */
int oracle_conv_plan(uint64_t la, uint64_t lb, uint64_t max_a, uint64_t max_b, int is_signed, int64_t* out);
int oracle_row_shape(uint64_t conv_len, uint64_t longest, uint64_t* out3);
int oracle_capacity(int count);
void oracle_schoolbook(uint64_t* dst, const uint64_t* a, uint64_t la, const uint64_t* b, uint64_t lb);
void oracle_operand(uint64_t* dst, uint64_t len, uint64_t seed);
int oracle_transform_check(int prime, int log_n, uint64_t seed);
#endif
