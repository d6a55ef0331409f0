// Generated by gen_crt_chains.py: multiword carry chains of the CRT, one
// inline-PTX statement per chain (the carry flag never crosses statements).
#pragma once
#include "ntt_arith.cuh"

namespace ntt {

template <int NP>
struct CrtChains;

template <>
struct CrtChains<1> {
    static __device__ __forceinline__ void accumulate(u32 (&S)[2], u32 y, const u32* M) {
        asm(
        "mad.lo.cc.u32 %0, %2, %3, %0;\n\t"
        "addc.u32 %1, %1, 0;\n\t"
        "mad.hi.cc.u32 %1, %2, %3, %1;\n\t"
        : "+r"(S[0]), "+r"(S[1])
        : "r"(y), "r"(M[0]));
    }
    static __device__ __forceinline__ void subtract(u32 (&x)[2], const u32 (&S)[2], const u32 (&U)[2]) {
        asm(
        "sub.cc.u32 %0, %2, %4;\n\t"
        "subc.u32 %1, %3, %5;\n\t"
        : "=r"(x[0]), "=r"(x[1])
        : "r"(S[0]), "r"(S[1]), "r"(U[0]), "r"(U[1]));
    }
};

template <>
struct CrtChains<2> {
    static __device__ __forceinline__ void accumulate(u32 (&S)[3], u32 y, const u32* M) {
        asm(
        "mad.lo.cc.u32 %0, %3, %4, %0;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        "mad.hi.cc.u32 %1, %3, %4, %1;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        : "+r"(S[0]), "+r"(S[1]), "+r"(S[2])
        : "r"(y), "r"(M[0]));
    }
    static __device__ __forceinline__ void subtract(u32 (&x)[3], const u32 (&S)[3], const u32 (&U)[3]) {
        asm(
        "sub.cc.u32 %0, %3, %6;\n\t"
        "subc.cc.u32 %1, %4, %7;\n\t"
        "subc.u32 %2, %5, %8;\n\t"
        : "=r"(x[0]), "=r"(x[1]), "=r"(x[2])
        : "r"(S[0]), "r"(S[1]), "r"(S[2]), "r"(U[0]), "r"(U[1]), "r"(U[2]));
    }
};

template <>
struct CrtChains<3> {
    static __device__ __forceinline__ void accumulate(u32 (&S)[4], u32 y, const u32* M) {
        asm(
        "mad.lo.cc.u32 %0, %4, %5, %0;\n\t"
        "madc.lo.cc.u32 %1, %4, %6, %1;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.u32 %3, %3, 0;\n\t"
        "mad.hi.cc.u32 %1, %4, %5, %1;\n\t"
        "madc.hi.cc.u32 %2, %4, %6, %2;\n\t"
        "addc.u32 %3, %3, 0;\n\t"
        : "+r"(S[0]), "+r"(S[1]), "+r"(S[2]), "+r"(S[3])
        : "r"(y), "r"(M[0]), "r"(M[1]));
    }
    static __device__ __forceinline__ void subtract(u32 (&x)[4], const u32 (&S)[4], const u32 (&U)[4]) {
        asm(
        "sub.cc.u32 %0, %4, %8;\n\t"
        "subc.cc.u32 %1, %5, %9;\n\t"
        "subc.cc.u32 %2, %6, %10;\n\t"
        "subc.u32 %3, %7, %11;\n\t"
        : "=r"(x[0]), "=r"(x[1]), "=r"(x[2]), "=r"(x[3])
        : "r"(S[0]), "r"(S[1]), "r"(S[2]), "r"(S[3]), "r"(U[0]), "r"(U[1]), "r"(U[2]), "r"(U[3]));
    }
};

template <>
struct CrtChains<4> {
    static __device__ __forceinline__ void accumulate(u32 (&S)[5], u32 y, const u32* M) {
        asm(
        "mad.lo.cc.u32 %0, %5, %6, %0;\n\t"
        "madc.lo.cc.u32 %1, %5, %7, %1;\n\t"
        "madc.lo.cc.u32 %2, %5, %8, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.hi.cc.u32 %1, %5, %6, %1;\n\t"
        "madc.hi.cc.u32 %2, %5, %7, %2;\n\t"
        "madc.hi.cc.u32 %3, %5, %8, %3;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        : "+r"(S[0]), "+r"(S[1]), "+r"(S[2]), "+r"(S[3]), "+r"(S[4])
        : "r"(y), "r"(M[0]), "r"(M[1]), "r"(M[2]));
    }
    static __device__ __forceinline__ void subtract(u32 (&x)[5], const u32 (&S)[5], const u32 (&U)[5]) {
        asm(
        "sub.cc.u32 %0, %5, %10;\n\t"
        "subc.cc.u32 %1, %6, %11;\n\t"
        "subc.cc.u32 %2, %7, %12;\n\t"
        "subc.cc.u32 %3, %8, %13;\n\t"
        "subc.u32 %4, %9, %14;\n\t"
        : "=r"(x[0]), "=r"(x[1]), "=r"(x[2]), "=r"(x[3]), "=r"(x[4])
        : "r"(S[0]), "r"(S[1]), "r"(S[2]), "r"(S[3]), "r"(S[4]), "r"(U[0]), "r"(U[1]), "r"(U[2]), "r"(U[3]), "r"(U[4]));
    }
};

template <>
struct CrtChains<5> {
    static __device__ __forceinline__ void accumulate(u32 (&S)[6], u32 y, const u32* M) {
        asm(
        "mad.lo.cc.u32 %0, %6, %7, %0;\n\t"
        "madc.lo.cc.u32 %1, %6, %8, %1;\n\t"
        "madc.lo.cc.u32 %2, %6, %9, %2;\n\t"
        "madc.lo.cc.u32 %3, %6, %10, %3;\n\t"
        "addc.cc.u32 %4, %4, 0;\n\t"
        "addc.u32 %5, %5, 0;\n\t"
        "mad.hi.cc.u32 %1, %6, %7, %1;\n\t"
        "madc.hi.cc.u32 %2, %6, %8, %2;\n\t"
        "madc.hi.cc.u32 %3, %6, %9, %3;\n\t"
        "madc.hi.cc.u32 %4, %6, %10, %4;\n\t"
        "addc.u32 %5, %5, 0;\n\t"
        : "+r"(S[0]), "+r"(S[1]), "+r"(S[2]), "+r"(S[3]), "+r"(S[4]), "+r"(S[5])
        : "r"(y), "r"(M[0]), "r"(M[1]), "r"(M[2]), "r"(M[3]));
    }
    static __device__ __forceinline__ void subtract(u32 (&x)[6], const u32 (&S)[6], const u32 (&U)[6]) {
        asm(
        "sub.cc.u32 %0, %6, %12;\n\t"
        "subc.cc.u32 %1, %7, %13;\n\t"
        "subc.cc.u32 %2, %8, %14;\n\t"
        "subc.cc.u32 %3, %9, %15;\n\t"
        "subc.cc.u32 %4, %10, %16;\n\t"
        "subc.u32 %5, %11, %17;\n\t"
        : "=r"(x[0]), "=r"(x[1]), "=r"(x[2]), "=r"(x[3]), "=r"(x[4]), "=r"(x[5])
        : "r"(S[0]), "r"(S[1]), "r"(S[2]), "r"(S[3]), "r"(S[4]), "r"(S[5]), "r"(U[0]), "r"(U[1]), "r"(U[2]), "r"(U[3]), "r"(U[4]), "r"(U[5]));
    }
};

template <>
struct CrtChains<6> {
    static __device__ __forceinline__ void accumulate(u32 (&S)[7], u32 y, const u32* M) {
        asm(
        "mad.lo.cc.u32 %0, %7, %8, %0;\n\t"
        "madc.lo.cc.u32 %1, %7, %9, %1;\n\t"
        "madc.lo.cc.u32 %2, %7, %10, %2;\n\t"
        "madc.lo.cc.u32 %3, %7, %11, %3;\n\t"
        "madc.lo.cc.u32 %4, %7, %12, %4;\n\t"
        "addc.cc.u32 %5, %5, 0;\n\t"
        "addc.u32 %6, %6, 0;\n\t"
        "mad.hi.cc.u32 %1, %7, %8, %1;\n\t"
        "madc.hi.cc.u32 %2, %7, %9, %2;\n\t"
        "madc.hi.cc.u32 %3, %7, %10, %3;\n\t"
        "madc.hi.cc.u32 %4, %7, %11, %4;\n\t"
        "madc.hi.cc.u32 %5, %7, %12, %5;\n\t"
        "addc.u32 %6, %6, 0;\n\t"
        : "+r"(S[0]), "+r"(S[1]), "+r"(S[2]), "+r"(S[3]), "+r"(S[4]), "+r"(S[5]), "+r"(S[6])
        : "r"(y), "r"(M[0]), "r"(M[1]), "r"(M[2]), "r"(M[3]), "r"(M[4]));
    }
    static __device__ __forceinline__ void subtract(u32 (&x)[7], const u32 (&S)[7], const u32 (&U)[7]) {
        asm(
        "sub.cc.u32 %0, %7, %14;\n\t"
        "subc.cc.u32 %1, %8, %15;\n\t"
        "subc.cc.u32 %2, %9, %16;\n\t"
        "subc.cc.u32 %3, %10, %17;\n\t"
        "subc.cc.u32 %4, %11, %18;\n\t"
        "subc.cc.u32 %5, %12, %19;\n\t"
        "subc.u32 %6, %13, %20;\n\t"
        : "=r"(x[0]), "=r"(x[1]), "=r"(x[2]), "=r"(x[3]), "=r"(x[4]), "=r"(x[5]), "=r"(x[6])
        : "r"(S[0]), "r"(S[1]), "r"(S[2]), "r"(S[3]), "r"(S[4]), "r"(S[5]), "r"(S[6]), "r"(U[0]), "r"(U[1]), "r"(U[2]), "r"(U[3]), "r"(U[4]), "r"(U[5]), "r"(U[6]));
    }
};

template <>
struct CrtChains<7> {
    static __device__ __forceinline__ void accumulate(u32 (&S)[8], u32 y, const u32* M) {
        asm(
        "mad.lo.cc.u32 %0, %8, %9, %0;\n\t"
        "madc.lo.cc.u32 %1, %8, %10, %1;\n\t"
        "madc.lo.cc.u32 %2, %8, %11, %2;\n\t"
        "madc.lo.cc.u32 %3, %8, %12, %3;\n\t"
        "madc.lo.cc.u32 %4, %8, %13, %4;\n\t"
        "madc.lo.cc.u32 %5, %8, %14, %5;\n\t"
        "addc.cc.u32 %6, %6, 0;\n\t"
        "addc.u32 %7, %7, 0;\n\t"
        "mad.hi.cc.u32 %1, %8, %9, %1;\n\t"
        "madc.hi.cc.u32 %2, %8, %10, %2;\n\t"
        "madc.hi.cc.u32 %3, %8, %11, %3;\n\t"
        "madc.hi.cc.u32 %4, %8, %12, %4;\n\t"
        "madc.hi.cc.u32 %5, %8, %13, %5;\n\t"
        "madc.hi.cc.u32 %6, %8, %14, %6;\n\t"
        "addc.u32 %7, %7, 0;\n\t"
        : "+r"(S[0]), "+r"(S[1]), "+r"(S[2]), "+r"(S[3]), "+r"(S[4]), "+r"(S[5]), "+r"(S[6]), "+r"(S[7])
        : "r"(y), "r"(M[0]), "r"(M[1]), "r"(M[2]), "r"(M[3]), "r"(M[4]), "r"(M[5]));
    }
    static __device__ __forceinline__ void subtract(u32 (&x)[8], const u32 (&S)[8], const u32 (&U)[8]) {
        asm(
        "sub.cc.u32 %0, %8, %16;\n\t"
        "subc.cc.u32 %1, %9, %17;\n\t"
        "subc.cc.u32 %2, %10, %18;\n\t"
        "subc.cc.u32 %3, %11, %19;\n\t"
        "subc.cc.u32 %4, %12, %20;\n\t"
        "subc.cc.u32 %5, %13, %21;\n\t"
        "subc.cc.u32 %6, %14, %22;\n\t"
        "subc.u32 %7, %15, %23;\n\t"
        : "=r"(x[0]), "=r"(x[1]), "=r"(x[2]), "=r"(x[3]), "=r"(x[4]), "=r"(x[5]), "=r"(x[6]), "=r"(x[7])
        : "r"(S[0]), "r"(S[1]), "r"(S[2]), "r"(S[3]), "r"(S[4]), "r"(S[5]), "r"(S[6]), "r"(S[7]), "r"(U[0]), "r"(U[1]), "r"(U[2]), "r"(U[3]), "r"(U[4]), "r"(U[5]), "r"(U[6]), "r"(U[7]));
    }
};

template <>
struct CrtChains<8> {
    static __device__ __forceinline__ void accumulate(u32 (&S)[9], u32 y, const u32* M) {
        asm(
        "mad.lo.cc.u32 %0, %9, %10, %0;\n\t"
        "madc.lo.cc.u32 %1, %9, %11, %1;\n\t"
        "madc.lo.cc.u32 %2, %9, %12, %2;\n\t"
        "madc.lo.cc.u32 %3, %9, %13, %3;\n\t"
        "madc.lo.cc.u32 %4, %9, %14, %4;\n\t"
        "madc.lo.cc.u32 %5, %9, %15, %5;\n\t"
        "madc.lo.cc.u32 %6, %9, %16, %6;\n\t"
        "addc.cc.u32 %7, %7, 0;\n\t"
        "addc.u32 %8, %8, 0;\n\t"
        "mad.hi.cc.u32 %1, %9, %10, %1;\n\t"
        "madc.hi.cc.u32 %2, %9, %11, %2;\n\t"
        "madc.hi.cc.u32 %3, %9, %12, %3;\n\t"
        "madc.hi.cc.u32 %4, %9, %13, %4;\n\t"
        "madc.hi.cc.u32 %5, %9, %14, %5;\n\t"
        "madc.hi.cc.u32 %6, %9, %15, %6;\n\t"
        "madc.hi.cc.u32 %7, %9, %16, %7;\n\t"
        "addc.u32 %8, %8, 0;\n\t"
        : "+r"(S[0]), "+r"(S[1]), "+r"(S[2]), "+r"(S[3]), "+r"(S[4]), "+r"(S[5]), "+r"(S[6]), "+r"(S[7]), "+r"(S[8])
        : "r"(y), "r"(M[0]), "r"(M[1]), "r"(M[2]), "r"(M[3]), "r"(M[4]), "r"(M[5]), "r"(M[6]));
    }
    static __device__ __forceinline__ void subtract(u32 (&x)[9], const u32 (&S)[9], const u32 (&U)[9]) {
        asm(
        "sub.cc.u32 %0, %9, %18;\n\t"
        "subc.cc.u32 %1, %10, %19;\n\t"
        "subc.cc.u32 %2, %11, %20;\n\t"
        "subc.cc.u32 %3, %12, %21;\n\t"
        "subc.cc.u32 %4, %13, %22;\n\t"
        "subc.cc.u32 %5, %14, %23;\n\t"
        "subc.cc.u32 %6, %15, %24;\n\t"
        "subc.cc.u32 %7, %16, %25;\n\t"
        "subc.u32 %8, %17, %26;\n\t"
        : "=r"(x[0]), "=r"(x[1]), "=r"(x[2]), "=r"(x[3]), "=r"(x[4]), "=r"(x[5]), "=r"(x[6]), "=r"(x[7]), "=r"(x[8])
        : "r"(S[0]), "r"(S[1]), "r"(S[2]), "r"(S[3]), "r"(S[4]), "r"(S[5]), "r"(S[6]), "r"(S[7]), "r"(S[8]), "r"(U[0]), "r"(U[1]), "r"(U[2]), "r"(U[3]), "r"(U[4]), "r"(U[5]), "r"(U[6]), "r"(U[7]), "r"(U[8]));
    }
};

}  // namespace ntt
