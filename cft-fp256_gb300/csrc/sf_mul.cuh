// sf_mul.cuh - the significand product on the IMAD pipe.
//
// mul_ptx and mul_ptx_split: product scanning (columns), below;
// mul_row_wide: one word times N words by wide multiply-adds (the square
// root's and the narrow divisions' multiply-subtract). MulPtx::row, the row
// of operand scanning that binary256 division's multiply-subtract uses:
// r (2N words) = a * b (N words each), for each word
// a[i], one carry chain adds the low halves of a[i]*b[j] into r[i..i+N]
// (mad.lo.cc / madc.lo.cc, then addc into r[i+N]) and a second adds the
// high halves into r[i+1..i+N] (mad.hi.cc / madc.hi.cc). After rows 0..i
// the partial sum is below 2^(32(i+1+N)), so r[i+N] is zero when row i
// starts and the last high-half add carries out nothing. Each chain is one
// asm block because the carry flag does not survive between blocks.
#pragma once
#include <cstdint>

namespace sfw {

template <int N> struct MulPtx;

template <> struct MulPtx<1> {
    static __device__ __forceinline__ void row(uint32_t *r, uint32_t a, const uint32_t (&b)[1])
    {
        asm("mad.lo.cc.u32 %0, %2, %3, %0;\n\taddc.u32 %1, %1, 0;\n\tmad.hi.u32 %1, %2, %3, %1;"
            : "+r"(r[0]), "+r"(r[1])
            : "r"(a), "r"(b[0]));
    }
};

template <> struct MulPtx<2> {
    static __device__ __forceinline__ void row(uint32_t *r, uint32_t a, const uint32_t (&b)[2])
    {
        asm("mad.lo.cc.u32 %0, %3, %4, %0;\n\tmadc.lo.cc.u32 %1, %3, %5, %1;\n\taddc.u32 %2, %2, 0;\n\tmad.hi.cc.u32 %1, %3, %4, %1;\n\tmadc.hi.u32 %2, %3, %5, %2;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2])
            : "r"(a), "r"(b[0]), "r"(b[1]));
    }
};

template <> struct MulPtx<4> {
    static __device__ __forceinline__ void row(uint32_t *r, uint32_t a, const uint32_t (&b)[4])
    {
        asm("mad.lo.cc.u32 %0, %5, %6, %0;\n\tmadc.lo.cc.u32 %1, %5, %7, %1;\n\tmadc.lo.cc.u32 %2, %5, %8, %2;\n\tmadc.lo.cc.u32 %3, %5, %9, %3;\n\taddc.u32 %4, %4, 0;\n\tmad.hi.cc.u32 %1, %5, %6, %1;\n\tmadc.hi.cc.u32 %2, %5, %7, %2;\n\tmadc.hi.cc.u32 %3, %5, %8, %3;\n\tmadc.hi.u32 %4, %5, %9, %4;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4])
            : "r"(a), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
    }
};

template <> struct MulPtx<8> {
    static __device__ __forceinline__ void row(uint32_t *r, uint32_t a, const uint32_t (&b)[8])
    {
        asm("mad.lo.cc.u32 %0, %9, %10, %0;\n\tmadc.lo.cc.u32 %1, %9, %11, %1;\n\tmadc.lo.cc.u32 %2, %9, %12, %2;\n\tmadc.lo.cc.u32 %3, %9, %13, %3;\n\tmadc.lo.cc.u32 %4, %9, %14, %4;\n\tmadc.lo.cc.u32 %5, %9, %15, %5;\n\tmadc.lo.cc.u32 %6, %9, %16, %6;\n\tmadc.lo.cc.u32 %7, %9, %17, %7;\n\taddc.u32 %8, %8, 0;\n\tmad.hi.cc.u32 %1, %9, %10, %1;\n\tmadc.hi.cc.u32 %2, %9, %11, %2;\n\tmadc.hi.cc.u32 %3, %9, %12, %3;\n\tmadc.hi.cc.u32 %4, %9, %13, %4;\n\tmadc.hi.cc.u32 %5, %9, %14, %5;\n\tmadc.hi.cc.u32 %6, %9, %15, %6;\n\tmadc.hi.cc.u32 %7, %9, %16, %7;\n\tmadc.hi.u32 %8, %9, %17, %8;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8])
            : "r"(a), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
    }
};

// r (N + 1 words) = a * b (N words): each word's 64-bit product plus the
// carry from the word below, one wide multiply-add a word (the low half is
// the word, the high half the next carry), in place of MulPtx::row's two
// carry chains of halves.
template <int N>
__device__ __forceinline__ void mul_row_wide(uint32_t (&r)[N + 1], uint32_t a, const uint32_t (&b)[N])
{
    uint32_t c = 0u;
#pragma unroll
    for (int j = 0; j < N; j++) {
        const uint64_t t = (uint64_t)a * b[j] + c;
        r[j] = (uint32_t)t;
        c = (uint32_t)(t >> 32);
    }
    r[N] = c;
}

// u (K words) -= t (K words); returns the borrow out (1 when u < t). One
// borrow chain; K = N + 1 for the division's multiply-subtract.
template <int K> struct SubPtx;

template <> struct SubPtx<3> {
    static __device__ __forceinline__ uint32_t sub(uint32_t *u, const uint32_t *t)
    {
        uint32_t b;
        asm("sub.cc.u32 %0, %0, %4;\n\tsubc.cc.u32 %1, %1, %5;\n\tsubc.cc.u32 %2, %2, %6;\n\tsubc.u32 %3, 0, 0;"
            : "+r"(u[0]), "+r"(u[1]), "+r"(u[2]), "=r"(b)
            : "r"(t[0]), "r"(t[1]), "r"(t[2]));
        return b & 1u;
    }
};

template <> struct SubPtx<5> {
    static __device__ __forceinline__ uint32_t sub(uint32_t *u, const uint32_t *t)
    {
        uint32_t b;
        asm("sub.cc.u32 %0, %0, %6;\n\tsubc.cc.u32 %1, %1, %7;\n\tsubc.cc.u32 %2, %2, %8;\n\tsubc.cc.u32 %3, %3, %9;\n\tsubc.cc.u32 %4, %4, %10;\n\tsubc.u32 %5, 0, 0;"
            : "+r"(u[0]), "+r"(u[1]), "+r"(u[2]), "+r"(u[3]), "+r"(u[4]), "=r"(b)
            : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]), "r"(t[4]));
        return b & 1u;
    }
};

template <> struct SubPtx<9> {
    static __device__ __forceinline__ uint32_t sub(uint32_t *u, const uint32_t *t)
    {
        uint32_t b;
        asm("sub.cc.u32 %0, %0, %10;\n\tsubc.cc.u32 %1, %1, %11;\n\tsubc.cc.u32 %2, %2, %12;\n\tsubc.cc.u32 %3, %3, %13;\n\tsubc.cc.u32 %4, %4, %14;\n\tsubc.cc.u32 %5, %5, %15;\n\tsubc.cc.u32 %6, %6, %16;\n\tsubc.cc.u32 %7, %7, %17;\n\tsubc.cc.u32 %8, %8, %18;\n\tsubc.u32 %9, 0, 0;"
            : "+r"(u[0]), "+r"(u[1]), "+r"(u[2]), "+r"(u[3]), "+r"(u[4]), "+r"(u[5]), "+r"(u[6]), "+r"(u[7]), "+r"(u[8]), "=r"(b)
            : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]), "r"(t[4]), "r"(t[5]), "r"(t[6]), "r"(t[7]), "r"(t[8]));
        return b & 1u;
    }
};

// r += x + cin (N words, cin 0 or 1); returns the carry out. One carry
// chain: the first instruction only sets the carry flag from cin.
template <int N> struct AddPtx;
template <> struct AddPtx<2> {
    static __device__ __forceinline__ uint32_t add(uint32_t (&r)[2], const uint32_t (&x)[2], uint32_t cin)
    {
        uint32_t c;
        [[maybe_unused]] uint32_t scratch;   // carries cin into the chain's carry flag
        asm("add.cc.u32 %3, %6, -1;\n\taddc.cc.u32 %0, %0, %4;\n\taddc.cc.u32 %1, %1, %5;\n\taddc.u32 %2, 0, 0;"
            : "+r"(r[0]), "+r"(r[1]), "=r"(c), "=r"(scratch)
            : "r"(x[0]), "r"(x[1]), "r"(cin));
        return c;
    }
};
template <> struct AddPtx<4> {
    static __device__ __forceinline__ uint32_t add(uint32_t (&r)[4], const uint32_t (&x)[4], uint32_t cin)
    {
        uint32_t c;
        [[maybe_unused]] uint32_t scratch;   // carries cin into the chain's carry flag
        asm("add.cc.u32 %5, %10, -1;\n\taddc.cc.u32 %0, %0, %6;\n\taddc.cc.u32 %1, %1, %7;\n\taddc.cc.u32 %2, %2, %8;\n\taddc.cc.u32 %3, %3, %9;\n\taddc.u32 %4, 0, 0;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "=r"(c), "=r"(scratch)
            : "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(cin));
        return c;
    }
};
template <> struct AddPtx<8> {
    static __device__ __forceinline__ uint32_t add(uint32_t (&r)[8], const uint32_t (&x)[8], uint32_t cin)
    {
        uint32_t c;
        [[maybe_unused]] uint32_t scratch;   // carries cin into the chain's carry flag
        asm("add.cc.u32 %9, %18, -1;\n\taddc.cc.u32 %0, %0, %10;\n\taddc.cc.u32 %1, %1, %11;\n\taddc.cc.u32 %2, %2, %12;\n\taddc.cc.u32 %3, %3, %13;\n\taddc.cc.u32 %4, %4, %14;\n\taddc.cc.u32 %5, %5, %15;\n\taddc.cc.u32 %6, %6, %16;\n\taddc.cc.u32 %7, %7, %17;\n\taddc.u32 %8, 0, 0;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "=r"(c), "=r"(scratch)
            : "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]), "r"(x[6]), "r"(x[7]), "r"(cin));
        return c;
    }
};
template <> struct AddPtx<16> {
    static __device__ __forceinline__ uint32_t add(uint32_t (&r)[16], const uint32_t (&x)[16], uint32_t cin)
    {
        uint32_t c;
        [[maybe_unused]] uint32_t scratch;   // carries cin into the chain's carry flag
        asm("add.cc.u32 %17, %34, -1;\n\taddc.cc.u32 %0, %0, %18;\n\taddc.cc.u32 %1, %1, %19;\n\taddc.cc.u32 %2, %2, %20;\n\taddc.cc.u32 %3, %3, %21;\n\taddc.cc.u32 %4, %4, %22;\n\taddc.cc.u32 %5, %5, %23;\n\taddc.cc.u32 %6, %6, %24;\n\taddc.cc.u32 %7, %7, %25;\n\taddc.cc.u32 %8, %8, %26;\n\taddc.cc.u32 %9, %9, %27;\n\taddc.cc.u32 %10, %10, %28;\n\taddc.cc.u32 %11, %11, %29;\n\taddc.cc.u32 %12, %12, %30;\n\taddc.cc.u32 %13, %13, %31;\n\taddc.cc.u32 %14, %14, %32;\n\taddc.cc.u32 %15, %15, %33;\n\taddc.u32 %16, 0, 0;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "=r"(c), "=r"(scratch)
            : "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]), "r"(x[6]), "r"(x[7]), "r"(x[8]), "r"(x[9]), "r"(x[10]), "r"(x[11]), "r"(x[12]), "r"(x[13]), "r"(x[14]), "r"(x[15]), "r"(cin));
        return c;
    }
};

// r += 1 (N words); returns the carry out. One carry chain.
template <int N> struct IncPtx;
template <> struct IncPtx<2> {
    static __device__ __forceinline__ uint32_t inc(uint32_t (&r)[2])
    {
        uint32_t c;
        asm("add.cc.u32 %0, %0, 1;\n\taddc.cc.u32 %1, %1, 0;\n\taddc.u32 %2, 0, 0;"
            : "+r"(r[0]), "+r"(r[1]), "=r"(c));
        return c;
    }
};
template <> struct IncPtx<4> {
    static __device__ __forceinline__ uint32_t inc(uint32_t (&r)[4])
    {
        uint32_t c;
        asm("add.cc.u32 %0, %0, 1;\n\taddc.cc.u32 %1, %1, 0;\n\taddc.cc.u32 %2, %2, 0;\n\taddc.cc.u32 %3, %3, 0;\n\taddc.u32 %4, 0, 0;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "=r"(c));
        return c;
    }
};
template <> struct IncPtx<8> {
    static __device__ __forceinline__ uint32_t inc(uint32_t (&r)[8])
    {
        uint32_t c;
        asm("add.cc.u32 %0, %0, 1;\n\taddc.cc.u32 %1, %1, 0;\n\taddc.cc.u32 %2, %2, 0;\n\taddc.cc.u32 %3, %3, 0;\n\taddc.cc.u32 %4, %4, 0;\n\taddc.cc.u32 %5, %5, 0;\n\taddc.cc.u32 %6, %6, 0;\n\taddc.cc.u32 %7, %7, 0;\n\taddc.u32 %8, 0, 0;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "=r"(c));
        return c;
    }
};
template <> struct IncPtx<16> {
    static __device__ __forceinline__ uint32_t inc(uint32_t (&r)[16])
    {
        uint32_t c;
        asm("add.cc.u32 %0, %0, 1;\n\taddc.cc.u32 %1, %1, 0;\n\taddc.cc.u32 %2, %2, 0;\n\taddc.cc.u32 %3, %3, 0;\n\taddc.cc.u32 %4, %4, 0;\n\taddc.cc.u32 %5, %5, 0;\n\taddc.cc.u32 %6, %6, 0;\n\taddc.cc.u32 %7, %7, 0;\n\taddc.cc.u32 %8, %8, 0;\n\taddc.cc.u32 %9, %9, 0;\n\taddc.cc.u32 %10, %10, 0;\n\taddc.cc.u32 %11, %11, 0;\n\taddc.cc.u32 %12, %12, 0;\n\taddc.cc.u32 %13, %13, 0;\n\taddc.cc.u32 %14, %14, 0;\n\taddc.cc.u32 %15, %15, 0;\n\taddc.u32 %16, 0, 0;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "=r"(c));
        return c;
    }
};

// The widths the square root's remainder takes (W + 2 words).
template <> struct MulPtx<3> {
    static __device__ __forceinline__ void row(uint32_t *r, uint32_t a, const uint32_t (&b)[3])
    {
        asm("mad.lo.cc.u32 %0, %4, %5, %0;\n\tmadc.lo.cc.u32 %1, %4, %6, %1;\n\tmadc.lo.cc.u32 %2, %4, %7, %2;\n\taddc.u32 %3, %3, 0;\n\tmad.hi.cc.u32 %1, %4, %5, %1;\n\tmadc.hi.cc.u32 %2, %4, %6, %2;\n\tmadc.hi.u32 %3, %4, %7, %3;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3])
            : "r"(a), "r"(b[0]), "r"(b[1]), "r"(b[2]));
    }
};
template <> struct MulPtx<6> {
    static __device__ __forceinline__ void row(uint32_t *r, uint32_t a, const uint32_t (&b)[6])
    {
        asm("mad.lo.cc.u32 %0, %7, %8, %0;\n\tmadc.lo.cc.u32 %1, %7, %9, %1;\n\tmadc.lo.cc.u32 %2, %7, %10, %2;\n\tmadc.lo.cc.u32 %3, %7, %11, %3;\n\tmadc.lo.cc.u32 %4, %7, %12, %4;\n\tmadc.lo.cc.u32 %5, %7, %13, %5;\n\taddc.u32 %6, %6, 0;\n\tmad.hi.cc.u32 %1, %7, %8, %1;\n\tmadc.hi.cc.u32 %2, %7, %9, %2;\n\tmadc.hi.cc.u32 %3, %7, %10, %3;\n\tmadc.hi.cc.u32 %4, %7, %11, %4;\n\tmadc.hi.cc.u32 %5, %7, %12, %5;\n\tmadc.hi.u32 %6, %7, %13, %6;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6])
            : "r"(a), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]));
    }
};
template <> struct MulPtx<10> {
    static __device__ __forceinline__ void row(uint32_t *r, uint32_t a, const uint32_t (&b)[10])
    {
        asm("mad.lo.cc.u32 %0, %11, %12, %0;\n\tmadc.lo.cc.u32 %1, %11, %13, %1;\n\tmadc.lo.cc.u32 %2, %11, %14, %2;\n\tmadc.lo.cc.u32 %3, %11, %15, %3;\n\tmadc.lo.cc.u32 %4, %11, %16, %4;\n\tmadc.lo.cc.u32 %5, %11, %17, %5;\n\tmadc.lo.cc.u32 %6, %11, %18, %6;\n\tmadc.lo.cc.u32 %7, %11, %19, %7;\n\tmadc.lo.cc.u32 %8, %11, %20, %8;\n\tmadc.lo.cc.u32 %9, %11, %21, %9;\n\taddc.u32 %10, %10, 0;\n\tmad.hi.cc.u32 %1, %11, %12, %1;\n\tmadc.hi.cc.u32 %2, %11, %13, %2;\n\tmadc.hi.cc.u32 %3, %11, %14, %3;\n\tmadc.hi.cc.u32 %4, %11, %15, %4;\n\tmadc.hi.cc.u32 %5, %11, %16, %5;\n\tmadc.hi.cc.u32 %6, %11, %17, %6;\n\tmadc.hi.cc.u32 %7, %11, %18, %7;\n\tmadc.hi.cc.u32 %8, %11, %19, %8;\n\tmadc.hi.cc.u32 %9, %11, %20, %9;\n\tmadc.hi.u32 %10, %11, %21, %10;"
            : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10])
            : "r"(a), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]));
    }
};
template <> struct SubPtx<4> {
    static __device__ __forceinline__ uint32_t sub(uint32_t *u, const uint32_t *t)
    {
        uint32_t b;
        asm("sub.cc.u32 %0, %0, %5;\n\tsubc.cc.u32 %1, %1, %6;\n\tsubc.cc.u32 %2, %2, %7;\n\tsubc.cc.u32 %3, %3, %8;\n\tsubc.u32 %4, 0, 0;"
            : "+r"(u[0]), "+r"(u[1]), "+r"(u[2]), "+r"(u[3]), "=r"(b)
            : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]));
        return b & 1u;
    }
};
template <> struct SubPtx<6> {
    static __device__ __forceinline__ uint32_t sub(uint32_t *u, const uint32_t *t)
    {
        uint32_t b;
        asm("sub.cc.u32 %0, %0, %7;\n\tsubc.cc.u32 %1, %1, %8;\n\tsubc.cc.u32 %2, %2, %9;\n\tsubc.cc.u32 %3, %3, %10;\n\tsubc.cc.u32 %4, %4, %11;\n\tsubc.cc.u32 %5, %5, %12;\n\tsubc.u32 %6, 0, 0;"
            : "+r"(u[0]), "+r"(u[1]), "+r"(u[2]), "+r"(u[3]), "+r"(u[4]), "+r"(u[5]), "=r"(b)
            : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]), "r"(t[4]), "r"(t[5]));
        return b & 1u;
    }
};
template <> struct SubPtx<10> {
    static __device__ __forceinline__ uint32_t sub(uint32_t *u, const uint32_t *t)
    {
        uint32_t b;
        asm("sub.cc.u32 %0, %0, %11;\n\tsubc.cc.u32 %1, %1, %12;\n\tsubc.cc.u32 %2, %2, %13;\n\tsubc.cc.u32 %3, %3, %14;\n\tsubc.cc.u32 %4, %4, %15;\n\tsubc.cc.u32 %5, %5, %16;\n\tsubc.cc.u32 %6, %6, %17;\n\tsubc.cc.u32 %7, %7, %18;\n\tsubc.cc.u32 %8, %8, %19;\n\tsubc.cc.u32 %9, %9, %20;\n\tsubc.u32 %10, 0, 0;"
            : "+r"(u[0]), "+r"(u[1]), "+r"(u[2]), "+r"(u[3]), "+r"(u[4]), "+r"(u[5]), "+r"(u[6]), "+r"(u[7]), "+r"(u[8]), "+r"(u[9]), "=r"(b)
            : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]), "r"(t[4]), "r"(t[5]), "r"(t[6]), "r"(t[7]), "r"(t[8]), "r"(t[9]));
        return b & 1u;
    }
};

// r (2N words) = a * b by product scanning: column k of the result sums
// a[i] * b[k-i] over every i into a three-word accumulator (c0, c1, c2),
// each partial product's low and high halves added by one adjacent pair of
// mad.lo.cc / madc.hi.cc on the same operands and the carry into c2 by
// addc; then c0 is word k and the accumulator moves down a word. Measured
// on a GB300 against the row form (operand scanning, MulPtx::row): 112
// against 85 G binary256 products/s in a dependent loop, the same bits.
template <int N>
__device__ __forceinline__ void mul_ptx(uint32_t (&r)[2 * N], const uint32_t (&a)[N],
                                        const uint32_t (&b)[N])
{
    uint32_t c0 = 0u, c1 = 0u, c2 = 0u;
#pragma unroll
    for (int k = 0; k < 2 * N - 1; k++) {
#pragma unroll
        for (int i = 0; i < N; i++) {
            const int j = k - i;
            if (j < 0 || j >= N) continue;
            asm("mad.lo.cc.u32 %0, %3, %4, %0;\n\tmadc.hi.cc.u32 %1, %3, %4, %1;\n\taddc.u32 %2, %2, 0;"
                : "+r"(c0), "+r"(c1), "+r"(c2)
                : "r"(a[i]), "r"(b[j]));
        }
        r[k] = c0;
        c0 = c1;
        c1 = c2;
        c2 = 0u;
    }
    r[2 * N - 1] = c0;
}

// Columns of the product of a's words [LO, HI) with b, into r (2N words):
// mul_ptx's accumulation restricted to those rows.
template <int N, int LO, int HI>
__device__ __forceinline__ void mul_cols_rows(uint32_t (&r)[2 * N], const uint32_t (&a)[N],
                                              const uint32_t (&b)[N])
{
    uint32_t c0 = 0u, c1 = 0u, c2 = 0u;
#pragma unroll
    for (int k = 0; k < 2 * N - 1; k++) {
#pragma unroll
        for (int i = LO; i < HI; i++) {
            const int j = k - i;
            if (j < 0 || j >= N) continue;
            asm("mad.lo.cc.u32 %0, %3, %4, %0;\n\tmadc.hi.cc.u32 %1, %3, %4, %1;\n\taddc.u32 %2, %2, 0;"
                : "+r"(c0), "+r"(c1), "+r"(c2)
                : "r"(a[i]), "r"(b[j]));
        }
        r[k] = c0;
        c0 = c1;
        c1 = c2;
        c2 = 0u;
    }
    r[2 * N - 1] = c0;
}

// r (2N words) = a * b as two independent column sums, over a's low and
// high halves of rows, added at the end by one carry chain: the same value
// as mul_ptx, with two dependency chains the scheduler can interleave, so a
// lone warp waits less for the product (a dependent chain of binary256
// FMAs on one warp, measured on a GB300: 1,667 cycles an operation, against
// 1,712 with mul_ptx's one chain and 1,910 with two chains of rows).
template <int N>
__device__ __forceinline__ void mul_ptx_split(uint32_t (&r)[2 * N], const uint32_t (&a)[N],
                                              const uint32_t (&b)[N])
{
    if constexpr (N == 1) {
        mul_ptx<1>(r, a, b);
    } else {
        uint32_t R0[2 * N], R1[2 * N];
        mul_cols_rows<N, 0, N / 2>(R0, a, b);
        mul_cols_rows<N, N / 2, N>(R1, a, b);
        AddPtx<2 * N>::add(R0, R1, 0u);
#pragma unroll
        for (int i = 0; i < 2 * N; i++) r[i] = R0[i];
    }
}

}  // namespace sfw
