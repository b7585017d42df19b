// sf_words.cuh - fixed-width unsigned integers held in registers.
//
// Every value is an array of N 32-bit words, little-endian, with N known at
// compile time so that the arrays stay in registers after unrolling. All
// variable shifts are select networks (one stage per bit of the word count)
// plus a funnel shift, so no array is ever indexed by a run-time value.
#pragma once
#include <cstdint>

#define SFD __device__ __forceinline__

namespace sfw {

template <int N>
SFD void zero(uint32_t (&x)[N])
{
#pragma unroll
    for (int i = 0; i < N; i++) x[i] = 0u;
}

template <int N>
SFD bool is_zero(const uint32_t (&x)[N])
{
    uint32_t o = 0u;
#pragma unroll
    for (int i = 0; i < N; i++) o |= x[i];
    return o == 0u;
}

// Number of significant bits (0 for zero).
template <int N>
SFD int bitlen(const uint32_t (&x)[N])
{
    int L = 0;
#pragma unroll
    for (int i = 0; i < N; i++)
        if (x[i]) L = 32 * i + 32 - __clz(x[i]);
    return L;
}

// The word-shift stages one of the active lanes needs: a stage of the
// select network that no lane of the warp uses is skipped by the whole warp.
SFD int warp_stages(int ws)
{
    return (int)__reduce_or_sync(__activemask(), (unsigned)ws);
}

// x <<= s for 0 <= s < 32N, zero fill.
template <int N>
SFD void shl(uint32_t (&x)[N], int s)
{
    const int ws = s >> 5, bs = s & 31;
    const int need = warp_stages(ws);
#pragma unroll
    for (int b = 16; b >= 1; b >>= 1) {
        if (b < N && (need & b)) {
            const bool take = (ws & b) != 0;
#pragma unroll
            for (int i = N - 1; i >= 0; i--)
                x[i] = take ? (i - b >= 0 ? x[i - b] : 0u) : x[i];
        }
    }
#pragma unroll
    for (int i = N - 1; i >= 1; i--) x[i] = __funnelshift_l(x[i - 1], x[i], bs);
    x[0] <<= bs;
}

// x >>= s with every bit shifted out ORed into bit 0 ("jamming").
// Any s: s <= 0 leaves x alone, s >= 32N leaves only the jam. Branch-free.
// The jam is gathered as the words leave: each stage of the select network
// that shifts drops its low b words, and the funnel shift drops the low bs
// bits of what is then x[0].
template <int N>
SFD void shr_jam(uint32_t (&x)[N], int s)
{
    const int sc = s <= 0 ? 0 : (s >= 32 * N ? 32 * N : s);
    const int ws = sc >> 5, bs = sc & 31;                 // ws may be N
    uint32_t st = 0u;
    const int need = warp_stages(ws);
#pragma unroll
    for (int b = 16; b >= 1; b >>= 1) {
        if (b <= N && (need & b)) {
            const bool take = (ws & b) != 0;
            uint32_t out = 0u;
#pragma unroll
            for (int i = 0; i < b; i++) out |= x[i];
            st |= take ? out : 0u;
#pragma unroll
            for (int i = 0; i < N; i++)
                x[i] = take ? (i + b < N ? x[i + b] : 0u) : x[i];
        }
    }
    st |= x[0] & ((1u << bs) - 1u);
#pragma unroll
    for (int i = 0; i < N - 1; i++) x[i] = __funnelshift_r(x[i], x[i + 1], bs);
    x[N - 1] >>= bs;
    x[0] |= (st != 0u) ? 1u : 0u;
}

// shl and shr_jam for a lone warp waiting on the result: a shift of less
// than a word (the usual one: no deep cancellation, an addend of nearly the
// product's size) by funnel shifts alone, the others through the select
// network. Per lane, without the network's vote.
template <int N>
SFD void shl_small_first(uint32_t (&x)[N], int s)
{
    if (s < 32) {
#pragma unroll
        for (int i = N - 1; i >= 1; i--) x[i] = __funnelshift_l(x[i - 1], x[i], s);
        x[0] <<= s;
    } else {
        shl(x, s);
    }
}

template <int N>
SFD void shr_jam_small_first(uint32_t (&x)[N], int s)
{
    if (s <= 0) return;
    if (s < 32) {
        const uint32_t st = x[0] & ((1u << s) - 1u);
#pragma unroll
        for (int i = 0; i < N - 1; i++) x[i] = __funnelshift_r(x[i], x[i + 1], s);
        x[N - 1] >>= s;
        x[0] |= st ? 1u : 0u;
    } else {
        shr_jam(x, s);
    }
}

// 32-bit multiply-adds as the IMAD pipe runs them (kept as PTX so that a
// multiplier known to be 0 or 1 is not turned back into a select).
SFD uint32_t imul(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("mul.lo.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}
SFD uint32_t imad(uint32_t a, uint32_t b, uint32_t c)
{
    uint32_t r;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
    return r;
}

// shr_jam with the select network's word moves as multiply-adds by 0 and 1
// (x[i] = x[i+b] * take + x[i] * !take): the same bits, computed on the
// IMAD pipe instead of the integer ALU pipe, which the kernels around it
// keep busier.
template <int N>
SFD void shr_jam_imad(uint32_t (&x)[N], int s)
{
    const int sc = s <= 0 ? 0 : (s >= 32 * N ? 32 * N : s);
    const int ws = sc >> 5, bs = sc & 31;                 // ws may be N
    uint32_t st = 0u;
    const int need = warp_stages(ws);
#pragma unroll
    for (int b = 16; b >= 1; b >>= 1) {
        if (b <= N && (need & b)) {
            const uint32_t t = (uint32_t)(ws & b) / (uint32_t)b;   // 0 or 1
            const uint32_t nt = t ^ 1u;
            uint32_t out = 0u;
#pragma unroll
            for (int i = 0; i < b; i++) out |= x[i];
            st |= imul(out, t);
#pragma unroll
            for (int i = 0; i < N; i++)
                x[i] = (i + b < N) ? imad(x[i + b], t, imul(x[i], nt)) : imul(x[i], nt);
        }
    }
    st |= x[0] & ((1u << bs) - 1u);
#pragma unroll
    for (int i = 0; i < N - 1; i++) x[i] = __funnelshift_r(x[i], x[i + 1], bs);
    x[N - 1] >>= bs;
    x[0] |= (st != 0u) ? 1u : 0u;
}

// shl with the word moves and the bit shift as multiply-adds: x[i] << bs
// is the low word of x[i] * 2^bs and x[i-1] >> (32 - bs) its high word.
template <int N>
SFD void shl_imad(uint32_t (&x)[N], int s)
{
    const int ws = s >> 5, bs = s & 31;
    const int need = warp_stages(ws);
#pragma unroll
    for (int b = 16; b >= 1; b >>= 1) {
        if (b < N && (need & b)) {
            const uint32_t t = (uint32_t)(ws & b) / (uint32_t)b;
            const uint32_t nt = t ^ 1u;
#pragma unroll
            for (int i = N - 1; i >= 0; i--)
                x[i] = (i - b >= 0) ? imad(x[i - b], t, imul(x[i], nt)) : imul(x[i], nt);
        }
    }
    const uint32_t m = 1u << bs;
#pragma unroll
    for (int i = N - 1; i >= 1; i--) {
        uint32_t r;
        asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(x[i - 1]), "r"(m), "r"(imul(x[i], m)));
        x[i] = r;
    }
    x[0] = imul(x[0], m);
}

// x >>= s for 0 <= s < 32N, logical (no jam).
template <int N>
SFD void shr(uint32_t (&x)[N], int s)
{
    const int ws = s >> 5, bs = s & 31;
    const int need = warp_stages(ws);
#pragma unroll
    for (int b = 16; b >= 1; b >>= 1) {
        if (b < N && (need & b)) {
            const bool take = (ws & b) != 0;
#pragma unroll
            for (int i = 0; i < N; i++)
                x[i] = take ? (i + b < N ? x[i + b] : 0u) : x[i];
        }
    }
#pragma unroll
    for (int i = 0; i < N - 1; i++) x[i] = __funnelshift_r(x[i], x[i + 1], bs);
    x[N - 1] >>= bs;
}

// x <<= S for a compile-time 0 <= S < 32N, zero fill.
template <int S, int N>
SFD void shl_const(uint32_t (&x)[N])
{
    constexpr int ws = S >> 5, bs = S & 31;
#pragma unroll
    for (int i = N - 1; i >= 0; i--) {
        const uint32_t hi = (i - ws >= 0) ? x[i - ws] : 0u;
        const uint32_t lo = (i - ws - 1 >= 0) ? x[i - ws - 1] : 0u;
        x[i] = bs ? __funnelshift_l(lo, hi, bs) : hi;
    }
}

// x >>= s for a compile-time 0 <= S < 32N (no jam).
template <int S, int N>
SFD void shr_const(uint32_t (&x)[N])
{
    constexpr int ws = S >> 5, bs = S & 31;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t lo = (i + ws < N) ? x[i + ws] : 0u;
        const uint32_t hi = (i + ws + 1 < N) ? x[i + ws + 1] : 0u;
        x[i] = bs ? __funnelshift_r(lo, hi, bs) : lo;
    }
}

// r = a + b, returns the carry out.
template <int N>
SFD uint32_t add(uint32_t (&r)[N], const uint32_t (&a)[N], const uint32_t (&b)[N])
{
    uint32_t c = 0u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t t = (uint64_t)a[i] + b[i] + c;
        r[i] = (uint32_t)t;
        c = (uint32_t)(t >> 32);
    }
    return c;
}

// r = a - b, returns the borrow out (1 when a < b).
template <int N>
SFD uint32_t sub(uint32_t (&r)[N], const uint32_t (&a)[N], const uint32_t (&b)[N])
{
    uint32_t br = 0u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t t = (uint64_t)a[i] - b[i] - br;
        r[i] = (uint32_t)t;
        br = (uint32_t)(t >> 63);
    }
    return br;
}

// x = -x modulo 2^(32N)
template <int N>
SFD void neg(uint32_t (&x)[N])
{
    uint32_t c = 1u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t t = (uint64_t)(~x[i]) + c;
        x[i] = (uint32_t)t;
        c = (uint32_t)(t >> 32);
    }
}

// x += 1, returns the carry out
template <int N>
SFD uint32_t inc(uint32_t (&x)[N])
{
    uint32_t c = 1u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint64_t t = (uint64_t)x[i] + c;
        x[i] = (uint32_t)t;
        c = (uint32_t)(t >> 32);
    }
    return c;
}

// -1, 0, 1
template <int N>
SFD int cmp(const uint32_t (&a)[N], const uint32_t (&b)[N])
{
    int r = 0;
#pragma unroll
    for (int i = 0; i < N; i++)
        if (a[i] != b[i]) r = a[i] < b[i] ? -1 : 1;
    return r;
}

// r (2N words) = a * b, schoolbook with 64-bit partial products.
template <int N>
SFD void mul(uint32_t (&r)[2 * N], const uint32_t (&a)[N], const uint32_t (&b)[N])
{
#pragma unroll
    for (int i = 0; i < 2 * N; i++) r[i] = 0u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        uint32_t c = 0u;
#pragma unroll
        for (int j = 0; j < N; j++) {
            const uint64_t t = (uint64_t)a[i] * b[j] + r[i + j] + c;
            r[i + j] = (uint32_t)t;
            c = (uint32_t)(t >> 32);
        }
        r[i + N] = c;
    }
}

// bit i (compile-time) of x
template <int I, int N>
SFD uint32_t bit(const uint32_t (&x)[N])
{
    return (x[I >> 5] >> (I & 31)) & 1u;
}

// any of bits [0, K) of x, K compile-time
template <int K, int N>
SFD bool low_any(const uint32_t (&x)[N])
{
    uint32_t o = 0u;
#pragma unroll
    for (int i = 0; i < N; i++) {
        if (32 * i + 32 <= K) o |= x[i];
        else if (32 * i < K) o |= x[i] & ((1u << (K - 32 * i)) - 1u);
    }
    return o != 0u;
}

}  // namespace sfw
