// softfloat.cuh - the element arithmetic on the GPU, one template per format.
//
// Semantics are the reference's (host/src/softfloat.c, with division and
// square root as python/cft_golden/softfloat.py:440-505 defines them): five
// rounding attributes, tininess detected after rounding, underflow only when
// tiny AND inexact, one canonical quiet NaN, ADD/SUB/MUL as the FMA with
// steered operands. The algorithms are this library's own:
//
//  * FMA: a fixed window of 2W words (W = the element's words) instead of the
//    reference's bounded alignment. The product of the two significands,
//    normalised to the top of the window, and the addend, aligned to it, are
//    combined exactly wherever they overlap; bits shifted below the window
//    are jammed into bit 0, which then acts as a sticky bit that is provably
//    at least two places below the rounding point (see fma_general).
//  * round_pack: normalise the window to its top bit with one variable
//    shift, read kept/guard/sticky at fixed positions, and denormalise only
//    for results below the normal range.
//  * div: base-2^32 long division (Knuth's Algorithm D) to at least p+3
//    quotient bits plus a remainder sticky; sqrt: the base-2^32
//    digit-by-digit integer root to at least p+3 bits plus sticky.
//    Both are exact quotient/root computations, so they round to the same
//    bits as any other exact method.
#pragma once
#include "sf_words.cuh"
#include "sf_mul.cuh"

namespace sf {

// Flag bits (host/src/softfloat.h:50-55)
constexpr uint32_t F_INVALID = 1u, F_DIVZERO = 2u, F_OVERFLOW = 4u, F_UNDERFLOW = 8u,
                   F_INEXACT = 16u;
// Rounding attributes (host/src/softfloat.h:57-62)
constexpr int RNE = 0, RTZ = 1, RDN = 2, RUP = 3, RMM = 4;
// IEEE 754-2019 9.5's roundTiesTowardZero: an internal direction of the
// augmented operations only (nearest, ties to the smaller magnitude,
// overflow to infinity), never a caller's attribute.
constexpr int RTTZ = 5;

// Format geometry (host/src/softfloat.c:10-16). W = 32-bit words an element.
template <int FMT> struct Fmt;
template <> struct Fmt<0> { static constexpr int W = 1, P = 24, MANW = 23, EXPW = 8, BIAS = 127, EMAX = 127, EMIN = -126; };
template <> struct Fmt<1> { static constexpr int W = 2, P = 53, MANW = 52, EXPW = 11, BIAS = 1023, EMAX = 1023, EMIN = -1022; };
template <> struct Fmt<2> { static constexpr int W = 4, P = 113, MANW = 112, EXPW = 15, BIAS = 16383, EMAX = 16383, EMIN = -16382; };
template <> struct Fmt<3> { static constexpr int W = 8, P = 237, MANW = 236, EXPW = 19, BIAS = 262143, EMAX = 262143, EMIN = -262142; };

enum { C_ZERO = 0, C_SUB = 1, C_NORM = 2, C_INF = 3, C_NAN = 4 };

template <int FMT>
struct Unp {
    static constexpr int W = Fmt<FMT>::W;
    int cls, sign, snan;
    int ve;             // exponent of the leading significand bit (finite non-zero)
    uint32_t m[W];      // significand, normalised so its leading bit is bit 32W-1
};

// position of the exponent field's low bit inside the top word
template <int FMT> __host__ __device__ constexpr int exp_shift() { return Fmt<FMT>::MANW - 32 * (Fmt<FMT>::W - 1); }
template <int FMT> __host__ __device__ constexpr uint32_t exp_mask() { return (1u << Fmt<FMT>::EXPW) - 1u; }

template <int FMT>
SFD uint32_t exp_field(const uint32_t (&x)[Fmt<FMT>::W])
{
    return (x[Fmt<FMT>::W - 1] >> exp_shift<FMT>()) & exp_mask<FMT>();
}

template <int FMT>
SFD int sign_of(const uint32_t (&x)[Fmt<FMT>::W])
{
    return (int)(x[Fmt<FMT>::W - 1] >> 31);
}

// Classify and unpack (host/src/softfloat.c:85-116 gives the classes). A
// finite non-zero significand is normalised with its leading bit at bit LB
// of the W words (32W-1 unless a caller wants it lower).
template <int FMT, int LB = 32 * Fmt<FMT>::W - 1>
SFD void unpack(const uint32_t (&x)[Fmt<FMT>::W], Unp<FMT> &u)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W;
    const uint32_t ef = exp_field<FMT>(x);
    u.sign = sign_of<FMT>(x);
#pragma unroll
    for (int i = 0; i < W; i++) u.m[i] = x[i];
    u.m[W - 1] &= (1u << exp_shift<FMT>()) - 1u;          // fraction only
    u.snan = 0;
    u.ve = 0;
    if (ef == exp_mask<FMT>()) {
        const bool fz = sfw::is_zero(u.m);
        u.cls = fz ? C_INF : C_NAN;
        u.snan = (!fz && !((x[(F::MANW - 1) >> 5] >> ((F::MANW - 1) & 31)) & 1u)) ? 1 : 0;
        return;
    }
    if (ef == 0u) {
        if (sfw::is_zero(u.m)) { u.cls = C_ZERO; return; }
        u.cls = C_SUB;
        // a subnormal's leading bit is nearly always in its top word
        const int L = u.m[W - 1] ? 32 * W - __clz(u.m[W - 1]) : sfw::bitlen(u.m);
        u.ve = F::EMIN - F::MANW + L - 1;
        sfw::shl(u.m, LB + 1 - L);
        return;
    }
    u.cls = C_NORM;
    u.m[W - 1] |= 1u << exp_shift<FMT>();                  // hidden bit
    u.ve = (int)ef - F::BIAS;
    sfw::shl_const<LB - F::MANW>(u.m);
}

// ---- encodings ---------------------------------------------------------

template <int FMT>
SFD void enc_zero(uint32_t (&o)[Fmt<FMT>::W], int sign)
{
    sfw::zero(o);
    o[Fmt<FMT>::W - 1] = (uint32_t)sign << 31;
}

template <int FMT>
SFD void enc_inf(uint32_t (&o)[Fmt<FMT>::W], int sign)
{
    sfw::zero(o);
    o[Fmt<FMT>::W - 1] = ((uint32_t)sign << 31) | (exp_mask<FMT>() << exp_shift<FMT>());
}

// The canonical quiet NaN: sign 0, exponent all ones, top fraction bit set
// (host/src/softfloat.c:50-56).
template <int FMT>
SFD void enc_qnan(uint32_t (&o)[Fmt<FMT>::W])
{
    using F = Fmt<FMT>;
    sfw::zero(o);
    o[F::W - 1] = exp_mask<FMT>() << exp_shift<FMT>();
    o[(F::MANW - 1) >> 5] |= 1u << ((F::MANW - 1) & 31);
}

template <int FMT>
SFD void enc_max_normal(uint32_t (&o)[Fmt<FMT>::W], int sign)
{
    constexpr int W = Fmt<FMT>::W;
#pragma unroll
    for (int i = 0; i < W; i++) o[i] = 0xFFFFFFFFu;
    o[W - 1] = ((uint32_t)sign << 31) | ((exp_mask<FMT>() - 1u) << exp_shift<FMT>()) |
               ((1u << exp_shift<FMT>()) - 1u);
}

template <int FMT>
SFD void enc_one(uint32_t (&o)[Fmt<FMT>::W], int sign)
{
    sfw::zero(o);
    o[Fmt<FMT>::W - 1] = ((uint32_t)sign << 31) | ((uint32_t)Fmt<FMT>::BIAS << exp_shift<FMT>());
}

// ---- rounding (semantics: host/src/softfloat.c:120-261) ----------------

SFD bool round_up(int rnd, int sign, bool guard, bool sticky, bool lsb)
{
    switch (rnd) {
    case RNE: return guard && (sticky || lsb);
    case RTZ: return false;
    case RDN: return sign && (guard || sticky);
    case RUP: return !sign && (guard || sticky);
    case RTTZ: return guard && sticky;
    default:  return guard;                                   // RMM
    }
}

// round_up by selects: a warp whose lanes round under different attributes
// (a trajectory's bundle) takes no branch
SFD bool round_up_sel(int rnd, int sign, bool guard, bool sticky, bool lsb)
{
    const bool gs = guard || sticky;
    bool r = false;                                           // RTZ
    r = rnd == RNE ? (guard && (sticky || lsb)) : r;
    r = rnd == RDN ? (sign && gs) : r;
    r = rnd == RUP ? (!sign && gs) : r;
    r = rnd == RTTZ ? (guard && sticky) : r;
    r = rnd == RMM ? guard : r;
    return r;
}

SFD bool overflow_to_inf(int rnd, int sign)
{
    return rnd == RTZ ? false : rnd == RDN ? (sign != 0) : rnd == RUP ? (sign == 0) : true;
}

// kept = the P bits of m below bit 32N (m normalised to its top bit),
// guard = the next bit, sticky = any bit below it.
template <int FMT, int N>
SFD void take_top(const uint32_t (&m)[N], uint32_t (&kept)[Fmt<FMT>::W], bool &guard, bool &sticky)
{
    using F = Fmt<FMT>;
    constexpr int SH = 32 * N - F::P;             // bits below the kept ones
    static_assert(SH >= 2, "window too narrow for rounding");
    uint32_t t[N];
#pragma unroll
    for (int i = 0; i < N; i++) t[i] = m[i];
    sfw::shr_const<SH>(t);
#pragma unroll
    for (int i = 0; i < F::W; i++) kept[i] = t[i];
    guard = sfw::bit<SH - 1>(m) != 0u;
    sticky = sfw::low_any<SH - 1>(m);
}

// Round the exact non-zero value m * 2^e (m an N-word integer; its bit 0 may
// carry a jammed sticky, which must sit at least two places below the
// rounding point) into the format. Writes the encoding and the flags.
// ZERO: m may be zero (an exact cancellation), which gives +0, or -0 under
// roundTowardNegative, with no flag. LAT: the form for a lone warp waiting
// on one result (shifts as selects on the integer ALU; see fma_general).
template <int FMT, int N, bool ZERO = false, bool LAT = false>
SFD void round_pack(int sign, uint32_t (&m)[N], int e, int rnd, uint32_t (&out)[Fmt<FMT>::W],
                    uint32_t &flags)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W;
    // An exact cancellation leaves with its zero first, so that the lanes
    // left can take the fast paths below.
    if constexpr (ZERO) {
        if ((m[N - 1] | m[N - 2]) == 0u && sfw::is_zero(m)) {
            enc_zero<FMT>(out, rnd == RDN ? 1 : 0);
            flags = 0u;
            return;
        }
    }
    // Most results keep their leading bit in the top word or the one below
    // (sums without deep cancellation, quotients, roots): when every lane of
    // the warp has it there, one clz. LAT: each lane on its own (a vote
    // costs a lone warp more than the clz it saves).
    int L;
    if constexpr (LAT) {
        if (m[N - 1]) L = 32 * N - __clz(m[N - 1]);
        else if (m[N - 2]) L = 32 * (N - 1) - __clz(m[N - 2]);
        else L = sfw::bitlen(m);
    } else {
        const unsigned am = __activemask();
        if (__all_sync(am, m[N - 1] != 0u)) L = 32 * N - __clz(m[N - 1]);
        else if (__all_sync(am, m[N - 1] == 0u && m[N - 2] != 0u)) L = 32 * (N - 1) - __clz(m[N - 2]);
        else L = sfw::bitlen(m);
    }
    const int e_norm = e + L - 1;                 // exponent of the leading bit
    // leading bit to the top; narrow windows shift on the IMAD pipe, wide
    // ones (whose products already load it) on the integer ALU; LAT: a
    // shift of less than a word (the usual one) without the select network
    // and its vote
    if constexpr (N <= 5 && !LAT) sfw::shl_imad(m, 32 * N - L);
    else if constexpr (LAT) sfw::shl_small_first(m, 32 * N - L);
    else sfw::shl(m, 32 * N - L);

    uint32_t kept[W];
    bool guard, sticky;
    take_top<FMT, N>(m, kept, guard, sticky);
    bool up = LAT ? round_up_sel(rnd, sign, guard, sticky, kept[0] & 1u)
                  : round_up(rnd, sign, guard, sticky, kept[0] & 1u);

    const int d = F::EMIN - e_norm;              // > 0: below the normal range
    bool carry_unb = false;
    if (d > 0) {
        // Rounded as if the exponent range were unbounded: does it carry out?
        uint32_t ones[W];
#pragma unroll
        for (int i = 0; i < W; i++) ones[i] = 0xFFFFFFFFu;
        ones[W - 1] = (F::P % 32) ? ((1u << (F::P % 32)) - 1u) : 0xFFFFFFFFu;
        carry_unb = up && sfw::cmp(kept, ones) == 0;
        sfw::shr_jam(m, d);
        take_top<FMT, N>(m, kept, guard, sticky);
        up = round_up(rnd, sign, guard, sticky, kept[0] & 1u);
    }
    const bool inexact = guard || sticky;
    uint32_t fl = inexact ? F_INEXACT : 0u;
    if constexpr (LAT && W >= 2) {
        // the increment as a carry chain with up as its carry in, no branch
        uint32_t zw[W];
#pragma unroll
        for (int i = 0; i < W; i++) zw[i] = 0u;
        sfw::AddPtx<W>::add(kept, zw, up ? 1u : 0u);
    } else if (up) {
        if constexpr (W >= 2) sfw::IncPtx<W>::inc(kept);
        else sfw::inc(kept);
    }

    if (d > 0) {
        // Subnormal (or rounded up into the smallest normal, whose bits are
        // exactly kept's with the hidden bit landing in the exponent field).
        const bool tiny = d >= 2 || !carry_unb;
        if (tiny && inexact) fl |= F_UNDERFLOW;
        if (sfw::is_zero(kept)) fl |= F_UNDERFLOW;  // rounded past the least subnormal
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = kept[i];
        out[W - 1] |= (uint32_t)sign << 31;
        flags = fl;
        return;
    }
    int e_res = e_norm;
    // carry out of the top: kept == 2^P
    static_assert(F::P < 32 * W, "kept needs room for the carry bit");
    if (sfw::bit<F::P, W>(kept)) {
        e_res += 1;
        sfw::zero(kept);
        kept[(F::P - 1) >> 5] = 1u << ((F::P - 1) & 31);
    }
    if (e_res > F::EMAX) {
        if (overflow_to_inf(rnd, sign)) enc_inf<FMT>(out, sign);
        else enc_max_normal<FMT>(out, sign);
        flags = fl | F_OVERFLOW | F_INEXACT;
        return;
    }
#pragma unroll
    for (int i = 0; i < W; i++) out[i] = kept[i];
    out[W - 1] &= (1u << exp_shift<FMT>()) - 1u;   // drop the hidden bit
    out[W - 1] |= ((uint32_t)sign << 31) | ((uint32_t)(e_res + F::BIAS) << exp_shift<FMT>());
    flags = fl;
}

// ---- fused multiply-add ---------------------------------------------------

template <int FMT>
SFD bool any_snan(const Unp<FMT> &a, const Unp<FMT> &b, const Unp<FMT> &c)
{
    return (a.cls == C_NAN && a.snan) || (b.cls == C_NAN && b.snan) || (c.cls == C_NAN && c.snan);
}

// The steered operand kinds: FMA a*b+c; ADD a*1+c; SUB a*1+(-c); MUL a*b+(+-0)
// (host/src/softfloat.c:438-468).
enum { OP_FMA = 0, OP_ADD = 1, OP_SUB = 2, OP_MUL = 3 };

// The general path: finite non-zero a and b; c finite (zero allowed).
//
// Window: N = 2W words. a's significand arrives with its leading bit at
// 32W-2 and b's at 32W-1 (unpack<FMT, LB>), so their product's leading bit
// is at 64W-3 or 64W-2 and bit 64W-1 is free for a carry. Its low 64W-2P-1
// bits are zero. The addend (leading bit at 32W-2) goes to the top half, its
// leading bit at 64W-2, its low 64W-P-1 bits zero.
// With delta = (addend exponent) - (product's nominal exponent) - 1:
//  * delta > 0: the product is shifted right by delta. Exact for delta <= 1
//    (the only shifts after which the two can cancel to fewer than P+2
//    bits); for delta >= 2 the difference keeps its leading bit at 64W-3 or
//    above, so a jammed bit 0 is far below the rounding point.
//  * delta < 0: the addend is shifted right by -delta; bits are lost only
//    when its leading bit falls below bit P, where it cannot cancel the
//    product's leading bits.
// A jammed bit 0 makes the computed window W' satisfy: bits >= 1 of W' are
// floor(exact/2) and bit 0 is set iff the exact value is not an integer
// (operands' true low bits are zero there, so subtracting a jammed operand
// leaves bit 0 set). Rounding at any position >= 2 then reads the right
// kept bits, guard and sticky.
//
// LAT selects the form for a warp that waits on this one result (a
// trajectory's dependent chain on a lightly loaded scheduler) rather than
// for many warps sharing the integer pipes: the product as two independent
// column sums (mul_ptx_split), and the selects, the alignment
// shift and the complement as selects and XORs on the integer ALU pipe
// (one instruction a word) instead of multiply-adds (two a word on the
// IMAD pipe, which balance the pipes under load but lengthen a lone
// chain). The same bits either way.
template <int FMT, int OP, bool LAT = false>
SFD void fma_general(const Unp<FMT> &ua, const Unp<FMT> &ub, const Unp<FMT> &uc, int sc, int rnd,
                     uint32_t (&out)[Fmt<FMT>::W], uint32_t &flags)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W, N = 2 * W;
    uint32_t P[N];
    const int sp = ua.sign ^ ub.sign;
    int ew;                                        // weight of window bit 0
    if constexpr (OP == OP_ADD || OP == OP_SUB) {
        // a * 1.0 needs no multiply: the product is a's significand placed
        // where the multiply would have put it, leading bit at 64W-3.
#pragma unroll
        for (int i = 0; i < W; i++) P[i] = 0u;
#pragma unroll
        for (int i = 0; i < W; i++) P[W + i] = ua.m[i];   // leading bit at 64W-2
        sfw::shr_const<1>(P);                              // leading bit at 64W-3
        ew = ua.ve - (64 * W - 3);
    } else {
        if constexpr (LAT) sfw::mul_ptx_split<W>(P, ua.m, ub.m);
        else sfw::mul_ptx<W>(P, ua.m, ub.m);
        ew = ua.ve + ub.ve - (64 * W - 3);
    }

    int rs = sp;
    if constexpr (OP != OP_MUL) {
        // The addend, leading bit at 64W-2 (a zero addend stays all zero).
        uint32_t C[N];
#pragma unroll
        for (int i = 0; i < W; i++) C[i] = 0u;
#pragma unroll
        for (int i = 0; i < W; i++) C[W + i] = uc.m[i];    // a zero's significand is zero
        const bool czero = uc.cls == C_ZERO;
        // Branch-free alignment: Y keeps its place, X (the term with the
        // smaller exponent) is shifted right by |delta| with jamming.
        const int delta = czero ? -(1 << 28) : uc.ve - (ew + 64 * W - 2);
        const bool pbig = delta <= 0;
        uint32_t X[N], Y[N];
        if constexpr (LAT) {
#pragma unroll
            for (int i = 0; i < N; i++) {
                X[i] = pbig ? C[i] : P[i];
                Y[i] = pbig ? P[i] : C[i];
            }
        } else {
            // the selections as multiply-adds by 0 and 1 (IMAD pipe)
            const uint32_t pb = pbig ? 1u : 0u, npb = pb ^ 1u;
#pragma unroll
            for (int i = 0; i < N; i++) {
                if (i < W) {                          // C's low words are zero
                    X[i] = sfw::imul(P[i], npb);
                    Y[i] = sfw::imul(P[i], pb);
                } else {
                    X[i] = sfw::imad(C[i], pb, sfw::imul(P[i], npb));
                    Y[i] = sfw::imad(P[i], pb, sfw::imul(C[i], npb));
                }
            }
        }
        // LAT: a zero addend (every MUL through the run-time dispatch) is
        // already aligned - it is all zero - so its shift is skipped
        if constexpr (LAT) sfw::shr_jam_small_first(X, czero ? 0 : (pbig ? -delta : delta));
        else sfw::shr_jam_imad(X, pbig ? -delta : delta);
        if (!pbig) ew += delta;
        const int s_big = pbig ? sp : sc, s_small = pbig ? sc : sp;
        // Y + X, or Y - X in two's complement, then the magnitude.
        const bool sub = sp != sc;
        const uint32_t mk = sub ? 0xFFFFFFFFu : 0u;
        // X ^ mk as X * m1 + mk (~X is -X - 1 modulo 2^32), on the IMAD pipe
        const uint32_t m1 = sub ? 0xFFFFFFFFu : 1u;
#pragma unroll
        for (int i = 0; i < N; i++) {
            P[i] = Y[i];
            X[i] = LAT ? X[i] ^ mk : sfw::imad(X[i], m1, mk);
        }
        const uint32_t cy = sfw::AddPtx<N>::add(P, X, sub ? 1u : 0u);
        const bool neg = sub && !cy;               // Y < X: the result is X - Y
        // the negation only where some lane of the warp needs it (the
        // smaller-exponent term is the larger magnitude only under deep
        // cancellation); LAT: where this lane needs it, without the vote
        if (LAT ? neg : __any_sync(__activemask(), neg)) {
            const uint32_t m2 = neg ? 0xFFFFFFFFu : 0u;
            uint32_t z[N];
#pragma unroll
            for (int i = 0; i < N; i++) {
                P[i] ^= m2;
                z[i] = 0u;
            }
            sfw::AddPtx<N>::add(P, z, neg ? 1u : 0u);
        }
        rs = neg ? s_small : s_big;
    }
    // an exact cancellation (only an effective subtraction gives one) leaves
    // P zero, which round_pack answers with the zero of the attribute
    round_pack<FMT, N, OP != OP_MUL, LAT>(rs, P, ew, rnd, out, flags);
}

// The steered operands of FMA/ADD/SUB/MUL, unpacked: x/y/z are the
// caller's a, b, c (b unused for ADD/SUB, c unused for MUL); csteer is the
// steered addend's encoding (host/src/softfloat.c:438-468).
template <int FMT, int OP>
SFD void steer_unpack(const uint32_t (&x)[Fmt<FMT>::W], const uint32_t (&y)[Fmt<FMT>::W],
                      const uint32_t (&z)[Fmt<FMT>::W], Unp<FMT> &ua, Unp<FMT> &ub,
                      Unp<FMT> &uc, uint32_t (&csteer)[Fmt<FMT>::W])
{
    constexpr int W = Fmt<FMT>::W;
    uint32_t bsteer[W];
    if constexpr (OP == OP_ADD || OP == OP_SUB) {
        enc_one<FMT>(bsteer, 0);
    } else {
#pragma unroll
        for (int i = 0; i < W; i++) bsteer[i] = y[i];
    }
    if constexpr (OP == OP_MUL) {
        enc_zero<FMT>(csteer, sign_of<FMT>(x) ^ sign_of<FMT>(y));
    } else {
#pragma unroll
        for (int i = 0; i < W; i++) csteer[i] = z[i];
        if constexpr (OP == OP_SUB) csteer[W - 1] ^= 0x80000000u;
    }
    unpack<FMT, 32 * W - 2>(x, ua);
    unpack<FMT, 32 * W - 1>(bsteer, ub);
    unpack<FMT, 32 * W - 2>(csteer, uc);
}

// The special cases in the reference's order (host/src/softfloat.c:335-373):
// true, with the result and flags, when an operand is a NaN or an infinity
// or a factor is zero; false when the element needs fma_general.
template <int FMT>
SFD bool arith_special_case(const Unp<FMT> &ua, const Unp<FMT> &ub, const Unp<FMT> &uc,
                            const uint32_t (&csteer)[Fmt<FMT>::W], int rnd,
                            uint32_t (&out)[Fmt<FMT>::W], uint32_t &flags)
{
    constexpr int W = Fmt<FMT>::W;
    flags = 0u;
    if (ua.cls == C_NAN || ub.cls == C_NAN || uc.cls == C_NAN) {
        enc_qnan<FMT>(out);
        flags = any_snan(ua, ub, uc) ? F_INVALID : 0u;
        return true;
    }
    const int sp = ua.sign ^ ub.sign;
    if (ua.cls == C_INF || ub.cls == C_INF) {
        if (ua.cls == C_ZERO || ub.cls == C_ZERO || (uc.cls == C_INF && uc.sign != sp)) {
            enc_qnan<FMT>(out);                    // inf * 0, inf - inf
            flags = F_INVALID;
            return true;
        }
        enc_inf<FMT>(out, sp);
        return true;
    }
    if (uc.cls == C_INF) {
        enc_inf<FMT>(out, uc.sign);
        return true;
    }
    if (ua.cls == C_ZERO || ub.cls == C_ZERO) {
        if (uc.cls == C_ZERO) {
            enc_zero<FMT>(out, uc.sign == sp ? uc.sign : (rnd == RDN ? 1 : 0));
            return true;
        }
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = csteer[i];   // 0*b + c is c, exactly
        return true;
    }
    return false;
}

// unpack for an operand known to be normal (unpack's last case alone)
template <int FMT, int LB>
SFD void unpack_normal(const uint32_t (&x)[Fmt<FMT>::W], Unp<FMT> &u)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W;
    u.sign = sign_of<FMT>(x);
    u.snan = 0;
    u.cls = C_NORM;
    u.ve = (int)exp_field<FMT>(x) - F::BIAS;
#pragma unroll
    for (int i = 0; i < W; i++) u.m[i] = x[i];
    u.m[W - 1] = (u.m[W - 1] & ((1u << exp_shift<FMT>()) - 1u)) | (1u << exp_shift<FMT>());
    sfw::shl_const<LB - F::MANW>(u.m);
}

// One element of FMA/ADD/SUB/MUL: the special cases, else the general path.
// LAT (a lone warp waiting on the result, fma_general): the usual operands -
// a and b normal, c normal or zero, which take no special case - are told
// apart by one test and unpacked without unpack's class branches.
template <int FMT, int OP, bool LAT = false>
SFD void arith(const uint32_t (&x)[Fmt<FMT>::W], const uint32_t (&y)[Fmt<FMT>::W],
               const uint32_t (&z)[Fmt<FMT>::W], int rnd, uint32_t (&out)[Fmt<FMT>::W],
               uint32_t &flags)
{
    constexpr int W = Fmt<FMT>::W;
    if constexpr (LAT && OP == OP_FMA) {
        constexpr uint32_t EM = exp_mask<FMT>();
        uint32_t zm = z[W - 1] & 0x7FFFFFFFu;
#pragma unroll
        for (int i = 0; i < W - 1; i++) zm |= z[i];
        const bool cz = zm == 0u;
        const uint32_t ea = exp_field<FMT>(x), eb = exp_field<FMT>(y), ec = exp_field<FMT>(z);
        if ((ea - 1u) < EM - 1u && (eb - 1u) < EM - 1u && ((ec - 1u) < EM - 1u || cz)) {
            Unp<FMT> ua, ub, uc;
            unpack_normal<FMT, 32 * W - 2>(x, ua);
            unpack_normal<FMT, 32 * W - 1>(y, ub);
            unpack_normal<FMT, 32 * W - 2>(z, uc);
            if (cz) {
                uc.cls = C_ZERO;
                uc.ve = 0;
#pragma unroll
                for (int i = 0; i < W; i++) uc.m[i] = 0u;
            }
            fma_general<FMT, OP, true>(ua, ub, uc, uc.sign, rnd, out, flags);
            return;
        }
    }
    Unp<FMT> ua, ub, uc;
    uint32_t csteer[Fmt<FMT>::W];
    steer_unpack<FMT, OP>(x, y, z, ua, ub, uc, csteer);
    if (arith_special_case<FMT>(ua, ub, uc, csteer, rnd, out, flags)) return;
    fma_general<FMT, OP, LAT>(ua, ub, uc, uc.sign, rnd, out, flags);
}

// FMA/ADD/SUB/MUL with the operation chosen at run time, all through the one
// FMA code path: ADD/SUB steer b to +1 (a*1 is exact) and SUB flips c's sign,
// MUL steers c to a zero of the product's sign, exactly the reference's
// steering; the special cases then see the steered operands. One copy of
// the code serves every arithmetic opcode, which keeps an interpreter's
// instruction footprint small and lets threads that run different opcodes
// of this family stay converged. LAT: see arith.
template <int FMT, bool LAT = false>
SFD void arith_rt(int op, const uint32_t (&x)[Fmt<FMT>::W], const uint32_t (&y)[Fmt<FMT>::W],
                  const uint32_t (&z)[Fmt<FMT>::W], int rnd, uint32_t (&out)[Fmt<FMT>::W],
                  uint32_t &flags)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W;
    constexpr int ES = exp_shift<FMT>();
    const bool addsub = op == OP_ADD || op == OP_SUB;
    uint32_t b[W], c[W];
#pragma unroll
    for (int i = 0; i < W; i++) {
        b[i] = addsub ? 0u : y[i];
        c[i] = op == OP_MUL ? 0u : z[i];
    }
    if (addsub) b[W - 1] = (uint32_t)F::BIAS << ES;                       // +1
    if (op == OP_SUB) c[W - 1] ^= 0x80000000u;
    if (op == OP_MUL) c[W - 1] = (x[W - 1] ^ y[W - 1]) & 0x80000000u;    // +-0
    arith<FMT, OP_FMA, LAT>(x, b, c, rnd, out, flags);
}

// ---- exact division of significands ---------------------------------------

// A two-word by one-word division by a normalised divisor d (top bit set)
// through its precomputed reciprocal v = floor((2^64 - 1) / d) - 2^32
// (Moller and Granlund, "Improved division by invariant integers", IEEE
// Trans. Computers 60(2), 2011, Algorithm 4): u1 < d; returns floor((u1 *
// 2^32 + u0) / d) and the remainder in r. One multiply and two corrections
// in place of a 64-by-32-bit division per quotient digit.
SFD uint32_t recip_norm(uint32_t d)
{
    return (uint32_t)(0xFFFFFFFFFFFFFFFFull / d - 0x100000000ull);
}

SFD uint32_t div_2by1(uint32_t u1, uint32_t u0, uint32_t d, uint32_t v, uint32_t &r)
{
    const uint64_t q = (uint64_t)v * u1 + (((uint64_t)u1 << 32) | u0);
    uint32_t q1 = (uint32_t)(q >> 32) + 1u;
    const uint32_t q0 = (uint32_t)q;
    uint32_t rr = u0 - q1 * d;
    if (rr > q0) {
        q1--;
        rr += d;
    }
    if (rr >= d) {
        q1++;
        rr -= d;
    }
    r = rr;
    return q1;
}

// q (W+1 words) = floor(X * 2^(32W) / Y) and rnz = (remainder != 0), for X, Y
// of W words with their top bits set. Base-2^32 long division (Knuth,
// TAOCP vol. 2, 4.3.1, Algorithm D): each quotient digit is estimated from
// the top two remainder words over Y's top word (by the reciprocal of that
// word, computed once), refined against Y's second word, and fixed by at
// most one add-back after the multiply-subtract.
template <int W>
SFD void divrem_top(const uint32_t (&X)[W], const uint32_t (&Y)[W], uint32_t (&q)[W + 1],
                    uint32_t &rnz)
{
    if constexpr (W == 1) {
        const uint64_t u = (uint64_t)X[0] << 32;
        const uint64_t qq = u / Y[0];
        q[0] = (uint32_t)qq;
        q[1] = (uint32_t)(qq >> 32);
        rnz = (uint32_t)(u - qq * Y[0]) != 0u;
    } else {
        constexpr int n = W, m = W;             // divisor words, quotient digits - 1
        uint32_t u[m + n + 1];                  // X * 2^(32W), one spare top word
#pragma unroll
        for (int i = 0; i < n; i++) u[i] = 0u;
#pragma unroll
        for (int i = 0; i < n; i++) u[n + i] = X[i];
        u[m + n] = 0u;
        const uint32_t vt = Y[n - 1], vs = Y[n - 2];
        const uint32_t vinv = recip_norm(vt);
        // the top digit is 0 or 1 (X < 2Y): X >= Y, and subtract Y if so
        {
            uint32_t d[n];
            const uint32_t br = sfw::sub(d, X, Y);
            q[m] = br ? 0u : 1u;
#pragma unroll
            for (int i = 0; i < n; i++) u[m + i] = br ? u[m + i] : d[i];
        }
#pragma unroll
        for (int j = m - 1; j >= 0; j--) {
            // the digit estimate is a word: 32 x 32-bit products below
            uint32_t qd;
            uint64_t rhat;
            if (u[j + n] >= vt) {
                qd = 0xFFFFFFFFu;
                rhat = (((uint64_t)u[j + n] << 32) | u[j + n - 1]) - 0xFFFFFFFFull * vt;
            } else {
                uint32_t r32;
                qd = div_2by1(u[j + n], u[j + n - 1], vt, vinv, r32);
                rhat = r32;
            }
            // at most two corrections make qd exact or one too large
            for (int k = 0; k < 2; k++) {
                if (rhat <= 0xFFFFFFFFull && (uint64_t)qd * vs > ((rhat << 32) | u[j + n - 2])) {
                    qd--;
                    rhat += vt;
                }
            }
            // u[j .. j+n] -= qd * Y: the row by wide multiply-adds, one borrow chain
            // (binary256 keeps the two carry chains of halves: its wide row
            // took 70 registers against 48 and measured 2 % slower)
            uint32_t row[n + 1];
            if constexpr (n <= 4) {
                sfw::mul_row_wide<n>(row, qd, Y);
            } else {
#pragma unroll
                for (int i = 0; i <= n; i++) row[i] = 0u;
                sfw::MulPtx<n>::row(row, qd, Y);
            }
            if (sfw::SubPtx<n + 1>::sub(u + j, row)) {   // one too large: add Y back
                qd--;
                uint32_t c = 0u;
#pragma unroll
                for (int i = 0; i < n; i++) {
                    const uint64_t a2 = (uint64_t)u[i + j] + Y[i] + c;
                    u[i + j] = (uint32_t)a2;
                    c = (uint32_t)(a2 >> 32);
                }
                u[j + n] += c;
            }
            q[j] = qd;
        }
        uint32_t o = 0u;
#pragma unroll
        for (int i = 0; i < n; i++) o |= u[i];
        rnz = o != 0u;
    }
}

// ---- division (definition: python/cft_golden/softfloat.py:440-471) ------

template <int FMT>
SFD void div(const uint32_t (&x)[Fmt<FMT>::W], const uint32_t (&y)[Fmt<FMT>::W], int rnd,
             uint32_t (&out)[Fmt<FMT>::W], uint32_t &flags)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W;
    Unp<FMT> ua, ub;
    unpack<FMT>(x, ua);
    unpack<FMT>(y, ub);
    flags = 0u;
    if (ua.cls == C_NAN || ub.cls == C_NAN) {
        enc_qnan<FMT>(out);
        flags = ((ua.cls == C_NAN && ua.snan) || (ub.cls == C_NAN && ub.snan)) ? F_INVALID : 0u;
        return;
    }
    const int sq = ua.sign ^ ub.sign;
    if (ua.cls == C_INF) {
        if (ub.cls == C_INF) { enc_qnan<FMT>(out); flags = F_INVALID; return; }
        enc_inf<FMT>(out, sq);
        return;
    }
    if (ub.cls == C_INF) { enc_zero<FMT>(out, sq); return; }
    if (ub.cls == C_ZERO) {
        if (ua.cls == C_ZERO) { enc_qnan<FMT>(out); flags = F_INVALID; return; }
        enc_inf<FMT>(out, sq);
        flags = F_DIVZERO;
        return;
    }
    if (ua.cls == C_ZERO) { enc_zero<FMT>(out, sq); return; }

    // Both significands have their leading bit at 32W-1. The quotient of
    // X * 2^(32W) by Y, exact with its remainder, by long division in base
    // 2^32 (Knuth, TAOCP vol. 2, 4.3.1, Algorithm D; Y is already
    // normalised). Q has W+1 words and at least 32W >= P+3 significant
    // bits, since X/Y > 1/2.
    uint32_t q[W + 1], rnz;
    divrem_top<W>(ua.m, ub.m, q, rnz);
    // fold the remainder in as a sticky bit below the quotient
    uint32_t m[W + 1];
#pragma unroll
    for (int i = W; i >= 1; i--) m[i] = __funnelshift_l(q[i - 1], q[i], 1);
    m[0] = (q[0] << 1) | (rnz ? 1u : 0u);
    // |a/b| = (X/Y) 2^(ve_a - ve_b) = Q 2^(ve_a - ve_b - 32W) (+ remainder)
    const int e = ua.ve - ub.ve - 32 * W - 1;
    round_pack<FMT, W + 1>(sq, m, e, rnd, out, flags);
}

// ---- exact integer square root of a significand ----------------------------

// floor(sqrt(t)) for t < 2^64, bit by bit.
SFD uint32_t isqrt64(uint64_t t)
{
    uint32_t r = 0u;
#pragma unroll
    for (int b = 31; b >= 0; b--) {
        const uint32_t c = r | (1u << b);
        if ((uint64_t)c * c <= t) r = c;
    }
    return r;
}

// S (W words) = floor(sqrt(N)) and rnz = (N != S^2), for N of 2W words with
// N >= 2^(64W-2). Digit by digit in base B = 2^32, the pencil-and-paper
// method: the first digit is the exact root of N's top 64 bits; each next
// digit d is the largest with (2rB + d) d <= rem, where r is the root so
// far and rem = (N's prefix) - r^2. Its estimate is floor(rem / (2rB))
// taken from the top words (r is normalised: its top bit is set), which is
// never below d and at most three above it, so at most three add-backs of
// (2rB + 2d + 1) correct it.
template <int W>
SFD void isqrtrem(const uint32_t (&N)[2 * W], uint32_t (&S)[W], uint32_t &rnz)
{
    constexpr int RW = W + 2;                // remainder words
    uint32_t rem[RW], r[W + 1];
#pragma unroll
    for (int i = 0; i < RW; i++) rem[i] = 0u;
#pragma unroll
    for (int i = 0; i <= W; i++) r[i] = 0u;
    {
        const uint64_t t = ((uint64_t)N[2 * W - 1] << 32) | N[2 * W - 2];
        const uint32_t d = isqrt64(t);                         // >= 2^31
        const uint64_t e = t - (uint64_t)d * d;                // <= 2d < 2^33
        rem[0] = (uint32_t)e;
        rem[1] = (uint32_t)(e >> 32);
        r[0] = d;
    }
    const uint32_t rinv = recip_norm(r[0]);        // the estimates' divisor never changes
#pragma unroll
    for (int i = 1; i < W; i++) {
        // rem = rem * B^2 + the next two words of N  (rem < (2r + 1) B^2)
#pragma unroll
        for (int j = RW - 1; j >= 2; j--) rem[j] = rem[j - 2];
        rem[1] = N[2 * W - 1 - 2 * i];
        rem[0] = N[2 * W - 2 - 2 * i];
        // estimate floor(rem / (2 r B)) = floor((rem >> 1) / (r B)) from the
        // top two words of rem >> 1 over r's top word (r[i-1] >= 2^31)
        const uint32_t u1 = __funnelshift_r(rem[i + 1], rem[i + 2], 1);
        const uint32_t u0 = __funnelshift_r(rem[i], rem[i + 1], 1);
        const uint32_t rt = r[i - 1];             // the first digit, every step
        uint32_t d = 0xFFFFFFFFu;
        if (u1 < rt) {
            uint32_t rr;
            d = div_2by1(u1, u0, rt, rinv, rr);
        }
        // D = 2 r B + d (words: d, then 2r)
        uint32_t D[RW];
        D[0] = d;
#pragma unroll
        for (int j = 1; j < RW; j++) {
            const uint32_t hi = (j - 1 <= W) ? r[j - 1] : 0u;
            const uint32_t lo = (j >= 2 && j - 2 <= W) ? r[j - 2] : 0u;
            D[j] = __funnelshift_l(lo, hi, 1);
        }
        // rem -= D * d   (D * d < B^(i+3) <= B^RW: no carry out, so the
        // row's top word is zero): the row by wide multiply-adds, one borrow chain
        uint32_t row[RW + 1];
        sfw::mul_row_wide<RW>(row, d, D);
        // the estimate is never low and at most three high: while rem < 0,
        // d -= 1 and rem += 2 r B + 2 d + 1
        bool neg = sfw::SubPtx<RW>::sub(rem, row) != 0u;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (neg) {
                d -= 1u;
                uint32_t c = 0u;
#pragma unroll
                for (int j = 0; j < RW; j++) {
                    const uint32_t add = j == 0 ? (d << 1) | 1u : j == 1 ? D[1] + (d >> 31) : D[j];
                    const uint64_t a2 = (uint64_t)rem[j] + add + c;
                    rem[j] = (uint32_t)a2;
                    c = (uint32_t)(a2 >> 32);
                }
                neg = c == 0u;
            }
        }
        // r = r B + d
#pragma unroll
        for (int j = W; j >= 1; j--) r[j] = r[j - 1];
        r[0] = d;
    }
#pragma unroll
    for (int i = 0; i < W; i++) S[i] = r[i];
    uint32_t o = 0u;
#pragma unroll
    for (int i = 0; i < RW; i++) o |= rem[i];
    rnz = o != 0u;
}

// ---- square root (definition: python/cft_golden/softfloat.py:474-505) ---

template <int FMT>
SFD void sqrt(const uint32_t (&x)[Fmt<FMT>::W], int rnd, uint32_t (&out)[Fmt<FMT>::W],
              uint32_t &flags)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W;
    Unp<FMT> ua;
    unpack<FMT>(x, ua);
    flags = 0u;
    if (ua.cls == C_NAN) {
        enc_qnan<FMT>(out);
        flags = ua.snan ? F_INVALID : 0u;
        return;
    }
    if (ua.cls == C_ZERO) {
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = x[i];
        return;
    }
    if (ua.sign) { enc_qnan<FMT>(out); flags = F_INVALID; return; }
    if (ua.cls == C_INF) {
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = x[i];
        return;
    }
    // The radicand N: the significand (leading bit at 32W-1) placed in 2W
    // words with its leading bit at 64W-1 or 64W-2, whichever leaves the
    // exponent of N's bit 0 even. Its root S = floor(sqrt(N)) then has
    // exactly 32W >= P+3 bits (N >= 2^(64W-2)).
    uint32_t N[2 * W];
#pragma unroll
    for (int i = 0; i < W; i++) N[i] = 0u;
#pragma unroll
    for (int i = 0; i < W; i++) N[W + i] = ua.m[i];          // leading bit at 64W-1
    // N = m_top * 2^(ve - 64W + 1); make that exponent even
    const bool odd = ((ua.ve - 64 * W + 1) & 1) != 0;
    if (odd) sfw::shr_const<1>(N);                             // leading bit at 64W-2
    const int ex = ua.ve - 64 * W + 1 + (odd ? 1 : 0);         // even
    uint32_t S[W], rnz;
    isqrtrem<W>(N, S, rnz);
    uint32_t m[W + 1];
    m[W] = S[W - 1] >> 31;
#pragma unroll
    for (int i = W - 1; i >= 1; i--) m[i] = __funnelshift_l(S[i - 1], S[i], 1);
    m[0] = (S[0] << 1) | (rnz ? 1u : 0u);
    // sqrt(|x|) = sqrt(N) 2^(ex/2); m = 2S + sticky
    round_pack<FMT, W + 1>(0, m, (ex >> 1) - 1, rnd, out, flags);
}

}  // namespace sf
