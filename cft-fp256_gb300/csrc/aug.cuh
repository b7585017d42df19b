// aug.cuh - IEEE 754-2019 9.5's augmented operations on the GPU:
// augmentedAddition, augmentedSubtraction, augmentedMultiplication, each
// returning r = the result rounded with roundTiesTowardZero and e = the
// residual (x op y) - r. Semantics as python/cft_golden/augmented.py defines
// them (reference C: host/src/augmented.c); the computation is this
// library's fixed window:
//
//  * multiplication: the exact 2p-bit product of the significands in 2W
//    words (the FMA's product, no addend);
//  * addition: when the value exponents are within p + 1 of each other
//    (the reference's NEAR bound), both significands in one 2W-word window,
//    the larger's leading bit at 64W-3 and the smaller shifted by the
//    exponent gap - no bit leaves the window, so the sum is exact. Farther
//    apart (FAR), the smaller operand is less than half an ulp of the
//    larger in every direction: r is the larger operand and e the smaller,
//    exactly;
//  * r = round_pack(exact, RTTZ); an overflow gives (inf, inf,
//    OVERFLOW|INEXACT). Otherwise r is placed back in the window (its bits
//    all land on the window's grid) and e = exact - r is packed: exact for
//    addition, RTTZ-rounded for a product residual below the smallest
//    quantum (then UNDERFLOW|INEXACT); UNDERFLOW alone when e is non-zero
//    and below 2^emin; a zero e takes r's sign.
#pragma once
#include "softfloat.cuh"

namespace sf {

enum { AUG_ADD = 0, AUG_SUB = 1, AUG_MUL = 2 };

// The pair for the exact non-zero value (-1)^sign * T * 2^ew (T of N = 2W
// words, leading bit at or below 64W-2).
template <int FMT>
SFD void aug_pair(int sign, const uint32_t (&T)[2 * Fmt<FMT>::W], int ew, bool is_mul,
                  uint32_t (&r)[Fmt<FMT>::W], uint32_t (&e)[Fmt<FMT>::W], uint32_t &flags)
{
    constexpr int W = Fmt<FMT>::W, N = 2 * W;
    uint32_t t[N], rf = 0u;
#pragma unroll
    for (int i = 0; i < N; i++) t[i] = T[i];
    round_pack<FMT, N>(sign, t, ew, RTTZ, r, rf);
    if (rf & F_OVERFLOW) {
        enc_inf<FMT>(r, sign);
#pragma unroll
        for (int i = 0; i < W; i++) e[i] = r[i];
        flags = F_OVERFLOW | F_INEXACT;
        return;
    }
    // r in window units (bit 0 weighs 2^ew)
    Unp<FMT> ur;
    unpack<FMT>(r, ur);
    uint32_t R[N];
#pragma unroll
    for (int i = 0; i < N; i++) R[i] = 0u;
    if (ur.cls != C_ZERO) {
#pragma unroll
        for (int i = 0; i < W; i++) R[W + i] = ur.m[i];          // leading bit at 64W-1
        sfw::shr(R, 64 * W - 1 - (ur.ve - ew));
    }
    // D = |T - R|, with its sign
    uint32_t D[N];
    const uint32_t borrow = sfw::sub(D, T, R);
    int sign_e = sign;
    if (borrow) {
        sfw::neg(D);
        sign_e = !sign;
    }
    if (sfw::is_zero(D)) {
        enc_zero<FMT>(e, ur.sign);
        flags = 0u;
        return;
    }
    const bool tiny = ew + sfw::bitlen(D) - 1 < Fmt<FMT>::EMIN;
    uint32_t ef = 0u;
    round_pack<FMT, N>(sign_e, D, ew, RTTZ, e, ef);
    if (is_mul && (ef & F_INEXACT)) flags = F_UNDERFLOW | F_INEXACT;
    else flags = tiny ? F_UNDERFLOW : 0u;
}

template <int FMT>
SFD void augmented(int fn, const uint32_t (&x)[Fmt<FMT>::W], const uint32_t (&yin)[Fmt<FMT>::W],
                   uint32_t (&r)[Fmt<FMT>::W], uint32_t (&e)[Fmt<FMT>::W], uint32_t &flags)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W, N = 2 * W;
    uint32_t y[W];
#pragma unroll
    for (int i = 0; i < W; i++) y[i] = yin[i];
    if (fn == AUG_SUB) y[W - 1] ^= 0x80000000u;                  // x - y is x + (-y)
    Unp<FMT> ua, ub;
    unpack<FMT>(x, ua);
    unpack<FMT>(y, ub);
    flags = 0u;
    auto both = [&](const uint32_t (&v)[W]) {
#pragma unroll
        for (int i = 0; i < W; i++) {
            r[i] = v[i];
            e[i] = v[i];
        }
    };
    uint32_t v[W];
    if (ua.cls == C_NAN || ub.cls == C_NAN) {
        enc_qnan<FMT>(v);
        both(v);
        flags = ((ua.cls == C_NAN && ua.snan) || (ub.cls == C_NAN && ub.snan)) ? F_INVALID : 0u;
        return;
    }
    if (fn == AUG_MUL) {
        const int sp = ua.sign ^ ub.sign;
        if ((ua.cls == C_INF && ub.cls == C_ZERO) || (ua.cls == C_ZERO && ub.cls == C_INF)) {
            enc_qnan<FMT>(v);
            both(v);
            flags = F_INVALID;
            return;
        }
        if (ua.cls == C_INF || ub.cls == C_INF) { enc_inf<FMT>(v, sp); both(v); return; }
        if (ua.cls == C_ZERO || ub.cls == C_ZERO) { enc_zero<FMT>(v, sp); both(v); return; }
        uint32_t ma[W], T[N];
#pragma unroll
        for (int i = 0; i < W; i++) ma[i] = ua.m[i];
        sfw::shr_const<1>(ma);                                   // leading bit at 32W-2
        sfw::mul_ptx<W>(T, ma, ub.m);                            // leading at 64W-3 or -2
        aug_pair<FMT>(sp, T, ua.ve + ub.ve - (64 * W - 3), true, r, e, flags);
        return;
    }
    if (ua.cls == C_INF && ub.cls == C_INF && ua.sign != ub.sign) {
        enc_qnan<FMT>(v);
        both(v);
        flags = F_INVALID;
        return;
    }
    if (ua.cls == C_INF || ub.cls == C_INF) {
        enc_inf<FMT>(v, ua.cls == C_INF ? ua.sign : ub.sign);
        both(v);
        return;
    }
    if (ua.cls == C_ZERO && ub.cls == C_ZERO) {
        enc_zero<FMT>(v, ua.sign == ub.sign ? ua.sign : 0);
        both(v);
        return;
    }
    if (ua.cls == C_ZERO || ub.cls == C_ZERO) {
#pragma unroll
        for (int i = 0; i < W; i++) r[i] = ua.cls == C_ZERO ? y[i] : x[i];
        enc_zero<FMT>(e, (int)(r[W - 1] >> 31));
        return;
    }
    const bool xbig = ua.ve >= ub.ve;
    const int gap = xbig ? ua.ve - ub.ve : ub.ve - ua.ve;
    if (gap >= F::P + 2) {
        // FAR: r is the larger operand and e the smaller, exactly
#pragma unroll
        for (int i = 0; i < W; i++) {
            r[i] = xbig ? x[i] : y[i];
            e[i] = xbig ? y[i] : x[i];
        }
        flags = ((xbig ? ub.ve : ua.ve) < F::EMIN) ? F_UNDERFLOW : 0u;
        return;
    }
    // NEAR: the exact sum in the window, the larger's leading bit at 64W-3
    const Unp<FMT> &big = xbig ? ua : ub;
    const Unp<FMT> &sml = xbig ? ub : ua;
    uint32_t A[N], B[N];
#pragma unroll
    for (int i = 0; i < W; i++) {
        A[i] = 0u;
        B[i] = 0u;
        A[W + i] = big.m[i];
        B[W + i] = sml.m[i];
    }
    sfw::shr_const<2>(A);
    sfw::shr(B, 2 + gap);
    const int ew = big.ve - (64 * W - 3);
    uint32_t T[N];
    int sign = big.sign;
    if (big.sign == sml.sign) {
        sfw::add(T, A, B);
    } else if (sfw::sub(T, A, B)) {
        sfw::neg(T);
        sign = sml.sign;
    }
    if (sfw::is_zero(T)) {                                       // exact cancellation: +0
        enc_zero<FMT>(v, 0);
        both(v);
        return;
    }
    aug_pair<FMT>(sign, T, ew, false, r, e, flags);
}

}  // namespace sf
