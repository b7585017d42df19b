// simple_ops.cuh - the opcodes that do not round through the FMA: sign
// operations, minimum/maximum, select, comparisons, the integer group and
// the divide/square-root seeds. Semantics: host/src/softfloat.c:470-735.
#pragma once
#include "softfloat.cuh"

namespace sf {

template <int FMT>
SFD bool is_nan_enc(const uint32_t (&x)[Fmt<FMT>::W], bool &signaling)
{
    using F = Fmt<FMT>;
    uint32_t fr[F::W];
#pragma unroll
    for (int i = 0; i < F::W; i++) fr[i] = x[i];
    fr[F::W - 1] &= (1u << exp_shift<FMT>()) - 1u;
    signaling = !((x[(F::MANW - 1) >> 5] >> ((F::MANW - 1) & 31)) & 1u);
    return exp_field<FMT>(x) == exp_mask<FMT>() && !sfw::is_zero(fr);
}

template <int FMT>
SFD bool mag_zero(const uint32_t (&x)[Fmt<FMT>::W])
{
    uint32_t o = x[Fmt<FMT>::W - 1] & 0x7FFFFFFFu;
#pragma unroll
    for (int i = 0; i < Fmt<FMT>::W - 1; i++) o |= x[i];
    return o == 0u;
}

// unsigned comparison of the magnitudes (sign bit cleared)
template <int FMT>
SFD int mag_cmp(const uint32_t (&a)[Fmt<FMT>::W], const uint32_t (&b)[Fmt<FMT>::W])
{
    constexpr int W = Fmt<FMT>::W;
    uint32_t ma[W], mb[W];
#pragma unroll
    for (int i = 0; i < W; i++) { ma[i] = a[i]; mb[i] = b[i]; }
    ma[W - 1] &= 0x7FFFFFFFu;
    mb[W - 1] &= 0x7FFFFFFFu;
    return sfw::cmp(ma, mb);
}

// a < b for non-NaN operands; -0 == +0 (softfloat.c:488-505)
template <int FMT>
SFD bool numeric_lt(const uint32_t (&a)[Fmt<FMT>::W], const uint32_t (&b)[Fmt<FMT>::W])
{
    if (mag_zero<FMT>(a) && mag_zero<FMT>(b)) return false;
    const int sa = sign_of<FMT>(a), sb = sign_of<FMT>(b);
    if (sa != sb) return sa != 0;
    const int c = mag_cmp<FMT>(a, b);
    return sa ? c > 0 : c < 0;
}

template <int FMT>
SFD void copy(uint32_t (&o)[Fmt<FMT>::W], const uint32_t (&x)[Fmt<FMT>::W])
{
#pragma unroll
    for (int i = 0; i < Fmt<FMT>::W; i++) o[i] = x[i];
}

// 754-2019 9.6 minimum/maximum and the ...Number forms (softfloat.c:522-560)
template <int FMT>
SFD void minmax(const uint32_t (&a)[Fmt<FMT>::W], const uint32_t (&b)[Fmt<FMT>::W], bool want_max,
                bool number, uint32_t (&out)[Fmt<FMT>::W], uint32_t &flags)
{
    bool sa, sb;
    const bool an = is_nan_enc<FMT>(a, sa), bn = is_nan_enc<FMT>(b, sb);
    flags = ((an && sa) || (bn && sb)) ? F_INVALID : 0u;
    if (an || bn) {
        if (!number || (an && bn)) enc_qnan<FMT>(out);
        else copy<FMT>(out, an ? b : a);
        return;
    }
    if (mag_zero<FMT>(a) && mag_zero<FMT>(b)) {
        const int za = sign_of<FMT>(a), zb = sign_of<FMT>(b);
        if (za == zb) copy<FMT>(out, a);
        else if (want_max) copy<FMT>(out, za ? b : a);
        else copy<FMT>(out, za ? a : b);
        return;
    }
    const bool lt = numeric_lt<FMT>(a, b);
    if (want_max) copy<FMT>(out, lt ? b : a);
    else copy<FMT>(out, lt ? a : b);
}

// quiet comparisons yielding 1.0 or +0.0 (softfloat.c:565-585)
template <int FMT>
SFD void compare(const uint32_t (&a)[Fmt<FMT>::W], const uint32_t (&b)[Fmt<FMT>::W], int op,
                 uint32_t (&out)[Fmt<FMT>::W], uint32_t &flags)
{
    bool sa, sb;
    const bool an = is_nan_enc<FMT>(a, sa), bn = is_nan_enc<FMT>(b, sb);
    flags = ((an && sa) || (bn && sb)) ? F_INVALID : 0u;
    if (an || bn) { enc_zero<FMT>(out, 0); return; }
    const bool lt = numeric_lt<FMT>(a, b), gt = numeric_lt<FMT>(b, a), eq = !lt && !gt;
    const bool truth = op == 12 ? lt : op == 13 ? (lt || eq) : eq;
    if (truth) enc_one<FMT>(out, 0);
    else enc_zero<FMT>(out, 0);
}

// the reciprocal seed table entry: nearest integer to 2^18/(1+(i+1/2)/2^9),
// ties to even (softfloat.c:620-633)
SFD uint32_t recip_entry(uint32_t i)
{
    const uint32_t num = 1u << 28, den = 1024u + (i << 1) + 1u;
    uint32_t q = num / den;
    const uint32_t r = num - q * den;
    if (2u * r > den || (2u * r == den && (q & 1u))) q++;
    return q;
}

// nearest integer to 2^17/sqrt(mid), decided by exact integer comparison
// (softfloat.c:638-658)
SFD uint32_t rsqrt_entry(uint32_t j)
{
    const uint32_t odd = j >> 9, i = j & 511u;
    const uint64_t m2 = (uint64_t)(1024u + (i << 1) + 1u) << odd;
    const uint64_t t = (1ull << 44) / m2;
    uint64_t q = 0;
    for (uint64_t bit = 1ull << 17; bit; bit >>= 1)
        if ((q | bit) * (q | bit) <= t) q |= bit;
    while ((q + 1) * (q + 1) * m2 <= (1ull << 44)) q++;
    if ((2 * q + 1) * (2 * q + 1) * m2 < (1ull << 46)) q++;
    return (uint32_t)q;
}

template <int FMT>
SFD uint32_t frac_top9(const uint32_t (&x)[Fmt<FMT>::W])
{
    constexpr int lo = Fmt<FMT>::MANW - 9;
    const uint32_t w0 = x[lo >> 5], w1 = ((lo >> 5) + 1 < Fmt<FMT>::W) ? x[(lo >> 5) + 1] : 0u;
    const uint32_t v = (lo & 31) ? __funnelshift_r(w0, w1, lo & 31) : w0;
    return v & 511u;
}

template <int FMT>
SFD void seed_pack(int sign, uint32_t r, int e, uint32_t (&out)[Fmt<FMT>::W])
{
    uint32_t m[Fmt<FMT>::W];
    sfw::zero(m);
    m[0] = r;
    uint32_t fl;
    round_pack<FMT, Fmt<FMT>::W>(sign, m, e, RNE, out, fl);
}

template <int FMT>
SFD void recip_seed(const uint32_t (&x)[Fmt<FMT>::W], uint32_t (&out)[Fmt<FMT>::W])
{
    using F = Fmt<FMT>;
    const int sign = sign_of<FMT>(x);
    const uint32_t ef = exp_field<FMT>(x);
    if (ef == exp_mask<FMT>()) {
        bool s;
        if (is_nan_enc<FMT>(x, s)) enc_qnan<FMT>(out);    // NaN, quietly
        else enc_zero<FMT>(out, sign);                      // +-inf -> +-0
        return;
    }
    if (ef == 0u) { enc_inf<FMT>(out, sign); return; }
    const int E = (int)ef - F::BIAS, e_out = -E - 18;
    if (e_out + 17 > F::EMAX) { enc_inf<FMT>(out, sign); return; }
    seed_pack<FMT>(sign, recip_entry(frac_top9<FMT>(x)), e_out, out);
}

template <int FMT>
SFD void rsqrt_seed(const uint32_t (&x)[Fmt<FMT>::W], uint32_t (&out)[Fmt<FMT>::W])
{
    using F = Fmt<FMT>;
    const int sign = sign_of<FMT>(x);
    const uint32_t ef = exp_field<FMT>(x);
    bool s;
    if (is_nan_enc<FMT>(x, s)) { enc_qnan<FMT>(out); return; }
    if (ef == 0u) { enc_inf<FMT>(out, sign); return; }
    if (sign) { enc_qnan<FMT>(out); return; }
    if (ef == exp_mask<FMT>()) { enc_zero<FMT>(out, 0); return; }
    const int E = (int)ef - F::BIAS, odd = E & 1;
    const int e_out = -((E - odd) / 2) - 17;
    seed_pack<FMT>(0, rsqrt_entry(((uint32_t)odd << 9) | frac_top9<FMT>(x)), e_out, out);
}

// Every opcode that is not FMA/ADD/SUB/MUL; the unassigned ones (15, 32 and
// up) answer with the canonical quiet NaN and invalid (softfloat.c:939-1009).
template <int FMT>
SFD void simple(int op, const uint32_t (&a)[Fmt<FMT>::W], const uint32_t (&b)[Fmt<FMT>::W],
                const uint32_t (&c)[Fmt<FMT>::W], uint32_t (&out)[Fmt<FMT>::W], uint32_t &flags)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W;
    flags = 0u;
    switch (op) {
    case 4:                                           // ABS
        copy<FMT>(out, a);
        out[W - 1] &= 0x7FFFFFFFu;
        return;
    case 5:                                           // NEG
        copy<FMT>(out, a);
        out[W - 1] ^= 0x80000000u;
        return;
    case 6:                                           // COPYSIGN
        copy<FMT>(out, a);
        out[W - 1] = (out[W - 1] & 0x7FFFFFFFu) | (b[W - 1] & 0x80000000u);
        return;
    case 7:  minmax<FMT>(a, b, false, false, out, flags); return;
    case 8:  minmax<FMT>(a, b, true, false, out, flags); return;
    case 9:  minmax<FMT>(a, b, false, true, out, flags); return;
    case 10: minmax<FMT>(a, b, true, true, out, flags); return;
    case 11:                                          // SELECT: c != 0 ? a : b
        copy<FMT>(out, mag_zero<FMT>(c) ? b : a);
        return;
    case 12: case 13: case 14:
        compare<FMT>(a, b, op, out, flags);
        return;
    case 16:
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = a[i] & b[i];
        return;
    case 17:
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = a[i] | b[i];
        return;
    case 18:
#pragma unroll
        for (int i = 0; i < W; i++) out[i] = a[i] ^ b[i];
        return;
    case 19:                                          // IADD, wraps
        sfw::add(out, a, b);
        return;
    case 20:                                          // ISUB, wraps
        sfw::sub(out, a, b);
        return;
    case 21: {                                        // ISHL, count mod width
        copy<FMT>(out, a);
        sfw::shl(out, (int)(b[0] & (uint32_t)(32 * W - 1)));
        return;
    }
    case 22:                                          // ISHR, logical
        copy<FMT>(out, a);
        sfw::shr(out, (int)(b[0] & (uint32_t)(32 * W - 1)));
        return;
    case 23:                                          // ICMPLT, unsigned
        if (sfw::cmp(a, b) < 0) enc_one<FMT>(out, 0);
        else enc_zero<FMT>(out, 0);
        return;
    case 30:                                          // IMUL: low 32 of low 32s
        sfw::zero(out);
        out[0] = a[0] * b[0];
        return;
    case 26:
        recip_seed<FMT>(a, out);
        return;
    case 27:
        rsqrt_seed<FMT>(a, out);
        return;
    default:
        enc_qnan<FMT>(out);
        flags = F_INVALID;
        return;
    }
}

}  // namespace sf
