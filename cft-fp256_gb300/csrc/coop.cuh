// coop.cuh - one binary128/256 FMA/ADD/SUB/MUL spread over a group of W
// threads (W = the element's 32-bit words), for a trajectory lane whose
// every operation waits on the one before it.
//
// One thread computing an operation runs it as one long dependent chain
// (a 2W-word product, alignment, sum, normalisation and rounding, each a
// carry chain or a select network over the 2W-word window). Here thread j
// of the group owns window words 2j and 2j+1 and the chains become short
// per-thread steps joined by group votes:
//
//  * product: thread j sums the 64-bit partial products of columns 2j and
//    2j+1 (the factor b placed in the group's shared scratch, read at an
//    offset), the parts above its two words go to thread j+1 by one
//    shuffle, and the last one-bit carries ripple by carry lookahead on the
//    group's ballot (generate: this thread's add carried out; propagate:
//    its two words are all ones);
//  * alignment: the shifted term is written to shared memory and every
//    thread reads its two words back at the shift's word offset; the jam is
//    a vote on the bits shifted out;
//  * sum, negation, rounding increment: two-word adds with the lookahead;
//  * normalisation and rounding: the leading bit from the ballot of non-zero
//    pairs, then each thread takes its word of the kept significand from
//    shared memory at the leading bit's offset; guard is one shared read,
//    sticky a vote.
//
// The bits are those of sf::arith (the same exact sum, rounded once by the
// same rules). The group computes the usual case - a and b normal, c normal
// or zero, a normal result - and answers false, with nothing written, for
// everything else (special operands, subnormal or tiny results, overflow),
// which the caller then computes with the one-thread code.
#pragma once
#include "softfloat.cuh"

namespace coop {

using sf::Fmt;

// The group: W consecutive lanes of the warp starting at a multiple of W.
// Every lane of the warp runs the group code together, whether or not its
// group has an operation (the votes and shuffles below take the whole warp,
// so the warp's groups stay converged and issue each instruction once).
struct Group {
    int base;           // the group's first lane
    int j;              // this thread's index in the group
};

template <int W>
SFD Group group_of(int lane)
{
    Group g;
    g.base = lane & ~(W - 1);
    g.j = lane & (W - 1);
    return g;
}

// Words of the group's shared scratch for format words W: a window buffer
// of 3N words (N = 2W; [0, N) and [2N, 3N) stay zero, data in [N, 2N)) and
// the placed factor b in 3W words ([0, W) and [2W, 3W) stay zero).
template <int W>
__host__ __device__ constexpr int scratch_words() { return 6 * W + 3 * W; }

// Zero the scratch of every group of a warp (words [0, count)), once.
SFD void zero_scratch(uint32_t *sb, int count, int lane)
{
    for (int i = lane; i < count; i += 32) sb[i] = 0u;
}

// The warp's vote, the group's W bits of it (bit j: thread j).
template <int W>
SFD unsigned gballot(const Group &g, bool pred)
{
    return (__ballot_sync(0xFFFFFFFFu, pred) >> g.base) & ((W == 32) ? 0xFFFFFFFFu : ((1u << W) - 1u));
}

// Carry lookahead over the group: thread j's add generated a carry (gen)
// or its words are all ones (prop); cin0 enters thread 0. Returns the carry
// into this thread; cout the carry out of the top thread. The carries of
// A + B with A = G|P and B = G follow c(j+1) = G(j) | P(j) & c(j).
template <int W>
SFD uint32_t lookahead(const Group &g, bool gen, bool prop, uint32_t cin0, uint32_t &cout)
{
    const unsigned G = gballot<W>(g, gen), P = gballot<W>(g, prop);
    const unsigned A = G | P;
    const unsigned S = A + G + cin0;
    const unsigned C = S ^ A ^ G;                  // bit j: the carry into thread j
    cout = (C >> W) & 1u;
    return (C >> g.j) & 1u;
}

// (r1:r0) = (x1:x0) + (y1:y0) + cin; returns the carry out.
SFD uint32_t add2(uint32_t &r0, uint32_t &r1, uint32_t x0, uint32_t x1, uint32_t y0, uint32_t y1,
                  uint32_t cin)
{
    uint32_t c;
    [[maybe_unused]] uint32_t scratch;
    asm("add.cc.u32 %3, %7, -1;\n\taddc.cc.u32 %0, %4, %5;\n\taddc.cc.u32 %1, %6, %8;\n\t"
        "addc.u32 %2, 0, 0;"
        : "=&r"(r0), "=r"(r1), "=r"(c), "=&r"(scratch)
        : "r"(x0), "r"(y0), "r"(x1), "r"(cin), "r"(y1));
    return c;
}

// The group's FMA/ADD/SUB/MUL of x, y, z (every thread holds all W words of
// each, already steered by the caller's NEG folding). Called by every lane
// of the warp at once (a group without an operation passes any operands and
// ignores the answer). Returns whether the group took the element: then res
// is word j of the result and flags the operation's flags (the same in
// every thread of the group); otherwise the caller computes the element
// with the one-thread code. Shared-memory offsets stay inside the scratch
// whatever the operands.
template <int FMT>
SFD bool arith_group(const Group &g, int op, const uint32_t (&x)[Fmt<FMT>::W],
                     const uint32_t (&y)[Fmt<FMT>::W], const uint32_t (&z)[Fmt<FMT>::W], int rnd,
                     uint32_t *sb, uint32_t &res, uint32_t &flags)
{
    using F = Fmt<FMT>;
    constexpr int W = F::W, N = 2 * W, P = F::P;
    constexpr int ES = sf::exp_shift<FMT>();
    constexpr uint32_t EM = sf::exp_mask<FMT>();
    const int j = g.j;
    uint32_t *const sh = sb;                  // window buffer, 3N words
    uint32_t *const bb = sb + 3 * N;          // placed b, 3W words

    // ---- steering (host/src/softfloat.c:438-468, as sf::arith_rt)
    const bool addsub = op == sf::OP_ADD || op == sf::OP_SUB;
    uint32_t b[W], c[W];
#pragma unroll
    for (int i = 0; i < W; i++) {
        b[i] = addsub ? 0u : y[i];
        c[i] = op == sf::OP_MUL ? 0u : z[i];
    }
    if (addsub) b[W - 1] = (uint32_t)F::BIAS << ES;                       // +1
    if (op == sf::OP_SUB) c[W - 1] ^= 0x80000000u;
    if (op == sf::OP_MUL) c[W - 1] = (x[W - 1] ^ y[W - 1]) & 0x80000000u;

    // ---- the usual operands only (the others are unpacked as if normal,
    // computed through and refused at the end)
    uint32_t cm = c[W - 1] & 0x7FFFFFFFu;
#pragma unroll
    for (int i = 0; i < W - 1; i++) cm |= c[i];
    const bool cz = cm == 0u;
    const uint32_t ea = sf::exp_field<FMT>(x), eb = sf::exp_field<FMT>(b), ec = sf::exp_field<FMT>(c);
    bool ok = (ea - 1u) < EM - 1u && (eb - 1u) < EM - 1u && ((ec - 1u) < EM - 1u || cz);
    sf::Unp<FMT> ua, ub, uc;
    sf::unpack_normal<FMT, 32 * W - 2>(x, ua);
    sf::unpack_normal<FMT, 32 * W - 1>(b, ub);
    sf::unpack_normal<FMT, 32 * W - 2>(c, uc);
    const int sp = ua.sign ^ ub.sign, sc = uc.sign;

    // ---- product, columns 2j and 2j+1
#pragma unroll
    for (int i = 0; i < W; i++) bb[W + i] = ub.m[i];
    __syncwarp();
    uint64_t s0 = 0, s1 = 0, s2 = 0;
#pragma unroll
    for (int i = 0; i < W; i++) {
        const uint32_t b0 = bb[W + 2 * j - i], b1 = bb[W + 2 * j + 1 - i];   // zero outside b
        const uint64_t p0 = (uint64_t)ua.m[i] * b0, p1 = (uint64_t)ua.m[i] * b1;
        s0 += (uint32_t)p0;
        s1 += (p0 >> 32) + (uint32_t)p1;
        s2 += p1 >> 32;
    }
    // this thread's sum V = s0 + s1 2^32 + s2 2^64 in four words
    const uint64_t t1 = (s0 >> 32) + s1;
    const uint64_t t2 = s2 + (t1 >> 32);
    const uint32_t v0 = (uint32_t)s0, v1 = (uint32_t)t1, v2 = (uint32_t)t2, v3 = (uint32_t)(t2 >> 32);
    // words 2j+2 and 2j+3 belong to thread j+1
    uint32_t h2 = __shfl_up_sync(0xFFFFFFFFu, v2, 1), h3 = __shfl_up_sync(0xFFFFFFFFu, v3, 1);
    if (j == 0) h2 = h3 = 0u;
    uint32_t p0w, p1w;
    const uint32_t cg = add2(p0w, p1w, v0, v1, h2, h3, 0u);
    uint32_t top;
    uint32_t ci = lookahead<W>(g, cg != 0u, (p0w & p1w) == 0xFFFFFFFFu, 0u, top);
    add2(p0w, p1w, p0w, p1w, ci, 0u, 0u);
    int ew = ua.ve + ub.ve - (64 * W - 3);               // weight of window bit 0

    // ---- the addend's window words 2j, 2j+1 (its significand in the top half)
    uint32_t c0w = 0u, c1w = 0u;
#pragma unroll
    for (int i = 0; i < W; i++) {
        c0w = (2 * j == W + i) ? uc.m[i] : c0w;
        c1w = (2 * j + 1 == W + i) ? uc.m[i] : c1w;
    }
    if (cz) c0w = c1w = 0u;

    // ---- alignment: X (the smaller exponent) shifted right with a jam
    const int delta = cz ? -(1 << 28) : uc.ve - (ew + 64 * W - 2);
    const bool pbig = delta <= 0;
    const uint32_t x0 = pbig ? c0w : p0w, x1 = pbig ? c1w : p1w;
    const uint32_t y0 = pbig ? p0w : c0w, y1 = pbig ? p1w : c1w;
    int s = pbig ? -delta : delta;
    s = s < 32 * N - 1 ? s : 32 * N - 1;                 // X's top bit is clear
    const int ws = s >> 5, bs = s & 31;
    sh[N + 2 * j] = x0;
    sh[N + 2 * j + 1] = x1;
    __syncwarp();
    const uint32_t r0 = sh[N + 2 * j + ws], r1 = sh[N + 2 * j + 1 + ws], r2 = sh[N + 2 * j + 2 + ws];
    uint32_t xs0 = __funnelshift_r(r0, r1, bs), xs1 = __funnelshift_r(r1, r2, bs);
    const uint32_t lowm = (1u << bs) - 1u;
    const uint32_t out0 = 2 * j < ws ? x0 : (2 * j == ws ? (x0 & lowm) : 0u);
    const uint32_t out1 = 2 * j + 1 < ws ? x1 : (2 * j + 1 == ws ? (x1 & lowm) : 0u);
    const bool jam = gballot<W>(g, (out0 | out1) != 0u) != 0u;
    if (j == 0 && jam) xs0 |= 1u;
    if (!pbig) ew += delta;
    __syncwarp();                                        // the reads of sh are done

    // ---- Y + X, or Y - X in two's complement, then the magnitude
    const bool sub = sp != sc;
    const uint32_t mk = sub ? 0xFFFFFFFFu : 0u;
    uint32_t m0, m1;
    const uint32_t ca = add2(m0, m1, y0, y1, xs0 ^ mk, xs1 ^ mk, 0u);
    uint32_t cy;
    ci = lookahead<W>(g, ca != 0u, (m0 & m1) == 0xFFFFFFFFu, sub ? 1u : 0u, cy);
    add2(m0, m1, m0, m1, ci, 0u, 0u);
    const bool neg = sub && !cy;                          // Y < X: the result is X - Y
    {
        // the negation, in every group where some group needs it
        const uint32_t nm = neg ? 0xFFFFFFFFu : 0u;
        if (__any_sync(0xFFFFFFFFu, neg)) {
            m0 ^= nm;
            m1 ^= nm;
            uint32_t dummy;
            ci = lookahead<W>(g, false, (m0 & m1) == 0xFFFFFFFFu, neg ? 1u : 0u, dummy);
            add2(m0, m1, m0, m1, ci, 0u, 0u);
        }
    }
    const int s_big = pbig ? sp : sc, s_small = pbig ? sc : sp;
    const int sign = neg ? s_small : s_big;

    // ---- the leading bit: the top non-zero pair's (nz == 0: an exact
    // cancellation, +0 or -0 under roundTowardNegative, no flag)
    const unsigned nz = gballot<W>(g, (m0 | m1) != 0u);
    const int h = nz ? 31 - __clz((int)nz) : 0;
    const int bl = m1 ? 64 - __clz(m1) : (m0 ? 32 - __clz(m0) : 0);
    const int L = 64 * h + __shfl_sync(0xFFFFFFFFu, bl, g.base + h);
    const int e_norm = ew + L - 1;
    ok = ok && (nz == 0u || e_norm >= F::EMIN);           // subnormal or tiny: one thread

    // ---- kept bits [L-P, L), guard L-P-1, sticky below, from the window
    sh[N + 2 * j] = m0;
    sh[N + 2 * j + 1] = m1;
    __syncwarp();
    const int lo = L - P;                                 // may be negative (deep cancellation)
    const int q = (lo + 32 * j) >> 5, rb = lo & 31;
    uint32_t kept = __funnelshift_r(sh[N + q], sh[N + q + 1], rb);
    const int gp = lo - 1;                                // the guard bit's index
    const bool guard = gp >= 0 && ((sh[N + (gp >> 5)] >> (gp & 31)) & 1u);
    // bits below the guard bit in this thread's two words
    auto below = [&](uint32_t v, int k) -> uint32_t {
        const int w0 = 32 * k;
        return w0 + 32 <= gp ? v : (w0 < gp ? (v & ((1u << (gp - w0)) - 1u)) : 0u);
    };
    const bool sticky = gballot<W>(g, (below(m0, 2 * j) | below(m1, 2 * j + 1)) != 0u) != 0u;
    __syncwarp();                                        // the reads of sh are done

    // ---- rounding (semantics: host/src/softfloat.c:120-261)
    const uint32_t lsb = __shfl_sync(0xFFFFFFFFu, kept, g.base) & 1u;
    const bool up = sf::round_up(rnd, sign, guard, sticky, lsb != 0u);
    const unsigned ones = gballot<W>(g, kept == 0xFFFFFFFFu);
    const int t = __ffs(~ones) - 1;                       // threads 0..t-1 are all ones
    if (up && j <= t) kept += 1u;
    int e_res = e_norm;
    constexpr int TOPB = P - 32 * (W - 1);                // kept's bit P in the top word
    const uint32_t kt = __shfl_sync(0xFFFFFFFFu, kept, g.base + W - 1);
    if ((kt >> TOPB) & 1u) {                              // rounded up to 2^P
        e_res += 1;
        kept = j == W - 1 ? 1u << (TOPB - 1) : 0u;
    }
    ok = ok && (nz == 0u || e_res <= F::EMAX);             // overflow: one thread
    if (nz == 0u) {
        res = j == W - 1 ? (rnd == sf::RDN ? 0x80000000u : 0u) : 0u;
        flags = 0u;
    } else {
        res = j == W - 1 ? ((kept & ((1u << ES) - 1u)) | ((uint32_t)sign << 31) |
                            ((uint32_t)(e_res + F::BIAS) << ES))
                         : kept;
        flags = (guard || sticky) ? sf::F_INEXACT : 0u;
    }
    return ok;
}

}  // namespace coop
