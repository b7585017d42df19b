// elem_hw.cu - binary32 FMA/ADD/SUB/MUL under RNE, RTZ, RDN and RUP on the
// GPU's own correctly rounded floating-point units, for every element whose
// value and flags the hardware is known to give exactly as the reference's
// softfloat does; every other element goes through the integer path
// (softfloat.cuh) in the same launch.
//
// Which elements, and why their bits and flags are the reference's
// (host/src/softfloat.c:120-468 defines both):
//  * Operands are finite (no NaN, no infinity; zeros and subnormals are
//    fine: the hardware keeps subnormals, nothing here flushes them).
//  * The hardware result r, rounded in the element's direction, is a normal
//    number of biased exponent >= 2 (so |r| >= 2^(emin+1)) and is not the
//    largest finite magnitude.
// IEEE 754 fixes r for every direction, so it is the reference's value.
// Flags: with finite operands INVALID and DIVZERO cannot arise; OVERFLOW
// gives an infinity or the largest finite magnitude (excluded); a tiny
// result (below 2^emin before rounding to the format's precision) rounds
// to at most 2^emin (excluded), so UNDERFLOW cannot arise either. INEXACT
// remains: the exact value is representable iff rounding it down and
// rounding it up give the same number, so INEXACT = (RD(x) != RU(x)) - two
// more hardware operations (one, RD or RU, is r itself under RDN/RUP; RTZ
// is RD for a positive and RU for a negative result).
// Elements with a NaN or an infinity take the reference's special cases
// straight from their encodings (hw_special), in the same pass.
//
// The launch works in tiles of T*K elements a block. Each thread loads its
// K elements and finishes those the two rules above cover; the others
// (zero, subnormal and overflowing results) go to a shared-memory queue,
// which the block's threads work through densely after a block barrier, so
// a few such elements do not hold a warp of 32 on the integer path. Under
// RMM (no hardware direction for it) the integer kernels take the launch.
//
// Binary64 is left to the integer kernels: the same scheme on the FP64
// units (three fused operations an element under RNE) measured 10-30 %
// slower than the integer path on a GB300 (binary64 FMA 58.9 against 65.4
// Gelem/s, ADD 64.0 against 80.2, MUL 60.9 against 87.4 at n = 2^24),
// whose FP64 rate is a small fraction of its integer rate.
#include <cstdlib>
#include <cstring>

#include "cftg_internal.h"
#include "elem_io.cuh"

namespace cftg {

namespace {

template <int FMT> struct HwT;
template <> struct HwT<0> {
    using F = float;
    static constexpr int W = 1, EXPW = 8, EXP_SHIFT = 23;
    static constexpr uint64_t MAG_MAX = 0x7F7FFFFFull;
};
template <> struct HwT<1> {
    using F = double;
    static constexpr int W = 2, EXPW = 11, EXP_SHIFT = 52;
    static constexpr uint64_t MAG_MAX = 0x7FEFFFFFFFFFFFFFull;
};

template <int FMT>
SFD uint64_t bits_of(const uint32_t (&x)[HwT<FMT>::W])
{
    if constexpr (FMT == 0) return x[0];
    else return ((uint64_t)x[1] << 32) | x[0];
}

template <int FMT>
SFD typename HwT<FMT>::F value_of(uint64_t u)
{
    if constexpr (FMT == 0) return __uint_as_float((uint32_t)u);
    else return __longlong_as_double((long long)u);
}

template <int FMT>
SFD uint64_t bits_from(typename HwT<FMT>::F v)
{
    if constexpr (FMT == 0) return __float_as_uint(v);
    else return (uint64_t)__double_as_longlong(v);
}

template <int FMT>
SFD uint32_t exp_of(uint64_t u)
{
    return (uint32_t)(u >> HwT<FMT>::EXP_SHIFT) & ((1u << HwT<FMT>::EXPW) - 1u);
}

// The operation in one direction (ADD/SUB read a and c, MUL a and b).
template <int FMT, int KIND, int DIR>
SFD typename HwT<FMT>::F hw_op(typename HwT<FMT>::F a, typename HwT<FMT>::F b,
                               typename HwT<FMT>::F c)
{
    if constexpr (FMT == 0) {
        if constexpr (KIND == K_FMA) {
            if constexpr (DIR == sf::RNE) return __fmaf_rn(a, b, c);
            else if constexpr (DIR == sf::RTZ) return __fmaf_rz(a, b, c);
            else if constexpr (DIR == sf::RDN) return __fmaf_rd(a, b, c);
            else return __fmaf_ru(a, b, c);
        } else if constexpr (KIND == K_ADD) {
            if constexpr (DIR == sf::RNE) return __fadd_rn(a, c);
            else if constexpr (DIR == sf::RTZ) return __fadd_rz(a, c);
            else if constexpr (DIR == sf::RDN) return __fadd_rd(a, c);
            else return __fadd_ru(a, c);
        } else if constexpr (KIND == K_SUB) {
            if constexpr (DIR == sf::RNE) return __fsub_rn(a, c);
            else if constexpr (DIR == sf::RTZ) return __fsub_rz(a, c);
            else if constexpr (DIR == sf::RDN) return __fsub_rd(a, c);
            else return __fsub_ru(a, c);
        } else {
            if constexpr (DIR == sf::RNE) return __fmul_rn(a, b);
            else if constexpr (DIR == sf::RTZ) return __fmul_rz(a, b);
            else if constexpr (DIR == sf::RDN) return __fmul_rd(a, b);
            else return __fmul_ru(a, b);
        }
    } else {
        if constexpr (KIND == K_FMA) {
            if constexpr (DIR == sf::RNE) return __fma_rn(a, b, c);
            else if constexpr (DIR == sf::RTZ) return __fma_rz(a, b, c);
            else if constexpr (DIR == sf::RDN) return __fma_rd(a, b, c);
            else return __fma_ru(a, b, c);
        } else if constexpr (KIND == K_ADD) {
            if constexpr (DIR == sf::RNE) return __dadd_rn(a, c);
            else if constexpr (DIR == sf::RTZ) return __dadd_rz(a, c);
            else if constexpr (DIR == sf::RDN) return __dadd_rd(a, c);
            else return __dadd_ru(a, c);
        } else if constexpr (KIND == K_SUB) {
            if constexpr (DIR == sf::RNE) return __dsub_rn(a, c);
            else if constexpr (DIR == sf::RTZ) return __dsub_rz(a, c);
            else if constexpr (DIR == sf::RDN) return __dsub_rd(a, c);
            else return __dsub_ru(a, c);
        } else {
            if constexpr (DIR == sf::RNE) return __dmul_rn(a, b);
            else if constexpr (DIR == sf::RTZ) return __dmul_rz(a, b);
            else if constexpr (DIR == sf::RDN) return __dmul_rd(a, b);
            else return __dmul_ru(a, b);
        }
    }
}

// One element on the hardware: true and (o, fl) when it qualifies; false
// with `special` set when an operand is a NaN or an infinity.
template <int FMT, int KIND, int RND>
SFD bool hw_elem(const uint32_t (&a)[HwT<FMT>::W], const uint32_t (&b)[HwT<FMT>::W],
                 const uint32_t (&c)[HwT<FMT>::W], uint32_t (&o)[HwT<FMT>::W], uint32_t &fl,
                 bool &special)
{
    using H = HwT<FMT>;
    constexpr uint32_t EMASK = (1u << H::EXPW) - 1u;
    const uint64_t ua = bits_of<FMT>(a), ub = bits_of<FMT>(b), uc = bits_of<FMT>(c);
    bool fin = exp_of<FMT>(ua) != EMASK;
    if constexpr (KIND == K_FMA || KIND == K_MUL) fin = fin && exp_of<FMT>(ub) != EMASK;
    if constexpr (KIND != K_MUL) fin = fin && exp_of<FMT>(uc) != EMASK;
    special = !fin;
    const typename H::F fa = value_of<FMT>(ua), fb = value_of<FMT>(ub), fc = value_of<FMT>(uc);
    const typename H::F lo = hw_op<FMT, KIND, sf::RDN>(fa, fb, fc);
    const typename H::F hi = hw_op<FMT, KIND, sf::RUP>(fa, fb, fc);
    typename H::F r;
    if constexpr (RND == sf::RNE) r = hw_op<FMT, KIND, sf::RNE>(fa, fb, fc);
    else if constexpr (RND == sf::RDN) r = lo;
    else if constexpr (RND == sf::RUP) r = hi;
    else r = lo > (typename H::F)0 ? lo : hi;       // RTZ: toward zero (the result is not 0)
    const uint64_t ur = bits_from<FMT>(r);
    const uint32_t er = exp_of<FMT>(ur);
    const uint64_t mag = ur & (H::MAG_MAX | (H::MAG_MAX + 1u));   // sign cleared
    const bool ok = fin && er >= 2u && er != EMASK && mag != H::MAG_MAX;
    fl = lo != hi ? sf::F_INEXACT : 0u;
    if constexpr (FMT == 0) {
        o[0] = (uint32_t)ur;
    } else {
        o[0] = (uint32_t)ur;
        o[1] = (uint32_t)(ur >> 32);
    }
    return ok;
}

// The result of an element with a NaN or an infinity among its operands,
// from the encodings alone: the reference's special cases in its order
// (host/src/softfloat.c:335-373), with ADD/SUB steered to a*1 + (+-c) and
// MUL to a*b + (+-0).
template <int FMT, int KIND>
SFD void hw_special(const uint32_t (&a)[HwT<FMT>::W], const uint32_t (&b)[HwT<FMT>::W],
                    const uint32_t (&c)[HwT<FMT>::W], uint32_t (&o)[HwT<FMT>::W], uint32_t &fl)
{
    using H = HwT<FMT>;
    constexpr uint32_t EMASK = (1u << H::EXPW) - 1u;
    constexpr uint64_t FRAC = (1ull << H::EXP_SHIFT) - 1u;
    constexpr uint64_t QUIET = 1ull << (H::EXP_SHIFT - 1);
    constexpr uint64_t ONE = (uint64_t)((1u << (H::EXPW - 1)) - 1u) << H::EXP_SHIFT;
    constexpr int SB = 32 * H::W - 1;
    const uint64_t ua = bits_of<FMT>(a);
    const uint64_t ub = (KIND == K_ADD || KIND == K_SUB) ? ONE : bits_of<FMT>(b);
    uint64_t uc = KIND == K_MUL ? ((ua ^ ub) & (1ull << SB)) : bits_of<FMT>(c);
    if constexpr (KIND == K_SUB) uc ^= 1ull << SB;
    auto nan = [](uint64_t u) { return exp_of<FMT>(u) == EMASK && (u & FRAC) != 0u; };
    auto inf = [](uint64_t u) { return exp_of<FMT>(u) == EMASK && (u & FRAC) == 0u; };
    auto snan = [&](uint64_t u) { return nan(u) && !(u & QUIET); };
    auto zero = [](uint64_t u) { return (u & ~(1ull << SB)) == 0u; };
    const uint64_t qnan = ((uint64_t)EMASK << H::EXP_SHIFT) | QUIET;
    const uint64_t sp = (ua ^ ub) & (1ull << SB);
    uint64_t r;
    fl = 0u;
    if (nan(ua) || nan(ub) || nan(uc)) {
        r = qnan;
        fl = (snan(ua) || snan(ub) || snan(uc)) ? sf::F_INVALID : 0u;
    } else if (inf(ua) || inf(ub)) {
        if (zero(ua) || zero(ub) || (inf(uc) && (uc & (1ull << SB)) != sp)) {
            r = qnan;                                  // inf * 0, inf - inf
            fl = sf::F_INVALID;
        } else {
            r = sp | ((uint64_t)EMASK << H::EXP_SHIFT);
        }
    } else {
        r = uc;                                        // c is the infinity
    }
    o[0] = (uint32_t)r;
    if constexpr (H::W == 2) o[1] = (uint32_t)(r >> 32);
}

// The integer path for one queued element (one copy of its code a kernel).
template <int FMT, int KIND>
__device__ __noinline__ uint32_t slow_elem(const ElemLaunch &L, size_t i)
{
    constexpr int W = sf::Fmt<FMT>::W;
    uint32_t a[W], b[W], c[W], o[W], fl = 0u;
    fetch<W>(L.a, L.scalar_mask & 1u, L.ia, i, a);
    if constexpr (KIND == K_FMA || KIND == K_MUL) fetch<W>(L.b, L.scalar_mask & 2u, L.ib, i, b);
    else sfw::zero(b);
    if constexpr (KIND != K_MUL) fetch<W>(L.c, L.scalar_mask & 4u, L.ic, i, c);
    else sfw::zero(c);
    compute_elem<FMT, KIND>(L.op, L.rnd, a, b, c, o, fl);
    store_elem<W>(static_cast<uint32_t *>(L.d), i, o);
    if (L.lane_flags) L.lane_flags[i] = (uint8_t)fl;
    return fl;
}

constexpr int HW_T = 256;

template <int FMT> struct HwTile { static constexpr int K = FMT == 0 ? 8 : 4; };

template <int FMT, int KIND, int RND>
__global__ void __launch_bounds__(HW_T) k_elem_hw(const __grid_constant__ ElemLaunch L)
{
    constexpr int W = sf::Fmt<FMT>::W;
    constexpr int K = HwTile<FMT>::K;
    constexpr int CAP = HW_T * K;
    // the elements the integer path takes, as offsets in the tile
    __shared__ uint32_t q[CAP];
    __shared__ int nq;
    const int tid = threadIdx.x, lane = tid & 31;
    const unsigned lt = (1u << lane) - 1u;
    uint32_t acc = 0u;
    const size_t tiles = (L.n + CAP - 1) / CAP;
    for (size_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        if (tid == 0) nq = 0;
        __syncthreads();
        const size_t base = tile * CAP;
        uint32_t a[K][W], b[K][W], c[K][W];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const size_t i = base + (size_t)k * HW_T + tid;
            if (i < L.n) {
                fetch<W>(L.a, L.scalar_mask & 1u, L.ia, i, a[k]);
                if constexpr (KIND == K_FMA || KIND == K_MUL)
                    fetch<W>(L.b, L.scalar_mask & 2u, L.ib, i, b[k]);
                else sfw::zero(b[k]);
                if constexpr (KIND != K_MUL) fetch<W>(L.c, L.scalar_mask & 4u, L.ic, i, c[k]);
                else sfw::zero(c[k]);
            } else {
                sfw::zero(a[k]);
                sfw::zero(b[k]);
                sfw::zero(c[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint32_t off = (uint32_t)(k * HW_T + tid);
            const size_t i = base + off;
            uint32_t o[W], fl;
            bool special;
            bool ok = hw_elem<FMT, KIND, RND>(a[k], b[k], c[k], o, fl, special);
            if (special) {
                hw_special<FMT, KIND>(a[k], b[k], c[k], o, fl);
                ok = true;
            }
            const bool in = i < L.n;
            if (in && ok) {
                store_elem<W>(static_cast<uint32_t *>(L.d), i, o);
                if (L.lane_flags) L.lane_flags[i] = (uint8_t)fl;
                acc |= fl;
            }
            const bool qg = in && !ok;
            const unsigned mg = __ballot_sync(0xFFFFFFFFu, qg);
            if (mg) {
                int at = 0;
                if (lane == 0) at = atomicAdd(&nq, __popc(mg));
                at = __shfl_sync(0xFFFFFFFFu, at, 0);
                if (qg) q[at + __popc(mg & lt)] = off;
            }
        }
        __syncthreads();
        const int ng = nq;
        for (int j = tid; j < ng; j += HW_T) acc |= slow_elem<FMT, KIND>(L, base + q[j]);
        __syncthreads();                              // the queue is rebuilt next tile
    }
    acc = __reduce_or_sync(0xFFFFFFFFu, acc);
    if (lane == 0 && acc) atomicOr(L.flags, acc);
}

template <int FMT, int KIND, int RND>
cudaError_t go_hw(const ElemLaunch &L, cudaStream_t s)
{
    constexpr int CAP = HW_T * HwTile<FMT>::K;
    const size_t want = (L.n + CAP - 1) / CAP;
    const size_t cap = (size_t)sm_count() * (L.blocks_per_sm ? L.blocks_per_sm : 8u);
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    k_elem_hw<FMT, KIND, RND><<<blocks ? blocks : 1, HW_T, 0, s>>>(L);
    return cudaGetLastError();
}

template <int FMT, int KIND>
cudaError_t go_hw_rnd(const ElemLaunch &L, cudaStream_t s)
{
    switch (L.rnd) {
    case sf::RNE: return go_hw<FMT, KIND, sf::RNE>(L, s);
    case sf::RTZ: return go_hw<FMT, KIND, sf::RTZ>(L, s);
    case sf::RDN: return go_hw<FMT, KIND, sf::RDN>(L, s);
    default: return go_hw<FMT, KIND, sf::RUP>(L, s);
    }
}

template <int FMT>
cudaError_t go_hw_kind(const ElemLaunch &L, cudaStream_t s)
{
    switch (L.kind) {
    case K_FMA: return go_hw_rnd<FMT, K_FMA>(L, s);
    case K_ADD: return go_hw_rnd<FMT, K_ADD>(L, s);
    case K_SUB: return go_hw_rnd<FMT, K_SUB>(L, s);
    default: return go_hw_rnd<FMT, K_MUL>(L, s);
    }
}

}  // namespace

// CFTG_ELEM_HW=0 sends binary32/64 arithmetic to the integer kernels (for
// comparisons); read at every launch.
bool launch_elem_hw(const ElemLaunch &L, cudaStream_t s, cudaError_t *err)
{
    if (L.fmt != 0 || L.kind > K_MUL || L.rnd < sf::RNE || L.rnd > sf::RUP) return false;
    const char *e = getenv("CFTG_ELEM_HW");
    if (e && strcmp(e, "0") == 0) return false;
    *err = go_hw_kind<0>(L, s);
    return true;
}

}  // namespace cftg
