// elem_hw.cu - binary32 FMA/ADD/SUB/MUL under RNE, RTZ, RDN and RUP on the
// GPU's own correctly rounded floating-point units, for every element whose
// value and flags the hardware is known to give exactly as the reference's
// softfloat does; every other element goes through the integer path
// (softfloat.cuh) in the same launch.
//
// The hardware result r is rounded in the element's direction, so IEEE 754
// fixes it; the question is only which elements' value AND flags are the
// reference's (host/src/softfloat.c:120-468 defines both). With finite
// operands INVALID and DIVZERO cannot arise, and INEXACT is exact to
// compute: the exact value x is representable iff rounding it down and
// rounding it up agree, so INEXACT = (RD(x) != RU(x)) - two more hardware
// operations (under RDN/RUP one of them is r itself; RTZ is RD of a
// positive and RU of a negative result). Taken on the hardware:
//  * r normal with biased exponent >= 2 (|r| >= 2^(emin+1)) and not the
//    largest finite magnitude: no OVERFLOW (that gives an infinity or the
//    largest magnitude) and no UNDERFLOW (a tiny x rounds to at most
//    2^emin); the operands were finite, because a NaN or an infinity among
//    them gives a NaN or an infinity. Zeros and subnormals among the
//    operands are fine: the hardware keeps subnormals, nothing flushes them.
//  * an exact zero (RD(x) = RU(x) = 0): IEEE 754's signs of exact zero sums
//    and products are the reference's, and no flag;
//  * an infinite r from finite operands: an overflow rounded to the
//    infinity, as the reference rounds it, with OVERFLOW and INEXACT (a
//    largest-magnitude r may or may not be an overflow, so it is not taken);
//  * a NaN or an infinity among the operands: IEEE 754's NaN or infinity is
//    the reference's special case in value (the NaN made the canonical
//    quiet NaN), with INVALID worked out from the operands' encodings.
// What remains - subnormal and tiny results, and largest-magnitude ones -
// takes the integer path.
//
// The launch works in tiles of T*K elements a block. Each thread loads its
// K elements and finishes those the rules above cover; the others go to
// the block's shared-memory queue, which the block's threads run through
// the integer path densely only when it is nearly full (and once at the
// end), so the block keeps streaming in between and a few such elements do
// not hold a warp of 32 on the integer path. Under RMM (no hardware
// direction for it) the integer kernels take the launch.
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

constexpr uint32_t EXP32 = 0x7F800000u, MAG_MAX32 = 0x7F7FFFFFu, QNAN32 = 0x7FC00000u;
constexpr uint32_t SIGN32 = 0x80000000u;

// The operation in one direction (ADD/SUB read a and c, MUL a and b).
template <int KIND, int DIR>
SFD float hw_op(float a, float b, float c)
{
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
}

SFD bool nan32(uint32_t u) { return (u & ~SIGN32) > EXP32; }
SFD bool inf32(uint32_t u) { return (u & ~SIGN32) == EXP32; }
SFD bool snan32(uint32_t u) { return nan32(u) && !(u & (1u << 22)); }

// One element on the hardware: the encoding in o and the flags in fl, and
// whether the element is finished (false: it is for the integer path).
// Branch-free; the outcomes (see the rules above):
//  * a NaN result: the canonical quiet NaN; INVALID iff an operand the kind
//    reads is a signalling NaN, or no operand is a NaN (inf * 0, inf - inf);
//  * an infinite result: exact when an operand is infinite, else an
//    overflow (OVERFLOW, INEXACT);
//  * a normal result of biased exponent >= 2 that is not the largest
//    magnitude, or an exact zero: INEXACT = (RD(x) != RU(x)).
// IEEE 754's results for NaN and infinite operands are the reference's
// special cases (host/src/softfloat.c:335-373) in value, the NaN's
// encoding aside: inf * 0 and inf - inf give a NaN, an infinite product or
// addend gives the infinity of its sign, under the steering ADD/SUB =
// a*1 + (+-c) and MUL = a*b + (+-0).
template <int KIND, int RND>
SFD bool hw_elem(uint32_t a, uint32_t b, uint32_t c, uint32_t &o, uint32_t &fl)
{
    const float fa = __uint_as_float(a), fb = __uint_as_float(b), fc = __uint_as_float(c);
    const float lo = hw_op<KIND, sf::RDN>(fa, fb, fc);
    const float hi = hw_op<KIND, sf::RUP>(fa, fb, fc);
    float r;
    if constexpr (RND == sf::RNE) r = hw_op<KIND, sf::RNE>(fa, fb, fc);
    else if constexpr (RND == sf::RDN) r = lo;
    else if constexpr (RND == sf::RUP) r = hi;
    else r = lo > 0.0f ? lo : hi;                   // RTZ: toward zero
    const uint32_t u = __float_as_uint(r);
    const uint32_t e = u & EXP32, mag = u & ~SIGN32;
    const bool rb = KIND == K_FMA || KIND == K_MUL, rc = KIND != K_MUL;
    const bool any_nan = nan32(a) || (rb && nan32(b)) || (rc && nan32(c));
    const bool any_snan = snan32(a) || (rb && snan32(b)) || (rc && snan32(c));
    const bool any_inf = inf32(a) || (rb && inf32(b)) || (rc && inf32(c));
    const bool r_nan = mag > EXP32, r_inf = mag == EXP32;
    const uint32_t inexact = lo != hi ? sf::F_INEXACT : 0u;
    o = r_nan ? QNAN32 : u;
    fl = r_nan ? ((any_snan || !any_nan) ? sf::F_INVALID : 0u)
               : r_inf ? (any_inf ? 0u : sf::F_OVERFLOW | sf::F_INEXACT) : inexact;
    // an exact zero (RD and RU agree, so the exact value is 0): IEEE 754's
    // signs of an exact zero sum are the reference's (+0, or -0 under RDN,
    // when the signs differ; the common sign otherwise)
    return r_nan || r_inf || (e >= (2u << 23) && mag != MAG_MAX32) || (mag == 0u && lo == hi);
}

// The integer path for one queued element (one copy of its code a kernel).
template <int KIND>
__device__ __noinline__ uint32_t slow_elem(const ElemLaunch &L, size_t i)
{
    uint32_t a[1], b[1], c[1], o[1], fl = 0u;
    fetch<1>(L.a, L.scalar_mask & 1u, L.ia, i, a);
    if constexpr (KIND == K_FMA || KIND == K_MUL) fetch<1>(L.b, L.scalar_mask & 2u, L.ib, i, b);
    else b[0] = 0u;
    if constexpr (KIND != K_MUL) fetch<1>(L.c, L.scalar_mask & 4u, L.ic, i, c);
    else c[0] = 0u;
    compute_elem<0, KIND>(L.op, L.rnd, a, b, c, o, fl);
    static_cast<uint32_t *>(L.d)[i] = o[0];
    if (L.lane_flags) L.lane_flags[i] = (uint8_t)fl;
    return fl;
}

constexpr int HW_T = 256;
constexpr int HW_K = 8;                          // elements a thread a tile
constexpr int HW_TILE = HW_T * HW_K;
constexpr int HW_Q = 4096;                       // queued elements a block holds

// Entries are the block's element positions r = (its tile number) * HW_TILE
// + (offset in the tile); the block's tile t is the launch's tile
// blockIdx.x + t * gridDim.x.
template <int KIND>
SFD void hw_drain(const ElemLaunch &L, const uint32_t *q, int count, uint32_t &acc)
{
    for (int j = threadIdx.x; j < count; j += HW_T) {
        const uint32_t r = q[j];
        const size_t tile = blockIdx.x + (size_t)(r / HW_TILE) * gridDim.x;
        acc |= slow_elem<KIND>(L, tile * HW_TILE + r % HW_TILE);
    }
}

// PLAIN: every operand the kind reads is a device array read element by
// element (no scalar, no index table) - direct loads; otherwise fetch().
template <int KIND, int RND, bool PLAIN>
__global__ void __launch_bounds__(HW_T, 4) k_elem_hw(const __grid_constant__ ElemLaunch L)
{
    constexpr int K = HW_K;
    __shared__ uint32_t q[HW_Q];
    __shared__ int nq;
    const int tid = threadIdx.x, lane = tid & 31;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t *pa = static_cast<const uint32_t *>(L.a);
    const uint32_t *pb = static_cast<const uint32_t *>(L.b);
    const uint32_t *pc = static_cast<const uint32_t *>(L.c);
    uint32_t *pd = static_cast<uint32_t *>(L.d);
    uint8_t *plf = L.lane_flags;
    uint32_t acc = 0u;
    if (tid == 0) nq = 0;
    __syncthreads();
    const size_t tiles = (L.n + HW_TILE - 1) / HW_TILE;
    uint32_t mine = 0;                               // this block's tiles so far
    for (size_t tile = blockIdx.x; tile < tiles; tile += gridDim.x, mine++) {
        const size_t base = tile * HW_TILE;
        const uint32_t left = L.n - base < (size_t)HW_TILE ? (uint32_t)(L.n - base) : HW_TILE;
        uint32_t a[K], b[K], c[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint32_t off = (uint32_t)(k * HW_T + tid);
            const size_t i = base + off;
            a[k] = b[k] = c[k] = 0u;
            if (off < left) {
                if constexpr (PLAIN) {
                    a[k] = pa[i];
                    if constexpr (KIND == K_FMA || KIND == K_MUL) b[k] = pb[i];
                    if constexpr (KIND != K_MUL) c[k] = pc[i];
                } else {
                    uint32_t x[1];
                    fetch<1>(L.a, L.scalar_mask & 1u, L.ia, i, x);
                    a[k] = x[0];
                    if constexpr (KIND == K_FMA || KIND == K_MUL) {
                        fetch<1>(L.b, L.scalar_mask & 2u, L.ib, i, x);
                        b[k] = x[0];
                    }
                    if constexpr (KIND != K_MUL) {
                        fetch<1>(L.c, L.scalar_mask & 4u, L.ic, i, x);
                        c[k] = x[0];
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint32_t off = (uint32_t)(k * HW_T + tid);
            const size_t i = base + off;
            uint32_t o, fl;
            const bool ok = hw_elem<KIND, RND>(a[k], b[k], c[k], o, fl);
            const bool in = off < left;
            if (in && ok) {
                pd[i] = o;
                if (plf) plf[i] = (uint8_t)fl;
                acc |= fl;
            }
            const bool qg = in && !ok;
            const unsigned mg = __ballot_sync(0xFFFFFFFFu, qg);
            if (mg) {
                int at = 0;
                if (lane == 0) at = atomicAdd(&nq, __popc(mg));
                at = __shfl_sync(0xFFFFFFFFu, at, 0);
                if (qg) q[at + __popc(mg & lt)] = mine * HW_TILE + off;
            }
        }
        // the queue runs only when another tile might not fit in it: the
        // block's warps stay on the streaming path in between
        if (__syncthreads_or(tid == 0 && nq > HW_Q - HW_TILE)) {
            hw_drain<KIND>(L, q, nq, acc);
            __syncthreads();
            if (tid == 0) nq = 0;
            __syncthreads();
        }
    }
    __syncthreads();
    hw_drain<KIND>(L, q, nq, acc);
    acc = __reduce_or_sync(0xFFFFFFFFu, acc);
    if (lane == 0 && acc) atomicOr(L.flags, acc);
}

template <int KIND, int RND, bool PLAIN>
cudaError_t go_hw(const ElemLaunch &L, cudaStream_t s)
{
    static int fit = 0;                            // blocks an SM holds
    if (!fit) {
        int f = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, k_elem_hw<KIND, RND, PLAIN>, HW_T, 0) !=
                cudaSuccess || f < 1)
            f = 1;
        fit = f;
    }
    const size_t want = (L.n + HW_TILE - 1) / HW_TILE;
    const size_t cap = (size_t)sm_count() * (L.blocks_per_sm ? L.blocks_per_sm : (unsigned)fit);
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    k_elem_hw<KIND, RND, PLAIN><<<blocks ? blocks : 1, HW_T, 0, s>>>(L);
    return cudaGetLastError();
}

template <int KIND, int RND>
cudaError_t go_hw_plain(const ElemLaunch &L, cudaStream_t s)
{
    const bool reads_b = KIND == K_FMA || KIND == K_MUL, reads_c = KIND != K_MUL;
    const bool plain = L.scalar_mask == 0u && !L.ia && !L.ib && !L.ic && L.a &&
                       (!reads_b || L.b) && (!reads_c || L.c);
    return plain ? go_hw<KIND, RND, true>(L, s) : go_hw<KIND, RND, false>(L, s);
}

template <int KIND>
cudaError_t go_hw_rnd(const ElemLaunch &L, cudaStream_t s)
{
    switch (L.rnd) {
    case sf::RNE: return go_hw_plain<KIND, sf::RNE>(L, s);
    case sf::RTZ: return go_hw_plain<KIND, sf::RTZ>(L, s);
    case sf::RDN: return go_hw_plain<KIND, sf::RDN>(L, s);
    default: return go_hw_plain<KIND, sf::RUP>(L, s);
    }
}

}  // namespace

// CFTG_ELEM_HW=0 sends binary32 arithmetic to the integer kernels (for
// comparisons); read at every launch.
bool launch_elem_hw(const ElemLaunch &L, cudaStream_t s, cudaError_t *err)
{
    if (L.fmt != 0 || L.kind > K_MUL || L.rnd < sf::RNE || L.rnd > sf::RUP) return false;
    const char *e = getenv("CFTG_ELEM_HW");
    if (e && strcmp(e, "0") == 0) return false;
    switch (L.kind) {
    case K_FMA: *err = go_hw_rnd<K_FMA>(L, s); break;
    case K_ADD: *err = go_hw_rnd<K_ADD>(L, s); break;
    case K_SUB: *err = go_hw_rnd<K_SUB>(L, s); break;
    default: *err = go_hw_rnd<K_MUL>(L, s); break;
    }
    return true;
}

}  // namespace cftg
