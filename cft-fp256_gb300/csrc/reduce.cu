// reduce.cu - the reductions (SUM, DOT, SUMSQ, SUMABS, MAXALL) on the GPU,
// to the reference's fixed tree.
//
// The tree (reference host/src/softfloat.c:878-937, include/cft.h:1210-1296)
// splits a range so that its left child is the largest power of two strictly
// inside it; the add at a node is ADD(left, right) with the node's rounding
// attribute. So T(0, n) is the right-to-left fold of one PERFECT subtree for
// each set bit of n - the block for bit k holds 2^k items, blocks in index
// order from the highest bit down - and each perfect subtree is the plain
// pairwise tree over its items. That is what this file computes:
//
//  * k_red_chunks: one CTA a chunk of RC = 8192 items, the chunk's perfect
//    subtree: 32 consecutive items a thread folded by a binary counter whose
//    five partial results stay in registers (the pairwise tree over the 32,
//    node by node in index order), then the 256 threads' values pairwise -
//    by shuffles inside a warp, through shared memory across warps. More
//    items a thread keep more of the adds at full width: the levels across
//    threads run with fewer and fewer lanes busy. Blocks of 2^k >= RC items are
//    made of whole, aligned chunks, so the chunk results of one level form
//    the next level's items, and the same bits-of-n structure repeats there.
//  * k_red_final: one CTA folds everything else right to left: at every
//    level the tail (items past the last whole chunk, blocks smaller than a
//    chunk), lowest level first, each block's perfect subtree computed by
//    the whole CTA, then the last level's items.
//  * k_red_seg: the segmented form, one CTA a segment: chunks in order with
//    a binary counter of completed perfect blocks, then the tail, folded;
//    k_red_seg_w: segments of at most 1,024 items, one warp a segment.
//
// Leaves: SUM the element; DOT the rounded product a*b; SUMSQ a*a; SUMABS
// |a| (clearing the sign signals nothing); MAXALL the element, combined by
// the elementwise MAX (IEEE 754-2019 maximum is associative and commutative
// with its flags, so its bits do not depend on the shape). SUMSQ and SUMABS
// note infinities and signalling NaNs among the raw elements for 9.4's
// infinity rule, which replaces a NaN result by +inf (reference
// host/src/device.c:2640-2715).
#include "cftg_internal.h"
#include "simple_ops.cuh"

namespace cftg {

namespace {

constexpr int RT = 256;           // threads a CTA
constexpr int RE = 32;            // items a thread in a chunk
constexpr int RL = 5;             // log2(RE): the fold's partial results
constexpr uint32_t RC = RT * RE;  // items a chunk

template <int W>
SFD void rload(const void *p, size_t i, uint32_t (&x)[W])
{
    const uint32_t *q = static_cast<const uint32_t *>(p) + i * W;
    if constexpr (W == 8) {
        const uint4 v0 = reinterpret_cast<const uint4 *>(q)[0];
        const uint4 v1 = reinterpret_cast<const uint4 *>(q)[1];
        x[0] = v0.x; x[1] = v0.y; x[2] = v0.z; x[3] = v0.w;
        x[4] = v1.x; x[5] = v1.y; x[6] = v1.z; x[7] = v1.w;
    } else if constexpr (W == 4) {
        const uint4 v = reinterpret_cast<const uint4 *>(q)[0];
        x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
    } else if constexpr (W == 2) {
        const uint2 v = reinterpret_cast<const uint2 *>(q)[0];
        x[0] = v.x; x[1] = v.y;
    } else {
        x[0] = q[0];
    }
}

template <int W>
SFD void rstore(void *p, size_t i, const uint32_t (&x)[W])
{
    uint32_t *q = static_cast<uint32_t *>(p) + i * W;
#pragma unroll
    for (int w = 0; w < W; w++) q[w] = x[w];
}

// A node: ADD(left, right) - the right subtree in ADD's c operand - or MAX;
// arguments and result in registers, the arithmetic a call (compiled once
// a format, not inlined at every node: a binary256 add is a thousand
// instructions).
template <int W> struct Val {
    uint32_t w[W];
};
template <int W> struct ValF {
    uint32_t w[W];
    uint32_t f;
};

template <int FMT, bool MAX>
__device__ __noinline__ ValF<sf::Fmt<FMT>::W> comb_v(const Val<sf::Fmt<FMT>::W> l,
                                                     const Val<sf::Fmt<FMT>::W> r, int rnd)
{
    constexpr int W = sf::Fmt<FMT>::W;
    uint32_t x[W], y[W], z[W];
    ValF<W> o;
    o.f = 0u;
#pragma unroll
    for (int w = 0; w < W; w++) {
        x[w] = l.w[w];
        y[w] = r.w[w];
        z[w] = 0u;
    }
    if constexpr (MAX) sf::simple<FMT>(8, x, y, z, o.w, o.f);
    else sf::arith<FMT, sf::OP_ADD>(x, z, y, rnd, o.w, o.f);
    return o;
}

template <int FMT>
__device__ __noinline__ ValF<sf::Fmt<FMT>::W> mul_v(const Val<sf::Fmt<FMT>::W> x,
                                                    const Val<sf::Fmt<FMT>::W> y, int rnd)
{
    constexpr int W = sf::Fmt<FMT>::W;
    uint32_t a[W], b[W], z[W];
    ValF<W> o;
    o.f = 0u;
#pragma unroll
    for (int w = 0; w < W; w++) {
        a[w] = x.w[w];
        b[w] = y.w[w];
        z[w] = 0u;
    }
    sf::arith<FMT, sf::OP_MUL>(a, b, z, rnd, o.w, o.f);
    return o;
}

template <int FMT, int MODE>
SFD void comb(uint32_t (&l)[sf::Fmt<FMT>::W], const uint32_t (&r)[sf::Fmt<FMT>::W], int rnd,
              uint32_t &fl)
{
    constexpr int W = sf::Fmt<FMT>::W;
    Val<W> x, y;
#pragma unroll
    for (int w = 0; w < W; w++) {
        x.w[w] = l[w];
        y.w[w] = r[w];
    }
    const ValF<W> o = comb_v<FMT, MODE == RED_MAX>(x, y, rnd);
#pragma unroll
    for (int w = 0; w < W; w++) l[w] = o.w[w];
    fl |= o.f;
}

// 9.4's rule notes an infinity (bit 0) or a signalling NaN (bit 1) among the
// raw elements of SUMSQ and SUMABS.
template <int FMT>
SFD void note_special(const uint32_t (&v)[sf::Fmt<FMT>::W], uint32_t &seen)
{
    constexpr int W = sf::Fmt<FMT>::W;
    constexpr int ES = sf::exp_shift<FMT>();
    constexpr uint32_t EM = sf::exp_mask<FMT>();
    if (((v[W - 1] >> ES) & EM) == EM) {
        uint32_t frac = v[W - 1] & ((1u << ES) - 1u);
#pragma unroll
        for (int w = 0; w < W - 1; w++) frac |= v[w];
        const int qbit = sf::Fmt<FMT>::MANW - 1;
        const bool quiet = (v[qbit >> 5] >> (qbit & 31)) & 1u;
        if (!frac) seen |= 1u;
        else if (!quiet) seen |= 2u;
    }
}

// One item into x: a leaf at level 0 (SUM, SUMABS, MAXALL; the product
// leaves are item_v's), a stored partial result above it.
template <int FMT, int MODE, bool LEAF>
SFD void item(const void *a, const void *b, size_t i, int rnd, uint32_t (&x)[sf::Fmt<FMT>::W],
              uint32_t &fl, uint32_t &seen)
{
    constexpr int W = sf::Fmt<FMT>::W;
    uint32_t v[W];
    rload<W>(a, i, v);
    if constexpr (LEAF && (MODE == RED_SQ || MODE == RED_ABS)) note_special<FMT>(v, seen);
    if constexpr (LEAF && MODE == RED_ABS) v[W - 1] &= 0x7FFFFFFFu;
#pragma unroll
    for (int w = 0; w < W; w++) x[w] = v[w];
}

// item() with the leaf product through mul_v (registers, not memory).
template <int FMT, int MODE, bool LEAF>
SFD void item_v(const void *a, const void *b, size_t i, int rnd, uint32_t (&x)[sf::Fmt<FMT>::W],
                uint32_t &fl, uint32_t &seen)
{
    constexpr int W = sf::Fmt<FMT>::W;
    if constexpr (LEAF && (MODE == RED_DOT || MODE == RED_SQ)) {
        Val<W> p, q;
        rload<W>(a, i, p.w);
        if constexpr (MODE == RED_SQ) note_special<FMT>(p.w, seen);
        if constexpr (MODE == RED_DOT) rload<W>(b, i, q.w);
        else q = p;
        const ValF<W> o = mul_v<FMT>(p, q, rnd);
#pragma unroll
        for (int w = 0; w < W; w++) x[w] = o.w[w];
        fl |= o.f;
    } else {
        item<FMT, MODE, LEAF>(a, b, i, rnd, x, fl, seen);
    }
}

// The pairwise tree over E consecutive items from item i0 (E a power of two,
// 1..RE) by one thread: a binary counter, unrolled with its steps past E
// skipped (E is the same across the CTA or warp), so the pending left
// subtrees of each level are registers; each node is a by-value call.
template <int FMT, int MODE, bool LEAF>
SFD void thread_fold(const void *a, const void *b, size_t i0, uint32_t E, int rnd,
                     uint32_t (&v)[sf::Fmt<FMT>::W], uint32_t &fl, uint32_t &seen)
{
    constexpr int W = sf::Fmt<FMT>::W;
    Val<W> stk[RL], cur;
#pragma unroll
    for (int k = 0; k < RE; k++) {
        if ((uint32_t)k < E) {
            uint32_t x[W];
            item_v<FMT, MODE, LEAF>(a, b, i0 + k, rnd, x, fl, seen);
#pragma unroll
            for (int w = 0; w < W; w++) cur.w[w] = x[w];
#pragma unroll
            for (int lev = 0; lev < RL; lev++) {
                if (!((k >> lev) & 1)) {
                    stk[lev] = cur;
                    break;
                }
                const ValF<W> o = comb_v<FMT, MODE == RED_MAX>(stk[lev], cur, rnd);
#pragma unroll
                for (int w = 0; w < W; w++) cur.w[w] = o.w[w];
                fl |= o.f;
            }
        }
    }
#pragma unroll
    for (int w = 0; w < W; w++) v[w] = cur.w[w];
}

// The perfect subtree over `count` items (a power of two, 1..RC) from item
// `base`, by the whole CTA; the result in thread 0's v. Each thread first
// reduces E = count/RT consecutive items pairwise, then the threads' values
// pair up through shared memory. sm: RT x W words.
template <int FMT, int MODE, bool LEAF>
SFD void cta_perfect(const void *a, const void *b, size_t base, uint32_t count, int rnd,
                     uint32_t (&v)[sf::Fmt<FMT>::W], uint32_t &fl, uint32_t &seen, uint32_t *sm)
{
    constexpr int W = sf::Fmt<FMT>::W;
    const uint32_t t = threadIdx.x;
    const uint32_t E = count >= (uint32_t)RT ? count / RT : 1u;
    const uint32_t P = count >= (uint32_t)RT ? (uint32_t)RT : count;
    const bool have = t < P;
    if (have) thread_fold<FMT, MODE, LEAF>(a, b, base + (size_t)t * E, E, rnd, v, fl, seen);
    // the levels inside a warp by shuffles (no block barrier), the rest
    // through shared memory
    const uint32_t Pw = P < 32u ? P : 32u;
    for (uint32_t s = 1; s < Pw; s <<= 1) {
        uint32_t r[W];
#pragma unroll
        for (int w = 0; w < W; w++) r[w] = __shfl_down_sync(0xFFFFFFFFu, v[w], s);
        if (have && (t & (2 * s - 1)) == 0) comb<FMT, MODE>(v, r, rnd, fl);
    }
    for (uint32_t s = 32; s < P; s <<= 1) {
        __syncthreads();
        if (have && (t & (2 * s - 1)) == s) {
#pragma unroll
            for (int w = 0; w < W; w++) sm[w * RT + t] = v[w];
        }
        __syncthreads();
        if (have && (t & (2 * s - 1)) == 0) {
            uint32_t r[W];
#pragma unroll
            for (int w = 0; w < W; w++) r[w] = sm[w * RT + t + s];
            comb<FMT, MODE>(v, r, rnd, fl);
        }
    }
    __syncthreads();
}

// The CTA's flags and seen bits into thread 0 (sm2: two words).
SFD void cta_or(uint32_t &fl, uint32_t &seen, uint32_t *sm2)
{
    if (threadIdx.x == 0) { sm2[0] = 0u; sm2[1] = 0u; }
    __syncthreads();
    fl = __reduce_or_sync(0xFFFFFFFFu, fl);
    seen = __reduce_or_sync(0xFFFFFFFFu, seen);
    if ((threadIdx.x & 31) == 0) {
        if (fl) atomicOr(sm2 + 0, fl);
        if (seen) atomicOr(sm2 + 1, seen);
    }
    __syncthreads();
    fl = sm2[0];
    seen = sm2[1];
    __syncthreads();
}

// 9.4's rule on a finished result: a NaN becomes +inf when an element was
// an infinity, with INVALID iff an element was a signalling NaN - the
// flags REPLACED (reference host/src/device.c:3050-3062).
template <int FMT, int MODE>
SFD void inf_rule(uint32_t (&v)[sf::Fmt<FMT>::W], uint32_t &fl, uint32_t seen)
{
    if constexpr (MODE == RED_SQ || MODE == RED_ABS) {
        constexpr int W = sf::Fmt<FMT>::W;
        constexpr int ES = sf::exp_shift<FMT>();
        constexpr uint32_t EM = sf::exp_mask<FMT>();
        uint32_t frac = v[W - 1] & ((1u << ES) - 1u);
#pragma unroll
        for (int w = 0; w < W - 1; w++) frac |= v[w];
        const bool nan = ((v[W - 1] >> ES) & EM) == EM && frac;
        if (nan && (seen & 1u)) {
#pragma unroll
            for (int w = 0; w < W; w++) v[w] = 0u;
            v[W - 1] = EM << ES;
            fl = (seen & 2u) ? sf::F_INVALID : 0u;
        }
    }
}

template <int FMT, int MODE, bool LEAF>
__global__ void __launch_bounds__(RT) k_red_chunks(const void *a, const void *b, size_t nchunks,
                                                   void *out, int rnd, uint32_t *word)
{
    constexpr int W = sf::Fmt<FMT>::W;
    __shared__ uint32_t sm[RT * W];
    __shared__ uint32_t sm2[2];
    uint32_t fl = 0u, seen = 0u;
    for (size_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        uint32_t v[W];
        cta_perfect<FMT, MODE, LEAF>(a, b, c * RC, RC, rnd, v, fl, seen, sm);
        if (threadIdx.x == 0) rstore<W>(out, c, v);
    }
    cta_or(fl, seen, sm2);
    if (threadIdx.x == 0) {
        if (fl) atomicOr(word + 0, fl);
        if (seen) atomicOr(word + 1, seen);
    }
}

template <int FMT, int MODE>
__global__ void __launch_bounds__(RT) k_red_final(const RedLevels L, void *out, int rnd,
                                                  uint32_t *word)
{
    constexpr int W = sf::Fmt<FMT>::W;
    __shared__ uint32_t sm[RT * W];
    __shared__ uint32_t sm2[2];
    uint32_t fl = 0u, seen = 0u;
    uint32_t S[W], v[W];
    bool have = false;
    for (int l = 0; l < L.count; l++) {
        const RedLevel &lv = L.lev[l];
        for (int k = 0; k < 32; k++) {
            if (!((lv.len >> k) & 1u)) continue;
            const size_t start = lv.start + (lv.len & ~((2u << k) - 1u));
            if (lv.leaf) cta_perfect<FMT, MODE, true>(L.a, L.b, start, 1u << k, rnd, v, fl, seen, sm);
            else cta_perfect<FMT, MODE, false>(lv.src, nullptr, start, 1u << k, rnd, v, fl, seen, sm);
            if (threadIdx.x == 0) {
                if (have) {                                  // v is the LEFT block
                    comb<FMT, MODE>(v, S, rnd, fl);
                }
#pragma unroll
                for (int w = 0; w < W; w++) S[w] = v[w];
                have = true;
            }
        }
    }
    cta_or(fl, seen, sm2);
    if (threadIdx.x == 0) {
        fl |= word[0];
        seen |= word[1];
        if (!have) {
#pragma unroll
            for (int w = 0; w < W; w++) S[w] = 0u;
        }
        inf_rule<FMT, MODE>(S, fl, seen);
        rstore<W>(out, 0, S);
        word[0] = fl;
    }
}

template <int FMT, int MODE>
__global__ void __launch_bounds__(RT) k_red_seg(const void *a, const void *b, size_t nseg,
                                                size_t seg, void *out, int rnd, uint32_t *word)
{
    constexpr int W = sf::Fmt<FMT>::W;
    __shared__ uint32_t sm[RT * W];
    __shared__ uint32_t sm2[2];
    __shared__ uint32_t stk[48 * W];                 // completed perfect blocks of chunks
    __shared__ int stk_lev[48];
    for (size_t s = blockIdx.x; s < nseg; s += gridDim.x) {
        uint32_t fl = 0u, seen = 0u;
        const size_t base = s * seg;
        const size_t q = seg / RC;
        const uint32_t tail = (uint32_t)(seg - q * RC);
        int sp = 0;
        uint32_t v[W], S[W];
        for (size_t c = 0; c < q; c++) {
            cta_perfect<FMT, MODE, true>(a, b, base + c * RC, RC, rnd, v, fl, seen, sm);
            if (threadIdx.x == 0) {
                int lev = 0;
                while (sp > 0 && stk_lev[sp - 1] == lev) {   // equal blocks merge, older on the left
                    uint32_t left[W];
#pragma unroll
                    for (int w = 0; w < W; w++) left[w] = stk[(sp - 1) * W + w];
                    comb<FMT, MODE>(left, v, rnd, fl);
#pragma unroll
                    for (int w = 0; w < W; w++) v[w] = left[w];
                    sp--;
                    lev++;
                }
#pragma unroll
                for (int w = 0; w < W; w++) stk[sp * W + w] = v[w];
                stk_lev[sp] = lev;
                sp++;
            }
        }
        bool have = false;
        const size_t tbase = base + q * RC;
        for (int k = 0; k < 32; k++) {
            if (!((tail >> k) & 1u)) continue;
            const size_t start = tbase + (tail & ~((2u << k) - 1u));
            cta_perfect<FMT, MODE, true>(a, b, start, 1u << k, rnd, v, fl, seen, sm);
            if (threadIdx.x == 0) {
                if (have) comb<FMT, MODE>(v, S, rnd, fl);
#pragma unroll
                for (int w = 0; w < W; w++) S[w] = v[w];
                have = true;
            }
        }
        if (threadIdx.x == 0) {
            for (int i = sp - 1; i >= 0; i--) {              // smallest chunk block first
#pragma unroll
                for (int w = 0; w < W; w++) v[w] = stk[i * W + w];
                if (have) comb<FMT, MODE>(v, S, rnd, fl);
#pragma unroll
                for (int w = 0; w < W; w++) S[w] = v[w];
                have = true;
            }
        }
        cta_or(fl, seen, sm2);
        if (threadIdx.x == 0) {
            if (!have) {
#pragma unroll
                for (int w = 0; w < W; w++) S[w] = 0u;
            }
            inf_rule<FMT, MODE>(S, fl, seen);
            rstore<W>(out, s, S);
            if (fl) atomicOr(word, fl);
        }
        __syncthreads();
    }
}

// Segments of at most RSW elements: one warp a segment, so a thread folds up
// to 32 items of a 1,024-item block and only five levels run across lanes.
// Blocks of the segment's set bits, right to left as in k_red_seg.
constexpr size_t RSW = 1024;

template <int FMT, int MODE>
__global__ void __launch_bounds__(RT) k_red_seg_w(const void *a, const void *b, size_t nseg,
                                                  size_t seg, void *out, int rnd, uint32_t *word)
{
    constexpr int W = sf::Fmt<FMT>::W;
    const uint32_t lane = threadIdx.x & 31u;
    const size_t warps = (size_t)gridDim.x * (RT / 32);
    uint32_t wfl = 0u;
    for (size_t g = (size_t)blockIdx.x * (RT / 32) + threadIdx.x / 32; g < nseg; g += warps) {
        uint32_t fl = 0u, seen = 0u, S[W];
        bool have = false;
        const size_t base = g * seg;
        for (int k = 0; k <= 10; k++) {
            if (!((seg >> k) & 1u)) continue;
            const size_t start = base + (seg & ~(((size_t)2 << k) - 1u));
            const uint32_t cnt = 1u << k;
            const uint32_t P = cnt < 32u ? cnt : 32u, E = cnt / P;
            uint32_t v[W];
#pragma unroll
            for (int w = 0; w < W; w++) v[w] = 0u;
            if (lane < P) thread_fold<FMT, MODE, true>(a, b, start + (size_t)lane * E, E, rnd, v, fl, seen);
            for (uint32_t st = 1; st < P; st <<= 1) {
                uint32_t r[W];
#pragma unroll
                for (int w = 0; w < W; w++) r[w] = __shfl_down_sync(0xFFFFFFFFu, v[w], st);
                if (lane < P && (lane & (2 * st - 1)) == 0) comb<FMT, MODE>(v, r, rnd, fl);
            }
            if (lane == 0) {
                if (have) comb<FMT, MODE>(v, S, rnd, fl);          // v is the LEFT block
#pragma unroll
                for (int w = 0; w < W; w++) S[w] = v[w];
                have = true;
            }
        }
        fl = __reduce_or_sync(0xFFFFFFFFu, fl);
        seen = __reduce_or_sync(0xFFFFFFFFu, seen);
        if (lane == 0) {
            if (!have) {
#pragma unroll
                for (int w = 0; w < W; w++) S[w] = 0u;
            }
            inf_rule<FMT, MODE>(S, fl, seen);
            rstore<W>(out, g, S);
            wfl |= fl;
        }
    }
    if (lane == 0 && wfl) atomicOr(word, wfl);
}

int red_blocks(size_t want)
{
    const size_t cap = (size_t)sm_count() * 4;
    return (int)(want < cap ? (want ? want : 1) : cap);
}

template <int FMT, int MODE>
cudaError_t go_tree(const void *a, const void *b, size_t n, void *partials, void *out, int rnd,
                    uint32_t *word, cudaStream_t s)
{
    constexpr size_t esz = 4 * sf::Fmt<FMT>::W;
    RedLevels L;
    L.a = a;
    L.b = b;
    L.count = 0;
    const void *X = a;
    bool leaf = true;
    size_t len = n;
    uint8_t *P = static_cast<uint8_t *>(partials);
    cudaError_t e = cudaMemsetAsync(word, 0, 2 * sizeof(uint32_t), s);
    while (e == cudaSuccess && len >= RC) {
        const size_t m = len / RC;
        if (leaf) k_red_chunks<FMT, MODE, true><<<red_blocks(m), RT, 0, s>>>(a, b, m, P, rnd, word);
        else k_red_chunks<FMT, MODE, false><<<red_blocks(m), RT, 0, s>>>(X, nullptr, m, P, rnd, word);
        e = cudaGetLastError();
        L.lev[L.count++] = RedLevel{X, m * RC, (uint32_t)(len - m * RC), leaf};
        X = P;
        P += m * esz;
        len = m;
        leaf = false;
    }
    L.lev[L.count++] = RedLevel{X, 0, (uint32_t)len, leaf};
    if (e == cudaSuccess) {
        k_red_final<FMT, MODE><<<1, RT, 0, s>>>(L, out, rnd, word);
        e = cudaGetLastError();
    }
    return e;
}

template <int FMT, int MODE>
cudaError_t go_seg(const void *a, const void *b, size_t nseg, size_t seg, void *out, int rnd,
                   uint32_t *word, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(word, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    if (seg <= RSW)
        k_red_seg_w<FMT, MODE><<<red_blocks((nseg + RT / 32 - 1) / (RT / 32)), RT, 0, s>>>(
            a, b, nseg, seg, out, rnd, word);
    else
        k_red_seg<FMT, MODE><<<red_blocks(nseg), RT, 0, s>>>(a, b, nseg, seg, out, rnd, word);
    return cudaGetLastError();
}

template <int FMT>
cudaError_t tree_fmt(int mode, const void *a, const void *b, size_t n, void *partials, void *out,
                     int rnd, uint32_t *word, cudaStream_t s)
{
    switch (mode) {
    case RED_SUM: return go_tree<FMT, RED_SUM>(a, b, n, partials, out, rnd, word, s);
    case RED_DOT: return go_tree<FMT, RED_DOT>(a, b, n, partials, out, rnd, word, s);
    case RED_SQ: return go_tree<FMT, RED_SQ>(a, b, n, partials, out, rnd, word, s);
    case RED_ABS: return go_tree<FMT, RED_ABS>(a, b, n, partials, out, rnd, word, s);
    default: return go_tree<FMT, RED_MAX>(a, b, n, partials, out, rnd, word, s);
    }
}

template <int FMT>
cudaError_t seg_fmt(int mode, const void *a, const void *b, size_t nseg, size_t seg, void *out,
                    int rnd, uint32_t *word, cudaStream_t s)
{
    switch (mode) {
    case RED_SUM: return go_seg<FMT, RED_SUM>(a, b, nseg, seg, out, rnd, word, s);
    case RED_DOT: return go_seg<FMT, RED_DOT>(a, b, nseg, seg, out, rnd, word, s);
    case RED_SQ: return go_seg<FMT, RED_SQ>(a, b, nseg, seg, out, rnd, word, s);
    case RED_ABS: return go_seg<FMT, RED_ABS>(a, b, nseg, seg, out, rnd, word, s);
    default: return go_seg<FMT, RED_MAX>(a, b, nseg, seg, out, rnd, word, s);
    }
}

}  // namespace

size_t red_partial_elems(size_t n)
{
    size_t t = 0;
    while (n >= RC) {
        n /= RC;
        t += n;
    }
    return t;
}

cudaError_t launch_reduce(int fmt, int mode, const void *a, const void *b, size_t n, void *partials,
                          void *out, int rnd, uint32_t *word, cudaStream_t s)
{
    switch (fmt) {
    case 0: return tree_fmt<0>(mode, a, b, n, partials, out, rnd, word, s);
    case 1: return tree_fmt<1>(mode, a, b, n, partials, out, rnd, word, s);
    case 2: return tree_fmt<2>(mode, a, b, n, partials, out, rnd, word, s);
    default: return tree_fmt<3>(mode, a, b, n, partials, out, rnd, word, s);
    }
}

cudaError_t launch_reduce_seg(int fmt, int mode, const void *a, const void *b, size_t nseg,
                              size_t seg, void *out, int rnd, uint32_t *word, cudaStream_t s)
{
    switch (fmt) {
    case 0: return seg_fmt<0>(mode, a, b, nseg, seg, out, rnd, word, s);
    case 1: return seg_fmt<1>(mode, a, b, nseg, seg, out, rnd, word, s);
    case 2: return seg_fmt<2>(mode, a, b, nseg, seg, out, rnd, word, s);
    default: return seg_fmt<3>(mode, a, b, nseg, seg, out, rnd, word, s);
    }
}

}  // namespace cftg
