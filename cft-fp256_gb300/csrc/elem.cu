// elem.cu - the elementwise kernels: one template per (format, kind), a
// grid-stride loop of one element per thread per step, values and flags
// computed in registers, the call's flag word ORed once per warp.
//
// Elements are the caller's dense little-endian byte strings (the ABI's
// layout, reference host/include/cft.h:1172-1174): an fp256 element is two
// 16-byte vectors, fp128 one, fp64 an 8-byte pair, fp32 one word.
#include "cftg_internal.h"
#include "simple_ops.cuh"

namespace cftg {

template <int W>
SFD void load_elem(const uint32_t *__restrict__ base, size_t j, uint32_t (&x)[W])
{
    const uint32_t *p = base + j * W;
    if constexpr (W == 8) {
        const uint4 v0 = reinterpret_cast<const uint4 *>(p)[0];
        const uint4 v1 = reinterpret_cast<const uint4 *>(p)[1];
        x[0] = v0.x; x[1] = v0.y; x[2] = v0.z; x[3] = v0.w;
        x[4] = v1.x; x[5] = v1.y; x[6] = v1.z; x[7] = v1.w;
    } else if constexpr (W == 4) {
        const uint4 v = reinterpret_cast<const uint4 *>(p)[0];
        x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
    } else if constexpr (W == 2) {
        const uint2 v = reinterpret_cast<const uint2 *>(p)[0];
        x[0] = v.x; x[1] = v.y;
    } else {
        x[0] = p[0];
    }
}

template <int W>
SFD void store_elem(uint32_t *__restrict__ base, size_t j, const uint32_t (&x)[W])
{
    uint32_t *p = base + j * W;
    if constexpr (W == 8) {
        reinterpret_cast<uint4 *>(p)[0] = make_uint4(x[0], x[1], x[2], x[3]);
        reinterpret_cast<uint4 *>(p)[1] = make_uint4(x[4], x[5], x[6], x[7]);
    } else if constexpr (W == 4) {
        reinterpret_cast<uint4 *>(p)[0] = make_uint4(x[0], x[1], x[2], x[3]);
    } else if constexpr (W == 2) {
        reinterpret_cast<uint2 *>(p)[0] = make_uint2(x[0], x[1]);
    } else {
        p[0] = x[0];
    }
}

// Operand r of element i: +0 for a NULL operand or a CFT_IDX_NONE index,
// element 0 for a scalar, source[idx[i]] through a table, else element i.
template <int W>
SFD void fetch(const void *src, bool scalar, const uint32_t *idx, size_t i, uint32_t (&x)[W])
{
    if (!src) {
        sfw::zero(x);
        return;
    }
    size_t j = scalar ? 0 : i;
    if (idx) {
        const uint32_t t = idx[i];
        if (t == 0xFFFFFFFFu) {
            sfw::zero(x);
            return;
        }
        j = t;
    }
    load_elem<W>(static_cast<const uint32_t *>(src), j, x);
}

template <int FMT, int KIND>
__global__ void __launch_bounds__(256) k_elem(const ElemLaunch L)
{
    constexpr int W = sf::Fmt<FMT>::W;
    uint32_t acc = 0u;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < L.n; i += stride) {
        uint32_t a[W], b[W], c[W], o[W], fl = 0u;
        fetch<W>(L.a, L.scalar_mask & 1u, L.ia, i, a);
        if constexpr (KIND != K_SQRT && KIND != K_ADD && KIND != K_SUB) fetch<W>(L.b, L.scalar_mask & 2u, L.ib, i, b);
        else sfw::zero(b);
        if constexpr (KIND == K_FMA || KIND == K_ADD || KIND == K_SUB || KIND == K_SIMPLE)
            fetch<W>(L.c, L.scalar_mask & 4u, L.ic, i, c);
        else sfw::zero(c);
        if constexpr (KIND <= K_MUL) sf::arith<FMT, KIND>(a, b, c, L.rnd, o, fl);
        else if constexpr (KIND == K_DIV) sf::div<FMT>(a, b, L.rnd, o, fl);
        else if constexpr (KIND == K_SQRT) sf::sqrt<FMT>(a, L.rnd, o, fl);
        else sf::simple<FMT>(L.op, a, b, c, o, fl);
        store_elem<W>(static_cast<uint32_t *>(L.d), i, o);
        if (L.lane_flags) L.lane_flags[i] = (uint8_t)fl;
        acc |= fl;
    }
    acc = __reduce_or_sync(0xFFFFFFFFu, acc);
    if ((threadIdx.x & 31) == 0 && acc) atomicOr(L.flags, acc);
}

static int g_sms = 0;

int sm_count()
{
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    return g_sms;
}

template <int FMT, int KIND>
static cudaError_t go(const ElemLaunch &L, cudaStream_t s)
{
    constexpr int T = 256;
    const size_t want = (L.n + T - 1) / T;
    const size_t cap = (size_t)sm_count() * (L.blocks_per_sm ? L.blocks_per_sm : 8u);
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    k_elem<FMT, KIND><<<blocks ? blocks : 1, T, 0, s>>>(L);
    return cudaGetLastError();
}

template <int FMT>
static cudaError_t go_fmt(const ElemLaunch &L, cudaStream_t s)
{
    switch (L.kind) {
    case K_FMA: return go<FMT, K_FMA>(L, s);
    case K_ADD: return go<FMT, K_ADD>(L, s);
    case K_SUB: return go<FMT, K_SUB>(L, s);
    case K_MUL: return go<FMT, K_MUL>(L, s);
    case K_DIV: return go<FMT, K_DIV>(L, s);
    case K_SQRT: return go<FMT, K_SQRT>(L, s);
    default: return go<FMT, K_SIMPLE>(L, s);
    }
}

cudaError_t launch_elem(const ElemLaunch &L, cudaStream_t s)
{
    if (L.n == 0) return cudaSuccess;
    switch (L.fmt) {
    case 0: return go_fmt<0>(L, s);
    case 1: return go_fmt<1>(L, s);
    case 2: return go_fmt<2>(L, s);
    default: return go_fmt<3>(L, s);
    }
}

}  // namespace cftg
