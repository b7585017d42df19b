// elem.cu - the elementwise kernels: one template per (format, kind), a
// grid-stride loop of one element per thread per step, values and flags
// computed in registers, the call's flag word ORed once per warp.
//
// Elements are the caller's dense little-endian byte strings (the ABI's
// layout, reference host/include/cft.h:1172-1174): an fp256 element is two
// 16-byte vectors, fp128 one, fp64 an 8-byte pair, fp32 one word.
#include "cftg_internal.h"
#include "elem_io.cuh"

namespace cftg {

// Blocks of 256 an SM the compiler is asked to fit (registers a thread
// at most 65,536 / (256 x blocks)): binary256 FMA at five (48 registers, a
// few spilled, against 64 and four blocks unasked) gives its warps' memory
// and integer latencies more company (warps active 43 -> 51 %; 31.9 -> 32.1
// Gelem/s at n = 2^24); binary128 FMA, ADD and SUB at six (40 registers,
// none spilled, against 50 and five): FMA 48.8 -> 49.7, ADD 64.2 -> 65.9.
template <int FMT, int KIND>
__host__ __device__ constexpr int elem_min_blocks()
{
    return FMT == 3 && KIND == K_FMA ? 5
         : FMT == 2 && (KIND == K_FMA || KIND == K_ADD || KIND == K_SUB) ? 6
         : 1;
}

template <int FMT, int KIND>
__global__ void __launch_bounds__(256, elem_min_blocks<FMT, KIND>()) k_elem(const ElemLaunch L)
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
        compute_elem<FMT, KIND>(L.op, L.rnd, a, b, c, o, fl);
        store_elem<W>(static_cast<uint32_t *>(L.d), i, o);
        if (L.lane_flags) L.lane_flags[i] = (uint8_t)fl;
        acc |= fl;
    }
    // the call's flag word: an atomic OR only for bits not already there
    // (the word fills within the first warps; an OR of thousands of warps
    // into one word otherwise queues at the L2's atomic unit). A bit read
    // stale costs a redundant OR, never a lost one.
    acc = __reduce_or_sync(0xFFFFFFFFu, acc);
    if ((threadIdx.x & 31) == 0 && acc && (acc & ~__ldcg(L.flags))) atomicOr(L.flags, acc);
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
    // 64 blocks an SM, many more than fit at once: blocks that start late
    // fill the SMs whose earlier blocks finish early. Measured at n = 2^24
    // (binary256 / binary128 FMA, Gelem/s): one wave of exactly the resident
    // blocks 31.0 / 48.5, 8 an SM 32.0 / 50.7, 16 33.3 / 53.3, 64 33.8 /
    // 55.0, 256 33.9 / 53.9 (with the flag word's atomics skipped once set;
    // 22.1 / 31.3 without)
    const size_t want = (L.n + T - 1) / T;
    const size_t cap = (size_t)sm_count() * (L.blocks_per_sm ? L.blocks_per_sm : 64u);
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
    // the staged kernels when asked for (CFTG_ELEM_STAGING=bulk); else
    // binary32 arithmetic on the hardware's rounding (elem_hw.cu), and the
    // one-element-a-thread kernels here for everything else
    cudaError_t err = cudaSuccess;
    if (launch_elem_bulk(L, s, &err)) return err;
    if (launch_elem_hw(L, s, &err)) return err;
    switch (L.fmt) {
    case 0: return go_fmt<0>(L, s);
    case 1: return go_fmt<1>(L, s);
    case 2: return go_fmt<2>(L, s);
    default: return go_fmt<3>(L, s);
    }
}

}  // namespace cftg
