// elem_bulk.cu - the elementwise kernels for large arrays whose operands sit
// in device memory: each warp owns a two-stage ring in shared memory, its
// lane 0 fills a stage with one bulk copy (cp.async.bulk, the Tensor Memory
// Accelerator) per operand of the warp's next tile of 32 elements, and the
// lanes read their elements out of shared memory while the copy of the tile
// after next is in flight. No block-wide barrier: warps run free of each
// other, as in the direct kernel (elem.cu), whose arithmetic and per-element
// semantics these kernels share.
//
// Taken, when CFTG_ELEM_STAGING=bulk asks for it, for calls without index
// tables, n >= 65,536 and every streamed operand in device memory, 16-byte
// aligned. Scalar operands (element 0 for every i) and NULL operands (+0)
// are read as the direct kernel reads them. The last n mod 32 elements are
// computed by one warp with direct loads.
#include "bulk.cuh"
#include "cftg_internal.h"
#include "elem_io.cuh"

#include <cstdlib>
#include <cstring>

namespace cftg {

namespace {

constexpr int TW = 32;                        // elements a warp tile
constexpr int WARPS = 8;                      // warps a block
constexpr size_t BULK_MIN_N = (size_t)1 << 16;
constexpr uint64_t STAGE_LIMIT_NS = 1000000000ull;   // a stage that takes 1 s has failed

// Operands each kind reads (bit r: operand r), as k_elem reads them.
template <int KIND>
__host__ __device__ constexpr unsigned reads_of()
{
    return KIND == K_SQRT ? 1u
         : (KIND == K_ADD || KIND == K_SUB) ? 5u
         : (KIND == K_MUL || KIND == K_DIV) ? 3u
         : 7u;
}

template <int FMT, int KIND>
__global__ void __launch_bounds__(256) k_elem_bulk(const ElemLaunch L, const unsigned streamed,
                                                   const int ns)
{
    constexpr int W = sf::Fmt<FMT>::W;
    constexpr uint32_t TB = TW * W * 4;       // bytes of one operand's warp tile
    constexpr unsigned READS = reads_of<KIND>();
    extern __shared__ __align__(128) uint8_t sm[];
    __shared__ __align__(8) uint64_t bar[WARPS][2];

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t *const ring = sm + (size_t)warp * 2 * ns * TB;
    uint64_t *const wb = bar[warp];
    const void *const src[3] = {L.a, L.b, L.c};
    const size_t ntiles = L.n / TW;
    const size_t nw = (size_t)gridDim.x * WARPS, gw = (size_t)blockIdx.x * WARPS + warp;

    if (lane == 0) {
        bulk::bar_init(&wb[0], 1);
        bulk::bar_init(&wb[1], 1);
        bulk::fence_async_shared();
    }
    __syncwarp();
    // lane 0: stage s <- the streamed operands of tile t
    auto fill = [&](int s, size_t t) {
        bulk::bar_expect_tx(&wb[s], (uint32_t)ns * TB);
        uint8_t *dst = ring + (size_t)s * ns * TB;
#pragma unroll
        for (int r = 0; r < 3; r++)
            if ((streamed >> r) & 1u) {
                bulk::copy_g2s(dst, static_cast<const uint8_t *>(src[r]) + t * TB, TB, &wb[s]);
                dst += TB;
            }
    };
    if (lane == 0) {
        if (gw < ntiles) fill(0, gw);
        if (gw + nw < ntiles) fill(1, gw + nw);
    }

    uint32_t acc = 0u;
    uint32_t j = 0;
    bool failed = false;
    size_t t = gw;
    for (; t < ntiles; t += nw, j++) {
        const int s = (int)(j & 1u);
        if (!__all_sync(0xFFFFFFFFu, bulk::bar_wait(&wb[s], (j >> 1) & 1u, STAGE_LIMIT_NS))) {
            failed = true;
            break;
        }
        uint32_t x[3][W];
        const uint8_t *stage = ring + (size_t)s * ns * TB + (size_t)lane * (W * 4);
        const size_t i = t * TW + lane;
#pragma unroll
        for (int r = 0; r < 3; r++) {
            if (!((READS >> r) & 1u)) {
                sfw::zero(x[r]);
            } else if ((streamed >> r) & 1u) {
                load_elem<W>(reinterpret_cast<const uint32_t *>(stage), 0, x[r]);
                stage += TB;
            } else {
                fetch<W>(src[r], (L.scalar_mask >> r) & 1u, nullptr, i, x[r]);
            }
        }
        __syncwarp();
        // every lane has its operands: the stage takes the tile after next
        if (lane == 0 && t + 2 * nw < ntiles) {
            bulk::fence_async_shared();
            fill(s, t + 2 * nw);
        }
        uint32_t o[W], fl = 0u;
        compute_elem<FMT, KIND>(L.op, L.rnd, x[0], x[1], x[2], o, fl);
        store_elem<W>(static_cast<uint32_t *>(L.d), i, o);
        if (L.lane_flags) L.lane_flags[i] = (uint8_t)fl;
        acc |= fl;
    }
    if (failed) {
        // Let the copies still in flight into this warp's ring land (or run
        // out of time) before the block can exit, and report the failure.
        if (lane == 0) {
            bulk::bar_wait(&wb[j & 1u], (j >> 1) & 1u, STAGE_LIMIT_NS);
            if (t + nw < ntiles) bulk::bar_wait(&wb[(j + 1) & 1u], ((j + 1) >> 1) & 1u, STAGE_LIMIT_NS);
            atomicOr(L.flags, ELEM_ERR_STAGING);
        }
    } else if (gw == nw - 1) {
        // the ragged end, n mod 32 elements, with direct loads
        const size_t i = ntiles * TW + lane;
        if (i < L.n) {
            uint32_t x[3][W], o[W], fl = 0u;
#pragma unroll
            for (int r = 0; r < 3; r++) {
                if ((READS >> r) & 1u) fetch<W>(src[r], (L.scalar_mask >> r) & 1u, nullptr, i, x[r]);
                else sfw::zero(x[r]);
            }
            compute_elem<FMT, KIND>(L.op, L.rnd, x[0], x[1], x[2], o, fl);
            store_elem<W>(static_cast<uint32_t *>(L.d), i, o);
            if (L.lane_flags) L.lane_flags[i] = (uint8_t)fl;
            acc |= fl;
        }
    }
    acc = __reduce_or_sync(0xFFFFFFFFu, acc);
    if (lane == 0 && acc) atomicOr(L.flags, acc);
}

// p is 16-byte aligned memory of the current device (not host memory, not
// managed memory, not another GPU's).
bool in_hbm(const void *p)
{
    if (reinterpret_cast<uintptr_t>(p) & 15u) return false;
    cudaPointerAttributes at;
    int dev = -1;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice && at.device == dev;
}

// The ring's shared memory asks for the opt-in ceiling and the largest
// shared carveout, set once a device and kernel instance.
template <typename K>
cudaError_t attrs_once(K kernel, unsigned &done_mask)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned bit = 1u << (dev & 31);
    if (done_mask & bit) return cudaSuccess;
    int optin = 0;
    cudaFuncAttributes fa;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
    // the ceiling counts the kernel's static shared memory (its barriers) too
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) done_mask |= bit;
    return e;
}

template <int FMT, int KIND>
cudaError_t go(const ElemLaunch &L, unsigned streamed, int ns, cudaStream_t s)
{
    constexpr int W = sf::Fmt<FMT>::W;
    static unsigned done = 0;
    static int per_sm[4] = {0, 0, 0, 0};      // resident blocks an SM, by streamed-operand count
    auto kernel = k_elem_bulk<FMT, KIND>;
    cudaError_t e = attrs_once(kernel, done);
    if (e != cudaSuccess) return e;
    const size_t smem = (size_t)WARPS * 2 * ns * TW * W * 4;
    if (!per_sm[ns]) {
        int per = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, WARPS * 32, smem);
        if (e != cudaSuccess) return e;
        per_sm[ns] = per > 0 ? per : 1;
    }
    const size_t ntiles = L.n / TW;
    const size_t want = (ntiles + WARPS - 1) / WARPS;
    const size_t cap = (size_t)sm_count() * per_sm[ns];
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    kernel<<<blocks ? blocks : 1, WARPS * 32, smem, s>>>(L, streamed, ns);
    return cudaGetLastError();
}

template <int FMT>
cudaError_t go_fmt(const ElemLaunch &L, unsigned streamed, int ns, cudaStream_t s)
{
    switch (L.kind) {
    case K_FMA: return go<FMT, K_FMA>(L, streamed, ns, s);
    case K_ADD: return go<FMT, K_ADD>(L, streamed, ns, s);
    case K_SUB: return go<FMT, K_SUB>(L, streamed, ns, s);
    case K_MUL: return go<FMT, K_MUL>(L, streamed, ns, s);
    case K_DIV: return go<FMT, K_DIV>(L, streamed, ns, s);
    case K_SQRT: return go<FMT, K_SQRT>(L, streamed, ns, s);
    default: return go<FMT, K_SIMPLE>(L, streamed, ns, s);
    }
}

unsigned reads_of_kind(int kind)
{
    switch (kind) {
    case K_SQRT: return reads_of<K_SQRT>();
    case K_ADD: return reads_of<K_ADD>();
    case K_SUB: return reads_of<K_SUB>();
    case K_MUL: return reads_of<K_MUL>();
    case K_DIV: return reads_of<K_DIV>();
    case K_FMA: return reads_of<K_FMA>();
    default: return reads_of<K_SIMPLE>();
    }
}

}  // namespace

// Taken only under CFTG_ELEM_STAGING=bulk: on a GB300 the staged kernels
// run 6-14 % below the direct ones in every cell of the elementwise sweep
// (fp256 FMA 26.1 against 27.8 Gelem/s at n = 2^24). The arithmetic, not
// the loads, bounds these kernels - the integer ALU pipe is ~80 % busy and
// the direct kernel's DRAM traffic already equals the algorithmic bytes - so
// staging adds instructions (ring waits, votes, copy issue, shared-memory
// loads) and registers without removing any.
bool launch_elem_bulk(const ElemLaunch &L, cudaStream_t s, cudaError_t *err)
{
    if (L.n < BULK_MIN_N || L.ia || L.ib || L.ic) return false;
    const char *mode = getenv("CFTG_ELEM_STAGING");
    if (!mode || strcmp(mode, "bulk") != 0) return false;
    const void *src[3] = {L.a, L.b, L.c};
    const unsigned reads = reads_of_kind(L.kind);
    unsigned streamed = 0;
    int ns = 0;
    for (int r = 0; r < 3; r++) {
        if (!((reads >> r) & 1u) || !src[r] || ((L.scalar_mask >> r) & 1u)) continue;
        if (!in_hbm(src[r])) return false;
        streamed |= 1u << r;
        ns++;
    }
    if (!ns) return false;
    switch (L.fmt) {
    case 0: *err = go_fmt<0>(L, streamed, ns, s); break;
    case 1: *err = go_fmt<1>(L, streamed, ns, s); break;
    case 2: *err = go_fmt<2>(L, streamed, ns, s); break;
    default: *err = go_fmt<3>(L, streamed, ns, s); break;
    }
    return true;
}

}  // namespace cftg
