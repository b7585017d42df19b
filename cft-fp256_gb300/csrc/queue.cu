// queue.cu - many independent elementwise calls as ONE persistent launch.
//
// The calls of a batch are cut into tiles (a tile is one call's elements
// [start, start + len)). A resident grid of blocks takes tiles from one
// atomic counter until the list is exhausted; a block processes a whole
// tile, so the format/kind branch is uniform across the block and the
// calls of every format and operation share the device without a launch
// per call. Tiles are ordered heaviest first (a cost model per format and
// kind), so the expensive division and square-root tiles start early and
// the tail is cheap. Each call's flags are ORed into its own word.
//
// The elements computed are exactly those of the plain kernels (elem.cu):
// the same device functions, the same operand rules.
#include "cftg_internal.h"
#include "queue.h"
#include "simple_ops.cuh"

namespace cftg {

namespace {

template <int W>
SFD void qload(const void *base, size_t j, uint32_t (&x)[W])
{
    if (!base) {
        sfw::zero(x);
        return;
    }
    const uint32_t *p = static_cast<const uint32_t *>(base) + j * W;
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
SFD void qstore(void *base, size_t j, const uint32_t (&x)[W])
{
    uint32_t *p = static_cast<uint32_t *>(base) + j * W;
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

template <int FMT, int KIND>
SFD uint32_t tile_work(const QCall &c, uint64_t start, uint32_t len)
{
    constexpr int W = sf::Fmt<FMT>::W;
    uint32_t acc = 0u;
    for (uint32_t k = threadIdx.x; k < len; k += blockDim.x) {
        const size_t i = start + k;
        uint32_t a[W], b[W], cc[W], o[W], fl = 0u;
        qload<W>(c.a, (c.scalar & 1u) ? 0 : i, a);
        if constexpr (KIND != K_SQRT && KIND != K_ADD && KIND != K_SUB) qload<W>(c.b, (c.scalar & 2u) ? 0 : i, b);
        else sfw::zero(b);
        if constexpr (KIND == K_FMA || KIND == K_ADD || KIND == K_SUB || KIND == K_SIMPLE)
            qload<W>(c.c, (c.scalar & 4u) ? 0 : i, cc);
        else sfw::zero(cc);
        if constexpr (KIND <= K_MUL) sf::arith<FMT, KIND>(a, b, cc, c.rnd, o, fl);
        else if constexpr (KIND == K_DIV) sf::div<FMT>(a, b, c.rnd, o, fl);
        else if constexpr (KIND == K_SQRT) sf::sqrt<FMT>(a, c.rnd, o, fl);
        else sf::simple<FMT>(c.op, a, b, cc, o, fl);
        qstore<W>(c.d, i, o);
        acc |= fl;
    }
    return acc;
}

template <int FMT>
SFD uint32_t tile_fmt(const QCall &c, uint64_t start, uint32_t len)
{
    switch (c.kind) {
    case K_FMA: return tile_work<FMT, K_FMA>(c, start, len);
    case K_ADD: return tile_work<FMT, K_ADD>(c, start, len);
    case K_SUB: return tile_work<FMT, K_SUB>(c, start, len);
    case K_MUL: return tile_work<FMT, K_MUL>(c, start, len);
    case K_DIV: return tile_work<FMT, K_DIV>(c, start, len);
    case K_SQRT: return tile_work<FMT, K_SQRT>(c, start, len);
    default: return tile_work<FMT, K_SIMPLE>(c, start, len);
    }
}

}  // namespace

__global__ void __launch_bounds__(256) k_queue(const QCall *__restrict__ calls,
                                               const QTile *__restrict__ tiles, uint32_t ntiles,
                                               uint32_t *counter, uint32_t *call_flags)
{
    // the next tile's index is taken while this one is computed, so the
    // counter's round trip is hidden behind the work
    __shared__ uint32_t next;
    if (threadIdx.x == 0) next = atomicAdd(counter, 1u);
    for (;;) {
        __syncthreads();
        const uint32_t t = next;
        __syncthreads();
        if (t >= ntiles) break;
        if (threadIdx.x == 0) next = atomicAdd(counter, 1u);
        const QTile tl = tiles[t];
        const QCall c = calls[tl.call];
        uint32_t acc;
        switch (c.fmt) {
        case 0: acc = tile_fmt<0>(c, tl.start, tl.len); break;
        case 1: acc = tile_fmt<1>(c, tl.start, tl.len); break;
        case 2: acc = tile_fmt<2>(c, tl.start, tl.len); break;
        default: acc = tile_fmt<3>(c, tl.start, tl.len); break;
        }
        acc = __reduce_or_sync(0xFFFFFFFFu, acc);
        if ((threadIdx.x & 31) == 0 && acc) atomicOr(call_flags + tl.call, acc);
    }
}

__global__ void __launch_bounds__(256) k_queue_calls(const QCall *__restrict__ calls,
                                                     const uint32_t *__restrict__ prefix,
                                                     uint32_t ncalls, uint32_t *counter,
                                                     uint32_t *call_flags)
{
    __shared__ uint32_t next, which;
    const uint32_t total = prefix[ncalls];
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t t = atomicAdd(counter, 1u);
            uint32_t lo = 0, hi = ncalls - 1;        // the last call with prefix <= t
            if (t < total) {
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (prefix[mid] <= t) lo = mid;
                    else hi = mid - 1;
                }
            }
            next = t;
            which = lo;
        }
        __syncthreads();
        const uint32_t t = next, ci = which;
        __syncthreads();
        if (t >= total) break;
        const QCall c = calls[ci];
        const uint64_t start = (uint64_t)(t - prefix[ci]) * c.tile;
        const uint32_t len = (uint32_t)(c.n - start < c.tile ? c.n - start : c.tile);
        uint32_t acc;
        switch (c.fmt) {
        case 0: acc = tile_fmt<0>(c, start, len); break;
        case 1: acc = tile_fmt<1>(c, start, len); break;
        case 2: acc = tile_fmt<2>(c, start, len); break;
        default: acc = tile_fmt<3>(c, start, len); break;
        }
        acc = __reduce_or_sync(0xFFFFFFFFu, acc);
        if ((threadIdx.x & 31) == 0 && acc) atomicOr(call_flags + ci, acc);
    }
}

// Long trajectory launches share the SMs with the work queue in the serving
// loop; both kernels ask for the same L1/shared split, so that an SM holding
// one can take blocks of the other without draining to change it.
static void carveout_once()
{
    static bool done = false;
    if (done) return;
    done = true;
    cudaFuncSetAttribute(k_queue_calls, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(k_queue, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
}

cudaError_t launch_queue_calls(const QCall *calls, const uint32_t *prefix, uint32_t ncalls,
                               uint32_t *counter, uint32_t *call_flags, int blocks, cudaStream_t s)
{
    if (ncalls == 0) return cudaSuccess;
    carveout_once();
    k_queue_calls<<<blocks, 256, 0, s>>>(calls, prefix, ncalls, counter, call_flags);
    return cudaGetLastError();
}

cudaError_t launch_queue(const QCall *calls, const QTile *tiles, uint32_t ntiles, uint32_t *counter,
                         uint32_t *call_flags, int blocks, int threads, cudaStream_t s)
{
    if (ntiles == 0) return cudaSuccess;
    k_queue<<<blocks, threads, 0, s>>>(calls, tiles, ntiles, counter, call_flags);
    return cudaGetLastError();
}

int queue_calls_regs()
{
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, k_queue_calls) != cudaSuccess) {
        cudaGetLastError();
        return 255;
    }
    return fa.numRegs;
}

int queue_blocks_per_sm(int threads)
{
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_queue, threads, 0);
    return per > 0 ? per : 1;
}

}  // namespace cftg
