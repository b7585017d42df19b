// elem_q.cu - binary128 and binary256 FMA/ADD/SUB/MUL with the special
// elements sorted out of the warps that run the general path.
//
// In the one-element-a-thread kernel (elem.cu) a warp whose lanes hold a
// NaN, an infinity or a zero factor runs those lanes' short special case
// and then the general path with them idle: with a tenth of each operand
// special, about a quarter of the lanes of every warp sit out the general
// path, which is nearly all of the time. Here a block takes a tile of T*K
// elements: each thread loads its K elements, classifies each from the
// exponent fields (arith_is_special) and copies its operands into one of
// two shared-memory queues, special cases from the front, general ones from
// the back (structure of 16-byte vectors, so a warp's accesses are
// conflict-free). After a block barrier the block's threads run the
// special queue, then the general queue, densely: every lane of a warp on
// the general path has general work. Values and flags are those of
// sf::arith for every element (the same functions, only the order of work
// differs).
#include <atomic>
#include <cstdlib>
#include <cstring>

#include "cftg_internal.h"
#include "elem_io.cuh"

namespace cftg {

namespace {

constexpr int Q_T = 256;

template <int FMT> struct QTile;
template <> struct QTile<2> { static constexpr int K = 4; };    // 1,024 elements, 48 KB
template <> struct QTile<3> { static constexpr int K = 2; };    // 512 elements, 48 KB

template <int FMT, int KIND>
__global__ void __launch_bounds__(Q_T) k_elem_q(const __grid_constant__ ElemLaunch L)
{
    constexpr int W = sf::Fmt<FMT>::W;
    constexpr int V = W / 4;                       // 16-byte vectors an operand
    constexpr int CAP = Q_T * QTile<FMT>::K;
    extern __shared__ uint4 qv[];                  // [3 * V][CAP] operand vectors
    __shared__ uint32_t qoff[CAP];
    __shared__ int nq[2];
    const int tid = threadIdx.x, lane = tid & 31;
    const unsigned lt = (1u << lane) - 1u;
    uint32_t acc = 0u;
    const size_t tiles = (L.n + CAP - 1) / CAP;
    for (size_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        if (tid < 2) nq[tid] = 0;
        __syncthreads();
        const size_t base = tile * CAP;
        // every element's operands first (K loads in flight a thread), then
        // the queues
        constexpr int K = QTile<FMT>::K;
        uint32_t a[K][W], b[K][W], c[K][W];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const size_t i = base + (size_t)k * Q_T + tid;
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
            const uint32_t off = (uint32_t)(k * Q_T + tid);
            const bool in = base + off < L.n;
            const bool sp = sf::arith_is_special<FMT, KIND>(a[k], b[k], c[k]);
            const bool qs = in && sp, qg = in && !sp;
            const unsigned ms = __ballot_sync(0xFFFFFFFFu, qs), mg = __ballot_sync(0xFFFFFFFFu, qg);
            int at = 0;
            if (lane == 0) {
                const int s0 = ms ? atomicAdd(&nq[0], __popc(ms)) : 0;
                const int g0 = mg ? atomicAdd(&nq[1], __popc(mg)) : 0;
                at = (s0 << 16) | g0;
            }
            at = __shfl_sync(0xFFFFFFFFu, at, 0);
            if (in) {
                const int slot = qs ? (at >> 16) + __popc(ms & lt)
                                    : CAP - 1 - ((at & 0xFFFF) + __popc(mg & lt));
                qoff[slot] = off;
#pragma unroll
                for (int v = 0; v < V; v++) {
                    qv[(0 * V + v) * CAP + slot] =
                        make_uint4(a[k][4 * v], a[k][4 * v + 1], a[k][4 * v + 2], a[k][4 * v + 3]);
                    qv[(1 * V + v) * CAP + slot] =
                        make_uint4(b[k][4 * v], b[k][4 * v + 1], b[k][4 * v + 2], b[k][4 * v + 3]);
                    qv[(2 * V + v) * CAP + slot] =
                        make_uint4(c[k][4 * v], c[k][4 * v + 1], c[k][4 * v + 2], c[k][4 * v + 3]);
                }
            }
        }
        __syncthreads();
        const int ns = nq[0], ng = nq[1];
        // both queues, specials first: slots [0, ns) and [CAP - ng, CAP)
        for (int j = tid; j < ns + ng; j += Q_T) {
            const int slot = j < ns ? j : CAP - ng + (j - ns);
            uint32_t a[W], b[W], c[W], o[W], fl;
#pragma unroll
            for (int v = 0; v < V; v++) {
                const uint4 x = qv[(0 * V + v) * CAP + slot];
                const uint4 y = qv[(1 * V + v) * CAP + slot];
                const uint4 z = qv[(2 * V + v) * CAP + slot];
                a[4 * v] = x.x; a[4 * v + 1] = x.y; a[4 * v + 2] = x.z; a[4 * v + 3] = x.w;
                b[4 * v] = y.x; b[4 * v + 1] = y.y; b[4 * v + 2] = y.z; b[4 * v + 3] = y.w;
                c[4 * v] = z.x; c[4 * v + 1] = z.y; c[4 * v + 2] = z.z; c[4 * v + 3] = z.w;
            }
            sf::arith<FMT, KIND>(a, b, c, L.rnd, o, fl);
            const size_t i = base + qoff[slot];
            store_elem<W>(static_cast<uint32_t *>(L.d), i, o);
            if (L.lane_flags) L.lane_flags[i] = (uint8_t)fl;
            acc |= fl;
        }
        __syncthreads();                              // the queues are rebuilt next tile
    }
    acc = __reduce_or_sync(0xFFFFFFFFu, acc);
    if (lane == 0 && acc) atomicOr(L.flags, acc);
}

template <int FMT, int KIND>
cudaError_t go_q(const ElemLaunch &L, cudaStream_t s)
{
    constexpr int W = sf::Fmt<FMT>::W;
    constexpr int CAP = Q_T * QTile<FMT>::K;
    constexpr size_t SMEM = (size_t)3 * (W / 4) * CAP * sizeof(uint4);
    // the shared-memory opt-in, once per device (a bit per device ordinal)
    static std::atomic<uint64_t> attr_done{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(attr_done.load() & bit)) {
        const cudaError_t e = cudaFuncSetAttribute(k_elem_q<FMT, KIND>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)SMEM);
        if (e != cudaSuccess) return e;
        attr_done.fetch_or(bit);
    }
    const size_t want = (L.n + CAP - 1) / CAP;
    const size_t cap = (size_t)sm_count() * (L.blocks_per_sm ? L.blocks_per_sm : 4u);
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    k_elem_q<FMT, KIND><<<blocks ? blocks : 1, Q_T, SMEM, s>>>(L);
    return cudaGetLastError();
}

template <int FMT>
cudaError_t go_q_kind(const ElemLaunch &L, cudaStream_t s)
{
    switch (L.kind) {
    case K_FMA: return go_q<FMT, K_FMA>(L, s);
    case K_ADD: return go_q<FMT, K_ADD>(L, s);
    case K_SUB: return go_q<FMT, K_SUB>(L, s);
    default: return go_q<FMT, K_MUL>(L, s);
    }
}

}  // namespace

// CFTG_ELEM_SORT=0 sends these launches to the one-element-a-thread
// kernels (for comparisons); read at every launch.
bool launch_elem_q(const ElemLaunch &L, cudaStream_t s, cudaError_t *err)
{
    if (L.fmt < 2 || L.kind > K_MUL) return false;
    const char *e = getenv("CFTG_ELEM_SORT");
    if (e && strcmp(e, "0") == 0) return false;
    *err = L.fmt == 2 ? go_q_kind<2>(L, s) : go_q_kind<3>(L, s);
    return true;
}

}  // namespace cftg
