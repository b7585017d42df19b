// aug.cu - the augmented operations' elementwise kernel: one element pair a
// thread, grid-stride, both results written after both operands are read
// (so r or e may alias a or b), flags ORed into one device word.
#include "aug.cuh"
#include "cftg_internal.h"

namespace cftg {

namespace {

template <int W>
SFD void aload(const void *p, size_t i, uint32_t (&x)[W])
{
    const uint32_t *q = static_cast<const uint32_t *>(p) + i * W;
#pragma unroll
    for (int w = 0; w < W; w++) x[w] = q[w];
}

template <int FMT>
__global__ void k_aug(int fn, const void *a, const void *b, void *r, void *e, size_t n,
                      uint32_t *word)
{
    constexpr int W = sf::Fmt<FMT>::W;
    uint32_t acc = 0u;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t x[W], y[W], vr[W], ve[W], fl = 0u;
        aload<W>(a, i, x);
        aload<W>(b, i, y);
        sf::augmented<FMT>(fn, x, y, vr, ve, fl);
        uint32_t *pr = static_cast<uint32_t *>(r) + i * W;
        uint32_t *pe = static_cast<uint32_t *>(e) + i * W;
#pragma unroll
        for (int w = 0; w < W; w++) {
            pr[w] = vr[w];
            pe[w] = ve[w];
        }
        acc |= fl;
    }
    acc = __reduce_or_sync(__activemask(), acc);
    if ((threadIdx.x & 31) == 0 && acc) atomicOr(word, acc);
}

}  // namespace

cudaError_t launch_aug(int fmt, int fn, const void *a, const void *b, void *r, void *e, size_t n,
                       uint32_t *word, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const size_t want = (n + 255) / 256;
    const unsigned blocks = (unsigned)(want < (size_t)sm_count() * 8 ? want : (size_t)sm_count() * 8);
    switch (fmt) {
    case 0: k_aug<0><<<blocks, 256, 0, s>>>(fn, a, b, r, e, n, word); break;
    case 1: k_aug<1><<<blocks, 256, 0, s>>>(fn, a, b, r, e, n, word); break;
    case 2: k_aug<2><<<blocks, 256, 0, s>>>(fn, a, b, r, e, n, word); break;
    default: k_aug<3><<<blocks, 256, 0, s>>>(fn, a, b, r, e, n, word); break;
    }
    return cudaGetLastError();
}

}  // namespace cftg
