// queue.h - the persistent work-queue's tables (shared by queue.cu and the
// host side in batch.cpp).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cftg {

// One call of a batch, as the kernel reads it.
struct QCall {
    const void *a, *b, *c;   // device pointers; NULL reads +0
    void *d;
    uint64_t n;
    int32_t fmt, kind, op, rnd;
    uint32_t scalar;         // bit r: operand r is element 0 for every i
    uint32_t pad;
};

// One tile: elements [start, start + len) of call `call`.
struct QTile {
    uint64_t start;
    uint32_t call, len;
};

cudaError_t launch_queue(const QCall *calls, const QTile *tiles, uint32_t ntiles, uint32_t *counter,
                         uint32_t *call_flags, int blocks, cudaStream_t s);
int queue_blocks_per_sm();

}  // namespace cftg
