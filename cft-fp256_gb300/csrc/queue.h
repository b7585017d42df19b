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
    uint32_t tile;           // elements a tile (k_queue_calls only)
};

// One tile: elements [start, start + len) of call `call`.
struct QTile {
    uint64_t start;
    uint32_t call, len;
};

// k_queue over `blocks` blocks of `threads` (a multiple of 32, <= 256)
cudaError_t launch_queue(const QCall *calls, const QTile *tiles, uint32_t ntiles, uint32_t *counter,
                         uint32_t *call_flags, int blocks, int threads, cudaStream_t s);
// k_queue blocks of `threads` one SM holds
int queue_blocks_per_sm(int threads);
// Registers a thread of the table-free work-queue kernel uses.
int queue_calls_regs();

// The same work queue without a tile table: call i owns tiles
// [prefix[i], prefix[i+1]) of `tile` elements each (the last one short), so
// a batch costs the host O(calls) to describe. prefix has ncalls+1 entries.
cudaError_t launch_queue_calls(const QCall *calls, const uint32_t *prefix, uint32_t ncalls,
                               uint32_t *counter, uint32_t *call_flags, int blocks, cudaStream_t s);

// The tile table the batched forms share: elements a tile per (format,
// kind), the autotuner's choice once it has run, and a relative cost of
// one element used to order tiles heaviest first.
uint32_t queue_tile(int fmt, int kind);
double queue_cost(int fmt, int kind);

}  // namespace cftg
