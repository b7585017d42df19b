// batch.cpp - the batched form: many independent elementwise calls of
// uneven sizes, formats and operations as one persistent work-queue launch
// (queue.cu), optionally captured in a CUDA graph and replayed, with a tile
// length per (format, kind) chosen by an autotuner.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/cft_gb300.h"
#include "api_core.h"
#include "queue.h"

using namespace cftg;

namespace {

// relative cost of one element, per format and kind (FMA/ADD/SUB/MUL, DIV,
// SQRT, other): used to order tiles heaviest first
double cost(int fmt, int kind)
{
    static const double base[4] = {1.0, 2.0, 5.0, 13.0};
    const double k = (kind == K_DIV || kind == K_SQRT) ? 12.0 * (1 + fmt) : kind == K_SIMPLE ? 0.3 : 1.0;
    return base[fmt] * k;
}

// elements a tile, per (format, kind): the autotuner's table, with
// defaults that give every tile roughly the same amount of work
uint32_t g_tile[4][7];
bool g_tile_init = false;
// threads a block of the work-queue launch: the autotuner's choice (a
// block takes a whole tile, so a tile of t elements gives each thread
// t / threads of them)
int g_queue_threads = 256;

void tile_defaults()
{
    if (g_tile_init) return;
    for (int f = 0; f < 4; f++)
        for (int k = 0; k < 7; k++) {
            const double c = cost(f, k);
            uint32_t t = (uint32_t)(65536.0 / c);
            t = std::max<uint32_t>(256u, std::min<uint32_t>(65536u, t));
            g_tile[f][k] = (t + 255u) & ~255u;
        }
    g_tile_init = true;
}

}  // namespace

namespace cftg {
double queue_cost(int fmt, int kind) { return cost(fmt, kind); }
uint32_t queue_tile(int fmt, int kind)
{
    tile_defaults();
    return g_tile[fmt][kind];
}
}  // namespace cftg

struct cftg_batch {
    cft_device *dev = nullptr;
    QCall *d_calls = nullptr;
    QTile *d_tiles = nullptr;
    uint32_t *d_counter = nullptr;
    uint32_t *d_flags = nullptr;      // the caller's per-call words
    size_t ncalls = 0;
    uint32_t ntiles = 0;
    int blocks = 0, threads = 256;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" void cftg_batch_free(cftg_batch *b)
{
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_calls) cudaFree(b->d_calls);
    if (b->d_tiles) cudaFree(b->d_tiles);
    if (b->d_counter) cudaFree(b->d_counter);
    delete b;
}

extern "C" cft_status cftg_batch_create(cft_device *dev, const cftg_call *calls, size_t ncalls,
                                        uint32_t *d_call_flags, cftg_batch **out)
{
    clear_error();
    if (!dev || !out || (ncalls && (!calls || !d_call_flags))) {
        set_error("cftg_batch_create: a required pointer is NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    tile_defaults();
    std::vector<QCall> qc(ncalls);
    std::vector<QTile> tiles;
    for (size_t i = 0; i < ncalls; i++) {
        const cftg_call &c = calls[i];
        const int kind = c.kind == CFTG_KIND_DIV ? K_DIV : c.kind == CFTG_KIND_SQRT ? K_SQRT
                                                          : elem_kind_of_op(c.op);
        if (c.fmt < 0 || c.fmt > 3 || c.rnd < 0 || c.rnd > 4 || c.kind < 0 || c.kind > 2 ||
            (c.kind == CFTG_KIND_OP && (c.op < 0 || c.op > 255 || op_is_reduction(c.op))) ||
            (c.scalar_mask & ~7u)) {
            set_error("cftg_batch_create: call %lu has an argument out of range", (unsigned long)i);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        const unsigned need = c.kind == CFTG_KIND_DIV ? 3u : c.kind == CFTG_KIND_SQRT ? 1u
                                                                : op_operands(c.op);
        if (c.n && (!c.d || ((need & 1u) && !c.a) || ((need & 2u) && !c.b) ||
                    ((need & 4u) && !c.c))) {
            set_error("cftg_batch_create: call %lu lacks an operand its operation reads",
                      (unsigned long)i);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        qc[i] = QCall{c.a, c.b, c.c, c.d, (uint64_t)c.n, c.fmt, kind, c.op, c.rnd, c.scalar_mask, 0u};
        const uint32_t tl = g_tile[c.fmt][kind];
        for (uint64_t s = 0; s < c.n; s += tl)
            tiles.push_back(QTile{s, (uint32_t)i, (uint32_t)std::min<uint64_t>(tl, c.n - s)});
    }
    if (tiles.size() >= 0xFFFFFFFFull) {
        set_error("cftg_batch_create: the batch cuts into more than 2^32 tiles");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    // heaviest first
    std::stable_sort(tiles.begin(), tiles.end(), [&](const QTile &x, const QTile &y) {
        const QCall &cx = qc[x.call], &cy = qc[y.call];
        return cost(cx.fmt, cx.kind) * x.len > cost(cy.fmt, cy.kind) * y.len;
    });
    cftg_batch *b = new (std::nothrow) cftg_batch();
    if (!b) return CFT_ERR_OUT_OF_MEMORY;
    b->dev = dev;
    b->ncalls = ncalls;
    b->ntiles = (uint32_t)tiles.size();
    b->d_flags = d_call_flags;
    cudaSetDevice(dev->ordinal);
    bool ok = cudaMalloc(&b->d_calls, std::max<size_t>(1, ncalls) * sizeof(QCall)) == cudaSuccess &&
              cudaMalloc(&b->d_tiles, std::max<size_t>(1, tiles.size()) * sizeof(QTile)) == cudaSuccess &&
              cudaMalloc(&b->d_counter, sizeof(uint32_t)) == cudaSuccess;
    if (ok && ncalls)
        ok = cudaMemcpy(b->d_calls, qc.data(), ncalls * sizeof(QCall), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok && !tiles.empty())
        ok = cudaMemcpy(b->d_tiles, tiles.data(), tiles.size() * sizeof(QTile),
                        cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cftg_batch_free(b);
        set_error("cftg_batch_create: could not place the batch's tables on the device");
        return CFT_ERR_OUT_OF_MEMORY;
    }
    b->threads = g_queue_threads;
    b->blocks = sm_count() * queue_blocks_per_sm(b->threads);
    *out = b;
    return CFT_OK;
}

static cudaError_t enqueue(cftg_batch *b, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(b->d_counter, 0, sizeof(uint32_t), s);
    if (e == cudaSuccess && b->ncalls) e = cudaMemsetAsync(b->d_flags, 0, b->ncalls * sizeof(uint32_t), s);
    if (e == cudaSuccess)
        e = launch_queue(b->d_calls, b->d_tiles, b->ntiles, b->d_counter, b->d_flags, b->blocks,
                         b->threads, s);
    return e;
}

extern "C" cft_status cftg_batch_capture(cftg_batch *b, void *stream)
{
    clear_error();
    if (!b) return CFT_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (!s) {
        set_error("cftg_batch_capture: capture needs a stream other than the legacy default");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (b->exec) return CFT_OK;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e2 = enqueue(b, s);
        e = cudaStreamEndCapture(s, &b->graph);
        if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cftg_batch_capture: %s", cudaGetErrorString(e));
        return CFT_ERR_INTERNAL;
    }
    return CFT_OK;
}

extern "C" cft_status cftg_batch_launch(cftg_batch *b, void *stream)
{
    clear_error();
    if (!b) return CFT_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = b->exec ? cudaGraphLaunch(b->exec, s) : enqueue(b, s);
    if (e != cudaSuccess) return poison(b->dev, "cftg_batch_launch", e);
    return CFT_OK;
}

extern "C" uint32_t cftg_batch_tiles(const cftg_batch *b) { return b ? b->ntiles : 0u; }

// The autotuner, in two passes over the caller's device buffers (sized for
// n elements of fp256; their contents are the operands): first, for each
// (format, kind), the queue over one call at each candidate tile length,
// keeping the fastest; then the launch's block shape, 128 or 256 threads
// (the resident blocks an SM follow from occupancy), keeping the one whose
// summed time over the same calls, at their chosen tiles, is least.
extern "C" cft_status cftg_autotune(cft_device *dev, const void *d_a, const void *d_b,
                                    const void *d_c, void *d_d, size_t n, void *stream)
{
    clear_error();
    if (!dev || !d_a || !d_b || !d_c || !d_d || n < 4096) {
        set_error("cftg_autotune: needs a device and four device buffers of n >= 4096 elements");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    tile_defaults();
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *d_fl = nullptr;
    if (cudaMalloc(&d_fl, 64 * sizeof(uint32_t)) != cudaSuccess) return CFT_ERR_OUT_OF_MEMORY;
    static const uint32_t cand[6] = {256, 1024, 4096, 16384, 65536, 262144};
    static const int shapes[2] = {128, 256};
    const int kinds[4][2] = {{CFTG_KIND_OP, 0}, {CFTG_KIND_OP, 1}, {CFTG_KIND_DIV, 0}, {CFTG_KIND_SQRT, 0}};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // ms of three queue launches over one call of m elements (warm first)
    auto time_call = [&](int f, const int (&kk)[2], size_t m) -> float {
        cftg_call c;
        memset(&c, 0, sizeof c);
        c.kind = kk[0];
        c.op = kk[1];
        c.fmt = f;
        c.a = d_a;
        c.b = d_b;
        c.c = d_c;
        c.d = d_d;
        c.n = m;
        cftg_batch *b = nullptr;
        if (cftg_batch_create(dev, &c, 1, d_fl, &b) != CFT_OK) return 1e30f;
        enqueue(b, s);
        cudaEventRecord(e0, s);
        for (int r = 0; r < 3; r++) enqueue(b, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cftg_batch_free(b);
        return ms;
    };
    // fewer elements for the costly ones keeps the tuning quick
    auto elems = [&](int f, int kind) {
        size_t m = std::min(n, (size_t)(4u << 20) / (size_t)(cost(f, kind) > 20 ? 32 : 1));
        return std::max<size_t>(m, 4096);
    };
    auto kind_of = [](const int (&kk)[2]) {
        return kk[0] == CFTG_KIND_DIV ? K_DIV : kk[0] == CFTG_KIND_SQRT ? K_SQRT : elem_kind_of_op(kk[1]);
    };
    g_queue_threads = 256;
    for (int f = 0; f < 4; f++) {
        for (auto &kk : kinds) {
            const int kind = kind_of(kk);
            const size_t m = elems(f, kind);
            float best = 1e30f;
            uint32_t bestt = g_tile[f][kind];
            for (uint32_t t : cand) {
                if (t > m) break;
                g_tile[f][kind] = t;
                const float ms = time_call(f, kk, m);
                if (ms < best) {
                    best = ms;
                    bestt = t;
                }
            }
            g_tile[f][kind] = bestt;
            if (kind == K_FMA) {                           // ADD/SUB/MUL follow FMA's
                g_tile[f][K_SUB] = bestt;
                g_tile[f][K_MUL] = bestt;
            }
        }
    }
    float best_sum = 1e30f;
    int best_shape = 256;
    for (int th : shapes) {
        g_queue_threads = th;
        float sum = 0.f;
        for (int f = 0; f < 4; f++)
            for (auto &kk : kinds) sum += time_call(f, kk, elems(f, kind_of(kk)));
        if (sum < best_sum) {
            best_sum = sum;
            best_shape = th;
        }
    }
    g_queue_threads = best_shape;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_fl);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return poison(dev, "cftg_autotune", e);
    return CFT_OK;
}

extern "C" int cftg_queue_block_threads(void) { return g_queue_threads; }

extern "C" cft_status cftg_set_queue_block_threads(int threads)
{
    clear_error();
    if (threads < 32 || threads > 256 || threads % 32) {
        set_error("cftg_set_queue_block_threads: %d is not a multiple of 32 in 32..256", threads);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    g_queue_threads = threads;
    return CFT_OK;
}

extern "C" uint32_t cftg_tile_length(int fmt, int kind, int op)
{
    tile_defaults();
    if (fmt < 0 || fmt > 3) return 0;
    const int k = kind == CFTG_KIND_DIV ? K_DIV : kind == CFTG_KIND_SQRT ? K_SQRT : elem_kind_of_op(op);
    return g_tile[fmt][k];
}
