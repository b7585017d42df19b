// traj.cpp - the batched sequencer: thousands of trajectories of uneven
// length (a lane runs its program `segments[lane]` times, state carried
// through the scratch block) as ONE launch, optionally recorded in a CUDA
// graph. The reference runs such a workload as one cft_program_run_ex per
// segment with the scratch-out block fed back as the next scratch-in
// (its segmented runner, host/tools/segrun.c); each lane's runs here are
// those same runs, so every state is the one that loop produces.
#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "../../include/cft_gb300.h"
#include "api_core.h"
#include "bundle.h"

using namespace cftg;

struct cftg_traj {
    cft_device *dev = nullptr;
    TrajLaunch L;
    uint32_t *d_segments = nullptr, *d_order = nullptr, *d_word = nullptr;
    void *d_scratch = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" void cftg_traj_free(cftg_traj *t)
{
    if (!t) return;
    if (t->exec) cudaGraphExecDestroy(t->exec);
    if (t->graph) cudaGraphDestroy(t->graph);
    if (t->d_segments) cudaFree(t->d_segments);
    if (t->d_order) cudaFree(t->d_order);
    if (t->d_word) cudaFree(t->d_word);
    if (t->d_scratch) cudaFree(t->d_scratch);
    delete t;
}

extern "C" cft_status cftg_traj_create(cft_program *prog, const uint32_t *segments, size_t n,
                                       const void *d_a, const void *d_b, const void *d_c,
                                       const void *d_bank, void *d_state, void *d_snaps,
                                       uint32_t snap_every, uint32_t max_snaps,
                                       uint8_t *d_lane_flags, cftg_traj **out)
{
    clear_error();
    cft_device *dev = nullptr;
    const SeqProgram *pp = program_seq(prog, &dev);
    if (!pp || !out || (n && (!segments || !d_a))) {
        set_error("cftg_traj_create: prog, out, segments and a are required");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    const SeqProgram &P = *pp;
    if (P.max_deposits) {
        set_error("cftg_traj_create: the program deposits (max_deposits = %u); a trajectory run "
                  "carries state through its scratch block and collects no deposits",
                  P.max_deposits);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (P.n_scratch_in != P.n_scratch_out) {
        set_error("cftg_traj_create: the program's scratch block is %u in and %u out; a "
                  "trajectory feeds one run's block to the next, so the two must be equal",
                  P.n_scratch_in, P.n_scratch_out);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (P.n_scratch_out && !d_state) {
        set_error("cftg_traj_create: the state block (n x %u elements) is NULL", P.n_scratch_out);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if ((P.flags & CFT_PROG_FLAG_BANK_EXT) && P.n_consts && !d_bank) {
        set_error("cftg_traj_create: the program's constants arrive per run and d_bank is NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (d_snaps && (!snap_every || !max_snaps)) {
        set_error("cftg_traj_create: snapshots need snap_every and max_snaps");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cftg_traj *t = new (std::nothrow) cftg_traj();
    if (!t) return CFT_ERR_OUT_OF_MEMORY;
    t->dev = dev;
    // longest first, so a warp's lanes have similar lengths
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t x, uint32_t y) { return segments[x] > segments[y]; });
    const size_t esz = esz_of(P.fmt);
    cudaSetDevice(dev->ordinal);
    bool ok = cudaMalloc(&t->d_segments, std::max<size_t>(1, n) * 4) == cudaSuccess &&
              cudaMalloc(&t->d_order, std::max<size_t>(1, n) * 4) == cudaSuccess &&
              cudaMalloc(&t->d_word, 4 * sizeof(uint32_t)) == cudaSuccess;
    if (ok && P.reach)
        ok = cudaMalloc(&t->d_scratch, std::max<size_t>(1, n) * P.reach * esz) == cudaSuccess;
    if (ok && n)
        ok = cudaMemcpy(t->d_segments, segments, n * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(t->d_order, order.data(), n * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cftg_traj_free(t);
        set_error("cftg_traj_create: could not allocate the run's device tables and scratch");
        return CFT_ERR_OUT_OF_MEMORY;
    }
    TrajLaunch &L = t->L;
    L.P = P;
    if (P.flags & CFT_PROG_FLAG_BANK_EXT) L.P.d_consts = d_bank;
    L.n = n;
    L.a = d_a;
    L.b = d_b;
    L.c = d_c;
    L.segments = t->d_segments;
    L.order = t->d_order;
    L.state = d_state;
    L.snaps = d_snaps;
    L.snap_every = snap_every;
    L.max_snaps = max_snaps;
    L.scratch = t->d_scratch;
    L.lane_flags = d_lane_flags;
    L.word = t->d_word;
    std::vector<uint32_t> runs_desc(n);
    for (size_t i = 0; i < n; i++) runs_desc[i] = segments[order[i]];
    plan_lanes(prog, n, L, n ? runs_desc.data() : nullptr);
    *out = t;
    return CFT_OK;
}

static cudaError_t traj_enqueue(cftg_traj *t, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(t->d_word, 0, 4 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = launch_traj(t->L, s);
    return e;
}

extern "C" cft_status cftg_traj_capture(cftg_traj *t, void *stream)
{
    clear_error();
    if (!t || !stream) {
        set_error("cftg_traj_capture: needs a run and a stream other than the legacy default");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (t->exec) return CFT_OK;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e2 = traj_enqueue(t, s);
        e = cudaStreamEndCapture(s, &t->graph);
        if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&t->exec, t->graph, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cftg_traj_capture: %s", cudaGetErrorString(e));
        return CFT_ERR_INTERNAL;
    }
    return CFT_OK;
}

extern "C" cft_status cftg_traj_launch(cftg_traj *t, void *stream)
{
    clear_error();
    if (!t) return CFT_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = t->exec ? cudaGraphLaunch(t->exec, s) : traj_enqueue(t, s);
    if (e != cudaSuccess) return poison(t->dev, "cftg_traj_launch", e);
    return CFT_OK;
}

// Wait for the run on `stream` and report its flags and STATUS (the
// handle's status word takes the flags, as every run's do).
extern "C" cft_status cftg_traj_result(cftg_traj *t, uint32_t *flags_out, uint32_t *status_out,
                                       void *stream)
{
    clear_error();
    if (!t) return CFT_ERR_INVALID_ARGUMENT;
    uint32_t w[4] = {0, 0, 0, 0};
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(w, t->d_word, sizeof w, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return poison(t->dev, "cftg_traj_result", e);
    if (w[2]) {
        set_error("cftg_traj_result: the executor reported invariant failure 0x%x", w[2]);
        return CFT_ERR_INTERNAL;
    }
    flags_emit(t->dev, w[0] & CFT_FLAGS_ALL, flags_out);
    if (status_out) *status_out = w[1];
    return CFT_OK;
}

// Several trajectory runs (of different programs and formats) recorded as
// one CUDA graph: every run an independent branch, so one graph launch puts
// them all on the device at once and they share the SMs.
struct cftg_traj_group {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" void cftg_traj_group_free(cftg_traj_group *g)
{
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
}

extern "C" cft_status cftg_traj_group_capture(cftg_traj *const *runs, size_t count, void *stream,
                                              cftg_traj_group **out)
{
    clear_error();
    if (!out || !runs || !count || !stream) {
        set_error("cftg_traj_group_capture: needs runs, a count, a stream other than the legacy "
                  "default and out");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    for (size_t i = 0; i < count; i++)
        if (!runs[i] || runs[i]->dev != runs[0]->dev) {
            set_error("cftg_traj_group_capture: run %zu is NULL or on another device", i);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    cftg_traj_group *g = new (std::nothrow) cftg_traj_group();
    if (!g) return CFT_ERR_OUT_OF_MEMORY;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<cudaStream_t> side(count, nullptr);
    std::vector<cudaEvent_t> join(count, nullptr);
    cudaEvent_t fork = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    for (size_t i = 1; e == cudaSuccess && i < count; i++) {
        e = cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        // fork: every run after the first on its own captured stream, the
        // first on `stream`; then join them all back into `stream`
        cudaError_t e2 = cudaEventRecord(fork, s);
        for (size_t i = 1; e2 == cudaSuccess && i < count; i++) {
            e2 = cudaStreamWaitEvent(side[i], fork, 0);
            if (e2 == cudaSuccess) e2 = traj_enqueue(runs[i], side[i]);
            if (e2 == cudaSuccess) e2 = cudaEventRecord(join[i], side[i]);
        }
        if (e2 == cudaSuccess) e2 = traj_enqueue(runs[0], s);
        for (size_t i = 1; e2 == cudaSuccess && i < count; i++) e2 = cudaStreamWaitEvent(s, join[i], 0);
        e = cudaStreamEndCapture(s, &g->graph);
        if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    for (size_t i = 1; i < count; i++) {
        if (join[i]) cudaEventDestroy(join[i]);
        if (side[i]) cudaStreamDestroy(side[i]);
    }
    if (fork) cudaEventDestroy(fork);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cftg_traj_group_free(g);
        set_error("cftg_traj_group_capture: %s", cudaGetErrorString(e));
        return CFT_ERR_INTERNAL;
    }
    *out = g;
    return CFT_OK;
}

extern "C" cft_status cftg_traj_group_launch(cftg_traj_group *g, void *stream)
{
    clear_error();
    if (!g || !g->exec) return CFT_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cftg_traj_group_launch: %s", cudaGetErrorString(e));
        return CFT_ERR_INTERNAL;
    }
    return CFT_OK;
}
