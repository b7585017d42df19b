// serve.cpp - the serving loop: continuous batching of element calls and
// program (trajectory) requests of mixed formats and sizes, with their data
// resident in HBM and admission by a device-memory budget.
//
// One engine thread owns the device side. Each turn it (1) retires batches
// whose completion event has fired, freeing their memory and posting their
// requests' completions, (2) admits waiting requests, first come first
// served per class, while a batch slot and budget are free, and (3) launches
// each admitted group at once on the slot's own stream: element calls as
// one work-queue launch (the batched form's kernel and tile table),
// requests of one program as one trajectory launch. Up to max_inflight
// element batches and max_program_inflight program batches are on the
// device together, so requests that arrive while others run are admitted
// and overlap them instead of queueing behind them.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <numeric>
#include <thread>
#include <vector>

#include "../../include/cft_gb300.h"
#include "api_core.h"
#include "arena.h"
#include "bundle.h"
#include "queue.h"

using namespace cftg;

namespace {

constexpr size_t SERVE_INIT_STAGING = 16u << 20;   // a program slot's pinned initial blocks

uint64_t now_ns()
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Req {
    cftg_request r;
    std::vector<uint8_t> init;      // program requests: the initial blocks
    int kind = 0;                   // element kind (K_*) of an element request
    size_t esz = 0, out_bytes = 0, dev_bytes = 0;
    size_t off = 0;                 // element requests: the output's arena offset
    const SeqProgram *P = nullptr;
    bool out_pinned = false;        // host_out readable by an async copy
    void *out_dev = nullptr;        // host_out as the GPU addresses it, or NULL
    bool early = false;             // program request completed before its batch
    uint64_t t_arrival = 0, t_admit = 0;
};

struct Slot {
    bool busy = false, program = false;
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    uint32_t id = 0;
    // element batch tables
    QCall *h_calls = nullptr, *d_calls = nullptr;
    uint32_t *h_prefix = nullptr, *d_prefix = nullptr;
    uint32_t *d_counter = nullptr, *d_flags = nullptr, *h_flags = nullptr;
    // program batch tables
    uint32_t *h_seg = nullptr, *d_seg = nullptr, *h_order = nullptr, *d_order = nullptr;
    uint32_t *h_lstatus = nullptr, *d_lstatus = nullptr, *d_word = nullptr, *h_word = nullptr;
    uint8_t *h_lflags = nullptr, *d_lflags = nullptr;
    uint8_t *h_init = nullptr;       // pinned staging of the initial blocks
    size_t h_init_cap = 0;
    // completion a request at a time (TrajLaunch::req_of): per lane its
    // request; per request its first lane, lanes left, flags/STATUS and
    // output; the done records in mapped host memory
    uint32_t *h_req_of = nullptr, *d_req_of = nullptr;
    uint32_t *h_req_lane0 = nullptr, *d_req_lane0 = nullptr;
    uint32_t *h_req_left = nullptr, *d_req_left = nullptr, *d_req_acc = nullptr;
    void **h_req_out = nullptr, **d_req_out = nullptr;
    uint32_t *h_done = nullptr, *d_done = nullptr;
    size_t req_cap = 0;
    size_t prog_off = 0, prog_bytes = 0;
    std::vector<Req *> reqs;
    std::vector<size_t> lane0;
};

}  // namespace

struct cftg_server {
    cft_device *dev = nullptr;
    cftg_server_config cfg{};
    void *base = nullptr;           // the budget's device region
    Arena arena;
    std::vector<Slot> slots;        // [0, max_inflight) element, the rest program
    // Few streams, shared by the slots: a GPU runs work from a handful of
    // hardware queues, and streams beyond them share one - so a short
    // element batch could wait behind a long trajectory launch that merely
    // shares its queue. Two element streams (ahead in priority) and up to
    // three program streams stay within the queues.
    std::vector<cudaStream_t> streams;
    int queue_blocks = 0;
    // The registers and shared memory of an SM that trajectory blocks may
    // take: what the element batches' blocks leave. Each trajectory launch
    // asks its blocks for shared memory so that no more of them fit than
    // these registers hold, so element blocks always find room beside them,
    // however many program batches are in flight.
    uint32_t traj_sm_regs = 0, traj_sm_smem = 0;

    std::mutex mu;                  // intake, completions, counters below
    std::condition_variable cv_in, cv_done;
    std::deque<Req *> intake;
    std::vector<cftg_completion> done;
    bool stop = false, failed = false;
    cftg_server_stats st{};

    std::deque<Req *> elem_q, prog_q;   // engine thread only
    uint32_t batch_id = 0;
    std::thread th;

    void loop();
    bool launch_elem(Slot &sl);
    bool launch_prog(Slot &sl);
    void retire(Slot &sl, cudaError_t e);
    bool early_completions(Slot &sl);
    void complete(Req *q, int32_t result, uint32_t flags, uint32_t status, uint32_t batch,
                  uint64_t t_done, bool release = true);
};

void cftg_server::complete(Req *q, int32_t result, uint32_t flags, uint32_t status, uint32_t batch,
                           uint64_t t_done, bool release)
{
    cftg_completion c;
    memset(&c, 0, sizeof c);
    c.tag = q->r.tag;
    c.result = result;
    c.flags = flags;
    c.status = status;
    c.batch = batch;
    c.t_arrival_ns = q->t_arrival;
    c.t_admit_ns = q->t_admit;
    c.t_done_ns = t_done;
    std::lock_guard<std::mutex> g(mu);
    done.push_back(c);
    st.completed++;
    if (result != CFT_OK) st.failed++;
    else if (q->r.type == CFTG_REQ_ELEM) st.elements_done += q->r.n;
    else st.lane_runs_done += (uint64_t)q->r.lanes * q->r.runs;
    if (release) delete q;
    cv_done.notify_all();
}

// A program request whose output the GPU writes completes when its last lane
// has finished, not when its batch has: the trajectory kernel marks it done
// in the slot's mapped records (TrajLaunch::req_of).
static bool completes_early(const Req *q) { return !q->r.host_out || q->out_dev; }

bool cftg_server::early_completions(Slot &sl)
{
    bool any = false;
    for (size_t i = 0; i < sl.reqs.size(); i++) {
        Req *q = sl.reqs[i];
        if (q->early || !completes_early(q)) continue;
        const volatile uint32_t *d = sl.h_done + 4 * i;
        if (!d[2]) continue;
        std::atomic_thread_fence(std::memory_order_acquire);
        q->early = true;
        complete(q, CFT_OK, d[0] & CFT_FLAGS_ALL, d[1], sl.id, now_ns(), false);
        any = true;
    }
    return any;
}

// Element batch: requests taken from the head of elem_q while calls and
// budget last; at least one, or nothing when the head does not fit the free
// budget yet. The batch's calls are ordered heaviest first and described to
// the kernel by a prefix of their tile counts (no tile table to build).
bool cftg_server::launch_elem(Slot &sl)
{
    sl.reqs.clear();
    const uint64_t t = now_ns();
    uint64_t elems = 0;
    while (!elem_q.empty() && sl.reqs.size() < cfg.max_batch_calls) {
        Req *q = elem_q.front();
        if (cfg.max_batch_elements && !sl.reqs.empty() && elems + q->r.n > cfg.max_batch_elements) break;
        if (!arena.alloc(q->out_bytes, &q->off)) break;
        elems += q->r.n;
        elem_q.pop_front();
        q->t_admit = t;
        sl.reqs.push_back(q);
    }
    if (sl.reqs.empty()) return false;
    std::stable_sort(sl.reqs.begin(), sl.reqs.end(), [](const Req *x, const Req *y) {
        return queue_cost(x->r.fmt, x->kind) * (double)x->r.n > queue_cost(y->r.fmt, y->kind) * (double)y->r.n;
    });
    const size_t k = sl.reqs.size();
    uint64_t tiles = 0;
    for (size_t i = 0; i < k; i++) {
        Req *q = sl.reqs[i];
        const uint32_t tl = queue_tile(q->r.fmt, q->kind);
        QCall &c = sl.h_calls[i];
        c.a = q->r.d_a;
        c.b = q->r.d_b;
        c.c = q->r.d_c;
        c.d = static_cast<uint8_t *>(base) + q->off;
        c.n = q->r.n;
        c.fmt = q->r.fmt;
        c.kind = q->kind;
        c.op = q->r.op;
        c.rnd = q->r.rnd;
        c.scalar = 0u;
        c.tile = tl;
        sl.h_prefix[i] = (uint32_t)tiles;
        tiles += (q->r.n + tl - 1) / tl;
    }
    sl.h_prefix[k] = (uint32_t)tiles;
    const int blocks = (int)std::min<uint64_t>((uint64_t)queue_blocks, std::max<uint64_t>(1, tiles));
    cudaError_t e = cudaMemcpyAsync(sl.d_calls, sl.h_calls, k * sizeof(QCall), cudaMemcpyHostToDevice, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.d_prefix, sl.h_prefix, (k + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, sl.s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_counter, 0, sizeof(uint32_t), sl.s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_flags, 0, k * sizeof(uint32_t), sl.s);
    if (e == cudaSuccess)
        e = launch_queue_calls(sl.d_calls, sl.d_prefix, (uint32_t)k, sl.d_counter, sl.d_flags, blocks, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.h_flags, sl.d_flags, k * sizeof(uint32_t), cudaMemcpyDeviceToHost, sl.s);
    for (size_t i = 0; e == cudaSuccess && i < k; i++) {
        Req *q = sl.reqs[i];
        if (q->r.host_out && q->out_pinned)
            e = cudaMemcpyAsync(q->r.host_out, static_cast<uint8_t *>(base) + q->off, q->out_bytes,
                                cudaMemcpyDeviceToHost, sl.s);
    }
    if (e == cudaSuccess) e = cudaEventRecord(sl.ev, sl.s);
    sl.busy = true;
    sl.program = false;
    sl.id = ++batch_id;
    {
        std::lock_guard<std::mutex> g(mu);
        st.batches++;
        st.launches++;
        st.bytes_in_use = arena.used();
        st.bytes_peak = arena.peak();
    }
    if (e != cudaSuccess) retire(sl, e);
    return true;
}

// Program batch: the head request's program and bank, and every waiting
// request of the same program and bank behind it (in order) while lanes
// and budget last, as one trajectory launch.
bool cftg_server::launch_prog(Slot &sl)
{
    sl.reqs.clear();
    sl.lane0.clear();
    if (prog_q.empty()) return false;
    Req *head = prog_q.front();
    const SeqProgram &P = *head->P;
    const size_t esz = head->esz;
    const size_t per_lane = (size_t)(P.n_scratch_out + P.reach) * esz;
    const size_t state_lane = (size_t)P.n_scratch_out * esz;
    size_t lanes = 0;
    std::vector<Req *> take;
    for (auto it = prog_q.begin(); it != prog_q.end();) {
        Req *q = *it;
        if (q->r.prog != head->r.prog || q->r.d_bank != head->r.d_bank) {
            ++it;
            continue;
        }
        if (!take.empty() && (lanes + q->r.lanes > cfg.max_batch_lanes || take.size() >= sl.req_cap ||
                              (lanes + q->r.lanes) * state_lane > sl.h_init_cap))
            break;
        take.push_back(q);
        lanes += q->r.lanes;
        it = prog_q.erase(it);
        if (lanes >= cfg.max_batch_lanes) break;
    }
    // the largest prefix of the group the free budget holds (the head alone
    // at least, or nothing yet); the rest go back to the front of the queue
    size_t keep = take.size();
    for (;;) {
        if (arena.alloc(lanes * per_lane, &sl.prog_off)) break;
        if (keep == 1) {
            for (auto r = take.rbegin(); r != take.rend(); ++r) prog_q.push_front(*r);
            return false;
        }
        keep = (keep + 1) / 2;
        lanes = 0;
        for (size_t i = 0; i < keep; i++) lanes += take[i]->r.lanes;
    }
    for (size_t i = take.size(); i-- > keep;) prog_q.push_front(take[i]);
    take.resize(keep);
    const size_t bytes = lanes * per_lane;
    sl.prog_bytes = bytes;
    const uint64_t t = now_ns();
    uint8_t *state = static_cast<uint8_t *>(base) + sl.prog_off;
    uint8_t *scratch = state + lanes * P.n_scratch_out * esz;
    // the initial blocks through the slot's pinned staging (allocated once:
    // freeing pinned memory would wait for the whole device), so the copy is
    // truly asynchronous on a stream other batches share
    const size_t init_bytes = lanes * P.n_scratch_out * esz;
    cudaError_t e = cudaSuccess;
    size_t l = 0;
    for (Req *q : take) {
        q->t_admit = t;
        const size_t ri = sl.reqs.size();
        sl.reqs.push_back(q);
        sl.lane0.push_back(l);
        for (size_t j = 0; j < q->r.lanes; j++) {
            sl.h_seg[l + j] = q->r.runs;
            sl.h_req_of[l + j] = (uint32_t)ri;
        }
        sl.h_req_lane0[ri] = (uint32_t)l;
        sl.h_req_left[ri] = (uint32_t)q->r.lanes;
        sl.h_req_out[ri] = q->r.host_out ? q->out_dev : nullptr;
        memset(sl.h_done + 4 * ri, 0, 4 * sizeof(uint32_t));
        if (e == cudaSuccess && !q->init.empty())
            memcpy(sl.h_init + l * P.n_scratch_out * esz, q->init.data(), q->init.size());
        l += q->r.lanes;
    }
    if (e == cudaSuccess && init_bytes)
        e = cudaMemcpyAsync(state, sl.h_init, init_bytes, cudaMemcpyHostToDevice, sl.s);
    std::iota(sl.h_order, sl.h_order + lanes, 0u);
    std::stable_sort(sl.h_order, sl.h_order + lanes,
                     [&](uint32_t x, uint32_t y) { return sl.h_seg[x] > sl.h_seg[y]; });
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.d_seg, sl.h_seg, lanes * 4, cudaMemcpyHostToDevice, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.d_order, sl.h_order, lanes * 4, cudaMemcpyHostToDevice, sl.s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_word, 0, 4 * sizeof(uint32_t), sl.s);
    const size_t nreq = sl.reqs.size();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.d_req_of, sl.h_req_of, lanes * 4, cudaMemcpyHostToDevice, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.d_req_lane0, sl.h_req_lane0, nreq * 4, cudaMemcpyHostToDevice, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.d_req_left, sl.h_req_left, nreq * 4, cudaMemcpyHostToDevice, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.d_req_out, sl.h_req_out, nreq * sizeof(void *), cudaMemcpyHostToDevice,
                            sl.s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_req_acc, 0, nreq * 2 * 4, sl.s);
    TrajLaunch T;
    T.P = P;
    if (P.flags & CFT_PROG_FLAG_BANK_EXT) T.P.d_consts = head->r.d_bank;
    T.n = lanes;
    T.segments = sl.d_seg;
    T.order = sl.d_order;
    T.state = state;
    T.scratch = P.reach ? scratch : nullptr;
    T.lane_flags = sl.d_lflags;
    T.lane_status = sl.d_lstatus;
    T.word = sl.d_word;
    T.req_of = sl.d_req_of;
    T.req_lane0 = sl.d_req_lane0;
    T.req_left = sl.d_req_left;
    T.req_acc = sl.d_req_acc;
    T.req_done = sl.d_done;
    T.req_out = sl.d_req_out;
    plan_lanes(head->r.prog, lanes, T);
    T.sm_regs = traj_sm_regs;
    T.sm_smem = traj_sm_smem;
    if (e == cudaSuccess) e = launch_traj(T, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.h_lflags, sl.d_lflags, lanes, cudaMemcpyDeviceToHost, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.h_lstatus, sl.d_lstatus, lanes * 4, cudaMemcpyDeviceToHost, sl.s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.h_word, sl.d_word, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, sl.s);
    for (size_t i = 0; e == cudaSuccess && i < sl.reqs.size(); i++) {
        Req *q = sl.reqs[i];
        if (q->r.host_out && q->out_pinned && !q->out_dev)    // the kernel writes the others
            e = cudaMemcpyAsync(q->r.host_out, state + sl.lane0[i] * P.n_scratch_out * esz,
                                q->out_bytes, cudaMemcpyDeviceToHost, sl.s);
    }
    if (e == cudaSuccess) e = cudaEventRecord(sl.ev, sl.s);
    sl.busy = true;
    sl.program = true;
    sl.id = ++batch_id;
    {
        std::lock_guard<std::mutex> g(mu);
        st.batches++;
        st.launches++;
        st.bytes_in_use = arena.used();
        st.bytes_peak = arena.peak();
    }
    if (e != cudaSuccess) retire(sl, e);
    return true;
}

// The slot's work has finished (e == cudaSuccess) or failed: post its
// requests' completions and give its memory back.
void cftg_server::retire(Slot &sl, cudaError_t e)
{
    const uint64_t t = now_ns();
    if (e != cudaSuccess) {
        cudaGetLastError();
        std::lock_guard<std::mutex> g(mu);
        failed = true;
    }
    if (!sl.program) {
        for (size_t i = 0; i < sl.reqs.size(); i++) {
            Req *q = sl.reqs[i];
            int32_t res = e == cudaSuccess ? CFT_OK : CFT_ERR_INTERNAL;
            if (res == CFT_OK && q->r.host_out && !q->out_pinned &&
                cudaMemcpy(q->r.host_out, static_cast<uint8_t *>(base) + q->off, q->out_bytes,
                           cudaMemcpyDeviceToHost) != cudaSuccess)
                res = CFT_ERR_INTERNAL;
            arena.release(q->off, q->out_bytes);
            complete(q, res, e == cudaSuccess ? (sl.h_flags[i] & CFT_FLAGS_ALL) : 0u, 0u, sl.id, t);
        }
    } else {
        const SeqProgram *P = sl.reqs.empty() ? nullptr : sl.reqs[0]->P;
        const bool bad = e != cudaSuccess || sl.h_word[2] != 0u;
        if (e == cudaSuccess) early_completions(sl);     // the last ones, before any is freed
        for (size_t i = 0; i < sl.reqs.size(); i++) {
            Req *q = sl.reqs[i];
            if (q->early) {                       // posted when its last lane finished
                delete q;
                continue;
            }
            uint32_t fl = 0, stt = 0;
            for (size_t j = 0; !bad && j < q->r.lanes; j++) {
                fl |= sl.h_lflags[sl.lane0[i] + j] & CFT_FLAGS_ALL;
                stt |= sl.h_lstatus[sl.lane0[i] + j];
            }
            int32_t res = e != cudaSuccess ? CFT_ERR_INTERNAL : bad ? CFT_ERR_INTERNAL : CFT_OK;
            if (res == CFT_OK && q->r.host_out && !q->out_pinned) {
                const uint8_t *src = static_cast<uint8_t *>(base) + sl.prog_off +
                                     sl.lane0[i] * P->n_scratch_out * q->esz;
                if (cudaMemcpy(q->r.host_out, src, q->out_bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
                    res = CFT_ERR_INTERNAL;
            }
            complete(q, res, fl, stt, sl.id, t);
        }
        arena.release(sl.prog_off, sl.prog_bytes);
    }
    sl.reqs.clear();
    sl.busy = false;
    std::lock_guard<std::mutex> g(mu);
    st.bytes_in_use = arena.used();
    cv_done.notify_all();
}

void cftg_server::loop()
{
    cudaSetDevice(dev->ordinal);
    const size_t ne = cfg.max_inflight;
    for (;;) {
        {
            std::unique_lock<std::mutex> g(mu);
            while (!intake.empty()) {
                Req *q = intake.front();
                intake.pop_front();
                (q->r.type == CFTG_REQ_ELEM ? elem_q : prog_q).push_back(q);
            }
            bool busy = false;
            for (auto &sl : slots) busy |= sl.busy;
            if (stop && !busy && elem_q.empty() && prog_q.empty()) break;
            st.pending = (uint32_t)(elem_q.size() + prog_q.size());
        }
        bool did = false;
        const uint64_t t0 = now_ns();
        for (auto &sl : slots) {
            if (!sl.busy) continue;
            const cudaError_t e = cudaEventQuery(sl.ev);
            if (e == cudaErrorNotReady) {
                if (sl.program && early_completions(sl)) did = true;
                continue;
            }
            retire(sl, e);
            did = true;
        }
        const uint64_t t1 = now_ns();
        bool full = !elem_q.empty() || !prog_q.empty();
        for (size_t i = 0; i < ne && !elem_q.empty(); i++)
            if (!slots[i].busy) {
                full = false;
                if (launch_elem(slots[i])) did = true;
                else break;                          // the budget is short: wait for a retire
            }
        for (size_t i = ne; i < slots.size() && !prog_q.empty(); i++)
            if (!slots[i].busy) {
                full = false;
                if (launch_prog(slots[i])) did = true;
                else break;
            }
        const uint64_t t2 = now_ns();
        {
            std::lock_guard<std::mutex> g(mu);
            st.engine_retire_ns += t1 - t0;
            st.engine_launch_ns += t2 - t1;
            if (full) st.slot_full_turns++;
        }
        {
            std::lock_guard<std::mutex> g(mu);
            uint32_t inflight = 0;
            for (auto &sl : slots) inflight += sl.busy ? 1u : 0u;
            st.inflight = inflight;
        }
        if (!did) {
            std::unique_lock<std::mutex> g(mu);
            bool busy = false;
            for (auto &sl : slots) busy |= sl.busy;
            // with work on the device, look again soon; otherwise sleep
            // until a request arrives
            cv_in.wait_for(g, busy ? std::chrono::microseconds(20) : std::chrono::milliseconds(5),
                           [&] { return !intake.empty() || stop; });
        }
    }
}

static void free_slot(Slot &sl)
{
    if (sl.ev) cudaEventDestroy(sl.ev);
    for (void *p : {(void *)sl.d_calls, (void *)sl.d_prefix, (void *)sl.d_counter, (void *)sl.d_flags,
                    (void *)sl.d_seg, (void *)sl.d_order, (void *)sl.d_lstatus, (void *)sl.d_word,
                    (void *)sl.d_lflags, (void *)sl.d_req_of, (void *)sl.d_req_lane0,
                    (void *)sl.d_req_left, (void *)sl.d_req_acc, (void *)sl.d_req_out})
        if (p) cudaFree(p);
    for (void *p : {(void *)sl.h_calls, (void *)sl.h_prefix, (void *)sl.h_flags, (void *)sl.h_seg,
                    (void *)sl.h_order, (void *)sl.h_lstatus, (void *)sl.h_word, (void *)sl.h_lflags,
                    (void *)sl.h_init, (void *)sl.h_req_of, (void *)sl.h_req_lane0,
                    (void *)sl.h_req_left, (void *)sl.h_req_out, (void *)sl.h_done})
        if (p) cudaFreeHost(p);
}

extern "C" uint64_t cftg_clock_ns(void) { return now_ns(); }

extern "C" void cftg_server_free(cftg_server *s)
{
    if (!s) return;
    if (s->th.joinable()) {
        {
            std::lock_guard<std::mutex> g(s->mu);
            s->stop = true;
        }
        s->cv_in.notify_all();
        s->th.join();
    }
    cudaSetDevice(s->dev->ordinal);
    for (auto &sl : s->slots) free_slot(sl);
    for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
    if (s->base) cudaFree(s->base);
    for (Req *q : s->elem_q) delete q;
    for (Req *q : s->prog_q) delete q;
    for (Req *q : s->intake) delete q;
    delete s;
}

extern "C" cft_status cftg_server_create(cft_device *dev, const cftg_server_config *cfg,
                                         cftg_server **out)
{
    clear_error();
    // a config written before elem_blocks_per_sm existed is read with it 0
    if (!dev || !cfg || !out || cfg->struct_size < offsetof(cftg_server_config, elem_blocks_per_sm)) {
        set_error("cftg_server_create: needs a device, a config (struct_size set) and out");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (dev->poisoned) {
        set_error("cftg_server_create: the handle is poisoned by an earlier device failure");
        return CFT_ERR_INTERNAL;
    }
    cftg_server_config c{};
    memcpy(&c, cfg, std::min(cfg->struct_size, sizeof c));
    if (!c.hbm_budget || c.max_inflight < 1 || c.max_inflight > 16 || c.max_program_inflight > 16 ||
        c.max_batch_calls < 1 || c.max_batch_calls > (1u << 20) ||
        (c.max_program_inflight && (c.max_batch_lanes < 1 || c.max_batch_lanes > (1u << 24)))) {
        set_error("cftg_server_create: budget must be > 0, max_inflight 1..16, "
                  "max_program_inflight 0..16, max_batch_calls 1..2^20, max_batch_lanes 1..2^24");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cftg_server *s = new (std::nothrow) cftg_server();
    if (!s) return CFT_ERR_OUT_OF_MEMORY;
    s->dev = dev;
    s->cfg = c;
    {
        const int per = queue_blocks_per_sm(256);
        const int want = (int)std::min<uint32_t>(c.elem_blocks_per_sm ? c.elem_blocks_per_sm : 2u, (uint32_t)per);
        s->queue_blocks = sm_count() * want;
        int per_sm = 0, reserved = 0, regs_sm = 0;
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev->ordinal);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev->ordinal);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev->ordinal);
        const long elem_regs = (long)want * 256 * ((queue_calls_regs() * 32 + 255) / 256 * 256) / 32;
        const long regs_left = (long)regs_sm - elem_regs;
        const long smem_left = (long)per_sm - (long)want * (reserved + 1024);
        s->traj_sm_regs = regs_left > 0 ? (uint32_t)regs_left : 1u;
        s->traj_sm_smem = smem_left > 0 ? (uint32_t)smem_left : 0u;
    }
    cudaSetDevice(dev->ordinal);
    bool ok = cudaMalloc(&s->base, c.hbm_budget) == cudaSuccess;
    s->arena.init(c.hbm_budget);
    s->slots.resize((size_t)c.max_inflight + c.max_program_inflight);
    const size_t ne = std::min<size_t>(2, c.max_inflight);
    const size_t np = std::min<size_t>(3, c.max_program_inflight);
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    for (size_t i = 0; ok && i < ne + np; i++) {
        cudaStream_t st = nullptr;
        ok = cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, i < ne ? hi_prio : lo_prio) ==
             cudaSuccess;
        if (ok) s->streams.push_back(st);
    }
    for (size_t i = 0; ok && i < s->slots.size(); i++) {
        Slot &sl = s->slots[i];
        sl.s = i < c.max_inflight ? s->streams[i % ne] : s->streams[ne + (i - c.max_inflight) % np];
        ok = cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) == cudaSuccess;
        if (!ok) break;
        if (i < c.max_inflight) {
            const size_t k = c.max_batch_calls;
            ok = cudaMalloc(&sl.d_calls, k * sizeof(QCall)) == cudaSuccess &&
                 cudaMalloc(&sl.d_prefix, (k + 1) * sizeof(uint32_t)) == cudaSuccess &&
                 cudaMalloc(&sl.d_counter, sizeof(uint32_t)) == cudaSuccess &&
                 cudaMalloc(&sl.d_flags, k * sizeof(uint32_t)) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_calls, k * sizeof(QCall), 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_prefix, (k + 1) * sizeof(uint32_t), 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_flags, k * sizeof(uint32_t), 0) == cudaSuccess;
        } else {
            const size_t l = c.max_batch_lanes;
            ok = cudaMalloc(&sl.d_seg, l * 4) == cudaSuccess && cudaMalloc(&sl.d_order, l * 4) == cudaSuccess &&
                 cudaMalloc(&sl.d_lstatus, l * 4) == cudaSuccess &&
                 cudaMalloc(&sl.d_lflags, l) == cudaSuccess &&
                 cudaMalloc(&sl.d_word, 4 * sizeof(uint32_t)) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_seg, l * 4, 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_order, l * 4, 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_lstatus, l * 4, 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_lflags, l, 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_word, 4 * sizeof(uint32_t), 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_init, SERVE_INIT_STAGING, 0) == cudaSuccess;
            sl.h_init_cap = SERVE_INIT_STAGING;
            const size_t rq = std::min<size_t>(l, 65536);
            sl.req_cap = rq;
            ok = ok && cudaMalloc(&sl.d_req_of, l * 4) == cudaSuccess &&
                 cudaMalloc(&sl.d_req_lane0, rq * 4) == cudaSuccess &&
                 cudaMalloc(&sl.d_req_left, rq * 4) == cudaSuccess &&
                 cudaMalloc(&sl.d_req_acc, rq * 8) == cudaSuccess &&
                 cudaMalloc(&sl.d_req_out, rq * sizeof(void *)) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_req_of, l * 4, 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_req_lane0, rq * 4, 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_req_left, rq * 4, 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_req_out, rq * sizeof(void *), 0) == cudaSuccess &&
                 cudaHostAlloc(&sl.h_done, rq * 16, cudaHostAllocMapped) == cudaSuccess &&
                 cudaHostGetDevicePointer((void **)&sl.d_done, sl.h_done, 0) == cudaSuccess;
        }
    }
    if (!ok) {
        cudaGetLastError();
        cftg_server_free(s);
        set_error("cftg_server_create: could not allocate the budget (%llu bytes) and the batch "
                  "slots' tables", (unsigned long long)c.hbm_budget);
        return CFT_ERR_OUT_OF_MEMORY;
    }
    s->st.budget = c.hbm_budget;
    s->th = std::thread([s] { s->loop(); });
    *out = s;
    return CFT_OK;
}

extern "C" cft_status cftg_server_submit(cftg_server *s, const cftg_request *r)
{
    clear_error();
    if (!s || !r || r->struct_size < sizeof(cftg_request)) {
        set_error("cftg_server_submit: needs a server and a request (struct_size set)");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    Req *q = new (std::nothrow) Req();
    if (!q) return CFT_ERR_OUT_OF_MEMORY;
    q->r = *r;
    q->t_arrival = r->t_arrival_ns ? r->t_arrival_ns : now_ns();
    auto refuse = [&](cft_status stt, const char *why) {
        set_error("cftg_server_submit: %s", why);
        delete q;
        return stt;
    };
    if (r->type == CFTG_REQ_ELEM) {
        if (r->fmt < 0 || r->fmt > 3 || r->rnd < 0 || r->rnd > 4 || r->kind < 0 || r->kind > 2 ||
            (r->kind == CFTG_KIND_OP && (r->op < 0 || r->op > 255 || op_is_reduction(r->op))))
            return refuse(CFT_ERR_INVALID_ARGUMENT, "an element request's format, rounding, kind or "
                                                    "operation is out of range");
        const unsigned need = r->kind == CFTG_KIND_DIV ? 3u : r->kind == CFTG_KIND_SQRT ? 1u
                                                                 : op_operands(r->op);
        if (!r->n || r->n > (1ull << 30))
            return refuse(CFT_ERR_INVALID_ARGUMENT, "an element request needs 1..2^30 elements");
        if (((need & 1u) && !r->d_a) || ((need & 2u) && !r->d_b) || ((need & 4u) && !r->d_c))
            return refuse(CFT_ERR_INVALID_ARGUMENT, "an element request lacks an operand its "
                                                    "operation reads");
        q->kind = r->kind == CFTG_KIND_DIV ? K_DIV : r->kind == CFTG_KIND_SQRT ? K_SQRT
                                                        : elem_kind_of_op(r->op);
        q->esz = esz_of(r->fmt);
        q->out_bytes = r->n * q->esz;
        q->dev_bytes = round_up(q->out_bytes);
    } else if (r->type == CFTG_REQ_PROGRAM) {
        cft_device *pd = nullptr;
        const SeqProgram *P = r->prog ? program_seq(r->prog, &pd) : nullptr;
        if (!P || pd != s->dev)
            return refuse(CFT_ERR_INVALID_ARGUMENT, "a program request needs a program loaded on "
                                                    "the server's device");
        if (P->max_deposits || P->n_scratch_in != P->n_scratch_out)
            return refuse(CFT_ERR_INVALID_ARGUMENT, "a program request's program must deposit "
                                                    "nothing and carry equal scratch blocks in "
                                                    "and out");
        if (!r->lanes || !r->runs || r->lanes > s->cfg.max_batch_lanes || !s->cfg.max_program_inflight)
            return refuse(CFT_ERR_INVALID_ARGUMENT, "a program request needs 1..max_batch_lanes "
                                                    "lanes, at least one run and a server with "
                                                    "program slots");
        if ((P->flags & CFT_PROG_FLAG_BANK_EXT) && P->n_consts && !r->d_bank)
            return refuse(CFT_ERR_INVALID_ARGUMENT, "the program's constants arrive per run and "
                                                    "d_bank is NULL");
        q->P = P;
        q->esz = esz_of(P->fmt);
        q->out_bytes = r->lanes * P->n_scratch_out * q->esz;
        if (q->out_bytes > SERVE_INIT_STAGING)
            return refuse(CFT_ERR_INVALID_ARGUMENT, "a program request's initial blocks exceed "
                                                    "the 16 MiB a program batch stages");
        if (P->n_scratch_out) {
            if (!r->init)
                return refuse(CFT_ERR_INVALID_ARGUMENT, "a program request needs its initial blocks");
            const uint8_t *p = static_cast<const uint8_t *>(r->init);
            q->init.assign(p, p + q->out_bytes);
        }
        q->dev_bytes = round_up(r->lanes * (size_t)(P->n_scratch_out + P->reach) * q->esz);
    } else {
        return refuse(CFT_ERR_INVALID_ARGUMENT, "unknown request type");
    }
    if (q->dev_bytes > s->cfg.hbm_budget)
        return refuse(CFT_ERR_OUT_OF_MEMORY, "the request needs more device memory than the "
                                             "server's whole budget");
    if (r->host_out) {
        cudaPointerAttributes at;
        const bool known = cudaPointerGetAttributes(&at, r->host_out) == cudaSuccess;
        cudaGetLastError();
        q->out_pinned = known && at.type == cudaMemoryTypeHost;
        // where the GPU can write the caller's buffer itself: pinned memory
        // through its mapped address, any host memory where the GPU walks
        // the host's page tables
        if (q->out_pinned && at.devicePointer) q->out_dev = at.devicePointer;
        else if (known && at.type == cudaMemoryTypeUnregistered && s->dev->host_page_tables)
            q->out_dev = r->host_out;
    }
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->failed) {
            delete q;
            set_error("cftg_server_submit: the server stopped after a device failure");
            return CFT_ERR_INTERNAL;
        }
        s->intake.push_back(q);
        s->st.submitted++;
    }
    s->cv_in.notify_one();
    return CFT_OK;
}

extern "C" size_t cftg_server_poll(cftg_server *s, cftg_completion *out, size_t cap)
{
    if (!s || !out || !cap) return 0;
    std::lock_guard<std::mutex> g(s->mu);
    const size_t k = std::min(cap, s->done.size());
    std::copy(s->done.begin(), s->done.begin() + k, out);
    s->done.erase(s->done.begin(), s->done.begin() + k);
    return k;
}

extern "C" cft_status cftg_server_drain(cftg_server *s, uint32_t timeout_ms)
{
    clear_error();
    if (!s) return CFT_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> g(s->mu);
    const bool ok = s->cv_done.wait_for(g, std::chrono::milliseconds(timeout_ms),
                                        [&] { return s->st.completed == s->st.submitted; });
    if (!ok) {
        set_error("cftg_server_drain: %llu of %llu requests still open after %u ms",
                  (unsigned long long)(s->st.submitted - s->st.completed),
                  (unsigned long long)s->st.submitted, timeout_ms);
        return CFT_ERR_TIMEOUT;
    }
    return s->failed ? CFT_ERR_INTERNAL : CFT_OK;
}

extern "C" void cftg_server_get_stats(cftg_server *s, cftg_server_stats *out)
{
    if (!s || !out) return;
    std::lock_guard<std::mutex> g(s->mu);
    *out = s->st;
}
