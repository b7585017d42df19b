// cftg_internal.h - what the host layer (api.cpp, program.cpp) and the
// kernels (elem.cu, seq.cu, queue.cu) share. Nothing here is exported.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace cftg {

// Kinds of elementwise work one launch does.
enum ElemKind : int {
    K_FMA = 0, K_ADD = 1, K_SUB = 2, K_MUL = 3,   // the FMA core, steered
    K_DIV = 4, K_SQRT = 5,                        // the contract's div/sqrt
    K_SIMPLE = 6                                  // every other opcode
};

inline int elem_kind_of_op(int op)
{
    return (op >= 0 && op <= 3) ? op : K_SIMPLE;
}

// One elementwise launch over device memory. Every operand pointer is a
// device pointer; a NULL operand reads +0 (the reference's loop loads a
// zeroed element for an operand the caller did not pass).
struct ElemLaunch {
    int fmt = 0, kind = 0, op = 0, rnd = 0;
    const void *a = nullptr, *b = nullptr, *c = nullptr;
    void *d = nullptr;
    uint32_t scalar_mask = 0;                 // bit r: operand r is element 0 for all i
    const uint32_t *ia = nullptr, *ib = nullptr, *ic = nullptr;   // index tables
    size_t n = 0;
    uint32_t *flags = nullptr;                // device word, ORed into
    uint8_t *lane_flags = nullptr;            // optional, n bytes
    uint32_t blocks_per_sm = 0;               // grid cap in blocks an SM (0: eight)
};

// Bit 31 of an element launch's flag word: a bulk-staged launch
// (elem_bulk.cu) found a stage of its shared-memory ring not filled within
// the time limit; that launch's outputs are incomplete.
constexpr uint32_t ELEM_ERR_STAGING = 0x80000000u;

// Launch on `stream`; returns the launch status. The direct kernels
// (elem.cu) take every launch unless CFTG_ELEM_STAGING=bulk sends large
// arrays in device memory to the bulk-staged ones (elem_bulk.cu).
cudaError_t launch_elem(const ElemLaunch &L, cudaStream_t stream);
// The bulk-staged launch, when asked for and L qualifies (then *err is its
// status and the result true); false when the direct kernels take L.
bool launch_elem_bulk(const ElemLaunch &L, cudaStream_t stream, cudaError_t *err);

// Binary32 FMA/ADD/SUB/MUL under RNE/RTZ/RDN/RUP on the hardware's
// rounding, with the elements it cannot take on the integer path
// (elem_hw.cu): true (and *err its status) when it takes L.
bool launch_elem_hw(const ElemLaunch &L, cudaStream_t stream, cudaError_t *err);

// The kernels' dimensions for a given launch (used by the queue autotuner).
int sm_count();

// ---- augmented operations (aug.cu) ----------------------------------------

// r[i], e[i] = 9.5's augmented operation fn (0 add, 1 sub, 2 mul) of a[i],
// b[i]; *word |= the flags. Device pointers, element-aligned words.
cudaError_t launch_aug(int fmt, int fn, const void *a, const void *b, void *r, void *e, size_t n,
                       uint32_t *word, cudaStream_t s);

// ---- reductions (reduce.cu) -------------------------------------------------

enum RedMode : int { RED_SUM = 0, RED_DOT = 1, RED_SQ = 2, RED_ABS = 3, RED_MAX = 4 };

// One level of the tree's leftover items: [start, start + len) of `src`
// (leaves from the call's a/b when `leaf`).
struct RedLevel {
    const void *src;
    size_t start;
    uint32_t len;
    bool leaf;
};
struct RedLevels {
    const void *a, *b;
    int count;
    RedLevel lev[8];
};

// Elements of partial results a tree over n items needs.
size_t red_partial_elems(size_t n);
// d_out (one element) = the reduction of a/b[0, n) (n >= 1); word[0] gets
// the flags. partials: red_partial_elems(n) elements of device memory.
cudaError_t launch_reduce(int fmt, int mode, const void *a, const void *b, size_t n,
                          void *partials, void *out, int rnd, uint32_t *word, cudaStream_t s);
// out[s] = the reduction of slice s of `seg` elements, s < nseg; *word |= flags.
cudaError_t launch_reduce_seg(int fmt, int mode, const void *a, const void *b, size_t nseg,
                              size_t seg, void *out, int rnd, uint32_t *word, cudaStream_t s);

// ---- the sequencer ------------------------------------------------------

// A loaded program as the GPU executor reads it (built by program.cpp).
struct SeqProgram {
    int fmt = 0;
    uint32_t n_insns = 0, n_consts = 0, max_deposits = 0, flags = 0;
    uint32_t n_scratch_in = 0, n_scratch_out = 0;
    uint32_t scratch_used = 0, scratch_depth = 256, scratch_log2 = 8;
    int scratch_active = 0;
    uint32_t reach = 0;                       // slots a lane's scratch clears
    uint32_t nregs = 32;                      // registers the program names (highest + 1)
    const uint64_t *d_insns = nullptr;        // device copy of the instruction words
    const void *d_consts = nullptr;           // device constants (or the run's bank)
    const int32_t *d_endrep = nullptr;        // REPEAT pc -> matching ENDREP pc
};

struct SeqLaunch {
    SeqProgram P;
    size_t n = 0;
    const void *a = nullptr, *b = nullptr, *c = nullptr;
    const uint32_t *ia = nullptr, *ib = nullptr, *ic = nullptr, *isi = nullptr;
    const void *scratch_in = nullptr;
    void *scratch_out = nullptr;
    void *deposits = nullptr;
    uint32_t *counts = nullptr;
    const uint8_t *lane_mask = nullptr;
    uint8_t *lane_flags = nullptr;
    void *scratch = nullptr;                  // n * reach * esz device bytes (or null)
    uint32_t *word = nullptr;                 // [0] flags, [1] status, [2] error
};

cudaError_t launch_seq(const SeqLaunch &L, cudaStream_t stream);

// Many chained runs a lane (trajectories), state carried through the
// scratch block (seq.cu, k_traj).
struct TrajLaunch {
    SeqProgram P;
    size_t n = 0;
    const void *a = nullptr, *b = nullptr, *c = nullptr;   // streams, n elements or NULL
    const uint32_t *segments = nullptr;                      // runs a lane
    const uint32_t *order = nullptr;                         // thread -> lane, or NULL
    void *state = nullptr;        // n * n_scratch_out elements: the initial block in, final out
    void *snaps = nullptr;        // n * max_snaps * n_scratch_out elements, or NULL
    uint32_t snap_every = 0, max_snaps = 0;
    void *scratch = nullptr;      // n * reach * esz
    uint8_t *lane_flags = nullptr;
    uint32_t *lane_status = nullptr;   // n words: each lane's STATUS, or NULL
    uint32_t *word = nullptr;     // [0] flags, [1] status, [2] error
    // G > 1: each lane served by G threads through a bundle schedule
    // (bundle.cpp); G == 1: one thread a lane, the plain interpreter. K:
    // threads a micro-operation (1, or the element's words for the
    // cooperative binary128/256 arithmetic of coop.cuh), so a bundle holds
    // G / K micro-operations
    int G = 1, K = 1;
    uint32_t nb = 0, nloc = 0;                // bundles; a lane's locations
    const uint64_t *b_ops = nullptr;
    const uint32_t *b_ctl = nullptr, *b_arg = nullptr;
    const int32_t *b_match = nullptr;
    // A caller sharing the GPU with other kernels caps how many of this
    // launch's blocks an SM holds: at most as many as fit in sm_regs
    // registers, enforced by asking each block for a share of sm_smem bytes
    // of shared memory. 0: no cap.
    uint32_t sm_regs = 0, sm_smem = 0;
    // Completion a request at a time (the serving loop), when req_of is
    // set: lane l belongs to request req_of[l], whose lanes start at batch
    // lane req_lane0[r]. A lane that has run its last segment writes its
    // final block to state and, when req_out[r] is not NULL (host memory the
    // GPU writes), to req_out[r] at its place in the request; ORs its flags
    // and STATUS into req_acc[2r], req_acc[2r+1] and counts req_left[r]
    // down. The request's last lane writes the flags and STATUS to
    // req_done[4r], req_done[4r+1] and then 1 to req_done[4r+2], in host
    // memory, after a system-wide fence.
    const uint32_t *req_of = nullptr, *req_lane0 = nullptr;
    uint32_t *req_left = nullptr, *req_acc = nullptr, *req_done = nullptr;
    void *const *req_out = nullptr;
};

cudaError_t launch_traj(const TrajLaunch &L, cudaStream_t stream);

}  // namespace cftg
