/* cft_gb300.h - entry points this library adds beside the reference's C ABI
 * (include/cft.h). None replaces a reference call; each exists so that a
 * caller holding DEVICE memory (a PyTorch CUDA tensor, a buffer another
 * CUDA library produced) can run the same arithmetic without a host round
 * trip, and so the batched and serving forms have a C surface.
 *
 * Semantics are exactly cft_run's / cft_div's / cft_sqrt's for the same
 * element values: same bits, same flags. Pointers are device pointers;
 * elements are the same dense little-endian byte strings.
 */
#ifndef CFT_GB300_H
#define CFT_GB300_H

#include "cft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Work kinds for the device-pointer calls. */
#define CFTG_KIND_OP   0   /* opcode `op`, as cft_run */
#define CFTG_KIND_DIV  1   /* a / b, as cft_div */
#define CFTG_KIND_SQRT 2   /* sqrt(a), as cft_sqrt */

/* One elementwise launch over device memory, asynchronous on `stream`
 * (a cudaStream_t; NULL is the legacy default stream). The call's flags
 * are ORed into the device word *flags_word (the caller zeroes it and
 * reads it back); lane_flags, when non-NULL, receives each element's flag
 * byte. A NULL b or c reads +0. scalar_mask bit r makes operand r element
 * 0 for every i. The status word of the handle is NOT updated: the flags
 * stay on the device until the caller reads them. Bit 31 of the word
 * (CFTG_FLAG_STAGING_TIMEOUT), set only by the bulk-staged kernels that
 * CFTG_ELEM_STAGING=bulk selects, means a shared-memory stage was not
 * filled within one second and the outputs are incomplete. */
#define CFTG_FLAG_STAGING_TIMEOUT 0x80000000u
CFT_API cft_status cftg_run_device(cft_device *dev, int kind, cft_op op, cft_format fmt,
                                   cft_round rnd, const void *a, const void *b, const void *c,
                                   void *d, size_t n, uint32_t scalar_mask, uint8_t *lane_flags,
                                   uint32_t *flags_word, void *stream);

/* The CUDA device ordinal a handle runs on. */
CFT_API int cftg_device_ordinal(cft_device *dev);

/* The sequencer features this build publishes in cft_caps.seq_features. */
CFT_API uint32_t cftg_seq_features(void);

/* cft_program_load's decision over an image, taken on the host with no
 * device: CFT_OK for an image a handle opened at scratch depth
 * `max_scratch` (0 = 256) would load, else the status and sentence the
 * load would give. For tools that vet images before a GPU is at hand. */
CFT_API cft_status cftg_program_check(const void *image, size_t bytes, uint32_t max_scratch);

/* ---- the batched form -------------------------------------------------
 *
 * Many independent elementwise calls - uneven sizes, any mix of formats,
 * operations and rounding attributes - run as ONE persistent work-queue
 * launch: the calls are cut into tiles, a resident grid takes tiles from
 * one atomic counter, and each call's flags are ORed into its own device
 * word. Every element is computed exactly as cftg_run_device computes it.
 * A batch is prepared once (its tables live on the device) and launched
 * any number of times; cftg_batch_capture records the launch in a CUDA
 * graph so each replay is one graph launch. The caller keeps the operand
 * buffers and the flag words alive while the batch exists. */
typedef struct cftg_call {
    int kind;                   /* CFTG_KIND_OP, _DIV or _SQRT */
    int op;                     /* the opcode, for CFTG_KIND_OP */
    int fmt;                    /* cft_format */
    int rnd;                    /* cft_round */
    const void *a, *b, *c;      /* device pointers; an unread one may be NULL */
    void *d;                    /* device pointer, n elements */
    size_t n;
    uint32_t scalar_mask;       /* as cft_run_ex's */
} cftg_call;

typedef struct cftg_batch cftg_batch;

CFT_API cft_status cftg_batch_create(cft_device *dev, const cftg_call *calls, size_t ncalls,
                                     uint32_t *d_call_flags, cftg_batch **out);
CFT_API cft_status cftg_batch_launch(cftg_batch *b, void *stream);
CFT_API cft_status cftg_batch_capture(cftg_batch *b, void *stream);
CFT_API void cftg_batch_free(cftg_batch *b);
CFT_API uint32_t cftg_batch_tiles(const cftg_batch *b);

/* The work queue's autotuner: times the queue at candidate tile lengths
 * (elements a tile: 256 .. 262,144) for each format and for FMA, ADD, DIV
 * and SQRT over n elements of the caller's device buffers (each sized for
 * n binary256 elements), then the launch's block shape (128 or 256
 * threads), and keeps the fastest of each for every batch created later in
 * the process. */
CFT_API cft_status cftg_autotune(cft_device *dev, const void *d_a, const void *d_b,
                                 const void *d_c, void *d_d, size_t n, void *stream);
/* Elements a tile the batched form cuts a call of (fmt, kind, op) into. */
CFT_API uint32_t cftg_tile_length(int fmt, int kind, int op);
/* Threads a block of the batched form's work-queue launch (256 until the
 * autotuner has run), and the setter for callers that choose it
 * themselves (a multiple of 32 in 32..256; batches created later use it). */
CFT_API int cftg_queue_block_threads(void);
CFT_API cft_status cftg_set_queue_block_threads(int threads);

/* ---- trajectories: the batched sequencer ------------------------------
 *
 * Thousands of lanes of one program, each run `segments[lane]` times in a
 * row with its scratch-out block fed back as the next run's scratch-in
 * (programs whose scratch blocks are equal in and out and that deposit
 * nothing, e.g. the ODE segment programs), as ONE launch. Every run is a
 * complete run as cft_program_run_ex defines it, so each lane's states are
 * those a host loop of single runs would produce. d_state holds n x
 * n_scratch_out elements, lane-major: the initial block in, the final block
 * out. With d_snaps, every snap_every runs the block is also copied to
 * d_snaps[(lane * max_snaps + k) * n_scratch_out ...] for k = runs /
 * snap_every - 1 < max_snaps. Flags, STATUS and the per-lane flag byte are
 * ORed over every run. `segments` is a HOST array read at creation (lanes
 * are ordered longest first so a warp's lanes finish together). Device
 * pointers otherwise; the caller keeps them alive. */
typedef struct cftg_traj cftg_traj;
CFT_API cft_status cftg_traj_create(cft_program *prog, const uint32_t *segments, size_t n,
                                    const void *d_a, const void *d_b, const void *d_c,
                                    const void *d_bank, void *d_state, void *d_snaps,
                                    uint32_t snap_every, uint32_t max_snaps,
                                    uint8_t *d_lane_flags, cftg_traj **out);
CFT_API cft_status cftg_traj_launch(cftg_traj *t, void *stream);
CFT_API cft_status cftg_traj_capture(cftg_traj *t, void *stream);
CFT_API cft_status cftg_traj_result(cftg_traj *t, uint32_t *flags_out, uint32_t *status_out,
                                    void *stream);
CFT_API void cftg_traj_free(cftg_traj *t);

/* A trajectory launch of few lanes spreads each lane over G threads
 * (G = 1, 2, 4, ... 32, chosen per launch from the lane count and the
 * program's parallelism): every straight-line stretch of the program is
 * scheduled into bundles of at most G independent operations, run
 * together, each reading its operands before any writes its result. Only
 * programs whose control is REPEAT/ENDREP/HALT and whose scratch accesses
 * are LDL/STL are scheduled; results are those of one thread a lane.
 * Within a stretch each written value gets a location of its own, so only
 * true dependences order operations; LDL/STL become renames.
 * cftg_program_schedule returns that schedule for an image, with no device:
 * ops (nb x G micro-operations, all ones where a thread idles), ctl (0
 * operations, 1 REPEAT, 2 ENDREP, 3 HALT), arg (REPEAT counts) and match
 * (REPEAT <-> ENDREP bundle). A micro-operation names locations (registers
 * 0..31, scratch slots 32.., renamed values after them): bits 0-7 opcode,
 * 8-10 rounding attribute, 11-13 operand a/b/c is a constant index, 14 MOVE
 * (dest = a), 15 operand c is read with its sign bit flipped (a NEG folded
 * into the read), 16-27 dest, 28-39 a, 40-51 b, 52-63 c. The arrays are filled
 * when cap >= *nb; CFT_ERR_UNSUPPORTED for a program outside the scheduled
 * set. */
CFT_API cft_status cftg_program_schedule(const void *image, size_t bytes, uint32_t G,
                                         uint64_t *ops, uint32_t *ctl, uint32_t *arg,
                                         int32_t *match, size_t cap, size_t *nb);

/* Several trajectory runs of one device (different programs and formats
 * allowed) recorded as ONE CUDA graph, each run an independent branch: one
 * cftg_traj_group_launch puts all of them on the device together. Each
 * run's flags and STATUS are still read with cftg_traj_result on the
 * launching stream. The runs must outlive the group. */
typedef struct cftg_traj_group cftg_traj_group;
CFT_API cft_status cftg_traj_group_capture(cftg_traj *const *runs, size_t count, void *stream,
                                           cftg_traj_group **out);
CFT_API cft_status cftg_traj_group_launch(cftg_traj_group *g, void *stream);
CFT_API void cftg_traj_group_free(cftg_traj_group *g);

/* Seeded synthetic operands written on the device: n elements of format
 * `fmt` into d_out, 90% normals with unbiased exponents uniform in
 * [-exp_range, exp_range], special_ppm per million specials (+-0,
 * subnormals, +-inf, quiet and signalling NaNs, near-overflow values).
 * Each element is a hash of (seed, index), so any range regenerates alike. */
CFT_API cft_status cftg_fill_operands(int fmt, void *d_out, size_t n, uint64_t seed,
                                      int exp_range, uint32_t special_ppm, void *stream);

/* ---- reductions over device memory --------------------------------------
 *
 * cft_reduce / cft_reduce_seg (the reference's fixed tree, compositions and
 * 9.4 infinity rule, same bits and flags) over DEVICE operands, asynchronous
 * on `stream`: d_out receives the n / seg results (seg = n: one result),
 * d_flags[0] the flags (two device words, overwritten). For seg == n the
 * tree's partial results go to d_partials, cftg_reduce_partial_bytes(fmt, n)
 * bytes of device memory. Operands aligned to their element size (16 bytes
 * at most). */
CFT_API cft_status cftg_reduce_device(cft_device *dev, int op, int fmt, int rnd, const void *a,
                                      const void *b, void *d_out, size_t n, size_t seg,
                                      void *d_partials, uint32_t *d_flags, void *stream);
CFT_API size_t cftg_reduce_partial_bytes(int fmt, size_t n);

/* ---- a program run that allocates nothing ------------------------------
 *
 * No counterpart in the reference: an addition of this library. It exists
 * for callers that cannot let a library call cudaMalloc - a host that owns
 * every byte of device memory through its own pool or budget, or a
 * latency-critical loop that cannot afford cudaMalloc/cudaFree's implicit
 * device synchronisation. It runs a loaded program as cft_program_run_ex
 * does (same bits, flags and STATUS) over DEVICE buffers the caller holds:
 * a (n elements), b and c (n elements or NULL for +0), the bank of a
 * BANK_EXT program, the scratch-in and scratch-out blocks of a SCRATCH_IO
 * program (lane-major, as cft_run_args'), deposits (n * max_deposits
 * elements, zero-filled by the call) and counts (n words, or NULL). No
 * lane mask, index tables or per-lane flag bytes.
 *
 * The run's scratch - each lane's scratch slots and three flag words -
 * comes from one fixed device array inside the library, of
 * cftg_noalloc_scratch_bytes() usable bytes (16 MiB less 256), which every
 * GPU that loads the library holds until exit. A run needing more (n x the
 * program's scratch slots x the element size) is refused with
 * CFT_ERR_INVALID_ARGUMENT and a sentence saying by how much. Every call
 * shares the array: calls whose work overlaps on the GPU race, so issue
 * them one after another (each returns after `stream` has finished its
 * run), never from two threads or on two streams at once. The first call
 * on a device looks up the array's device address; make that first call
 * before any stream capture. That address is kept until the process
 * exits, so after a cudaDeviceReset (or anything else that destroys the
 * device's primary context) this entry point must not be used on that
 * device again. A handle that failed earlier is refused, as the other
 * entry points refuse it. */
CFT_API cft_status cftg_program_run_noalloc(cft_program *prog, const void *d_a, const void *d_b,
                                            const void *d_c, const void *d_bank,
                                            const void *d_scratch_in, void *d_scratch_out,
                                            void *d_deposits, uint32_t *d_counts, size_t n,
                                            uint32_t *flags_out, uint32_t *status_out,
                                            void *stream);
CFT_API size_t cftg_noalloc_scratch_bytes(void);

/* ---- serving: a continuous-batching request loop ----------------------
 *
 * A server owns one device region of hbm_budget bytes and an engine thread.
 * Requests are element calls (one cftg_call's worth over DEVICE operands the
 * caller keeps resident) or program requests (`lanes` lanes of a loaded
 * program run `runs` times each with the scratch block carried, as
 * cftg_traj_*; initial blocks from the host). The engine admits waiting
 * requests first come first served per class while a batch slot is free
 * and the budget holds their outputs (element: n elements; program: the
 * lanes' state and scratch), and launches each admitted group at once:
 * element calls as one work-queue launch, requests of one program and bank
 * as one trajectory launch, each batch on its own stream, up to
 * max_inflight element and max_program_inflight program batches on the
 * device together. Requests arriving meanwhile are admitted as slots and
 * budget free up, so their work overlaps what is running. Results are the
 * same bits and flags as each call or program run alone.
 *
 * A request's output lives in the budget until it completes; with host_out
 * it is copied there (asynchronously when host_out is pinned memory) before
 * the completion is posted, and the device copy is then released. Times
 * are on cftg_clock_ns's clock; t_arrival_ns = 0 takes the submit time. */
typedef struct cftg_server cftg_server;

typedef struct {
    size_t struct_size;             /* sizeof(cftg_server_config) */
    uint64_t hbm_budget;            /* bytes of device memory requests may hold together */
    uint32_t max_inflight;          /* element batches on the device at once, 1..16 */
    uint32_t max_program_inflight;  /* program batches on the device at once, 0..16 */
    uint32_t max_batch_calls;       /* element requests in one batch, 1..2^20 */
    uint32_t max_batch_lanes;       /* program lanes in one batch, 1..2^24 */
    uint64_t max_batch_elements;    /* elements of one element batch (0: no limit); a batch
                                       completes as a whole, so this bounds the wait of its
                                       smallest requests */
    uint32_t elem_blocks_per_sm;    /* work-queue blocks an SM per element batch (0: two;
                                       clamped to what fits an empty SM). A batch completes when
                                       its last block has run, so a block that does not fit
                                       beside the trajectory blocks already on an SM waits for
                                       them to finish: two leave room for them and keep every
                                       element block resident */
} cftg_server_config;

#define CFTG_REQ_ELEM    0
#define CFTG_REQ_PROGRAM 1

typedef struct {
    size_t struct_size;             /* sizeof(cftg_request) */
    int type;                       /* CFTG_REQ_ELEM or CFTG_REQ_PROGRAM */
    int kind, op, fmt, rnd;         /* element requests: as cftg_call */
    const void *d_a, *d_b, *d_c;    /* element requests: device operands, n elements */
    size_t n;                       /* element requests: 1..2^30 elements */
    cft_program *prog;              /* program requests: loaded on the server's device */
    const void *d_bank;             /* program requests: device bank of a BANK_EXT program */
    const void *init;               /* program requests: HOST, lanes x n_scratch_out elements */
    size_t lanes;                   /* program requests: lanes */
    uint32_t runs;                  /* program requests: runs a lane */
    void *host_out;                 /* optional HOST destination of the output */
    uint64_t t_arrival_ns;          /* arrival time (cftg_clock_ns), 0 = now */
    uint64_t tag;                   /* returned in the completion */
} cftg_request;

typedef struct {
    uint64_t tag;
    int32_t result;                 /* CFT_OK, or why the request failed */
    uint32_t flags;                 /* the request's IEEE flags */
    uint32_t status;                /* program requests: STATUS ORed over lanes */
    uint32_t batch;                 /* the batch that ran it */
    uint64_t t_arrival_ns, t_admit_ns, t_done_ns;
} cftg_completion;

typedef struct {
    uint64_t submitted, completed, failed, batches, launches;
    uint64_t elements_done, lane_runs_done;
    uint64_t bytes_in_use, bytes_peak, budget;
    uint32_t inflight, pending;
    uint64_t engine_launch_ns, engine_retire_ns;   /* engine thread time spent */
    uint64_t slot_full_turns;       /* engine turns that found work waiting and no free slot */
} cftg_server_stats;

CFT_API uint64_t cftg_clock_ns(void);
CFT_API cft_status cftg_server_create(cft_device *dev, const cftg_server_config *cfg,
                                      cftg_server **out);
/* Validates and queues a request (copying it and any initial blocks);
 * refuses at once a request that needs more than the whole budget. */
CFT_API cft_status cftg_server_submit(cftg_server *s, const cftg_request *r);
/* Moves up to cap completions, oldest first, into out; returns how many. */
CFT_API size_t cftg_server_poll(cftg_server *s, cftg_completion *out, size_t cap);
/* Waits until every submitted request has completed, up to timeout_ms. */
CFT_API cft_status cftg_server_drain(cftg_server *s, uint32_t timeout_ms);
CFT_API void cftg_server_get_stats(cftg_server *s, cftg_server_stats *out);
/* Finishes every queued request, stops the engine and frees the budget. */
CFT_API void cftg_server_free(cftg_server *s);

/* ---- programs as source: the `.cfta` assembler (host only) ------------
 *
 * The reference's text form (docs/PROGRAMS.md; python/cft_golden/asm.py,
 * host/tools/cft-asm.c) as library calls, so a client can submit SOURCE.
 * cftg_asm_assemble turns UTF-8 text into the exact `.cftp` image the
 * reference assembler writes (*image malloc'd, freed with cftg_asm_free),
 * or refuses with CFT_ERR_INVALID_ARGUMENT and "source:line: reason" in
 * cft_last_error(). cftg_asm_disassemble gives text that assembles back to
 * the same bytes; cftg_asm_info the header report of `cft-asm -i`. None
 * needs a device. cftg_program_load_source assembles and loads in one call.
 *
 * cftg_ode_bank writes the default bank of one of the reference's ODE
 * segment programs ("lorenz63-rk4", "lorenz96-rk4", "henonheiles-lf") for a
 * step h given as a decimal, as programs/gen_odes.py:bank_values derives
 * it: raw format-width values, dense, in declaration order. *bytes is set
 * to the size needed; bank NULL with cap 0 asks for it. */
CFT_API cft_status cftg_asm_assemble(const char *text, size_t len, const char *source,
                                     void **image, size_t *image_bytes);
CFT_API cft_status cftg_asm_disassemble(const void *image, size_t bytes, char **text);
CFT_API cft_status cftg_asm_info(const void *image, size_t bytes, char **text);
CFT_API void cftg_asm_free(void *p);
CFT_API cft_status cftg_ode_bank(const char *system, cft_format fmt, const char *h, void *bank,
                                 size_t cap, size_t *bytes);
CFT_API cft_status cftg_program_load_source(cft_device *dev, const char *text, size_t len,
                                            const char *source, cft_program **out);

/* One decimal (hex = 0) or hexadecimal-significand (hex = 1) sequence into
 * fmt under rnd, exactly as cft_from_decimal_char / cft_from_hex_char
 * convert each element, with no device: the form tools use. */
CFT_API cft_status cftg_from_char(int hex, cft_format fmt, cft_round rnd, const char *in, void *d,
                                  uint32_t *flags_out);

#ifdef __cplusplus
}
#endif

#endif /* CFT_GB300_H */
