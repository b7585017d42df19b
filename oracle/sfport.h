/* sfport.h - the oracle: a plain-C restatement of cft-fp256's element
 * arithmetic and sequencer, used ONLY as a test checker and as the timed
 * CPU baseline. Nothing in the shipped library links or calls it.
 *
 * It follows the reference's software backend (host/src/softfloat.c,
 * host/src/seq_exec.h) and, for division and square root, the golden
 * model's definition (python/cft_golden/softfloat.py:440-505). Parity of
 * this restatement is pinned against the reference library built from
 * its own sources (oracle/Makefile, target `ref`) and against golden
 * vectors produced by the reference's Python model (tests/golden/).
 *
 * Elements are dense little-endian byte strings of 4, 8, 16 or 32 bytes
 * (host/include/cft.h:1172-1174). Formats: 0 fp32, 1 fp64, 2 fp128,
 * 3 fp256. Rounding: 0 RNE, 1 RTZ, 2 RDN, 3 RUP, 4 RMM. Flags: 1 invalid,
 * 2 divide-by-zero, 4 overflow, 8 underflow, 16 inexact.
 */
#ifndef SFPORT_H
#define SFPORT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One element of opcode `op` (0..255). Returns 0, or 1 on an internal
 * invariant failure. Operands an opcode does not read may be NULL. */
int sfp_compute(int fmt, int op, int rnd, const uint8_t *a, const uint8_t *b,
                const uint8_t *c, uint8_t *d, uint32_t *flags);

/* The contract's division and square root (one element each). */
int sfp_div(int fmt, int rnd, const uint8_t *a, const uint8_t *b, uint8_t *d,
            uint32_t *flags);
int sfp_sqrt(int fmt, int rnd, const uint8_t *a, uint8_t *d, uint32_t *flags);

/* Elementwise over n elements, as cft_run's software loop does
 * (host/src/device.c:2154-2170): NULL operands read as +0, scalar_mask bit
 * r makes operand r element 0 for every i. `kind` 0 = opcode `op`,
 * 1 = division, 2 = square root. lane_flags (n bytes) may be NULL; *acc
 * receives the OR of every element's flags. Returns 0 or 1. */
/* Reductions (opcodes 24 SUM, 25 DOT, 28 SUMSQ, 29 SUMABS, 31 MAXALL): one
 * element into d, the reference's fixed tree and compositions; the
 * segmented form writes n / seg results. Return 0, or 1 on a refusal. */
int sfp_reduce(int fmt, int op, int rnd, const void *a, const void *b, void *d, size_t n,
               uint32_t *flags);
int sfp_reduce_seg(int fmt, int op, int rnd, const void *a, const void *b, void *d, size_t n,
                   size_t seg, uint32_t *flags);

/* IEEE 754-2019 9.5's augmented operations on one element pair: fn 0
 * augmentedAddition, 1 augmentedSubtraction, 2 augmentedMultiplication;
 * r and e receive the rounded result and the residual. */
int sfp_aug(int fmt, int fn, const uint8_t *x, const uint8_t *y, uint8_t *r, uint8_t *e,
            uint32_t *flags);

int sfp_run(int kind, int fmt, int op, int rnd, const void *a, const void *b,
            const void *c, void *d, size_t n, uint32_t scalar_mask,
            uint8_t *lane_flags, uint32_t *acc);

/* ---- sequencer (seqport.c) ------------------------------------------ */

/* Run a program image (already accepted by a loader) over n lanes, as the
 * reference's seq_program_run does for a software handle at scratch depth
 * `depth` (a power of two). Every pointer may be NULL where the run does
 * not use it; the byte counts are the caller's to get right. Returns 0,
 * or a non-zero code for an image this restatement cannot parse. */
typedef struct sfp_seq_args {
    const void *a, *b, *c;
    size_t n;
    const void *bank;               /* BANK_EXT constant bank, or NULL */
    const void *scratch_in;         /* n * n_scratch_in elements, or NULL */
    void *scratch_out;              /* n * n_scratch_out elements, or NULL */
    void *deposits;                 /* n * max_deposits elements */
    uint32_t *counts;               /* n, or NULL */
    const uint8_t *lane_mask;       /* (n + 7) / 8 bytes, or NULL */
    uint8_t *lane_flags;            /* n, or NULL */
    const uint32_t *idx_a, *idx_b, *idx_c, *idx_scratch_in;
    uint32_t depth;                 /* scratch slots a lane */
    uint32_t flags_out;             /* out: the run's IEEE flags */
    uint32_t status_out;            /* out: STATUS bits [6:4] */
} sfp_seq_args;

int sfp_seq_run(const void *image, size_t bytes, sfp_seq_args *args);

#ifdef __cplusplus
}
#endif

#endif /* SFPORT_H */
