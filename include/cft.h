/* cft.h - the C ABI of libcft_gb300, a GB300 (sm_103a) backend for
 * cft-fp256's batched elementwise softfloat path and its sequencer.
 *
 * Every declaration here is the reference's public interface for that
 * path, kept so that a caller of the reference - its ctypes binding
 * (bindings/python/cftmpfr/_lib.py), its C tests, its tools - can load
 * this library in its place. Names, enum values, struct layouts, status
 * codes and the argument meanings are the reference's; each block cites
 * the line of the reference's host/include/cft.h it replaces. The
 * implementation is this library's own: CUDA kernels for the arithmetic,
 * a C++ host layer for arguments, buffers and program images.
 *
 * What differs from the reference's software backend, by design:
 *   - cft_open(NULL, ...) and cft_open("cuda:N"/"hip:N"/"gpu", ...) open a
 *     GPU. There is no CPU fallback: without a GPU every open returns
 *     CFT_ERR_NO_DEVICE with a sentence saying so.
 *   - Operations outside the hot path (transcendentals, clause-5
 *     conversions, formatOf, the conversions to character sequences, NaN
 *     payloads) are exported so bindings load, and return
 *     CFT_ERR_UNSUPPORTED with a sentence naming the reason. The
 *     reductions, the augmented operations and the conversions FROM
 *     character sequences (which the program assembler needs) are built.
 */
#ifndef CFT_H
#define CFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__) && __GNUC__ >= 4
#define CFT_API __attribute__((visibility("default")))
#else
#define CFT_API
#endif

/* ABI version 0.18 (reference cft.h:111-129). */
#define CFT_ABI_VERSION_MAJOR 0
#define CFT_ABI_VERSION_MINOR 18
CFT_API uint32_t cft_abi_version(void);
CFT_API const char *cft_build_id(void);                         /* cft.h:239 */

/* Status codes (cft.h:244-267). */
typedef enum cft_status {
    CFT_OK = 0,
    CFT_ERR_INVALID_ARGUMENT,
    CFT_ERR_UNSUPPORTED,
    CFT_ERR_NO_DEVICE,
    CFT_ERR_ARTIFACT,
    CFT_ERR_BUS_FAULT,
    CFT_ERR_OUT_OF_MEMORY,
    CFT_ERR_TIMEOUT,
    CFT_ERR_INTERNAL
} cft_status;

CFT_API const char *cft_strerror(cft_status s);                 /* cft.h:270 */
/* The sentence of the call that just returned, or "" (cft.h:272-303).
 * Every entry point returning a status empties it first. One slot per
 * process, not thread-safe, as the reference's. */
CFT_API const char *cft_last_error(void);

/* Formats (cft.h:311-323): elements are dense little-endian byte strings
 * of 4, 8, 16 or 32 bytes. */
typedef enum cft_format { CFT_FP32 = 0, CFT_FP64 = 1, CFT_FP128 = 2, CFT_FP256 = 3 } cft_format;
CFT_API size_t cft_format_size(cft_format f);
CFT_API const char *cft_format_name(cft_format f);

/* Opcodes (cft.h:325-474). 15 and 32..255 are unassigned: cft_run answers
 * them with the canonical quiet NaN and invalid. */
typedef enum cft_op {
    CFT_FMA = 0, CFT_ADD = 1, CFT_SUB = 2, CFT_MUL = 3,
    CFT_ABS = 4, CFT_NEG = 5, CFT_COPYSIGN = 6,
    CFT_MIN = 7, CFT_MAX = 8, CFT_MINNUM = 9, CFT_MAXNUM = 10,
    CFT_SELECT = 11, CFT_CMPLT = 12, CFT_CMPLE = 13, CFT_CMPEQ = 14,
    CFT_IAND = 16, CFT_IOR = 17, CFT_IXOR = 18, CFT_IADD = 19,
    CFT_ISUB = 20, CFT_ISHL = 21, CFT_ISHR = 22, CFT_ICMPLT = 23,
    CFT_SUM = 24, CFT_DOT = 25, CFT_RECIP_SEED = 26, CFT_RSQRT_SEED = 27,
    CFT_SUMSQ = 28, CFT_SUMABS = 29, CFT_IMUL = 30, CFT_MAXALL = 31
} cft_op;
CFT_API const char *cft_op_name(cft_op op);                     /* cft.h:477 */

/* Rounding attributes (cft.h:481-488), RISC-V frm order. */
typedef enum cft_round { CFT_RNE = 0, CFT_RTZ = 1, CFT_RDN = 2, CFT_RUP = 3, CFT_RMM = 4 } cft_round;

/* Sticky exception flags (cft.h:491-501). */
typedef enum cft_exception {
    CFT_FLAG_INVALID = 1u << 0,
    CFT_FLAG_DIVBYZERO = 1u << 1,
    CFT_FLAG_OVERFLOW = 1u << 2,
    CFT_FLAG_UNDERFLOW = 1u << 3,
    CFT_FLAG_INEXACT = 1u << 4
} cft_exception;
#define CFT_FLAGS_ALL ((uint32_t)0x1Fu)

/* ---- devices (cft.h:506-579) ------------------------------------------ */
typedef struct cft_device cft_device;
CFT_API cft_status cft_open(const char *artifact, int index, cft_device **out);
CFT_API void cft_close(cft_device *dev);

typedef struct cft_open_args {
    size_t struct_size;
    const char *artifact;
    int index;
    uint32_t scratch_depth;     /* 0, or a power of two in 1..32768 */
} cft_open_args;
CFT_API cft_status cft_open_ex(const cft_open_args *args, cft_device **out);

/* Capabilities with the size handshake (cft.h:655-772). */
typedef struct cft_caps {
    size_t struct_size;
    uint32_t format_mask;
    uint32_t tiles;
    uint32_t abi_version;
    uint32_t device_version;
    int flags_readable;
    char backend[32];
    uint32_t max_deposits;
    uint32_t max_insns;
    uint32_t max_consts;
    uint32_t seq_features;
    uint32_t max_scratch;
    int buffers_resident;
} cft_caps;

/* seq_features bits (cft.h:785-1030) */
#define CFT_SEQ_FEAT_WIDE_CONST   0x01u
#define CFT_SEQ_FEAT_REGS32       0x02u
#define CFT_SEQ_FEAT_BANK_PTR     0x04u
#define CFT_SEQ_FEAT_KX9          0x08u
#define CFT_ALU_EXT_IMUL          0x10u
#define CFT_SEQ_FEAT_SCRATCH      0x100u
#define CFT_SEQ_FEAT_SCRATCH_IO   0x200u
#define CFT_SEQ_FEAT_SCRATCH_STRICT 0x400u
#define CFT_SEQ_FEAT_SCALAR       0x800u
#define CFT_FEAT_REDUCE_SEG       0x1000u
#define CFT_SEQ_FEAT_INDEXED      0x2000u
#define CFT_SEQ_FEAT_LANE_MASK    0x4000u
#define CFT_SEQ_FEAT_AUGADD       0x8000u
#define CFT_SEQ_FEAT_SCRATCH_STEP 0x10000u
#define CFT_SEQ_FEAT_LANE_FLAGS   0x20000u
#define CFT_SEQ_FEAT_FLAG_CONTROL 0x40000u
#define CFT_IDX_NONE 0xFFFFFFFFu

CFT_API cft_status cft_get_caps(cft_device *dev, cft_caps *out);
CFT_API int cft_supports(cft_device *dev, cft_op op, cft_format fmt);

/* The device image id (cft.h:1095-1159). Refused on this backend as on the
 * reference's software backend: there is no image. */
typedef struct cft_image_id {
    size_t struct_size;
    uint8_t sha256[32];
    uint64_t image_bytes;
    uint32_t version;
    uint32_t n_caps;
    uint32_t caps[4];
    char platform[256];
    char xrt_version[64];
    uint64_t clock_hz;
    char serial[256];
} cft_image_id;
CFT_API cft_status cft_get_image_id(cft_device *dev, cft_image_id *out);

/* ---- the hot path ------------------------------------------------------ */

/* d[i] = op(a[i], b[i], c[i]) for i in [0, n) (cft.h:1160-1208). b for
 * ADD/SUB and c for MUL may be NULL; d may alias a, b or c; n == 0 writes
 * nothing. flags_out receives the OR of every element's flags. */
CFT_API cft_status cft_run(cft_device *dev, cft_op op, cft_format fmt, cft_round rnd,
                           const void *a, const void *b, const void *c, void *d, size_t n,
                           uint32_t *flags_out, uint32_t *bus_out);

/* Correctly rounded a/b and sqrt(a) with 754 flags (cft.h:1385-1402). */
CFT_API cft_status cft_div(cft_device *dev, cft_format fmt, cft_round rnd, const void *a,
                           const void *b, void *d, size_t n, uint32_t *flags_out,
                           uint32_t *bus_out);
CFT_API cft_status cft_sqrt(cft_device *dev, cft_format fmt, cft_round rnd, const void *a,
                            void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);

/* Scalar operands and index tables (cft.h:3058-3136). */
typedef struct cft_elem_args {
    size_t struct_size;
    const void *a, *b, *c;
    void *d;
    size_t n;
    uint32_t scalar_mask;      /* bit 0 a, bit 1 b, bit 2 c */
    uint32_t *flags_out;
    uint32_t *bus_out;
    const uint32_t *idx_a, *idx_b, *idx_c;
    size_t idx_a_src, idx_b_src, idx_c_src;
} cft_elem_args;
CFT_API cft_status cft_run_ex(cft_device *dev, cft_op op, cft_format fmt, cft_round rnd,
                              const cft_elem_args *args);

/* Reductions (cft.h:1210-1340): SUM, DOT, SUMSQ, SUMABS and MAXALL over the
 * reference's fixed tree, whole arrays and fixed-length segments. */
CFT_API cft_status cft_reduce(cft_device *dev, cft_op op, cft_format fmt, cft_round rnd,
                              const void *a, const void *b, void *d, size_t n,
                              uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_reduce_seg(cft_device *dev, cft_op op, cft_format fmt, cft_round rnd,
                                  const void *a, const void *b, void *d, size_t n, size_t seg,
                                  uint32_t *flags_out, uint32_t *bus_out);

/* ---- augmented arithmetic, IEEE 754-2019 9.5 (cft.h:2351-2451) -------- *
 * r = x op y rounded with roundTiesTowardZero, e = the residual; no
 * rounding attribute (9.5 fixes it). r and e may alias a or b but not each
 * other. */
CFT_API cft_status cft_augmented_add(cft_device *dev, cft_format fmt, const void *a,
                                     const void *b, void *r, void *e, size_t n,
                                     uint32_t *flags_out);
CFT_API cft_status cft_augmented_sub(cft_device *dev, cft_format fmt, const void *a,
                                     const void *b, void *r, void *e, size_t n,
                                     uint32_t *flags_out);
CFT_API cft_status cft_augmented_mul(cft_device *dev, cft_format fmt, const void *a,
                                     const void *b, void *r, void *e, size_t n,
                                     uint32_t *flags_out);

/* ---- character sequences to encodings, 754-2019 5.12 (cft.h:1899-1960) *
 * Host operations: a batch of NUL-terminated sequences, each correctly
 * rounded under rnd into fmt with exact flags (OR across the batch); NaN
 * payloads and the signalling bit kept. A sequence outside the syntax
 * refuses the whole call with CFT_ERR_INVALID_ARGUMENT and its index in
 * *bad_index. cft_format_decimal_digits is 5.12.2's Pmin: 9, 17, 36, 73. */
CFT_API size_t cft_format_decimal_digits(cft_format fmt);
CFT_API cft_status cft_from_decimal_char(cft_device *dev, cft_format fmt, cft_round rnd,
                                         const char *const *in, void *d, size_t n,
                                         size_t *bad_index, uint32_t *flags_out);
CFT_API cft_status cft_from_hex_char(cft_device *dev, cft_format fmt, cft_round rnd,
                                     const char *const *in, void *d, size_t n, size_t *bad_index,
                                     uint32_t *flags_out);

/* ---- resident buffers (cft.h:2470-2705) ------------------------------- *
 * cft_alloc gives a pinned host mirror (the pointer callers use) and a
 * device copy. A run that names a pointer inside a buffer reads the device
 * copy, so a caller who fills once and runs many pays no transfer. The
 * authority rule is the reference's: write the mirror, then
 * cft_buffer_to_device; after a run wrote it, cft_buffer_from_device
 * brings the result home. */
typedef struct cft_buffer cft_buffer;
CFT_API cft_status cft_alloc(cft_device *dev, size_t bytes, cft_buffer **out);
CFT_API void *cft_buffer_data(cft_buffer *buf);
CFT_API cft_status cft_buffer_to_device(cft_buffer *buf);
CFT_API cft_status cft_buffer_from_device(cft_buffer *buf);
CFT_API void cft_buffer_free(cft_buffer *buf);

typedef struct cft_buffer_info {
    size_t struct_size;
    size_t bytes;
    int resident;
    int device_authority;
    uint64_t resident_binds;
    uint64_t staged_binds;
    char staged_why[112];
} cft_buffer_info;
CFT_API cft_status cft_buffer_get_info(cft_buffer *buf, cft_buffer_info *out);

/* ---- programs: the sequencer (cft.h:2707-3053) ------------------------ */
typedef struct cft_program cft_program;

#define CFT_STATUS_DEPOSIT_OVERFLOW (1u << 4)
#define CFT_STATUS_SCRATCH_RANGE (1u << 5)
#define CFT_STATUS_MARKED (1u << 6)
#define CFT_LANE_DEPOSIT_OVERFLOW (1u << 5)
#define CFT_LANE_SCRATCH_RANGE (1u << 6)
#define CFT_LANE_MARKED (1u << 7)

#define CFT_PROG_FLAG_BANK_EXT (1u << 0)
#define CFT_PROG_FLAG_SCRATCH_IO (1u << 1)
#define CFT_PROG_FLAG_SCRATCH_STRICT (1u << 2)

CFT_API cft_status cft_program_load(cft_device *dev, const void *image, size_t bytes,
                                    cft_program **out);
CFT_API void cft_program_free(cft_program *prog);

typedef struct cft_program_info {
    size_t struct_size;
    cft_format format;
    uint32_t max_deposits;
    uint32_t n_insns;
    uint32_t n_consts;
    uint32_t flags;
    uint32_t n_scratch_in;
    uint32_t n_scratch_out;
    uint32_t scratch_used;
} cft_program_info;
CFT_API cft_status cft_program_get_info(cft_program *prog, cft_program_info *out);

CFT_API cft_status cft_program_run(cft_program *prog, const void *a, const void *b,
                                   const void *c, void *deposits, uint32_t *counts, size_t n,
                                   uint32_t *flags, uint32_t *bus);
CFT_API cft_status cft_program_run_bank(cft_program *prog, const void *bank, size_t bank_bytes,
                                        const void *a, const void *b, const void *c,
                                        void *deposits, uint32_t *counts, size_t n,
                                        uint32_t *flags_out, uint32_t *bus_out);

typedef struct cft_run_args {
    size_t struct_size;
    const void *a, *b, *c;
    size_t n;
    const void *bank;        size_t bank_bytes;
    const void *scratch_in;  size_t scratch_in_bytes;
    void *scratch_out;       size_t scratch_out_bytes;
    void *deposits;          uint32_t *counts;
    uint32_t *flags_out;     uint32_t *bus_out;
    const uint32_t *idx_a, *idx_b, *idx_c;
    size_t idx_a_src, idx_b_src, idx_c_src;
    const uint32_t *idx_scratch_in;
    size_t idx_scratch_src;
    const uint8_t *lane_mask;
    size_t lane_mask_bytes;
    uint8_t *lane_flags;
    size_t lane_flags_bytes;
} cft_run_args;
CFT_API cft_status cft_program_run_ex(cft_program *prog, const cft_run_args *args);

/* SHA-256 digests (cft.h:3138-3167). */
CFT_API cft_status cft_program_digest(cft_program *prog, const void *bank, size_t bank_bytes,
                                      uint8_t out[32]);
CFT_API cft_status cft_sha256(const void *data, size_t bytes, uint8_t out[32]);

/* ---- the status word and 5.7.4's flag operations (cft.h:3169-3267) ---- */
CFT_API void cft_lower_flags(cft_device *dev, uint32_t mask);
CFT_API void cft_raise_flags(cft_device *dev, uint32_t mask);
CFT_API int cft_test_flags(cft_device *dev, uint32_t mask);
CFT_API uint32_t cft_save_all_flags(cft_device *dev);
CFT_API void cft_restore_flags(cft_device *dev, uint32_t saved, uint32_t mask);
CFT_API int cft_test_saved_flags(uint32_t saved, uint32_t mask);
CFT_API int cft_is754version1985(void);
CFT_API int cft_is754version2008(void);
CFT_API int cft_is754version2019(void);

#ifdef __cplusplus
}
#endif

/* the reference's entry points outside this backend's path, each a refusal
 * by name: with them this header declares every function the reference's
 * cft.h exports, so a C caller of the reference compiles and links here */
#include "cft_unsupported.h"

#endif /* CFT_H */
