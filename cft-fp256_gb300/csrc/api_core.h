// api_core.h - the handle, buffer and error machinery shared by the host
// translation units (api.cpp, program.cpp, queue.cpp, stubs.cpp).
#pragma once
#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <map>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cft.h"
#include "cftg_internal.h"

namespace cftg {

// The error sentence of the call that just returned (reference cft.h:272-303).
void clear_error();
void set_error(const char *fmt, ...) __attribute__((format(printf, 1, 2)));

// A growable device allocation.
struct DevMem {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes);
    void release();
};

enum BufState { B_STALE = 0, B_FRESH = 1, B_DIRTY = 2, B_LOST = 3 };

}  // namespace cftg

// A cft_alloc'd buffer: a pinned host mirror (what callers hold) and one
// device copy, with the reference's authority rule at buffer granularity.
struct cft_buffer {
    cft_device *dev = nullptr;
    size_t bytes = 0;
    uint8_t *host = nullptr;
    void *dptr = nullptr;
    int state = cftg::B_STALE;
    uint64_t resident_binds = 0, staged_binds = 0;
    char why[112] = {0};
};

struct cft_device {
    int ordinal = 0;
    uint32_t word = 0;            // the 7.1 status word
    int mute = 0;
    int poisoned = 0;
    uint32_t max_scratch = 256;
    int host_page_tables = 0;     // the GPU walks the host's page tables (ATS)
    cudaStream_t s[2] = {nullptr, nullptr};
    uint32_t *d_word = nullptr;   // device flag/status words, 64 of them
    uint32_t *h_word = nullptr;   // pinned host copy
    cftg::DevMem stage[2][4];     // per pipeline slot: a, b, c, d
    cftg::DevMem gath[3];         // whole indexed sources / scalars
    cftg::DevMem tabs[3];         // index tables
    cftg::DevMem lanef;           // per-element flag bytes
    std::map<uintptr_t, cft_buffer *> bufs;   // mirror base -> buffer
};

namespace cftg {

// Reference conventions (cft.h:1166-1208; device.c:1699-1810).
bool check_dev(cft_device *dev, const char *who);
// Emit a call's flags: ORed into the sticky word unless muted, and written
// to flags_out when non-NULL (reference softfloat.h:293-330).
void flags_emit(cft_device *dev, uint32_t acc, uint32_t *flags_out);
// Mark the handle unusable after a device failure (reference HOSTAPI:
// "close it and open it again").
cft_status poison(cft_device *dev, const char *who, cudaError_t e);

// The resident buffer containing [p, p+bytes), or null.
cft_buffer *find_buffer(cft_device *dev, const void *p, size_t bytes, size_t *offset);

// Bind an input window: returns a device pointer holding the bytes of
// [p, p+bytes) (the buffer's device copy when resident; else the staging
// slot `slot`), issuing copies on `s`.
cft_status bind_input(cft_device *dev, const void *p, size_t bytes, DevMem &slot, cudaStream_t s,
                      const void **out, const char *who);

// Opcode helpers (reference softfloat.c:770-848).
bool op_assigned(int op);
bool op_is_reduction(int op);
unsigned op_operands(int op);
size_t esz_of(int fmt);

// A loaded program's executor view and its handle (program.cpp).
const SeqProgram *program_seq(const cft_program *pr, cft_device **dev);

}  // namespace cftg
