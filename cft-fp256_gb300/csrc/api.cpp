// api.cpp - the C ABI's hot path on the GPU: handles, the error slot, the
// status word, resident buffers, and the elementwise entry points
// (cft_run, cft_run_ex, cft_div, cft_sqrt) with the reference's argument
// rules (host/src/device.c:1699-1990, host/src/divsqrt.c:1574-1700).
//
// A call with host operands runs as a pipeline of chunks over two streams:
// chunk k's upload, kernel and download are ordered on stream k%2, so the
// copies of one chunk overlap the kernel of the next. Operands that are
// resident buffers (cft_alloc) are read from their device copies in place.
#include "api_core.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/cft_gb300.h"

using namespace cftg;

// ---- the error slot (reference cft.h:272-303) -----------------------------

static char g_err[1024];

void cftg::clear_error() { g_err[0] = '\0'; }

void cftg::set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

extern "C" const char *cft_last_error(void) { return g_err; }

// ---- small tables ------------------------------------------------------------

extern "C" uint32_t cft_abi_version(void)
{
    return ((uint32_t)CFT_ABI_VERSION_MAJOR << 16) | CFT_ABI_VERSION_MINOR;
}

extern "C" const char *cft_build_id(void) { return "unknown"; }

extern "C" const char *cft_strerror(cft_status s)
{
    switch (s) {
    case CFT_OK: return "ok";
    case CFT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CFT_ERR_UNSUPPORTED: return "operation or format not available on this device";
    case CFT_ERR_NO_DEVICE: return "no such device";
    case CFT_ERR_ARTIFACT: return "artifact missing, unreadable, or not a tile";
    case CFT_ERR_BUS_FAULT: return "memory system fault: the output is not valid";
    case CFT_ERR_OUT_OF_MEMORY: return "out of memory";
    case CFT_ERR_TIMEOUT: return "timed out";
    case CFT_ERR_INTERNAL: return "internal error";
    }
    return "unknown status";
}

size_t cftg::esz_of(int fmt) { return (fmt >= 0 && fmt <= 3) ? (size_t)(4u << fmt) : 0; }

extern "C" size_t cft_format_size(cft_format f) { return esz_of((int)f); }

extern "C" const char *cft_format_name(cft_format f)
{
    static const char *const n[4] = {"fp32", "fp64", "fp128", "fp256"};
    return ((int)f >= 0 && (int)f <= 3) ? n[(int)f] : "invalid";
}

extern "C" const char *cft_op_name(cft_op op)
{
    static const char *const names[32] = {
        "fma", "add", "sub", "mul", "abs", "neg", "copysign", "min", "max", "minnum", "maxnum",
        "select", "cmplt", "cmple", "cmpeq", nullptr, "iand", "ior", "ixor", "iadd", "isub",
        "ishl", "ishr", "icmplt", "sum", "dot", "recip_seed", "rsqrt_seed", "sumsq", "sumabs",
        "imul", "maxall"};
    const int o = (int)op;
    return (o >= 0 && o < 32 && names[o]) ? names[o] : "reserved";
}

// assigned opcodes and operands (reference softfloat.c:770-848)
bool cftg::op_assigned(int op)
{
    return (op >= 0 && op <= 14) || (op >= 16 && op <= 23) || (op >= 24 && op <= 29) || op == 30 ||
           op == 31;
}

bool cftg::op_is_reduction(int op)
{
    return op == 24 || op == 25 || op == 28 || op == 29 || op == 31;
}

unsigned cftg::op_operands(int op)
{
    switch (op) {
    case 0: return 7u;
    case 1: case 2: return 5u;
    case 3: return 3u;
    case 4: case 5: case 26: case 27: return 1u;
    case 11: return 7u;
    case 24: case 28: case 29: case 31: return 1u;
    case 25: return 3u;
    default: return op_assigned(op) ? 3u : 0u;
    }
}

// ---- device memory -------------------------------------------------------------

cudaError_t DevMem::ensure(size_t bytes)
{
    if (bytes <= cap && p) return cudaSuccess;
    release();
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        cap = 0;
        return e;
    }
    cap = want;
    return cudaSuccess;
}

void DevMem::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

// ---- devices ---------------------------------------------------------------------

bool cftg::check_dev(cft_device *dev, const char *who)
{
    if (!dev) {
        set_error("%s: dev is NULL", who);
        return false;
    }
    return true;
}

cft_status cftg::poison(cft_device *dev, const char *who, cudaError_t e)
{
    dev->poisoned = 1;
    for (auto &kv : dev->bufs)
        if (kv.second->state == B_DIRTY) kv.second->state = B_LOST;
    set_error("%s: the GPU reported %s (%s) after work may have started; this handle is "
              "unusable now - close it and open it again",
              who, cudaGetErrorName(e), cudaGetErrorString(e));
    return CFT_ERR_INTERNAL;
}

static bool poisoned(cft_device *dev, const char *who)
{
    if (dev->poisoned) {
        set_error("%s: this handle failed after a launch may have started; close it and open it "
                  "again",
                  who);
        return true;
    }
    return false;
}

void cftg::flags_emit(cft_device *dev, uint32_t acc, uint32_t *flags_out)
{
    if (dev && !dev->mute) dev->word |= acc;
    if (flags_out) *flags_out = acc;
}

// Parse the artifact: NULL, "cuda", "cuda:N", "hip:N", "gpu", "gpu:N" open
// a GPU; anything else names no device this library can open.
static bool parse_artifact(const char *artifact, int index, int *ordinal)
{
    if (!artifact) {
        *ordinal = index;
        return true;
    }
    const char *pre[3] = {"cuda", "hip", "gpu"};
    for (const char *p : pre) {
        size_t L = strlen(p);
        if (strncmp(artifact, p, L) == 0) {
            const char *rest = artifact + L;
            if (*rest == '\0') {
                *ordinal = index;
                return true;
            }
            if (*rest == ':') {
                char *end = nullptr;
                long v = strtol(rest + 1, &end, 10);
                if (end && *end == '\0' && v >= 0 && v < 1024 && end != rest + 1) {
                    if (index != 0) return false;
                    *ordinal = (int)v;
                    return true;
                }
            }
            return false;
        }
    }
    return false;
}

static cft_status open_impl(const char *who, const char *artifact, int index, uint32_t depth,
                            cft_device **out)
{
    if (!out) {
        set_error("%s: out is NULL - it receives the handle", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    int ord = 0;
    if (!parse_artifact(artifact, index, &ord)) {
        set_error("%s: \"%s\" (index %d) names no device this library opens: it opens a GPU as "
                  "NULL, \"cuda\", \"cuda:N\", \"hip:N\" or \"gpu:N\"",
                  who, artifact ? artifact : "(null)", index);
        return CFT_ERR_NO_DEVICE;
    }
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= 0) {
        set_error("%s: no CUDA device is visible (%s); this library computes on a GPU only and "
                  "has no CPU fallback",
                  who, e != cudaSuccess ? cudaGetErrorString(e) : "count is 0");
        cudaGetLastError();
        return CFT_ERR_NO_DEVICE;
    }
    if (ord < 0 || ord >= count) {
        set_error("%s: GPU %d requested and %d visible", who, ord, count);
        return CFT_ERR_NO_DEVICE;
    }
    e = cudaSetDevice(ord);
    if (e != cudaSuccess) {
        set_error("%s: cudaSetDevice(%d): %s", who, ord, cudaGetErrorString(e));
        return CFT_ERR_NO_DEVICE;
    }
    cft_device *dev = new (std::nothrow) cft_device();
    if (!dev) return CFT_ERR_OUT_OF_MEMORY;
    dev->ordinal = ord;
    dev->max_scratch = depth ? depth : 256u;
    {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, ord) !=
            cudaSuccess) {
            cudaGetLastError();
            v = 0;
        }
        dev->host_page_tables = v;
    }
    bool ok = cudaStreamCreateWithFlags(&dev->s[0], cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&dev->s[1], cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&dev->d_word, 64 * sizeof(uint32_t)) == cudaSuccess &&
              cudaHostAlloc(&dev->h_word, 64 * sizeof(uint32_t), cudaHostAllocDefault) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cft_close(dev);
        set_error("%s: could not create the handle's streams and flag words on GPU %d", who, ord);
        return CFT_ERR_OUT_OF_MEMORY;
    }
    *out = dev;
    return CFT_OK;
}

extern "C" cft_status cft_open(const char *artifact, int index, cft_device **out)
{
    clear_error();
    return open_impl("cft_open", artifact, index, 0, out);
}

extern "C" cft_status cft_open_ex(const cft_open_args *args, cft_device **out)
{
    clear_error();
    if (!out) {
        set_error("cft_open_ex: out is NULL - it receives the handle");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (!args) {
        set_error("cft_open_ex: args is NULL - pass a zeroed cft_open_args with struct_size set");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (args->struct_size != sizeof(cft_open_args)) {
        set_error("cft_open_ex was given a %lu-byte cft_open_args and this library's is %lu bytes",
                  (unsigned long)args->struct_size, (unsigned long)sizeof(cft_open_args));
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const uint32_t depth = args->scratch_depth;
    if (depth && (depth > 32768u || (depth & (depth - 1u)))) {
        set_error("cft_open_ex: scratch_depth %lu is not a power of two in 1..32768",
                  (unsigned long)depth);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    return open_impl("cft_open_ex", args->artifact, args->index, depth, out);
}

extern "C" void cft_close(cft_device *dev)
{
    if (!dev) return;
    cudaSetDevice(dev->ordinal);
    for (auto &kv : dev->bufs) {
        // the buffer stays valid as plain host memory (reference cft.h:2605-2610)
        cft_buffer *b = kv.second;
        if (b->dptr) cudaFree(b->dptr);
        b->dptr = nullptr;
        b->dev = nullptr;
    }
    dev->bufs.clear();
    for (int s = 0; s < 2; s++)
        for (int r = 0; r < 4; r++) dev->stage[s][r].release();
    for (int r = 0; r < 3; r++) {
        dev->gath[r].release();
        dev->tabs[r].release();
    }
    dev->lanef.release();
    if (dev->d_word) cudaFree(dev->d_word);
    if (dev->h_word) cudaFreeHost(dev->h_word);
    for (int s = 0; s < 2; s++)
        if (dev->s[s]) cudaStreamDestroy(dev->s[s]);
    delete dev;
}

// Sequencer features this executor implements (reference cft.h:785-1030):
// everything the software backend publishes, augmented addition and the
// segmented reductions included.
static const uint32_t SEQ_FEATURES =
    CFT_SEQ_FEAT_WIDE_CONST | CFT_SEQ_FEAT_REGS32 | CFT_SEQ_FEAT_BANK_PTR | CFT_SEQ_FEAT_KX9 |
    CFT_ALU_EXT_IMUL | CFT_SEQ_FEAT_SCRATCH | CFT_SEQ_FEAT_SCRATCH_IO | CFT_FEAT_REDUCE_SEG |
    CFT_SEQ_FEAT_AUGADD |
    CFT_SEQ_FEAT_SCRATCH_STRICT | CFT_SEQ_FEAT_SCALAR | CFT_SEQ_FEAT_INDEXED |
    CFT_SEQ_FEAT_LANE_MASK | CFT_SEQ_FEAT_SCRATCH_STEP | CFT_SEQ_FEAT_LANE_FLAGS |
    CFT_SEQ_FEAT_FLAG_CONTROL;

extern "C" uint32_t cftg_seq_features(void) { return SEQ_FEATURES; }

extern "C" cft_status cft_get_caps(cft_device *dev, cft_caps *out)
{
    clear_error();
    if (!dev || !out) {
        set_error("cft_get_caps: %s is NULL", dev ? "out" : "dev");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cft_caps c;
    memset(&c, 0, sizeof c);
    c.format_mask = 0xFu;
    c.tiles = 1;
    c.abi_version = cft_abi_version();
    c.device_version = 0;
    c.flags_readable = 1;
    snprintf(c.backend, sizeof c.backend, "cuda");
    c.max_deposits = 1u << 20;
    c.max_insns = 0xFFFFFFFFu;
    c.max_consts = 512u;
    c.seq_features = SEQ_FEATURES;
    c.max_scratch = dev->max_scratch;
    c.buffers_resident = 1;
    size_t give = out->struct_size;
    if (give > sizeof c) give = sizeof c;
    if (give < sizeof(size_t)) {
        set_error("cft_get_caps: struct_size %lu is smaller than the struct_size field itself",
                  (unsigned long)out->struct_size);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    c.struct_size = give;
    memcpy(out, &c, give);
    return CFT_OK;
}

extern "C" int cft_supports(cft_device *dev, cft_op op, cft_format fmt)
{
    if (!dev || (int)fmt < 0 || (int)fmt > 3) return 0;
    const int o = (int)op;
    if (!op_assigned(o)) return 0;
    return 1;
}

extern "C" cft_status cft_get_image_id(cft_device *dev, cft_image_id *out)
{
    clear_error();
    if (!dev || !out) return CFT_ERR_INVALID_ARGUMENT;
    if (out->struct_size >= sizeof(size_t)) out->struct_size = 0;
    set_error("cft_get_image_id: a GPU handle runs no device image; there is nothing to name");
    return CFT_ERR_UNSUPPORTED;
}

// ---- the status word (reference cft.h:3169-3267) ---------------------------------

extern "C" void cft_lower_flags(cft_device *dev, uint32_t mask)
{
    if (dev) dev->word &= ~(mask & CFT_FLAGS_ALL);
}
extern "C" void cft_raise_flags(cft_device *dev, uint32_t mask)
{
    if (dev) dev->word |= mask & CFT_FLAGS_ALL;
}
extern "C" int cft_test_flags(cft_device *dev, uint32_t mask)
{
    return (dev && (dev->word & mask & CFT_FLAGS_ALL)) ? 1 : 0;
}
extern "C" uint32_t cft_save_all_flags(cft_device *dev) { return dev ? dev->word : 0u; }
extern "C" void cft_restore_flags(cft_device *dev, uint32_t saved, uint32_t mask)
{
    if (!dev) return;
    mask &= CFT_FLAGS_ALL;
    dev->word = (dev->word & ~mask) | (saved & mask);
}
extern "C" int cft_test_saved_flags(uint32_t saved, uint32_t mask)
{
    return (saved & mask & CFT_FLAGS_ALL) ? 1 : 0;
}
extern "C" int cft_is754version1985(void) { return 0; }
extern "C" int cft_is754version2008(void) { return 0; }
extern "C" int cft_is754version2019(void) { return 1; }

// ---- resident buffers (reference cft.h:2470-2705) ----------------------------------

cft_buffer *cftg::find_buffer(cft_device *dev, const void *p, size_t bytes, size_t *offset)
{
    if (!dev || !p || dev->bufs.empty()) return nullptr;
    const uintptr_t a = (uintptr_t)p;
    auto it = dev->bufs.upper_bound(a);
    if (it == dev->bufs.begin()) return nullptr;
    --it;
    cft_buffer *b = it->second;
    const uintptr_t base = it->first;
    if (a < base || a - base > b->bytes || bytes > b->bytes - (a - base)) return nullptr;
    if (offset) *offset = (size_t)(a - base);
    return b;
}

static void buf_why(cft_buffer *b, const char *why)
{
    snprintf(b->why, sizeof b->why, "%s", why);
}

// Make the device copy current with the mirror (STALE -> FRESH).
static cft_status buf_upload(cft_buffer *b, cudaStream_t s, const char *who)
{
    if (b->state == B_LOST) {
        set_error("%s: a resident buffer was LOST by a failed run; publish it with "
                  "cft_buffer_to_device first",
                  who);
        return CFT_ERR_INTERNAL;
    }
    if (b->state != B_STALE) return CFT_OK;
    cudaError_t e = cudaMemcpyAsync(b->dptr, b->host, b->bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return poison(b->dev, who, e);
    b->state = B_FRESH;
    return CFT_OK;
}

cft_status cftg::bind_input(cft_device *dev, const void *p, size_t bytes, DevMem &slot,
                            cudaStream_t s, const void **out, const char *who)
{
    *out = nullptr;
    if (!p) return CFT_OK;
    size_t off = 0;
    cft_buffer *b = find_buffer(dev, p, bytes, &off);
    if (b) {
        const int was = b->state;
        cft_status st = buf_upload(b, s, who);
        if (st != CFT_OK) return st;
        if (was == B_STALE) {
            b->staged_binds++;
            buf_why(b, "the mirror was newer than the device copy (first use or published)");
        } else {
            b->resident_binds++;
        }
        *out = (const uint8_t *)b->dptr + off;
        return CFT_OK;
    }
    cudaError_t e = slot.ensure(bytes);
    if (e != cudaSuccess) {
        set_error("%s: could not allocate %lu bytes of device staging", who, (unsigned long)bytes);
        cudaGetLastError();
        return CFT_ERR_OUT_OF_MEMORY;
    }
    e = cudaMemcpyAsync(slot.p, p, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return poison(dev, who, e);
    *out = slot.p;
    return CFT_OK;
}

extern "C" cft_status cft_alloc(cft_device *dev, size_t bytes, cft_buffer **out)
{
    clear_error();
    if (!dev || !out) {
        set_error("cft_alloc: %s is NULL", dev ? "out" : "dev");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (poisoned(dev, "cft_alloc")) return CFT_ERR_INTERNAL;
    cft_buffer *b = new (std::nothrow) cft_buffer();
    if (!b) return CFT_ERR_OUT_OF_MEMORY;
    const size_t want = bytes ? bytes : 1;
    cudaSetDevice(dev->ordinal);
    if (cudaHostAlloc((void **)&b->host, want, cudaHostAllocDefault) != cudaSuccess ||
        cudaMalloc(&b->dptr, want) != cudaSuccess) {
        cudaGetLastError();
        if (b->host) cudaFreeHost(b->host);
        delete b;
        set_error("cft_alloc: could not allocate %lu bytes of pinned host and device memory",
                  (unsigned long)bytes);
        return CFT_ERR_OUT_OF_MEMORY;
    }
    memset(b->host, 0, want);
    b->dev = dev;
    b->bytes = bytes;
    b->state = B_STALE;
    dev->bufs[(uintptr_t)b->host] = b;
    *out = b;
    return CFT_OK;
}

extern "C" void *cft_buffer_data(cft_buffer *buf) { return buf ? buf->host : nullptr; }

extern "C" cft_status cft_buffer_to_device(cft_buffer *buf)
{
    clear_error();
    if (!buf) {
        set_error("cft_buffer_to_device: buf is NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (buf->state == B_DIRTY) {
        set_error("cft_buffer_to_device: this buffer holds a run's results that nobody has read "
                  "back; call cft_buffer_from_device first, then write the mirror and publish");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    // Moves nothing: the mirror becomes the truth, uploaded at the next bind.
    buf->state = B_STALE;
    buf->why[0] = '\0';
    return CFT_OK;
}

extern "C" cft_status cft_buffer_from_device(cft_buffer *buf)
{
    clear_error();
    if (!buf) {
        set_error("cft_buffer_from_device: buf is NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (buf->state == B_LOST) {
        set_error("cft_buffer_from_device: the buffer is LOST - a run that wrote it failed after "
                  "it may have started, so neither copy can be vouched for");
        return CFT_ERR_INTERNAL;
    }
    if (buf->state != B_DIRTY || !buf->dev) return CFT_OK;
    cft_device *dev = buf->dev;
    cudaError_t e = cudaMemcpyAsync(buf->host, buf->dptr, buf->bytes, cudaMemcpyDeviceToHost,
                                    dev->s[0]);
    if (e == cudaSuccess) e = cudaStreamSynchronize(dev->s[0]);
    if (e != cudaSuccess) return poison(dev, "cft_buffer_from_device", e);
    buf->state = B_FRESH;
    return CFT_OK;
}

extern "C" void cft_buffer_free(cft_buffer *buf)
{
    if (!buf) return;
    if (buf->dev) {
        buf->dev->bufs.erase((uintptr_t)buf->host);
        cudaStreamSynchronize(buf->dev->s[0]);
        cudaStreamSynchronize(buf->dev->s[1]);
        if (buf->dptr) cudaFree(buf->dptr);
    }
    if (buf->host) cudaFreeHost(buf->host);
    delete buf;
}

extern "C" cft_status cft_buffer_get_info(cft_buffer *buf, cft_buffer_info *out)
{
    clear_error();
    if (!buf || !out) return CFT_ERR_INVALID_ARGUMENT;
    cft_buffer_info i;
    memset(&i, 0, sizeof i);
    i.bytes = buf->bytes;
    i.resident = (buf->dev && buf->state != B_STALE) ? 1 : 0;
    i.device_authority = buf->state == B_DIRTY ? 1 : 0;
    i.resident_binds = buf->resident_binds;
    i.staged_binds = buf->staged_binds;
    if (buf->state == B_LOST)
        snprintf(i.staged_why, sizeof i.staged_why, "LOST: a run that wrote this buffer failed");
    else
        snprintf(i.staged_why, sizeof i.staged_why, "%s", buf->why);
    size_t give = out->struct_size;
    if (give > sizeof i) give = sizeof i;
    if (give < sizeof(size_t)) return CFT_ERR_INVALID_ARGUMENT;
    i.struct_size = give;
    memcpy(out, &i, give);
    return CFT_OK;
}

// ---- the elementwise path ------------------------------------------------------------

namespace {

struct Operand {
    const void *host = nullptr;   // the caller's pointer
    cft_buffer *buf = nullptr;     // resident buffer holding it, if any
    size_t off = 0;
    size_t count = 0;              // elements the window holds
    bool scalar = false;
    const uint32_t *idx = nullptr; // index table (host pointer)
    size_t src = 0;
    const void *dev = nullptr;     // device pointer of the whole window (when not chunked)
    const uint32_t *dtab = nullptr;
};

bool windows_overlap(const void *a, size_t an, const void *b, size_t bn)
{
    const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
    return x < y + bn && y < x + an;
}

}  // namespace

// The kernels load an element as 4-, 8- or 16-byte vectors, so an operand
// must start on that boundary; anything else is staged through aligned
// device memory by cudaMemcpy, which takes any alignment.
static bool aligned_for(const void *p, size_t esz)
{
    const uintptr_t a = esz >= 16 ? 16 : esz;
    return ((uintptr_t)p % a) == 0;
}

// A pointer a kernel can dereference for the caller's host memory, or NULL:
// pinned host memory through its mapped device pointer, and on a system
// whose GPU walks the host page tables (Grace's NVLink-C2C with ATS) any
// host pointer as it is.
static const void *device_view(cft_device *dev, const void *p, size_t esz)
{
    if (!p || !aligned_for(p, esz)) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    const void *v = nullptr;
    if ((at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeDevice ||
         at.type == cudaMemoryTypeManaged) && at.devicePointer)
        v = at.devicePointer;
    else if (at.type == cudaMemoryTypeUnregistered && dev->host_page_tables)
        v = p;
    return (v && aligned_for(v, esz)) ? v : nullptr;
}

// The direct route: every operand and the output are reachable by the
// kernel where they are, so one launch reads and writes them in place (no
// staging copies; the host link carries only the bytes the kernel touches).
static bool exec_direct(const char *who, cft_device *dev, int kind, int op, int fmt, int rnd,
                        const void *const opnd[3], void *d, size_t n, uint32_t scalar_mask,
                        uint32_t *flags_out, cft_status *st)
{
    const size_t esz = esz_of(fmt);
    const char *mode = getenv("CFTG_HOST_ACCESS");
    if (mode && strcmp(mode, "stage") == 0) return false;
    const void *v[3] = {nullptr, nullptr, nullptr};
    for (int r = 0; r < 3; r++) {
        if (!opnd[r]) continue;
        if (find_buffer(dev, opnd[r], esz, nullptr)) return false;
        v[r] = device_view(dev, opnd[r], esz);
        if (!v[r]) return false;
    }
    if (find_buffer(dev, d, esz, nullptr)) return false;
    void *vd = const_cast<void *>(device_view(dev, d, esz));
    if (!vd) return false;
    cudaStream_t s = dev->s[0];
    ElemLaunch L;
    L.fmt = fmt;
    L.kind = kind;
    L.op = op;
    L.rnd = rnd;
    L.a = v[0];
    L.b = v[1];
    L.c = v[2];
    L.d = vd;
    L.n = n;
    L.scalar_mask = scalar_mask & 7u;
    L.flags = dev->d_word;
    // Two blocks an SM: the host link carries ~211 GB/s, which a few warps an
    // SM saturate, and more requests in flight over it lower what it carries
    // (fp256 FMA in place: 2.13 Gelem/s at one or two blocks an SM, 1.83 at
    // three, 1.65 at four). CFTG_HOST_BLOCKS_PER_SM overrides.
    {
        static const int per = [] {
            const char *v = getenv("CFTG_HOST_BLOCKS_PER_SM");
            return v && atoi(v) > 0 ? atoi(v) : 2;
        }();
        L.blocks_per_sm = (uint32_t)per;
    }
    cudaError_t e = cudaMemsetAsync(dev->d_word, 0, sizeof(uint32_t), s);
    if (e == cudaSuccess) e = launch_elem(L, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dev->h_word, dev->d_word, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        *st = poison(dev, who, e);
        return true;
    }
    if (dev->h_word[0] & ELEM_ERR_STAGING) {
        set_error("%s: a staged operand load did not complete in time; outputs are incomplete", who);
        *st = CFT_ERR_INTERNAL;
        return true;
    }
    flags_emit(dev, dev->h_word[0] & CFT_FLAGS_ALL, flags_out);
    *st = CFT_OK;
    return true;
}

// One elementwise run after the reference's argument checks have passed.
static cft_status exec_elem(const char *who, cft_device *dev, int kind, int op, int fmt, int rnd,
                            const void *a, const void *b, const void *c, void *d, size_t n,
                            uint32_t scalar_mask, const uint32_t *const idx[3],
                            const size_t src[3], uint32_t *flags_out)
{
    const size_t esz = esz_of(fmt);
    cudaSetDevice(dev->ordinal);
    const unsigned need = (kind == K_DIV) ? 3u : (kind == K_SQRT) ? 1u : op_operands(op);
    Operand o[3];
    const void *ptr[3] = {a, b, c};
    if (!idx) {
        const void *read[3];
        for (int r = 0; r < 3; r++) read[r] = ((need >> r) & 1u) ? ptr[r] : nullptr;
        cft_status st;
        if (exec_direct(who, dev, kind, op, fmt, rnd, read, d, n, scalar_mask, flags_out, &st))
            return st;
    }
    for (int r = 0; r < 3; r++) {
        if (!ptr[r] || !((need >> r) & 1u)) continue;   // unread operands read as +0
        o[r].host = ptr[r];
        o[r].scalar = (scalar_mask >> r) & 1u;
        o[r].idx = idx ? idx[r] : nullptr;
        o[r].src = src ? src[r] : 0;
        o[r].count = o[r].idx ? o[r].src : (o[r].scalar ? 1 : n);
        o[r].buf = find_buffer(dev, ptr[r], o[r].count * esz, &o[r].off);
    }
    size_t doff = 0;
    cft_buffer *dbuf = find_buffer(dev, d, n * esz, &doff);
    if (dbuf && dbuf->state == B_LOST) {
        set_error("%s: the output is a LOST resident buffer; publish it first", who);
        return CFT_ERR_INTERNAL;
    }

    // Resident inputs that overlap a resident output other than exactly
    // (same pointer, dense) are copied aside: lanes run in no fixed order.
    bool copy_aside[3] = {false, false, false};
    for (int r = 0; r < 3; r++) {
        if (!o[r].host || !o[r].buf || !dbuf || o[r].buf != dbuf) continue;
        const bool same = o[r].host == d && !o[r].scalar && !o[r].idx;
        if (!same && windows_overlap(o[r].host, o[r].count * esz, d, n * esz)) copy_aside[r] = true;
    }
    for (int r = 0; r < 3; r++)
        if (o[r].buf && !aligned_for(o[r].host, esz)) copy_aside[r] = true;
    // An output inside a resident buffer at an offset the kernels cannot
    // store to is written through the mirror instead: the run's bytes come
    // home first if the device held newer ones, and the buffer is stale after.
    cft_buffer *dbuf_mirror = nullptr;
    if (dbuf && !aligned_for(d, esz)) {
        if (dbuf->state == B_DIRTY) {
            cft_status st0 = cft_buffer_from_device(dbuf);
            if (st0 != CFT_OK) return st0;
        }
        dbuf_mirror = dbuf;
        dbuf = nullptr;
    }

    cudaStream_t s0 = dev->s[0];
    cft_status st;
    // Whole-window operands: scalar, indexed, resident or copied aside.
    for (int r = 0; r < 3; r++) {
        if (!o[r].host) continue;
        const bool whole = o[r].scalar || o[r].idx || o[r].buf;
        if (!whole) continue;
        if (o[r].buf && !copy_aside[r]) {
            st = bind_input(dev, o[r].host, o[r].count * esz, dev->gath[r], s0, &o[r].dev, who);
        } else if (o[r].buf && copy_aside[r]) {
            const void *res = nullptr;
            st = bind_input(dev, o[r].host, o[r].count * esz, dev->gath[r], s0, &res, who);
            if (st == CFT_OK) {
                if (dev->gath[r].ensure(o[r].count * esz) != cudaSuccess) {
                    cudaGetLastError();
                    return CFT_ERR_OUT_OF_MEMORY;
                }
                cudaError_t e = cudaMemcpyAsync(dev->gath[r].p, res, o[r].count * esz,
                                                cudaMemcpyDeviceToDevice, s0);
                if (e != cudaSuccess) return poison(dev, who, e);
                o[r].dev = dev->gath[r].p;
            }
        } else {
            st = bind_input(dev, o[r].host, o[r].count * esz, dev->gath[r], s0, &o[r].dev, who);
        }
        if (st != CFT_OK) return st;
        if (o[r].idx) {
            const void *t = nullptr;
            st = bind_input(dev, o[r].idx, n * sizeof(uint32_t), dev->tabs[r], s0, &t, who);
            if (st != CFT_OK) return st;
            o[r].dtab = (const uint32_t *)t;
        }
    }
    // The output: a resident buffer's device copy, made current first so
    // the bytes around the window stay the mirror's.
    void *dd = nullptr;
    if (dbuf) {
        st = buf_upload(dbuf, s0, who);
        if (st != CFT_OK) return st;
        dd = (uint8_t *)dbuf->dptr + doff;
    }

    // Chunks: host dense operands and a host output are streamed.
    bool any_stream = !dbuf;
    for (int r = 0; r < 3; r++)
        if (o[r].host && !o[r].dev) any_stream = true;
    const size_t chunk_bytes = (size_t)32 << 20;
    size_t chunk = any_stream ? (chunk_bytes / esz) : n;
    if (chunk == 0) chunk = 1;
    if (chunk > n) chunk = n;
    const size_t nchunks = (n + chunk - 1) / chunk;

    cudaEvent_t ready = nullptr;
    if (nchunks > 0) {
        // stream 1 must see stream 0's whole-window uploads
        if (cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return CFT_ERR_INTERNAL;
        }
        cudaEventRecord(ready, s0);
        cudaStreamWaitEvent(dev->s[1], ready, 0);
    }
    for (int slot = 0; slot < 2; slot++)
        cudaMemsetAsync(dev->d_word + slot, 0, sizeof(uint32_t), dev->s[slot]);

    for (size_t k = 0; k < nchunks; k++) {
        const int slot = (int)(k & 1);
        cudaStream_t s = dev->s[slot];
        const size_t start = k * chunk, cnt = (n - start < chunk) ? n - start : chunk;
        ElemLaunch L;
        L.fmt = fmt;
        L.kind = kind;
        L.op = op;
        L.rnd = rnd;
        L.n = cnt;
        L.flags = dev->d_word + slot;
        L.scalar_mask = scalar_mask & 7u;
        const void **lp[3] = {&L.a, &L.b, &L.c};
        const uint32_t **lt[3] = {&L.ia, &L.ib, &L.ic};
        for (int r = 0; r < 3; r++) {
            if (!o[r].host) {
                *lp[r] = nullptr;
                continue;
            }
            if (o[r].dev) {
                if (o[r].idx) {
                    *lp[r] = o[r].dev;
                    *lt[r] = o[r].dtab + start;
                } else if (o[r].scalar) {
                    *lp[r] = o[r].dev;
                } else {
                    *lp[r] = (const uint8_t *)o[r].dev + start * esz;
                }
                continue;
            }
            DevMem &m = dev->stage[slot][r];
            if (m.ensure(chunk * esz) != cudaSuccess) {
                cudaGetLastError();
                set_error("%s: could not allocate device staging", who);
                if (ready) cudaEventDestroy(ready);
                return CFT_ERR_OUT_OF_MEMORY;
            }
            cudaError_t e = cudaMemcpyAsync(m.p, (const uint8_t *)o[r].host + start * esz,
                                            cnt * esz, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) {
                if (ready) cudaEventDestroy(ready);
                return poison(dev, who, e);
            }
            *lp[r] = m.p;
        }
        if (dbuf) {
            L.d = (uint8_t *)dd + start * esz;
        } else {
            DevMem &m = dev->stage[slot][3];
            if (m.ensure(chunk * esz) != cudaSuccess) {
                cudaGetLastError();
                set_error("%s: could not allocate device staging", who);
                if (ready) cudaEventDestroy(ready);
                return CFT_ERR_OUT_OF_MEMORY;
            }
            L.d = m.p;
        }
        cudaError_t e = launch_elem(L, s);
        if (e == cudaSuccess && !dbuf)
            e = cudaMemcpyAsync((uint8_t *)d + start * esz, L.d, cnt * esz, cudaMemcpyDeviceToHost,
                                s);
        if (e != cudaSuccess) {
            if (ready) cudaEventDestroy(ready);
            return poison(dev, who, e);
        }
    }
    for (int slot = 0; slot < 2; slot++)
        cudaMemcpyAsync(dev->h_word + slot, dev->d_word + slot, sizeof(uint32_t),
                        cudaMemcpyDeviceToHost, dev->s[slot]);
    cudaError_t e0 = cudaStreamSynchronize(dev->s[0]);
    cudaError_t e1 = cudaStreamSynchronize(dev->s[1]);
    if (ready) cudaEventDestroy(ready);
    if (e0 != cudaSuccess || e1 != cudaSuccess)
        return poison(dev, who, e0 != cudaSuccess ? e0 : e1);
    if ((dev->h_word[0] | dev->h_word[1]) & ELEM_ERR_STAGING) {
        // a resident output holds a partial run: LOST, as after a failed run
        if (dbuf) dbuf->state = B_LOST;
        set_error("%s: a staged operand load did not complete in time; outputs are incomplete", who);
        return CFT_ERR_INTERNAL;
    }
    if (dbuf) dbuf->state = B_DIRTY;
    if (dbuf_mirror) dbuf_mirror->state = B_STALE;
    flags_emit(dev, (dev->h_word[0] | dev->h_word[1]) & CFT_FLAGS_ALL, flags_out);
    return CFT_OK;
}

// The reference's argument rules for an elementwise run, in its order
// (host/src/device.c:1699-1990).
static cft_status run_impl(const char *who, cft_device *dev, int op, int fmt, int rnd,
                           const void *a, const void *b, const void *c, void *d, size_t n,
                           uint32_t scalar_mask, const uint32_t *const idx[3], const size_t src[3],
                           uint32_t *flags_out, uint32_t *bus_out)
{
    if (bus_out) *bus_out = 0;
    if (!check_dev(dev, who)) return CFT_ERR_INVALID_ARGUMENT;
    if (fmt < 0 || fmt > 3) {
        set_error("%s: format %d is not a cft_format (CFT_FP32 to CFT_FP256, 0 to 3)", who, fmt);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (rnd < 0 || rnd > 4) {
        set_error("%s: rounding attribute %d is not a cft_round (CFT_RNE to CFT_RMM, 0 to 4)", who,
                  rnd);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (op < 0 || op > 255) {
        set_error("%s: opcode %d does not fit the device's opcode byte (0 to 255)", who, op);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (op_is_reduction(op)) {
        set_error("%s: opcode %d (%s) is a reduction - n inputs, one output - and is issued "
                  "through cft_reduce, which %s does not take",
                  who, op, cft_op_name((cft_op)op), who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (poisoned(dev, who)) return CFT_ERR_INTERNAL;
    if (n == 0) {
        flags_emit(dev, 0, flags_out);
        return CFT_OK;
    }
    if (!d) {
        set_error("%s: d is NULL, and %llu elements are to be written to it", who,
                  (unsigned long long)n);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const unsigned need = op_operands(op);
    if (((need & 1u) && !a) || ((need & 2u) && !b) || ((need & 4u) && !c)) {
        set_error("%s: opcode %d (%s) reads operand %c, which is NULL", who, op,
                  cft_op_name((cft_op)op),
                  ((need & 1u) && !a) ? 'a' : ((need & 2u) && !b) ? 'b' : 'c');
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const size_t esz = esz_of(fmt);
    if (n > ((size_t)-1) / esz) {
        set_error("%s: n = %llu elements of %lu bytes are more bytes than a size_t counts", who,
                  (unsigned long long)n, (unsigned long)esz);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    bool tables = idx && (idx[0] || idx[1] || idx[2]);
    if (tables) {
        const void *opnd[3] = {a, b, c};
        for (int r = 0; r < 3; r++) {
            if (!opnd[r]) continue;
            const size_t ob = (idx[r] ? src[r] : ((scalar_mask >> r) & 1u) ? 1u : n) * esz;
            if (windows_overlap(d, n * esz, opnd[r], ob)) {
                set_error("%s: d overlaps operand %c, and a run with an index table may not write "
                          "over any of its operands; give the gather its own output",
                          who, 'a' + r);
                return CFT_ERR_INVALID_ARGUMENT;
            }
        }
        for (int r = 0; r < 3; r++) {
            if (!idx[r]) continue;
            // a resident table is read on the host from its current bytes
            size_t off = 0;
            cft_buffer *tb = find_buffer(dev, idx[r], n * 4, &off);
            if (tb && tb->state == B_DIRTY) {
                cft_status st = cft_buffer_from_device(tb);
                if (st != CFT_OK) return st;
            }
            for (size_t e = 0; e < n; e++) {
                const uint32_t t = idx[r][e];
                if (t != CFT_IDX_NONE && (size_t)t >= src[r]) {
                    set_error("%s: idx_%c[%lu] = %lu is at or past the %lu elements idx_%c_src "
                              "says operand %c holds",
                              who, 'a' + r, (unsigned long)e, (unsigned long)t,
                              (unsigned long)src[r], 'a' + r, 'a' + r);
                    return CFT_ERR_INVALID_ARGUMENT;
                }
            }
        }
    }
    return exec_elem(who, dev, elem_kind_of_op(op), op, fmt, rnd, a, b, c, d, n, scalar_mask,
                     tables ? idx : nullptr, tables ? src : nullptr, flags_out);
}

extern "C" cft_status cft_run(cft_device *dev, cft_op op, cft_format fmt, cft_round rnd,
                              const void *a, const void *b, const void *c, void *d, size_t n,
                              uint32_t *flags_out, uint32_t *bus_out)
{
    clear_error();
    return run_impl("cft_run", dev, (int)op, (int)fmt, (int)rnd, a, b, c, d, n, 0, nullptr,
                    nullptr, flags_out, bus_out);
}

extern "C" cft_status cft_run_ex(cft_device *dev, cft_op op, cft_format fmt, cft_round rnd,
                                 const cft_elem_args *args)
{
    clear_error();
    if (!dev || !args) {
        set_error("cft_run_ex: %s is NULL", dev ? "args" : "dev");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (args->struct_size != sizeof(cft_elem_args)) {
        set_error("cft_run_ex was given a %lu-byte cft_elem_args and this library's is %lu bytes",
                  (unsigned long)args->struct_size, (unsigned long)sizeof(cft_elem_args));
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (args->scalar_mask & ~7u) {
        set_error("cft_run_ex: scalar_mask 0x%lx sets bits above the three operands",
                  (unsigned long)args->scalar_mask);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (((args->scalar_mask & 1u) && !args->a) || ((args->scalar_mask & 2u) && !args->b) ||
        ((args->scalar_mask & 4u) && !args->c)) {
        set_error("cft_run_ex: scalar_mask names a NULL operand as one element every lane reads");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const uint32_t *idx[3] = {args->idx_a, args->idx_b, args->idx_c};
    const size_t src[3] = {args->idx_a_src, args->idx_b_src, args->idx_c_src};
    const void *opnd[3] = {args->a, args->b, args->c};
    for (int r = 0; r < 3; r++) {
        if (!idx[r]) {
            if (src[r]) {
                set_error("cft_run_ex: idx_%c_src = %lu names a source length for operand %c, "
                          "which has no index table",
                          'a' + r, (unsigned long)src[r], 'a' + r);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            continue;
        }
        if (!opnd[r]) {
            set_error("cft_run_ex: idx_%c indexes operand %c, which is NULL", 'a' + r, 'a' + r);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        if (args->scalar_mask & (1u << r)) {
            set_error("cft_run_ex: operand %c is both scalar and indexed", 'a' + r);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        if (src[r] == 0) {
            set_error("cft_run_ex: idx_%c is set and idx_%c_src is zero", 'a' + r, 'a' + r);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    }
    const int o = (int)op;
    if (o >= 0 && o <= 255 && !op_is_reduction(o)) {
        const unsigned need = op_operands(o);
        for (int r = 0; r < 3; r++)
            if (idx[r] && !((need >> r) & 1u)) {
                set_error("cft_run_ex: idx_%c gathers operand %c and opcode %d (%s) does not read "
                          "it",
                          'a' + r, 'a' + r, o, cft_op_name(op));
                return CFT_ERR_INVALID_ARGUMENT;
            }
    }
    return run_impl("cft_run_ex", dev, o, (int)fmt, (int)rnd, args->a, args->b, args->c, args->d,
                    args->n, args->scalar_mask, idx, src, args->flags_out, args->bus_out);
}

// cft_div / cft_sqrt (reference divsqrt.c:1574-1700): the contract's
// correctly rounded quotient and root, one kernel pass each.
static cft_status divsqrt(const char *who, cft_device *dev, int fmt, int rnd, const void *a,
                          const void *b, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out,
                          bool is_div)
{
    if (bus_out) *bus_out = 0;
    if (!dev) {
        set_error("%s: dev is NULL", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (fmt < 0 || fmt > 3 || rnd < 0 || rnd > 4) {
        set_error("%s: format %d or rounding attribute %d is out of range", who, fmt, rnd);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (poisoned(dev, who)) return CFT_ERR_INTERNAL;
    if (n == 0) {
        flags_emit(dev, 0, flags_out);
        return CFT_OK;
    }
    if (!a || !d || (is_div && !b)) {
        set_error("%s: %s is NULL", who, !a ? "a" : !d ? "d" : "b");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const size_t esz = esz_of(fmt);
    if (n > ((size_t)-1) / esz) {
        set_error("%s: n = %llu elements is more bytes than a size_t counts", who,
                  (unsigned long long)n);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    return exec_elem(who, dev, is_div ? K_DIV : K_SQRT, is_div ? 0 : 0, fmt, rnd, a,
                     is_div ? b : nullptr, nullptr, d, n, 0, nullptr, nullptr, flags_out);
}

extern "C" cft_status cft_div(cft_device *dev, cft_format fmt, cft_round rnd, const void *a,
                              const void *b, void *d, size_t n, uint32_t *flags_out,
                              uint32_t *bus_out)
{
    clear_error();
    return divsqrt("cft_div", dev, (int)fmt, (int)rnd, a, b, d, n, flags_out, bus_out, true);
}

extern "C" cft_status cft_sqrt(cft_device *dev, cft_format fmt, cft_round rnd, const void *a,
                               void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out)
{
    clear_error();
    return divsqrt("cft_sqrt", dev, (int)fmt, (int)rnd, a, nullptr, d, n, flags_out, bus_out,
                   false);
}

// ---- device-pointer entry points (include/cft_gb300.h) -------------------------------

extern "C" cft_status cftg_run_device(cft_device *dev, int kind, cft_op op, cft_format fmt,
                                      cft_round rnd, const void *a, const void *b, const void *c,
                                      void *d, size_t n, uint32_t scalar_mask,
                                      uint8_t *lane_flags, uint32_t *flags_word, void *stream)
{
    clear_error();
    if (!check_dev(dev, "cftg_run_device")) return CFT_ERR_INVALID_ARGUMENT;
    if ((int)fmt < 0 || (int)fmt > 3 || (int)rnd < 0 || (int)rnd > 4 || (int)op < 0 ||
        (int)op > 255 || kind < 0 || kind > 2 || (scalar_mask & ~7u)) {
        set_error("cftg_run_device: an argument is out of range");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (kind == 0 && op_is_reduction((int)op)) {
        set_error("cftg_run_device: opcode %d is a reduction", (int)op);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (poisoned(dev, "cftg_run_device")) return CFT_ERR_INTERNAL;
    if (n == 0) return CFT_OK;
    if (!d || !a || !flags_word) {
        set_error("cftg_run_device: d, a and flags_word must be device pointers");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    ElemLaunch L;
    L.fmt = (int)fmt;
    L.kind = kind == 1 ? K_DIV : kind == 2 ? K_SQRT : elem_kind_of_op((int)op);
    L.op = (int)op;
    L.rnd = (int)rnd;
    L.a = a;
    L.b = b;
    L.c = c;
    L.d = d;
    L.n = n;
    L.scalar_mask = scalar_mask;
    L.flags = flags_word;
    L.lane_flags = lane_flags;
    cudaError_t e = launch_elem(L, (cudaStream_t)stream);
    if (e != cudaSuccess) return poison(dev, "cftg_run_device", e);
    return CFT_OK;
}

extern "C" int cftg_device_ordinal(cft_device *dev) { return dev ? dev->ordinal : -1; }
