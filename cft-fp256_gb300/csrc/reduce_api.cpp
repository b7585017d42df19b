// reduce_api.cpp - cft_reduce and cft_reduce_seg (reference include/cft.h:
// 1210-1330, host/src/device.c:2731-3420) over the GPU tree of reduce.cu,
// and cftg_reduce_device over device memory.
//
// Argument rules in the reference's order: dev, format, rounding attribute,
// reduction opcode, d; n == 0 gives the identity (+0, MAXALL -inf) with no
// flags before the operand check; then the operands the opcode reads; for
// the segmented form a segment of at least one element that divides n.
#include <algorithm>
#include <cstring>

#include "../../include/cft_gb300.h"
#include "api_core.h"

using namespace cftg;

namespace {

int mode_of(int op)
{
    switch (op) {
    case 24: return RED_SUM;
    case 25: return RED_DOT;
    case 28: return RED_SQ;
    case 29: return RED_ABS;
    default: return RED_MAX;
    }
}

bool aligned(const void *p, size_t esz)
{
    const size_t need = esz < 16 ? esz : 16;
    return ((uintptr_t)p % need) == 0;
}

// The common checks; *done when the call is already answered (n == 0).
cft_status check(const char *who, cft_device *dev, int op, int fmt, int rnd, const void *a,
                 const void *b, void *d, size_t n, size_t nres, uint32_t *flags_out, bool *done)
{
    *done = false;
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
    if (!op_is_reduction(op)) {
        set_error("%s: opcode %d (%s) is not a reduction, and elementwise opcodes are issued "
                  "through cft_run", who, op, cft_op_name((cft_op)op));
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (!d) {
        set_error("%s: d is NULL, and %s written there", who,
                  nres == 1 ? "the result is one element" : "one result per segment is");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (dev->poisoned) {
        set_error("%s: this handle is unusable after a device failure - close it and open it "
                  "again", who);
        return CFT_ERR_INTERNAL;
    }
    const size_t esz = esz_of(fmt);
    if (n == 0) {
        *done = true;
        return CFT_OK;
    }
    const unsigned need = op == 25 ? 3u : 1u;
    if (((need & 1u) && !a) || ((need & 2u) && !b)) {
        set_error("%s: opcode %d (%s) reads operand %c, which is NULL", who, op,
                  cft_op_name((cft_op)op), ((need & 1u) && !a) ? 'a' : 'b');
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (n > ((size_t)-1) / esz) {
        set_error("%s: n = %llu elements of %lu bytes are more bytes than a size_t counts", who,
                  (unsigned long long)n, (unsigned long)esz);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    (void)flags_out;
    return CFT_OK;
}

// An operand on the device, vector-aligned: the resident copy or staging.
cft_status operand(cft_device *dev, const void *p, size_t bytes, size_t esz, DevMem &slot,
                   DevMem &aside, cudaStream_t s, const void **out, const char *who)
{
    cft_status st = bind_input(dev, p, bytes, slot, s, out, who);
    if (st != CFT_OK || !*out || aligned(*out, esz)) return st;
    cudaError_t e = aside.ensure(bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("%s: could not allocate %lu bytes to realign an operand", who, (unsigned long)bytes);
        return CFT_ERR_OUT_OF_MEMORY;
    }
    e = cudaMemcpyAsync(aside.p, *out, bytes, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return poison(dev, who, e);
    *out = aside.p;
    return CFT_OK;
}

// The result written on the host: a resident buffer holding d has its
// device bytes brought home first and is marked for upload after
// (reference softfloat.h's cft_host_out).
cft_status host_out_begin(cft_device *dev, void *d, size_t bytes, cft_buffer **buf)
{
    size_t off = 0;
    *buf = find_buffer(dev, d, bytes, &off);
    if (*buf && (*buf)->state == B_DIRTY) return cft_buffer_from_device(*buf);
    return CFT_OK;
}

void host_out_end(cft_buffer *buf)
{
    if (buf && buf->state != B_LOST) buf->state = B_STALE;
}

void identity(int op, int fmt, void *d)
{
    const size_t esz = esz_of(fmt);
    memset(d, 0, esz);
    if (op == 31) {                              // -inf
        static const uint32_t top[4] = {0xFF800000u, 0xFFF00000u, 0xFFFF0000u, 0xFFFFF000u};
        uint32_t w = top[fmt];
        memcpy(static_cast<uint8_t *>(d) + esz - 4, &w, 4);
    }
}

}  // namespace

extern "C" cft_status cft_reduce(cft_device *dev, cft_op op, cft_format fmt, cft_round rnd,
                                 const void *a, const void *b, void *d, size_t n,
                                 uint32_t *flags_out, uint32_t *bus_out)
{
    clear_error();
    if (bus_out) *bus_out = 0;
    const char *who = "cft_reduce";
    bool done = false;
    cft_status st = check(who, dev, (int)op, (int)fmt, (int)rnd, a, b, d, n, 1, flags_out, &done);
    if (st != CFT_OK) return st;
    const size_t esz = esz_of((int)fmt);
    cft_buffer *ob = nullptr;
    st = host_out_begin(dev, d, esz, &ob);
    if (st != CFT_OK) return st;
    if (done) {
        identity((int)op, (int)fmt, d);
        host_out_end(ob);
        flags_emit(dev, 0u, flags_out);
        return CFT_OK;
    }
    cudaSetDevice(dev->ordinal);
    cudaStream_t s = dev->s[0];
    const void *da = nullptr, *db = nullptr;
    st = operand(dev, a, n * esz, esz, dev->gath[0], dev->stage[0][0], s, &da, who);
    if (st == CFT_OK && op == 25)
        st = operand(dev, b, n * esz, esz, dev->gath[1], dev->stage[0][1], s, &db, who);
    if (st != CFT_OK) return st;
    const size_t np = red_partial_elems(n);
    cudaError_t e = dev->tabs[0].ensure((np + 1) * esz);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("%s: could not allocate the tree's %lu partial results", who, (unsigned long)np);
        return CFT_ERR_OUT_OF_MEMORY;
    }
    uint8_t *part = static_cast<uint8_t *>(dev->tabs[0].p);
    void *dout = part + np * esz;
    e = launch_reduce((int)fmt, mode_of((int)op), da, db, n, part, dout, (int)rnd, dev->d_word, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dev->h_word, dev->d_word, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, dout, esz, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return poison(dev, who, e);
    host_out_end(ob);
    flags_emit(dev, dev->h_word[0] & CFT_FLAGS_ALL, flags_out);
    return CFT_OK;
}

extern "C" cft_status cft_reduce_seg(cft_device *dev, cft_op op, cft_format fmt, cft_round rnd,
                                     const void *a, const void *b, void *d, size_t n, size_t seg,
                                     uint32_t *flags_out, uint32_t *bus_out)
{
    clear_error();
    if (bus_out) *bus_out = 0;
    const char *who = "cft_reduce_seg";
    bool done = false;
    if (seg == 0 && dev && d && fmt >= 0 && fmt <= 3 && rnd >= 0 && rnd <= 4 &&
        op_is_reduction((int)op)) {
        set_error("cft_reduce_seg: a segment is at least one element");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const size_t nres = seg ? n / seg : 0;
    cft_status st = check(who, dev, (int)op, (int)fmt, (int)rnd, a, b, d, n, nres == 1 ? 1 : 2,
                          flags_out, &done);
    if (st != CFT_OK) return st;
    if (n % seg) {
        set_error("cft_reduce_seg: n = %lu is not a whole number of segments of %lu - the last "
                  "%lu elements would belong to no result", (unsigned long)n, (unsigned long)seg,
                  (unsigned long)(n % seg));
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (done) {
        flags_emit(dev, 0u, flags_out);
        return CFT_OK;
    }
    if (seg == n) return cft_reduce(dev, op, fmt, rnd, a, b, d, n, flags_out, bus_out);
    const size_t esz = esz_of((int)fmt);
    cft_buffer *ob = nullptr;
    st = host_out_begin(dev, d, nres * esz, &ob);
    if (st != CFT_OK) return st;
    cudaSetDevice(dev->ordinal);
    cudaStream_t s = dev->s[0];
    const void *da = nullptr, *db = nullptr;
    st = operand(dev, a, n * esz, esz, dev->gath[0], dev->stage[0][0], s, &da, who);
    if (st == CFT_OK && op == 25)
        st = operand(dev, b, n * esz, esz, dev->gath[1], dev->stage[0][1], s, &db, who);
    if (st != CFT_OK) return st;
    cudaError_t e = dev->tabs[1].ensure(nres * esz);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("%s: could not allocate %lu results", who, (unsigned long)nres);
        return CFT_ERR_OUT_OF_MEMORY;
    }
    void *dout = dev->tabs[1].p;
    // few long segments: each one's tree over the whole GPU; else one CTA a
    // segment
    const bool wide = nres < (size_t)sm_count() && seg >= ((size_t)1 << 16);
    uint32_t fl = 0;
    if (wide) {
        const size_t np = red_partial_elems(seg);
        e = dev->tabs[0].ensure((np + 1) * esz);
        for (size_t i = 0; e == cudaSuccess && i < nres; i++) {
            const uint8_t *sa = static_cast<const uint8_t *>(da) + i * seg * esz;
            const uint8_t *sb = db ? static_cast<const uint8_t *>(db) + i * seg * esz : nullptr;
            e = launch_reduce((int)fmt, mode_of((int)op), sa, sb, seg, dev->tabs[0].p,
                              static_cast<uint8_t *>(dout) + i * esz, (int)rnd, dev->d_word, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(dev->h_word, dev->d_word, 4, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e == cudaSuccess) fl |= dev->h_word[0];
        }
    } else {
        e = launch_reduce_seg((int)fmt, mode_of((int)op), da, db, nres, seg, dout, (int)rnd,
                              dev->d_word, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dev->h_word, dev->d_word, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) fl = dev->h_word[0];
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, dout, nres * esz, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return poison(dev, who, e);
    host_out_end(ob);
    flags_emit(dev, fl & CFT_FLAGS_ALL, flags_out);
    return CFT_OK;
}

// The same over DEVICE memory, asynchronous on `stream`: d_out receives
// the n / seg results (seg = n for one), d_flags[0] the flags (d_flags is
// two device words the call overwrites). d_partials: cftg_reduce_partial_
// bytes(fmt, n) bytes of device scratch for seg == n (unused otherwise).
extern "C" size_t cftg_reduce_partial_bytes(int fmt, size_t seg)
{
    if (fmt < 0 || fmt > 3) return 0;
    return (red_partial_elems(seg) + 1) * esz_of(fmt);
}

extern "C" cft_status cftg_reduce_device(cft_device *dev, int op, int fmt, int rnd, const void *a,
                                         const void *b, void *d_out, size_t n, size_t seg,
                                         void *d_partials, uint32_t *d_flags, void *stream)
{
    clear_error();
    const char *who = "cftg_reduce_device";
    bool done = false;
    if (!seg || (n % seg)) {
        set_error("%s: seg must be at least one element and divide n", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cft_status st = check(who, dev, op, fmt, rnd, a, b, d_out, n, n / seg, nullptr, &done);
    if (st != CFT_OK) return st;
    if (done) return CFT_OK;
    const size_t esz = esz_of(fmt);
    if (!aligned(a, esz) || (b && !aligned(b, esz)) || !aligned(d_out, esz) || !d_flags) {
        set_error("%s: device operands must be aligned to their element size (16 bytes at most) "
                  "and d_flags given", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    if (seg == n) {
        if (red_partial_elems(n) && !d_partials) {
            set_error("%s: this length needs %lu bytes of d_partials", who,
                      (unsigned long)cftg_reduce_partial_bytes(fmt, n));
            return CFT_ERR_INVALID_ARGUMENT;
        }
        e = launch_reduce(fmt, mode_of(op), a, b, n, d_partials, d_out, rnd, d_flags, s);
    } else {
        e = launch_reduce_seg(fmt, mode_of(op), a, b, n / seg, seg, d_out, rnd, d_flags, s);
    }
    if (e != cudaSuccess) return poison(dev, who, e);
    return CFT_OK;
}
