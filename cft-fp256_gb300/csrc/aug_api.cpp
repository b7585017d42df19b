// aug_api.cpp - cft_augmented_add / _sub / _mul (reference host/src/
// augmented.c:408-570) over the GPU kernel of aug.cu: argument rules in the
// reference's order (dev, format, n == 0 answered with no flags, the four
// pointers, r != e), operands bound like cft_run's (resident buffers read
// in place, else staged), both results copied back.
#include <cstring>

#include "../../include/cft_gb300.h"
#include "api_core.h"

using namespace cftg;

namespace {

cft_status aug_call(const char *who, cft_device *dev, int fmt, int fn, const void *a,
                    const void *b, void *r, void *e, size_t n, uint32_t *flags_out)
{
    clear_error();
    if (!dev) {
        set_error("%s: dev is NULL", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (fmt < 0 || fmt > 3) {
        set_error("%s: format %d is not a cft_format (CFT_FP32 to CFT_FP256, 0 to 3)", who, fmt);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) {
        flags_emit(dev, 0u, flags_out);
        return CFT_OK;
    }
    if (!a || !b || !r || !e) {
        set_error("%s: a, b, r and e are all required", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (r == e) {
        set_error("%s: r and e are the same buffer - two outputs of one operation", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const size_t esz = esz_of(fmt);
    if (n > ((size_t)-1) / esz) {
        set_error("%s: n = %llu elements are more bytes than a size_t counts", who,
                  (unsigned long long)n);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (dev->poisoned) {
        set_error("%s: this handle is unusable after a device failure - close it and open it "
                  "again", who);
        return CFT_ERR_INTERNAL;
    }
    const size_t bytes = n * esz;
    // outputs written on the host: resident buffers holding them come home first
    for (void *out : {r, e}) {
        size_t off = 0;
        cft_buffer *ob = find_buffer(dev, out, bytes, &off);
        if (ob && ob->state == B_DIRTY) {
            cft_status st = cft_buffer_from_device(ob);
            if (st != CFT_OK) return st;
        }
    }
    cudaSetDevice(dev->ordinal);
    cudaStream_t s = dev->s[0];
    const void *da = nullptr, *db = nullptr;
    cft_status st = bind_input(dev, a, bytes, dev->gath[0], s, &da, who);
    if (st == CFT_OK) st = bind_input(dev, b, bytes, dev->gath[1], s, &db, who);
    if (st != CFT_OK) return st;
    // a resident operand at an offset that is not word-aligned is copied
    // aside first (the kernel reads 32-bit words)
    const void **ops[2] = {&da, &db};
    for (int k = 0; k < 2; k++) {
        if (!((uintptr_t)*ops[k] & 3u)) continue;
        cudaError_t e2 = dev->stage[1][k].ensure(bytes);
        if (e2 == cudaSuccess)
            e2 = cudaMemcpyAsync(dev->stage[1][k].p, *ops[k], bytes, cudaMemcpyDeviceToDevice, s);
        if (e2 != cudaSuccess) return poison(dev, who, e2);
        *ops[k] = dev->stage[1][k].p;
    }
    cudaError_t ce = dev->stage[1][2].ensure(bytes);
    if (ce == cudaSuccess) ce = dev->stage[1][3].ensure(bytes);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        set_error("%s: could not allocate %lu bytes of results", who, (unsigned long)bytes);
        return CFT_ERR_OUT_OF_MEMORY;
    }
    void *dr = dev->stage[1][2].p, *de = dev->stage[1][3].p;
    ce = cudaMemsetAsync(dev->d_word, 0, sizeof(uint32_t), s);
    if (ce == cudaSuccess) ce = launch_aug(fmt, fn, da, db, dr, de, n, dev->d_word, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(r, dr, bytes, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(e, de, bytes, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(dev->h_word, dev->d_word, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return poison(dev, who, ce);
    for (void *out : {r, e}) {
        size_t off = 0;
        cft_buffer *ob = find_buffer(dev, out, bytes, &off);
        if (ob && ob->state != B_LOST) ob->state = B_STALE;
    }
    flags_emit(dev, dev->h_word[0] & CFT_FLAGS_ALL, flags_out);
    return CFT_OK;
}

}  // namespace

extern "C" cft_status cft_augmented_add(cft_device *dev, cft_format fmt, const void *a,
                                        const void *b, void *r, void *e, size_t n,
                                        uint32_t *flags_out)
{
    return aug_call("cft_augmented_add", dev, (int)fmt, 0, a, b, r, e, n, flags_out);
}

extern "C" cft_status cft_augmented_sub(cft_device *dev, cft_format fmt, const void *a,
                                        const void *b, void *r, void *e, size_t n,
                                        uint32_t *flags_out)
{
    return aug_call("cft_augmented_sub", dev, (int)fmt, 1, a, b, r, e, n, flags_out);
}

extern "C" cft_status cft_augmented_mul(cft_device *dev, cft_format fmt, const void *a,
                                        const void *b, void *r, void *e, size_t n,
                                        uint32_t *flags_out)
{
    return aug_call("cft_augmented_mul", dev, (int)fmt, 2, a, b, r, e, n, flags_out);
}
