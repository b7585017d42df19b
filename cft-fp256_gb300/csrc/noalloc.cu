// noalloc.cu - a program run that allocates nothing.
//
// cft_program_run_ex sizes its lane scratch and its flag words per run and
// takes them with cudaMalloc. Some callers cannot let a library do that:
// a host that owns every byte of device memory through its own pool or
// budget (a serving process admitting work against a fixed HBM budget, a
// framework whose caching allocator must see every allocation), and a
// latency-critical caller for whom cudaMalloc and cudaFree - which may
// synchronise the whole device - are not acceptable in the run loop. For
// them, cftg_program_run_noalloc runs the same executor (seq.cu) on device
// buffers the caller already holds, with the run's scratch - each lane's
// scratch slots and the three flag/status/error words - carved from one
// file-scope device array of fixed size, NOALLOC_SCRATCH_BYTES.
//
// That array is part of the library image: every GPU that loads the
// library holds it until the process exits. Every call shares it and it
// keeps the last call's contents, so each call clears what must start at
// zero (the words here, each lane's slots in the kernel), and calls whose
// work overlaps on the GPU race on it: a caller issues them one after the
// other (the call returns only after its stream has finished the run).
//
// In host code the array's name is a host-side stand-in, not a device
// address. Its device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made
// on that device; that first call should therefore come before any stream
// capture. The address is kept for the life of the process: a caller that
// resets a device (cudaDeviceReset) or otherwise destroys its primary
// context reloads the library's module there, at another address, so such
// a caller must not use this entry point on that device afterwards.
#include <mutex>

#include "../../include/cft_gb300.h"
#include "api_core.h"

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)16 << 20;   // 16 MiB
constexpr size_t WORDS_BYTES = 256;                          // flags, status, error

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_addr_lock;
void *g_addr[64] = {nullptr};                                // per device ordinal

// The array's device address on the current device (set-up on first use).
cudaError_t scratch_address(int ordinal, unsigned char **out)
{
    if (ordinal < 0 || ordinal >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_addr_lock);
    if (!g_addr[ordinal]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[ordinal] = p;
    }
    *out = static_cast<unsigned char *>(g_addr[ordinal]);
    return cudaSuccess;
}

}  // namespace

extern "C" size_t cftg_noalloc_scratch_bytes(void) { return NOALLOC_SCRATCH_BYTES - WORDS_BYTES; }

extern "C" cft_status cftg_program_run_noalloc(cft_program *prog, const void *d_a, const void *d_b,
                                               const void *d_c, const void *d_bank,
                                               const void *d_scratch_in, void *d_scratch_out,
                                               void *d_deposits, uint32_t *d_counts, size_t n,
                                               uint32_t *flags_out, uint32_t *status_out,
                                               void *stream)
{
    using namespace cftg;
    clear_error();
    if (status_out) *status_out = 0;
    cft_device *dev = nullptr;
    const SeqProgram *pp = program_seq(prog, &dev);
    if (!pp || !dev) {
        set_error("cftg_program_run_noalloc: prog is NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    SeqProgram P = *pp;
    if (dev->poisoned) {
        set_error("cftg_program_run_noalloc: this handle failed earlier; close it and open it "
                  "again");
        return CFT_ERR_INTERNAL;
    }
    if (n == 0) {
        flags_emit(dev, 0, flags_out);
        return CFT_OK;
    }
    const size_t esz = esz_of(P.fmt);
    if (!d_a || (P.max_deposits && !d_deposits) ||
        ((P.flags & CFT_PROG_FLAG_BANK_EXT) && P.n_consts && !d_bank) ||
        (P.n_scratch_in && !d_scratch_in) || (P.n_scratch_out && !d_scratch_out)) {
        set_error("cftg_program_run_noalloc: a buffer this program reads or writes is NULL "
                  "(a, deposits, bank, scratch in or out)");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    // the whole run's lane scratch must fit the fixed array
    const size_t per_lane = (size_t)P.reach * esz;
    if (per_lane && n > (NOALLOC_SCRATCH_BYTES - WORDS_BYTES) / per_lane) {
        set_error("cftg_program_run_noalloc: %lu lanes x %u scratch slots x %lu bytes need %llu "
                  "bytes of scratch and this entry point has %lu (a fixed array; it allocates "
                  "nothing) - run fewer lanes a call, or use cft_program_run_ex",
                  (unsigned long)n, P.reach, (unsigned long)esz,
                  (unsigned long long)n * per_lane,
                  (unsigned long)(NOALLOC_SCRATCH_BYTES - WORDS_BYTES));
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (P.max_deposits && n > ((size_t)-1) / P.max_deposits / esz) {
        set_error("cftg_program_run_noalloc: n = %lu lanes is more than this library can size",
                  (unsigned long)n);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(dev->ordinal);
    unsigned char *base = nullptr;
    cudaError_t e = scratch_address(dev->ordinal, &base);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("cftg_program_run_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return CFT_ERR_INTERNAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *words = reinterpret_cast<uint32_t *>(base);
    e = cudaMemsetAsync(words, 0, 3 * sizeof(uint32_t), s);
    if (e == cudaSuccess && P.max_deposits)
        e = cudaMemsetAsync(d_deposits, 0, n * (size_t)P.max_deposits * esz, s);
    if (e != cudaSuccess) return poison(dev, "cftg_program_run_noalloc", e);
    if (P.flags & CFT_PROG_FLAG_BANK_EXT) P.d_consts = d_bank;

    SeqLaunch L;
    L.P = P;
    L.n = n;
    L.a = d_a;
    L.b = d_b;
    L.c = d_c;
    L.scratch_in = d_scratch_in;
    L.scratch_out = d_scratch_out;
    L.deposits = d_deposits;
    L.counts = d_counts;
    L.scratch = per_lane ? base + WORDS_BYTES : nullptr;
    L.word = words;
    e = launch_seq(L, s);
    uint32_t host_words[3] = {0, 0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host_words, words, sizeof host_words, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return poison(dev, "cftg_program_run_noalloc", e);
    if (host_words[2]) {
        set_error("cftg_program_run_noalloc: the executor reported invariant failure 0x%x",
                  host_words[2]);
        return CFT_ERR_INTERNAL;
    }
    flags_emit(dev, host_words[0] & CFT_FLAGS_ALL, flags_out);
    if (status_out) *status_out = host_words[1];
    return CFT_OK;
}
