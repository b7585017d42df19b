// gen.cu - seeded synthetic operands generated on the device, for the
// benchmark and serving workloads whose arrays (tens of GB) are too large to
// build on the host. The mix matches cftgb/workload.py's per-operand mix:
// 90% normals (random sign, random fraction, unbiased exponent uniform in
// [-exp_range, exp_range]) and 10% specials (+-0, subnormals, +-inf, quiet
// and signalling NaNs with payloads, values within 2 ulp of the largest
// normal). Every word is a counter-based hash of (seed, element, word), so
// any sub-range can be regenerated independently and on any device.
#include "cftg_internal.h"
#include "softfloat.cuh"

#include "../../include/cft_gb300.h"

namespace cftg {

namespace {

// SplitMix64's finaliser (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014), used as a counter hash.
SFD uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

SFD uint64_t h3(uint64_t seed, uint64_t i, uint64_t k)
{
    return mix64(mix64(seed ^ mix64(i)) + k);
}

template <int FMT>
__global__ void k_gen(uint32_t *out, size_t n, uint64_t seed, int exp_range, uint32_t special_ppm)
{
    using F = sf::Fmt<FMT>;
    constexpr int W = F::W;
    constexpr int ES = sf::exp_shift<FMT>();
    constexpr uint32_t EXPMAX = sf::exp_mask<FMT>();
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t x[W];
#pragma unroll
        for (int w = 0; w < W; w++) x[w] = (uint32_t)h3(seed, i, 16 + w);
        const uint64_t r = h3(seed, i, 1);
        const uint32_t sign = (uint32_t)(r >> 63);
        const uint32_t frac_top = x[W - 1] & ((1u << ES) - 1u);
        const bool special = (uint32_t)(r % 1000000u) < special_ppm;
        if (!special) {
            const int e = (int)((r >> 20) % (uint64_t)(2 * exp_range + 1)) - exp_range;
            x[W - 1] = (sign << 31) | ((uint32_t)(e + F::BIAS) << ES) | frac_top;
        } else {
            switch ((r >> 24) % 6u) {
            case 0:                                   // +-0
#pragma unroll
                for (int w = 0; w < W; w++) x[w] = 0u;
                x[W - 1] = sign << 31;
                break;
            case 1:                                   // subnormal
                x[W - 1] = (sign << 31) | frac_top;
                x[0] |= 1u;
                break;
            case 2:                                   // +-inf
#pragma unroll
                for (int w = 0; w < W; w++) x[w] = 0u;
                x[W - 1] = (sign << 31) | (EXPMAX << ES);
                break;
            case 3:                                   // quiet NaN
                x[W - 1] = (sign << 31) | (EXPMAX << ES) | frac_top;
                x[(F::MANW - 1) >> 5] |= 1u << ((F::MANW - 1) & 31);
                break;
            case 4:                                   // signalling NaN
                x[W - 1] = (sign << 31) | (EXPMAX << ES) | frac_top;
                x[(F::MANW - 1) >> 5] &= ~(1u << ((F::MANW - 1) & 31));
                x[0] |= 1u;
                break;
            default:                                  // within 2 ulp of max normal
#pragma unroll
                for (int w = 0; w < W; w++) x[w] = 0xFFFFFFFFu;
                x[W - 1] = (sign << 31) | ((EXPMAX - 1u) << ES) | ((1u << ES) - 1u);
                x[0] -= (uint32_t)((r >> 40) % 3u);
                break;
            }
        }
        uint32_t *p = out + i * W;
#pragma unroll
        for (int w = 0; w < W; w++) p[w] = x[w];
    }
}

}  // namespace

}  // namespace cftg

extern "C" cft_status cftg_fill_operands(int fmt, void *d_out, size_t n, uint64_t seed,
                                         int exp_range, uint32_t special_ppm, void *stream)
{
    using namespace cftg;
    if (fmt < 0 || fmt > 3 || !d_out || exp_range < 0 || exp_range > 100 || special_ppm > 1000000u)
        return CFT_ERR_INVALID_ARGUMENT;
    if (n == 0) return CFT_OK;
    const size_t want = (n + 255) / 256;
    const unsigned blocks = (unsigned)(want < (size_t)sm_count() * 16 ? want : (size_t)sm_count() * 16);
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *o = static_cast<uint32_t *>(d_out);
    switch (fmt) {
    case 0: k_gen<0><<<blocks, 256, 0, s>>>(o, n, seed, exp_range, special_ppm); break;
    case 1: k_gen<1><<<blocks, 256, 0, s>>>(o, n, seed, exp_range, special_ppm); break;
    case 2: k_gen<2><<<blocks, 256, 0, s>>>(o, n, seed, exp_range, special_ppm); break;
    default: k_gen<3><<<blocks, 256, 0, s>>>(o, n, seed, exp_range, special_ppm); break;
    }
    return cudaGetLastError() == cudaSuccess ? CFT_OK : CFT_ERR_INTERNAL;
}
