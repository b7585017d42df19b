// sha256.cpp - SHA-256 (FIPS 180-4) for cft_sha256 and cft_program_digest.
//
// The round constants and the initial hash value are DERIVED at first use
// from their definitions in FIPS 180-4 (4.2.2: the first 32 bits of the
// fractional parts of the cube roots of the first 64 primes; 5.3.3: of the
// square roots of the first 8 primes), with exact integer roots, rather
// than written out as tables.
#include "sha256.h"

#include <cstring>

namespace cftg {

namespace {

uint32_t K[64], H0[8];
bool ready = false;

using u128 = unsigned __int128;

// floor(cbrt(x)) for x < 2^110
uint64_t icbrt(u128 x)
{
    uint64_t lo = 0, hi = (uint64_t)1 << 37;
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo + 1) / 2;
        if ((u128)mid * mid * mid <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// floor(sqrt(x)) for x < 2^70
uint64_t isqrt(u128 x)
{
    uint64_t lo = 0, hi = (uint64_t)1 << 36;
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo + 1) / 2;
        if ((u128)mid * mid <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

void derive()
{
    int primes[64], np = 0;
    for (int c = 2; np < 64; c++) {
        bool p = true;
        for (int d = 2; d * d <= c; d++)
            if (c % d == 0) { p = false; break; }
        if (p) primes[np++] = c;
    }
    for (int i = 0; i < 64; i++) K[i] = (uint32_t)icbrt((u128)primes[i] << 96);   // frac * 2^32
    for (int i = 0; i < 8; i++) H0[i] = (uint32_t)isqrt((u128)primes[i] << 64);
    ready = true;
}

inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

void block(uint32_t h[8], const uint8_t *p)
{
    uint32_t w[64];
    for (int i = 0; i < 16; i++)
        w[i] = ((uint32_t)p[4 * i] << 24) | ((uint32_t)p[4 * i + 1] << 16) |
               ((uint32_t)p[4 * i + 2] << 8) | p[4 * i + 3];
    for (int i = 16; i < 64; i++) {
        const uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
        const uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
        w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
    for (int i = 0; i < 64; i++) {
        const uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
        const uint32_t ch = (e & f) ^ (~e & g);
        const uint32_t t1 = hh + S1 + ch + K[i] + w[i];
        const uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
        const uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
        const uint32_t t2 = S0 + mj;
        hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
}

}  // namespace

void Sha256::init()
{
    if (!ready) derive();
    for (int i = 0; i < 8; i++) h[i] = H0[i];
    len = 0;
    fill = 0;
}

void Sha256::update(const void *data, size_t n)
{
    const uint8_t *p = static_cast<const uint8_t *>(data);
    len += n;
    while (n) {
        const size_t take = (64 - fill) < n ? (64 - fill) : n;
        memcpy(buf + fill, p, take);
        fill += take;
        p += take;
        n -= take;
        if (fill == 64) {
            block(h, buf);
            fill = 0;
        }
    }
}

void Sha256::final(uint8_t out[32])
{
    const uint64_t bits = len * 8;
    const uint8_t one = 0x80, zero = 0;
    update(&one, 1);
    while (fill != 56) update(&zero, 1);
    uint8_t L[8];
    for (int i = 0; i < 8; i++) L[i] = (uint8_t)(bits >> (56 - 8 * i));
    update(L, 8);
    for (int i = 0; i < 8; i++) {
        out[4 * i] = (uint8_t)(h[i] >> 24);
        out[4 * i + 1] = (uint8_t)(h[i] >> 16);
        out[4 * i + 2] = (uint8_t)(h[i] >> 8);
        out[4 * i + 3] = (uint8_t)h[i];
    }
}

}  // namespace cftg
