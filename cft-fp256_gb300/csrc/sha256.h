// sha256.h - SHA-256 (FIPS 180-4), host side.
#pragma once
#include <cstddef>
#include <cstdint>

namespace cftg {

struct Sha256 {
    uint32_t h[8];
    uint64_t len;
    uint8_t buf[64];
    size_t fill;
    void init();
    void update(const void *data, size_t n);
    void final(uint8_t out[32]);
};

}  // namespace cftg
