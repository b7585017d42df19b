// chars.h - character sequences to encodings (754-2019 5.12.2, 5.12.3) on
// the host, in exact integer arithmetic: a decimal sequence's value is a
// rational, a hexadecimal one's a dyadic rational, and each is rounded
// once into the format. Semantics as python/cft_golden/chars.py defines
// them (reference C: host/src/chars.c): correctly rounded under the
// caller's attribute at any digit count, exact flags, NaN payloads and the
// signalling bit kept, a sequence outside the syntax refused.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cftg {
namespace chars {

// A natural number, 32-bit words little-endian, no leading zero words.
struct Nat {
    std::vector<uint32_t> w;
    bool zero() const { return w.empty(); }
    int64_t bits() const;                       // bit length (0 for zero)
    bool bit(int64_t i) const;
    bool any_below(int64_t i) const;            // a set bit below position i
    void trim();
    static Nat of(uint64_t v);
};

void mul_small(Nat &a, uint32_t m, uint32_t add);
void shl(Nat &a, int64_t s);
Nat shr(const Nat &a, int64_t s);
Nat mul(const Nat &a, const Nat &b);
int cmp(const Nat &a, const Nat &b);
void sub_in(Nat &a, const Nat &b);             // a -= b, a >= b
Nat pow10(int64_t k);                           // k >= 0
// floor(n / d) when it has at most qbits bits; *rem_nz = remainder != 0.
Nat div_bounded(const Nat &n, const Nat &d, int qbits, bool *rem_nz);

// An encoding of up to 256 bits, 32-bit words little-endian.
struct Enc {
    uint32_t w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

// Round the exact non-zero value (-1)^sign * m * 2^e into format fmt
// (0..3) under rnd (0..4), with the flags the reference's round_pack
// gives (tininess after rounding; python/cft_golden/softfloat.py:269-322).
Enc round_pack(int fmt, int sign, const Nat &m, int64_t e, int rnd, uint32_t *flags);
// (-1)^sign * num / den, num and den > 0 (chars.py:180-231).
Enc round_rational(int fmt, int sign, const Nat &num, const Nat &den, int rnd, uint32_t *flags);

// A decimal or hexadecimal-significand sequence (NUL-free, whole) into
// fmt. Returns false with *why set for a sequence outside the syntax.
bool from_decimal(int fmt, const std::string &s, int rnd, Enc *out, uint32_t *flags,
                  std::string *why);
bool from_hex(int fmt, const std::string &s, int rnd, Enc *out, uint32_t *flags, std::string *why);

// Format geometry.
struct Geo {
    int width, man_w, exp_w, prec;
    int64_t bias, emin, emax;
};
const Geo &geo(int fmt);

// The value of a finite non-zero encoding as (-1)^sign m 2^e; false for a
// zero, an infinity or a NaN.
bool decode_finite(int fmt, const Enc &x, int *sign, Nat *m, int64_t *e);

}  // namespace chars
}  // namespace cftg
