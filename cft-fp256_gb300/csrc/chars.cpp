// chars.cpp - exact character-sequence conversions on the host (see
// chars.h), and the two C-ABI batch entry points that carry them,
// cft_from_decimal_char and cft_from_hex_char (reference cft.h:1857-1960,
// host/src/chars.c:1477-1553).
//
// The arithmetic is a small natural-number type: the value of a decimal
// sequence is digits * 10^k, a rational; its binary window is one bounded
// division (p + 3 or p + 4 quotient bits and a remainder sticky), then one
// rounding - the construction chars.py's module docstring gives. Two
// bands are answered without materialising 10^k, as chars.py:234-268 does:
// a value whose leading bit is above emax + 1 overflows under every
// attribute, one whose leading bit is at or below emin - man_w - 2 is
// below half the smallest subnormal, and each band's answer depends only
// on the sign and the attribute, so one representative inside the band
// gives it.
#include "chars.h"

#include <cstring>

#include "api_core.h"

namespace cftg {
namespace chars {

// ---- natural numbers --------------------------------------------------

int64_t Nat::bits() const
{
    if (w.empty()) return 0;
    return 32 * (int64_t)(w.size() - 1) + (32 - __builtin_clz(w.back()));
}

bool Nat::bit(int64_t i) const
{
    if (i < 0 || i >= 32 * (int64_t)w.size()) return false;
    return (w[(size_t)(i >> 5)] >> (i & 31)) & 1u;
}

bool Nat::any_below(int64_t i) const
{
    if (i <= 0 || w.empty()) return false;
    const int64_t top = i >> 5;
    for (int64_t k = 0; k < top && k < (int64_t)w.size(); k++)
        if (w[(size_t)k]) return true;
    if (top < (int64_t)w.size() && (i & 31)) {
        const uint32_t mask = (1u << (i & 31)) - 1u;
        if (w[(size_t)top] & mask) return true;
    }
    return false;
}

void Nat::trim()
{
    while (!w.empty() && w.back() == 0u) w.pop_back();
}

Nat Nat::of(uint64_t v)
{
    Nat r;
    r.w.push_back((uint32_t)v);
    r.w.push_back((uint32_t)(v >> 32));
    r.trim();
    return r;
}

void mul_small(Nat &a, uint32_t m, uint32_t add)
{
    uint64_t carry = add;
    for (auto &x : a.w) {
        const uint64_t t = (uint64_t)x * m + carry;
        x = (uint32_t)t;
        carry = t >> 32;
    }
    if (carry) a.w.push_back((uint32_t)carry);
    a.trim();
}

void shl(Nat &a, int64_t s)
{
    if (a.zero() || s <= 0) return;
    const size_t words = (size_t)(s >> 5);
    const int b = (int)(s & 31);
    std::vector<uint32_t> r(a.w.size() + words + 1, 0u);
    for (size_t i = 0; i < a.w.size(); i++) {
        const uint64_t v = (uint64_t)a.w[i] << b;
        r[i + words] |= (uint32_t)v;
        r[i + words + 1] |= (uint32_t)(v >> 32);
    }
    a.w.swap(r);
    a.trim();
}

Nat shr(const Nat &a, int64_t s)
{
    if (s <= 0) return a;
    Nat r;
    const int64_t words = s >> 5;
    if (words >= (int64_t)a.w.size()) return r;
    const int b = (int)(s & 31);
    r.w.resize(a.w.size() - (size_t)words);
    for (size_t i = 0; i < r.w.size(); i++) {
        const uint64_t lo = a.w[i + (size_t)words];
        const uint64_t hi = (i + (size_t)words + 1 < a.w.size()) ? a.w[i + (size_t)words + 1] : 0u;
        r.w[i] = (uint32_t)(((hi << 32) | lo) >> b);
    }
    r.trim();
    return r;
}

Nat mul(const Nat &a, const Nat &b)
{
    Nat r;
    if (a.zero() || b.zero()) return r;
    r.w.assign(a.w.size() + b.w.size(), 0u);
    for (size_t i = 0; i < a.w.size(); i++) {
        uint64_t carry = 0;
        for (size_t j = 0; j < b.w.size(); j++) {
            const uint64_t t = (uint64_t)a.w[i] * b.w[j] + r.w[i + j] + carry;
            r.w[i + j] = (uint32_t)t;
            carry = t >> 32;
        }
        r.w[i + b.w.size()] = (uint32_t)carry;
    }
    r.trim();
    return r;
}

int cmp(const Nat &a, const Nat &b)
{
    if (a.w.size() != b.w.size()) return a.w.size() < b.w.size() ? -1 : 1;
    for (size_t i = a.w.size(); i-- > 0;)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    return 0;
}

void sub_in(Nat &a, const Nat &b)
{
    int64_t borrow = 0;
    for (size_t i = 0; i < a.w.size(); i++) {
        int64_t t = (int64_t)a.w[i] - (i < b.w.size() ? (int64_t)b.w[i] : 0) - borrow;
        borrow = t < 0;
        a.w[i] = (uint32_t)(t + (borrow ? ((int64_t)1 << 32) : 0));
    }
    a.trim();
}

Nat pow10(int64_t k)
{
    Nat r = Nat::of(1);
    for (; k >= 9; k -= 9) mul_small(r, 1000000000u, 0u);
    static const uint32_t small[9] = {1u, 10u, 100u, 1000u, 10000u, 100000u, 1000000u, 10000000u,
                                      100000000u};
    mul_small(r, small[k], 0u);
    return r;
}

Nat div_bounded(const Nat &n, const Nat &d, int qbits, bool *rem_nz)
{
    Nat rem = n, q;
    q.w.assign((size_t)(qbits + 31) / 32, 0u);
    for (int b = qbits - 1; b >= 0; b--) {
        Nat t = d;
        shl(t, b);
        if (cmp(rem, t) >= 0) {
            sub_in(rem, t);
            q.w[(size_t)(b >> 5)] |= 1u << (b & 31);
        }
    }
    q.trim();
    *rem_nz = !rem.zero();
    return q;
}

// ---- formats and encodings --------------------------------------------

const Geo &geo(int fmt)
{
    static const Geo g[4] = {
        {32, 23, 8, 24, 127, -126, 127},
        {64, 52, 11, 53, 1023, -1022, 1023},
        {128, 112, 15, 113, 16383, -16382, 16383},
        {256, 236, 19, 237, 262143, -262142, 262143},
    };
    return g[fmt];
}

static void or_nat(Enc &x, const Nat &v, int shift)
{
    for (size_t i = 0; i < v.w.size(); i++) {
        const int lo = shift + 32 * (int)i;
        const uint64_t t = (uint64_t)v.w[i] << (lo & 31);
        if (lo / 32 < 8) x.w[lo / 32] |= (uint32_t)t;
        if (lo / 32 + 1 < 8) x.w[lo / 32 + 1] |= (uint32_t)(t >> 32);
    }
}

static void set_sign(int fmt, Enc &x, int sign)
{
    if (sign) x.w[(geo(fmt).width - 1) / 32] |= 1u << ((geo(fmt).width - 1) & 31);
}

static Enc zero_enc(int fmt, int sign)
{
    Enc x;
    set_sign(fmt, x, sign);
    return x;
}

static Enc exp_all_ones(int fmt, int sign)
{
    const Geo &g = geo(fmt);
    Enc x;
    Nat ones;
    ones.w.push_back((1u << g.exp_w) - 1u);
    or_nat(x, ones, g.man_w);
    set_sign(fmt, x, sign);
    return x;
}

static Enc max_normal(int fmt, int sign)
{
    const Geo &g = geo(fmt);
    Enc x;
    Nat top;
    top.w.push_back((1u << g.exp_w) - 2u);
    or_nat(x, top, g.man_w);
    for (int i = 0; i < g.man_w; i++) x.w[i / 32] |= 1u << (i & 31);
    set_sign(fmt, x, sign);
    return x;
}

bool decode_finite(int fmt, const Enc &x, int *sign, Nat *m, int64_t *e)
{
    const Geo &g = geo(fmt);
    auto bit = [&](int i) { return (x.w[i / 32] >> (i & 31)) & 1u; };
    *sign = (int)bit(g.width - 1);
    uint32_t biased = 0;
    for (int i = 0; i < g.exp_w; i++) biased |= bit(g.man_w + i) << i;
    Nat frac;
    frac.w.assign((size_t)(g.man_w + 32) / 32, 0u);
    for (int i = 0; i < g.man_w; i++) frac.w[(size_t)(i / 32)] |= bit(i) << (i & 31);
    frac.trim();
    if (biased == (1u << g.exp_w) - 1u) return false;
    if (biased == 0) {
        if (frac.zero()) return false;
        *m = frac;
        *e = g.emin - g.man_w;
        return true;
    }
    Nat lead = Nat::of(1);
    shl(lead, g.man_w);
    frac.w.resize(std::max(frac.w.size(), lead.w.size()), 0u);
    for (size_t i = 0; i < lead.w.size(); i++) frac.w[i] |= lead.w[i];
    frac.trim();
    *m = frac;
    *e = (int64_t)biased - g.bias - g.man_w;
    return true;
}

// ---- rounding -----------------------------------------------------------

// m * 2^e to a multiple of 2^q under rnd: the count of 2^q kept, and
// whether anything was dropped (softfloat.py's _round_at).
static Nat round_at(const Nat &m, int64_t e, int64_t q, int sign, int rnd, bool *inexact)
{
    if (q <= e) {
        Nat k = m;
        shl(k, e - q);
        *inexact = false;
        return k;
    }
    const int64_t s = q - e;
    Nat kept = shr(m, s);
    const bool guard = m.bit(s - 1), sticky = m.any_below(s - 1);
    *inexact = guard || sticky;
    bool up = false;
    switch (rnd) {
    case 0: up = guard && (sticky || kept.bit(0)); break;          // ties to even
    case 1: up = false; break;                                       // toward zero
    case 2: up = sign && *inexact; break;                            // toward -inf
    case 3: up = !sign && *inexact; break;                           // toward +inf
    case 4: up = guard; break;                                       // ties away
    }
    if (up) mul_small(kept, 1u, 1u);
    return kept;
}

Enc round_pack(int fmt, int sign, const Nat &m, int64_t e, int rnd, uint32_t *flags)
{
    const Geo &g = geo(fmt);
    const int64_t p = g.prec;
    const int64_t e_norm = e + m.bits() - 1;
    bool ix;
    // tininess after rounding: the unbounded-exponent rounding's exponent
    const int64_t q_unb = e_norm - (p - 1);
    const Nat ku = round_at(m, e, q_unb, sign, rnd, &ix);
    const bool tiny = q_unb + ku.bits() - 1 < g.emin;
    const int64_t q = std::max(e_norm, g.emin) - (p - 1);
    bool inexact;
    Nat kept = round_at(m, e, q, sign, rnd, &inexact);
    uint32_t fl = inexact ? (uint32_t)CFT_FLAG_INEXACT : 0u;
    if (kept.zero()) {
        *flags = fl | CFT_FLAG_UNDERFLOW;
        return zero_enc(fmt, sign);
    }
    const int64_t e_res = q + kept.bits() - 1;
    if (e_res > g.emax) {
        *flags = fl | CFT_FLAG_OVERFLOW | CFT_FLAG_INEXACT;
        const bool to_inf = rnd == 0 || rnd == 4 || (rnd == 3 && !sign) || (rnd == 2 && sign);
        return to_inf ? exp_all_ones(fmt, sign) : max_normal(fmt, sign);
    }
    if (tiny && inexact) fl |= CFT_FLAG_UNDERFLOW;
    *flags = fl;
    Enc x = zero_enc(fmt, sign);
    if (e_res < g.emin) {                       // subnormal: kept is the fraction
        or_nat(x, kept, 0);
        return x;
    }
    if (kept.bits() == p + 1) kept = shr(kept, 1);
    kept.w.resize((size_t)(g.man_w + 32) / 32, 0u);
    kept.w[(size_t)(g.man_w / 32)] &= ~(1u << (g.man_w & 31));   // drop the hidden bit
    kept.trim();
    or_nat(x, kept, 0);
    or_nat(x, Nat::of((uint64_t)(e_res + g.bias)), g.man_w);
    return x;
}

// p + 3 bits of quotient plus a sticky (chars.py's _WINDOW).
static constexpr int WINDOW = 3;

Enc round_rational(int fmt, int sign, const Nat &num, const Nat &den, int rnd, uint32_t *flags)
{
    const int64_t w = geo(fmt).prec + WINDOW;
    const int64_t q = (num.bits() - den.bits()) - w;
    bool rem;
    Nat m;
    if (q >= 0) {
        Nat d = den;
        shl(d, q);
        m = div_bounded(num, d, (int)w + 2, &rem);
    } else {
        Nat n = num;
        shl(n, -q);
        m = div_bounded(n, den, (int)w + 2, &rem);
    }
    if (rem) {
        shl(m, 1);
        mul_small(m, 1u, 1u);
        return round_pack(fmt, sign, m, q - 1, rnd, flags);
    }
    return round_pack(fmt, sign, m, q, rnd, flags);
}

// ---- the bands ------------------------------------------------------------

static __int128 floor_div(__int128 a, __int128 b)      // b > 0
{
    __int128 q = a / b;
    if ((a % b) != 0 && a < 0) q -= 1;
    return q;
}

// lo <= t log2(10) <= hi, from 3.321928 < log2(10) < 3.321929.
static void log2_10_bounds(int64_t t, __int128 *lo, __int128 *hi)
{
    const __int128 L = 3321928, H = 3321929, D = 1000000;
    if (t >= 0) {
        *lo = floor_div((__int128)t * L, D);
        *hi = -floor_div(-(__int128)t * H, D);
    } else {
        *lo = floor_div((__int128)t * H, D);
        *hi = -floor_div(-(__int128)t * L, D);
    }
}

static bool clamped(int fmt, int sign, __int128 e_lo, __int128 e_hi, int rnd, Enc *out,
                    uint32_t *flags)
{
    const Geo &g = geo(fmt);
    const int64_t w = g.prec + WINDOW;
    Nat rep = Nat::of(1);
    shl(rep, w);
    mul_small(rep, 1u, 1u);                      // 2^w + 1
    if (e_lo > g.emax + 1) {
        *out = round_pack(fmt, sign, rep, g.emax + 1 - w, rnd, flags);
        return true;
    }
    if (e_hi <= g.emin - g.man_w - 2) {
        *out = round_pack(fmt, sign, rep, g.emin - g.man_w - 2 - w, rnd, flags);
        return true;
    }
    return false;
}

// ---- the lexer --------------------------------------------------------------

static bool is_dec(char c) { return c >= '0' && c <= '9'; }
static bool is_hex(char c)
{
    return is_dec(c) || (c >= 'a' && c <= 'f') || (c >= 'A' && c <= 'F');
}
static int hex_val(char c)
{
    return is_dec(c) ? c - '0' : (c >= 'a' && c <= 'f') ? c - 'a' + 10 : c - 'A' + 10;
}

static std::string lower(const std::string &s)
{
    std::string r = s;
    for (auto &c : r)
        if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
    return r;
}

static Nat nat_dec(const std::string &d)
{
    Nat r;
    size_t i = 0;
    const size_t head = d.size() % 9;
    auto chunk = [&](size_t from, size_t len) {
        uint32_t v = 0, scale = 1;
        for (size_t k = 0; k < len; k++) {
            v = v * 10u + (uint32_t)(d[from + k] - '0');
            scale *= 10u;
        }
        mul_small(r, scale, v);
    };
    if (head) {
        chunk(0, head);
        i = head;
    }
    for (; i < d.size(); i += 9) chunk(i, 9);
    return r;
}

static Nat nat_hex(const std::string &h)
{
    Nat r;
    r.w.assign(h.size() / 8 + 1, 0u);
    for (size_t k = 0; k < h.size(); k++) {
        const size_t pos = h.size() - 1 - k;              // nibble index from the bottom
        r.w[pos / 8] |= (uint32_t)hex_val(h[k]) << (4 * (pos % 8));
    }
    r.trim();
    return r;
}

// A decimal exponent's digits, saturated at 10^15: every exponent that far
// out lies in a band for any significand a source can hold.
static int64_t dec_sat(const std::string &d)
{
    int64_t v = 0;
    for (char c : d) {
        v = v * 10 + (c - '0');
        if (v > 1000000000000000LL) return 1000000000000000LL;
    }
    return v;
}

static void split_sign(const std::string &s, int *sign, std::string *body)
{
    if (!s.empty() && (s[0] == '-' || s[0] == '+')) {
        *sign = s[0] == '-';
        *body = s.substr(1);
    } else {
        *sign = 0;
        *body = s;
    }
}

// 5.12.1's words: 1 with *out set, 0 when body is not one, -1 for a
// payload the format cannot hold (a refusal; chars.py:297-340).
static int lex_special(int fmt, const std::string &body, int sign, Enc *out, std::string *why)
{
    const Geo &g = geo(fmt);
    const std::string low = lower(body);
    if (low == "inf" || low == "infinity") {
        *out = exp_all_ones(fmt, sign);
        return 1;
    }
    std::string head = low;
    bool have_payload = false;
    Nat payload;
    if (!low.empty() && low.back() == ')') {
        const size_t open = low.find('(');
        if (open == std::string::npos) return 0;
        head = low.substr(0, open);
        const std::string inner = body.substr(open + 1, body.size() - open - 2);
        if (inner.size() >= 2 && inner[0] == '0' && (inner[1] == 'x' || inner[1] == 'X')) {
            const std::string t = inner.substr(2);
            if (t.empty()) return 0;
            for (char c : t)
                if (!is_hex(c)) return 0;
            payload = nat_hex(t);
        } else {
            if (inner.empty()) return 0;
            for (char c : inner)
                if (!is_dec(c)) return 0;
            payload = nat_dec(inner);
        }
        have_payload = true;
    }
    if (head != "nan" && head != "snan") return 0;
    const bool sig = head == "snan";
    if (!have_payload) payload = Nat::of(sig ? 1 : 0);
    if (payload.bits() > g.man_w - 1 || (sig && payload.zero())) {
        *why = std::string("the payload is not admissible in ") + cft_format_name((cft_format)fmt) +
               (sig ? " (a signalling NaN needs a non-zero payload below 2^(man_w-1))"
                    : " (a payload is below 2^(man_w-1))");
        return -1;
    }
    Enc x = exp_all_ones(fmt, sign);
    or_nat(x, payload, 0);
    if (!sig) x.w[(g.man_w - 1) / 32] |= 1u << ((g.man_w - 1) & 31);
    *out = x;
    return 1;
}

// The exponent part: "" or mark sign? digit+ (chars.py:343-353).
static bool lex_exponent(const std::string &rest, const char *marks, int64_t *exp)
{
    *exp = 0;
    if (rest.empty()) return true;
    if (rest[0] != marks[0] && rest[0] != marks[1]) return false;
    int es;
    std::string body;
    split_sign(rest.substr(1), &es, &body);
    if (body.empty()) return false;
    for (char c : body)
        if (!is_dec(c)) return false;
    const int64_t v = dec_sat(body);
    *exp = es ? -v : v;
    return true;
}

bool from_decimal(int fmt, const std::string &s, int rnd, Enc *out, uint32_t *flags,
                  std::string *why)
{
    *flags = 0;
    int sign;
    std::string body;
    split_sign(s, &sign, &body);
    if (body.empty()) {
        *why = "an empty sequence";
        return false;
    }
    const int sp = lex_special(fmt, body, sign, out, why);
    if (sp < 0) return false;
    if (sp > 0) return true;
    size_t i = 0;
    std::string digits;
    while (i < body.size() && is_dec(body[i])) digits += body[i++];
    size_t nfrac = 0;
    if (i < body.size() && body[i] == '.') {
        i++;
        while (i < body.size() && is_dec(body[i])) {
            digits += body[i++];
            nfrac++;
        }
    }
    int64_t exp;
    if (digits.empty() || !lex_exponent(body.substr(i), "eE", &exp)) {
        *why = "not a decimal sequence";
        return false;
    }
    size_t lead = 0;
    while (lead < digits.size() && digits[lead] == '0') lead++;
    if (lead == digits.size()) {                   // a zero keeps its sign
        *out = zero_enc(fmt, sign);
        return true;
    }
    const Nat d = nat_dec(digits.substr(lead));
    const int64_t k = exp - (int64_t)nfrac;
    __int128 lo, hi;
    log2_10_bounds(k, &lo, &hi);
    const int64_t b = d.bits();
    if (clamped(fmt, sign, (__int128)b - 2 + lo, (__int128)b + hi, rnd, out, flags)) return true;
    if (k >= 0) *out = round_rational(fmt, sign, mul(d, pow10(k)), Nat::of(1), rnd, flags);
    else *out = round_rational(fmt, sign, d, pow10(-k), rnd, flags);
    return true;
}

bool from_hex(int fmt, const std::string &s, int rnd, Enc *out, uint32_t *flags, std::string *why)
{
    *flags = 0;
    int sign;
    std::string body;
    split_sign(s, &sign, &body);
    if (body.empty()) {
        *why = "an empty sequence";
        return false;
    }
    const int sp = lex_special(fmt, body, sign, out, why);
    if (sp < 0) return false;
    if (sp > 0) return true;
    if (body.size() < 2 || body[0] != '0' || (body[1] != 'x' && body[1] != 'X')) {
        *why = "not a hexadecimal sequence";
        return false;
    }
    size_t i = 2;
    std::string digits;
    while (i < body.size() && is_hex(body[i])) digits += body[i++];
    size_t nfrac = 0;
    if (i < body.size() && body[i] == '.') {
        i++;
        while (i < body.size() && is_hex(body[i])) {
            digits += body[i++];
            nfrac++;
        }
    }
    if (digits.empty()) {
        *why = "not a hexadecimal sequence";
        return false;
    }
    if (i == body.size()) {
        *why = "no binary exponent: 5.12.3's grammar requires one (p+0 for a value that needs no scaling)";
        return false;
    }
    int64_t exp;
    if (!lex_exponent(body.substr(i), "pP", &exp)) {
        *why = "not a hexadecimal sequence";
        return false;
    }
    const Nat m = nat_hex(digits);
    if (m.zero()) {
        *out = zero_enc(fmt, sign);
        return true;
    }
    const int64_t e = exp - 4 * (int64_t)nfrac;
    const __int128 lead = (__int128)e + m.bits() - 1;
    if (clamped(fmt, sign, lead, lead, rnd, out, flags)) return true;
    *out = round_pack(fmt, sign, m, e, rnd, flags);
    return true;
}

}  // namespace chars
}  // namespace cftg

// ---- the C ABI ------------------------------------------------------------

using namespace cftg;

static cft_status from_char_batch(cft_device *dev, cft_format fmt, cft_round rnd,
                                  const char *const *in, void *d, size_t n, size_t *bad_index,
                                  uint32_t *flags_out, bool hex, const char *who)
{
    if (bad_index) *bad_index = 0;
    if (!check_dev(dev, who)) return CFT_ERR_INVALID_ARGUMENT;
    if ((int)fmt < 0 || (int)fmt > 3 || (int)rnd < 0 || (int)rnd > 4) {
        set_error("%s: format %d or rounding attribute %d is outside the ABI's range", who, (int)fmt,
                  (int)rnd);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) {
        flags_emit(dev, 0u, flags_out);
        return CFT_OK;
    }
    if (!in || !d) {
        set_error("%s: the sequence array and the destination must not be NULL", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const size_t esz = esz_of((int)fmt);
    if (n > SIZE_MAX / esz) {
        set_error("%s: %lu elements overflow the destination's size", who, (unsigned long)n);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    // d is written on the host: a resident buffer's device bytes come home
    // first and the buffer is uploaded at its next use.
    size_t off = 0;
    cft_buffer *ob = find_buffer(dev, d, n * esz, &off);
    if (ob && ob->state == B_DIRTY) {
        const cft_status st = cft_buffer_from_device(ob);
        if (st != CFT_OK) return st;
    }
    uint32_t acc = 0u;
    for (size_t i = 0; i < n; i++) {
        chars::Enc v;
        uint32_t fl = 0u;
        std::string why;
        if (!in[i]) {
            if (bad_index) *bad_index = i;
            set_error("%s: sequence %lu is NULL", who, (unsigned long)i);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        const std::string s(in[i]);
        const bool ok = hex ? chars::from_hex((int)fmt, s, (int)rnd, &v, &fl, &why)
                            : chars::from_decimal((int)fmt, s, (int)rnd, &v, &fl, &why);
        if (!ok) {
            if (bad_index) *bad_index = i;
            set_error("%s: sequence %lu is refused: %s", who, (unsigned long)i, why.c_str());
            return CFT_ERR_INVALID_ARGUMENT;
        }
        acc |= fl;
        memcpy(static_cast<uint8_t *>(d) + i * esz, v.w, esz);
    }
    if (ob && ob->state != B_LOST) ob->state = B_STALE;
    flags_emit(dev, acc, flags_out);
    return CFT_OK;
}

// 5.12.2's Pmin = 1 + ceil(p log10 2): the smallest k with 10^k >= 2^p, plus one.
extern "C" CFT_API size_t cft_format_decimal_digits(cft_format fmt)
{
    if ((int)fmt < 0 || (int)fmt > 3) return 0;
    chars::Nat ten = chars::Nat::of(1), two = chars::Nat::of(1);
    chars::shl(two, chars::geo((int)fmt).prec);
    size_t k = 0;
    while (chars::cmp(ten, two) < 0) {
        chars::mul_small(ten, 10u, 0u);
        k++;
    }
    return 1 + k;
}

extern "C" CFT_API cft_status cft_from_decimal_char(cft_device *dev, cft_format fmt, cft_round rnd,
                                                    const char *const *in, void *d, size_t n,
                                                    size_t *bad_index, uint32_t *flags_out)
{
    clear_error();
    return from_char_batch(dev, fmt, rnd, in, d, n, bad_index, flags_out, false,
                           "cft_from_decimal_char");
}

extern "C" CFT_API cft_status cft_from_hex_char(cft_device *dev, cft_format fmt, cft_round rnd,
                                                const char *const *in, void *d, size_t n,
                                                size_t *bad_index, uint32_t *flags_out)
{
    clear_error();
    return from_char_batch(dev, fmt, rnd, in, d, n, bad_index, flags_out, true,
                           "cft_from_hex_char");
}

// One sequence, no device: for tools that run where no GPU is open (the
// assembler's literals go through the same routine).
extern "C" CFT_API cft_status cftg_from_char(int hex, cft_format fmt, cft_round rnd, const char *in,
                                             void *d, uint32_t *flags_out)
{
    clear_error();
    if (flags_out) *flags_out = 0u;
    if ((int)fmt < 0 || (int)fmt > 3 || (int)rnd < 0 || (int)rnd > 4 || !in || !d) {
        set_error("cftg_from_char: fmt 0..3, rnd 0..4, and in and d not NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    chars::Enc v;
    uint32_t fl = 0u;
    std::string why;
    const bool ok = hex ? chars::from_hex((int)fmt, in, (int)rnd, &v, &fl, &why)
                        : chars::from_decimal((int)fmt, in, (int)rnd, &v, &fl, &why);
    if (!ok) {
        set_error("cftg_from_char: the sequence is refused: %s", why.c_str());
        return CFT_ERR_INVALID_ARGUMENT;
    }
    memcpy(d, v.w, esz_of((int)fmt));
    if (flags_out) *flags_out = fl;
    return CFT_OK;
}
