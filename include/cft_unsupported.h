/* cft_unsupported.h - reference entry points outside this backend's scope.
 *
 * The reference's Python binding declares every one of these at import
 * (bindings/python/cftmpfr/_lib.py:181-372), so a library that omits one
 * cannot be loaded in the reference's place. This backend carries the
 * batched elementwise path and the sequencer only; each function below
 * returns CFT_ERR_UNSUPPORTED and leaves a sentence in cft_last_error()
 * naming itself. Prototypes are the reference's (host/include/cft.h, the
 * line cited beside each group).
 */
#ifndef CFT_UNSUPPORTED_H
#define CFT_UNSUPPORTED_H

#include "cft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* transcendentals, unary (cft.h:1648-1666, 1759-1786, 2092-2109, 2201-2227) */
CFT_API cft_status cft_exp(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_expm1(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_exp2(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_log(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_log1p(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_log2(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_log10(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_sinpi(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cospi(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_tanpi(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_asin(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_acos(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_atan(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_asinpi(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_acospi(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_atanpi(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_sin(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cos(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_tan(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_sinh(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cosh(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_tanh(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_asinh(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_acosh(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_atanh(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_exp2m1(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_exp10(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_exp10m1(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_log2p1(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_log10p1(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_rsqrt(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
/* transcendentals, binary (cft.h:1672-1676, 1789-1794, 2112) */
CFT_API cft_status cft_pow(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_hypot(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_atan2(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_atan2pi(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_powr(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
/* integer-exponent functions (cft.h:2119-2128) */
CFT_API cft_status cft_pown(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const int64_t *nexp, void *d, size_t count, uint32_t *flags_out);
CFT_API cft_status cft_compound(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const int64_t *nexp, void *d, size_t count, uint32_t *flags_out);
CFT_API cft_status cft_rootn(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const int64_t *nexp, void *d, size_t count, uint32_t *flags_out);
/* scaled products, 754-2019 9.4 (cft.h:2335-2347) */
CFT_API cft_status cft_scaled_prod(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, void *pr, int64_t *scale_out, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_scaled_prod_sum(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const void *b, void *pr, int64_t *scale_out, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_scaled_prod_diff(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, const void *b, void *pr, int64_t *scale_out, size_t n, uint32_t *flags_out);
/* formatOf arithmetic, 754-2019 5.4.1 (cft.h:3511-3542) */
CFT_API cft_status cft_formatof_add(cft_device *dev, cft_format sfmt, cft_format dfmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_formatof_sub(cft_device *dev, cft_format sfmt, cft_format dfmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_formatof_mul(cft_device *dev, cft_format sfmt, cft_format dfmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_formatof_div(cft_device *dev, cft_format sfmt, cft_format dfmt, cft_round rnd, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_formatof_sqrt(cft_device *dev, cft_format sfmt, cft_format dfmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_formatof_fma(cft_device *dev, cft_format sfmt, cft_format dfmt, cft_round rnd, const void *a, const void *b, const void *c, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
/* conversions to character sequences and payloads, 754-2019 5.12 and 9.7 (cft.h:1936-2002) */
CFT_API cft_status cft_to_decimal_char(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, size_t digits, char *out, size_t cap, size_t *len, uint32_t *flags_out);
CFT_API cft_status cft_to_hex_char(cft_device *dev, cft_format fmt, const void *a, char *out, size_t cap, size_t *len);
CFT_API cft_status cft_get_payload(cft_device *dev, cft_format fmt, const void *a, void *d, size_t n);
CFT_API cft_status cft_set_payload(cft_device *dev, cft_format fmt, const void *a, void *d, size_t n);
CFT_API cft_status cft_set_payload_signaling(cft_device *dev, cft_format fmt, const void *a, void *d, size_t n);
/* the magnitude forms of 754-2019 9.6 (cft.h:3360-3371) */
CFT_API cft_status cft_min_mag(cft_device *dev, cft_format fmt, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_max_mag(cft_device *dev, cft_format fmt, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_minnum_mag(cft_device *dev, cft_format fmt, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_maxnum_mag(cft_device *dev, cft_format fmt, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);

/* clause-5 operations off the hot path: roundToIntegral, scaleB, signaling
 * comparisons, conversions between formats and to and from integers, logB,
 * nextUp/nextDown, class, totalOrder, remainder (cft.h:1438-1569) */
typedef enum cft_class_value {
    CFT_CLASS_NEG_INF = 0, CFT_CLASS_NEG_NORM = 1, CFT_CLASS_NEG_SUB = 2, CFT_CLASS_NEG_ZERO = 3,
    CFT_CLASS_POS_ZERO = 4, CFT_CLASS_POS_SUB = 5, CFT_CLASS_POS_NORM = 6, CFT_CLASS_POS_INF = 7,
    CFT_CLASS_SNAN = 8, CFT_CLASS_QNAN = 9
} cft_class_value;
CFT_API cft_status cft_rint(cft_device *dev, cft_format fmt, cft_round rnd, int exact, const void *a, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_scaleb(cft_device *dev, cft_format fmt, cft_round rnd, const void *a, int64_t nexp, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_cmp_sig(cft_device *dev, cft_op cmp, cft_format fmt, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out, uint32_t *bus_out);
CFT_API cft_status cft_convert(cft_device *dev, cft_format sfmt, cft_format dfmt, cft_round rnd, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cvt_from_i32(cft_device *dev, cft_format fmt, cft_round rnd, const int32_t *src, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cvt_from_u32(cft_device *dev, cft_format fmt, cft_round rnd, const uint32_t *src, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cvt_from_i64(cft_device *dev, cft_format fmt, cft_round rnd, const int64_t *src, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cvt_from_u64(cft_device *dev, cft_format fmt, cft_round rnd, const uint64_t *src, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cvt_to_i32(cft_device *dev, cft_format fmt, cft_round rnd, int exact, const void *a, int32_t *dst, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cvt_to_u32(cft_device *dev, cft_format fmt, cft_round rnd, int exact, const void *a, uint32_t *dst, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cvt_to_i64(cft_device *dev, cft_format fmt, cft_round rnd, int exact, const void *a, int64_t *dst, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_cvt_to_u64(cft_device *dev, cft_format fmt, cft_round rnd, int exact, const void *a, uint64_t *dst, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_logb(cft_device *dev, cft_format fmt, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_next_up(cft_device *dev, cft_format fmt, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_next_down(cft_device *dev, cft_format fmt, const void *a, void *d, size_t n, uint32_t *flags_out);
CFT_API cft_status cft_class(cft_device *dev, cft_format fmt, const void *a, uint8_t *cls, size_t n);
CFT_API cft_status cft_total_order(cft_device *dev, cft_format fmt, const void *a, const void *b, void *d, size_t n);
CFT_API cft_status cft_total_order_mag(cft_device *dev, cft_format fmt, const void *a, const void *b, void *d, size_t n);
CFT_API cft_status cft_rem(cft_device *dev, cft_format fmt, const void *a, const void *b, void *d, size_t n, uint32_t *flags_out);
/* the replay of the reference's published vector sets (cft.h:3397): the
 * sets are the reference's, replayed by its own tests against this library */
CFT_API cft_status cft_conformance(cft_device *dev, const char *dir, char *report, size_t report_size, uint64_t *cases_checked);

#ifdef __cplusplus
}
#endif

#endif /* CFT_UNSUPPORTED_H */
