// stubs.cpp - the reference entry points outside this backend's scope
// (include/cft_unsupported.h). Each refuses by name so that a binding
// written for the reference loads and a call outside the hot path says why
// it cannot run here, instead of computing on the CPU.
#include "../../include/cft_unsupported.h"
#include "api_core.h"

using cftg::clear_error;
using cftg::set_error;

static cft_status refuse(const char *who)
{
    set_error("%s: this GB300 backend carries the elementwise arithmetic path (cft_run, cft_run_ex, "
              "cft_div, cft_sqrt) and the sequencer; %s is outside it",
              who, who);
    return CFT_ERR_UNSUPPORTED;
}

extern "C" cft_status cft_exp(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_exp"); }
extern "C" cft_status cft_expm1(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_expm1"); }
extern "C" cft_status cft_exp2(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_exp2"); }
extern "C" cft_status cft_log(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_log"); }
extern "C" cft_status cft_log1p(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_log1p"); }
extern "C" cft_status cft_log2(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_log2"); }
extern "C" cft_status cft_log10(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_log10"); }
extern "C" cft_status cft_sinpi(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_sinpi"); }
extern "C" cft_status cft_cospi(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_cospi"); }
extern "C" cft_status cft_tanpi(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_tanpi"); }
extern "C" cft_status cft_asin(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_asin"); }
extern "C" cft_status cft_acos(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_acos"); }
extern "C" cft_status cft_atan(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_atan"); }
extern "C" cft_status cft_asinpi(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_asinpi"); }
extern "C" cft_status cft_acospi(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_acospi"); }
extern "C" cft_status cft_atanpi(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_atanpi"); }
extern "C" cft_status cft_sin(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_sin"); }
extern "C" cft_status cft_cos(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_cos"); }
extern "C" cft_status cft_tan(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_tan"); }
extern "C" cft_status cft_sinh(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_sinh"); }
extern "C" cft_status cft_cosh(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_cosh"); }
extern "C" cft_status cft_tanh(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_tanh"); }
extern "C" cft_status cft_asinh(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_asinh"); }
extern "C" cft_status cft_acosh(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_acosh"); }
extern "C" cft_status cft_atanh(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_atanh"); }
extern "C" cft_status cft_exp2m1(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_exp2m1"); }
extern "C" cft_status cft_exp10(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_exp10"); }
extern "C" cft_status cft_exp10m1(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_exp10m1"); }
extern "C" cft_status cft_log2p1(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_log2p1"); }
extern "C" cft_status cft_log10p1(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_log10p1"); }
extern "C" cft_status cft_rsqrt(cft_device *, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_rsqrt"); }
extern "C" cft_status cft_pow(cft_device *, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_pow"); }
extern "C" cft_status cft_hypot(cft_device *, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_hypot"); }
extern "C" cft_status cft_atan2(cft_device *, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_atan2"); }
extern "C" cft_status cft_atan2pi(cft_device *, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_atan2pi"); }
extern "C" cft_status cft_powr(cft_device *, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_powr"); }
extern "C" cft_status cft_pown(cft_device *, cft_format, cft_round, const void *, const int64_t *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_pown"); }
extern "C" cft_status cft_compound(cft_device *, cft_format, cft_round, const void *, const int64_t *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_compound"); }
extern "C" cft_status cft_rootn(cft_device *, cft_format, cft_round, const void *, const int64_t *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_rootn"); }
extern "C" cft_status cft_scaled_prod(cft_device *, cft_format, cft_round, const void *, void *, int64_t *, size_t, uint32_t *) { clear_error(); return refuse("cft_scaled_prod"); }
extern "C" cft_status cft_scaled_prod_sum(cft_device *, cft_format, cft_round, const void *, const void *, void *, int64_t *, size_t, uint32_t *) { clear_error(); return refuse("cft_scaled_prod_sum"); }
extern "C" cft_status cft_scaled_prod_diff(cft_device *, cft_format, cft_round, const void *, const void *, void *, int64_t *, size_t, uint32_t *) { clear_error(); return refuse("cft_scaled_prod_diff"); }
extern "C" cft_status cft_formatof_add(cft_device *, cft_format, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_formatof_add"); }
extern "C" cft_status cft_formatof_sub(cft_device *, cft_format, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_formatof_sub"); }
extern "C" cft_status cft_formatof_mul(cft_device *, cft_format, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_formatof_mul"); }
extern "C" cft_status cft_formatof_div(cft_device *, cft_format, cft_format, cft_round, const void *, const void *, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_formatof_div"); }
extern "C" cft_status cft_formatof_sqrt(cft_device *, cft_format, cft_format, cft_round, const void *, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_formatof_sqrt"); }
extern "C" cft_status cft_formatof_fma(cft_device *, cft_format, cft_format, cft_round, const void *, const void *, const void *, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_formatof_fma"); }
extern "C" cft_status cft_to_decimal_char(cft_device *, cft_format, cft_round, const void *, size_t, char *, size_t, size_t *, uint32_t *) { clear_error(); return refuse("cft_to_decimal_char"); }
extern "C" cft_status cft_to_hex_char(cft_device *, cft_format, const void *, char *, size_t, size_t *) { clear_error(); return refuse("cft_to_hex_char"); }
extern "C" cft_status cft_get_payload(cft_device *, cft_format, const void *, void *, size_t) { clear_error(); return refuse("cft_get_payload"); }
extern "C" cft_status cft_set_payload(cft_device *, cft_format, const void *, void *, size_t) { clear_error(); return refuse("cft_set_payload"); }
extern "C" cft_status cft_set_payload_signaling(cft_device *, cft_format, const void *, void *, size_t) { clear_error(); return refuse("cft_set_payload_signaling"); }
extern "C" cft_status cft_min_mag(cft_device *, cft_format, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_min_mag"); }
extern "C" cft_status cft_max_mag(cft_device *, cft_format, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_max_mag"); }
extern "C" cft_status cft_minnum_mag(cft_device *, cft_format, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_minnum_mag"); }
extern "C" cft_status cft_maxnum_mag(cft_device *, cft_format, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_maxnum_mag"); }

extern "C" cft_status cft_rint(cft_device *, cft_format, cft_round, int, const void *, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_rint"); }
extern "C" cft_status cft_scaleb(cft_device *, cft_format, cft_round, const void *, int64_t, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_scaleb"); }
extern "C" cft_status cft_cmp_sig(cft_device *, cft_op, cft_format, const void *, const void *, void *, size_t, uint32_t *, uint32_t *) { clear_error(); return refuse("cft_cmp_sig"); }
extern "C" cft_status cft_convert(cft_device *, cft_format, cft_format, cft_round, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_convert"); }
extern "C" cft_status cft_cvt_from_i32(cft_device *, cft_format, cft_round, const int32_t *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_cvt_from_i32"); }
extern "C" cft_status cft_cvt_from_u32(cft_device *, cft_format, cft_round, const uint32_t *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_cvt_from_u32"); }
extern "C" cft_status cft_cvt_from_i64(cft_device *, cft_format, cft_round, const int64_t *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_cvt_from_i64"); }
extern "C" cft_status cft_cvt_from_u64(cft_device *, cft_format, cft_round, const uint64_t *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_cvt_from_u64"); }
extern "C" cft_status cft_cvt_to_i32(cft_device *, cft_format, cft_round, int, const void *, int32_t *, size_t, uint32_t *) { clear_error(); return refuse("cft_cvt_to_i32"); }
extern "C" cft_status cft_cvt_to_u32(cft_device *, cft_format, cft_round, int, const void *, uint32_t *, size_t, uint32_t *) { clear_error(); return refuse("cft_cvt_to_u32"); }
extern "C" cft_status cft_cvt_to_i64(cft_device *, cft_format, cft_round, int, const void *, int64_t *, size_t, uint32_t *) { clear_error(); return refuse("cft_cvt_to_i64"); }
extern "C" cft_status cft_cvt_to_u64(cft_device *, cft_format, cft_round, int, const void *, uint64_t *, size_t, uint32_t *) { clear_error(); return refuse("cft_cvt_to_u64"); }
extern "C" cft_status cft_logb(cft_device *, cft_format, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_logb"); }
extern "C" cft_status cft_next_up(cft_device *, cft_format, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_next_up"); }
extern "C" cft_status cft_next_down(cft_device *, cft_format, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_next_down"); }
extern "C" cft_status cft_class(cft_device *, cft_format, const void *, uint8_t *, size_t) { clear_error(); return refuse("cft_class"); }
extern "C" cft_status cft_total_order(cft_device *, cft_format, const void *, const void *, void *, size_t) { clear_error(); return refuse("cft_total_order"); }
extern "C" cft_status cft_total_order_mag(cft_device *, cft_format, const void *, const void *, void *, size_t) { clear_error(); return refuse("cft_total_order_mag"); }
extern "C" cft_status cft_rem(cft_device *, cft_format, const void *, const void *, void *, size_t, uint32_t *) { clear_error(); return refuse("cft_rem"); }
extern "C" cft_status cft_conformance(cft_device *, const char *, char *report, size_t report_size, uint64_t *cases_checked)
{
    clear_error();
    if (cases_checked)
        *cases_checked = 0;
    if (report && report_size)
        report[0] = 0;
    return refuse("cft_conformance");
}
