/* sfport.c - the oracle's element arithmetic (test infrastructure only).
 *
 * A plain-C restatement of the reference's software backend, function by
 * function, each citing the reference lines it follows. It is written to be
 * read beside them, not to be fast: the GPU kernels in the shipped library
 * use a different (fixed-window) FMA algorithm, so agreement between the
 * two is a real check rather than one implementation compared to itself.
 *
 * Division and square root follow the golden model's definition
 * (python/cft_golden/softfloat.py:424-505): an exact quotient or integer
 * root carried to at least p+3 bits, the remainder folded into one sticky
 * bit, then round_pack. The reference C library reaches the same bits by
 * a Newton composition (host/src/divsqrt.c); only the bits are contract.
 */
#include "sfport.h"

#include <stdlib.h>
#include <string.h>

/* ---- format geometry (host/src/softfloat.c:10-16) ------------------- */

typedef struct {
    int exp_w, man_w, width, prec;
    int32_t bias, emax, emin;
    uint32_t exp_mask;
} fmt_t;

static const fmt_t FMTS[4] = {
    {  8,  23,  32,  24,    127,    127,    -126,    255u },
    { 11,  52,  64,  53,   1023,   1023,   -1022,   2047u },
    { 15, 112, 128, 113,  16383,  16383,  -16382,  32767u },
    { 19, 236, 256, 237, 262143, 262143, -262142, 524287u },
};

/* ---- a small unsigned bignum (the role of host/src/bigint.c) -------- *
 * 32-bit limbs, little-endian, `n` significant limbs, every limb at or
 * above n kept zero. 1,536 bits: the widest intermediate below is the
 * FMA near case at about 5p+3 = 1,188 bits (softfloat.c:287-292). */

#define OBL 48
typedef struct { int n; uint32_t v[OBL]; } ob;

static void ob_fix(ob *r)
{
    while (r->n > 0 && r->v[r->n - 1] == 0)
        r->n--;
}

static void ob_zero(ob *r) { memset(r, 0, sizeof *r); }

static void ob_u32(ob *r, uint32_t x)
{
    ob_zero(r);
    r->v[0] = x;
    r->n = x ? 1 : 0;
}

static int ob_is_zero(const ob *a) { return a->n == 0; }

static int ob_bitlen(const ob *a)
{
    uint32_t t;
    int b = 0;
    if (a->n == 0)
        return 0;
    t = a->v[a->n - 1];
    while (t) { b++; t >>= 1; }
    return (a->n - 1) * 32 + b;
}

static int ob_bit(const ob *a, int i)
{
    if (i < 0 || i >= OBL * 32)
        return 0;
    return (int)((a->v[i >> 5] >> (i & 31)) & 1u);
}

static void ob_setbit(ob *r, int i)
{
    r->v[i >> 5] |= 1u << (i & 31);
    if (r->n < (i >> 5) + 1)
        r->n = (i >> 5) + 1;
}

static void ob_clearbit(ob *r, int i)
{
    r->v[i >> 5] &= ~(1u << (i & 31));
    ob_fix(r);
}

/* bits [lo, lo+nb) as an integer, nb <= 32 */
static uint32_t ob_extract(const ob *a, int lo, int nb)
{
    uint32_t r = 0;
    int i;
    for (i = 0; i < nb; i++)
        r |= (uint32_t)ob_bit(a, lo + i) << i;
    return r;
}

/* keep the low nb bits */
static void ob_mask(ob *r, int nb)
{
    int w = nb >> 5, i;
    if (w >= OBL)
        return;
    if (nb & 31) {
        r->v[w] &= (1u << (nb & 31)) - 1u;
        w++;
    }
    for (i = w; i < OBL; i++)
        r->v[i] = 0;
    if (r->n > w)
        r->n = w;
    ob_fix(r);
}

static int ob_cmp(const ob *a, const ob *b)
{
    int i;
    if (a->n != b->n)
        return a->n < b->n ? -1 : 1;
    for (i = a->n - 1; i >= 0; i--)
        if (a->v[i] != b->v[i])
            return a->v[i] < b->v[i] ? -1 : 1;
    return 0;
}

/* any of bits [0, k) set */
static int ob_low_nonzero(const ob *a, int k)
{
    int w, i;
    if (k <= 0)
        return 0;
    w = k >> 5;
    for (i = 0; i < w && i < a->n; i++)
        if (a->v[i])
            return 1;
    if ((k & 31) && w < OBL && (a->v[w] & ((1u << (k & 31)) - 1u)))
        return 1;
    return 0;
}

/* r = a << k; returns 1 if it would not fit */
static int ob_shl(ob *r, const ob *a, int k)
{
    ob t;
    int ws = k >> 5, bs = k & 31, i;
    if (a->n == 0) { ob_zero(r); return 0; }
    if (ob_bitlen(a) + k > OBL * 32)
        return 1;
    ob_zero(&t);
    for (i = a->n - 1; i >= 0; i--) {
        uint64_t x = (uint64_t)a->v[i] << bs;
        t.v[i + ws] |= (uint32_t)x;
        if (i + ws + 1 < OBL)
            t.v[i + ws + 1] |= (uint32_t)(x >> 32);
    }
    t.n = OBL;
    ob_fix(&t);
    *r = t;
    return 0;
}

/* r = a >> k */
static void ob_shr(ob *r, const ob *a, int k)
{
    ob t;
    int ws = k >> 5, bs = k & 31, i;
    ob_zero(&t);
    for (i = ws; i < a->n; i++) {
        uint64_t x = a->v[i];
        if (i + 1 < a->n)
            x |= (uint64_t)a->v[i + 1] << 32;
        t.v[i - ws] = (uint32_t)(x >> bs);
    }
    t.n = a->n - ws > 0 ? a->n - ws : 0;
    ob_fix(&t);
    *r = t;
}

static int ob_add(ob *r, const ob *a, const ob *b)
{
    ob t;
    uint64_t cy = 0;
    int i, n = a->n > b->n ? a->n : b->n;
    ob_zero(&t);
    for (i = 0; i < n; i++) {
        cy += (uint64_t)a->v[i] + b->v[i];
        t.v[i] = (uint32_t)cy;
        cy >>= 32;
    }
    if (cy) {
        if (n >= OBL)
            return 1;
        t.v[n++] = (uint32_t)cy;
    }
    t.n = n;
    ob_fix(&t);
    *r = t;
    return 0;
}

/* r = a - b, a >= b */
static void ob_sub(ob *r, const ob *a, const ob *b)
{
    ob t;
    int64_t br = 0;
    int i;
    ob_zero(&t);
    for (i = 0; i < a->n; i++) {
        int64_t x = (int64_t)a->v[i] - (int64_t)b->v[i] - br;
        br = x < 0;
        t.v[i] = (uint32_t)(x + (br ? ((int64_t)1 << 32) : 0));
    }
    t.n = a->n;
    ob_fix(&t);
    *r = t;
}

static int ob_mul(ob *r, const ob *a, const ob *b)
{
    ob t;
    int i, j;
    if (a->n + b->n > OBL)
        return 1;
    ob_zero(&t);
    for (i = 0; i < a->n; i++) {
        uint64_t cy = 0;
        for (j = 0; j < b->n; j++) {
            cy += (uint64_t)a->v[i] * b->v[j] + t.v[i + j];
            t.v[i + j] = (uint32_t)cy;
            cy >>= 32;
        }
        t.v[i + b->n] = (uint32_t)cy;
    }
    t.n = a->n + b->n;
    ob_fix(&t);
    *r = t;
    return 0;
}

static int ob_inc(ob *r)
{
    ob one;
    ob_u32(&one, 1);
    return ob_add(r, r, &one);
}

static void ob_dec(ob *r)
{
    ob one;
    ob_u32(&one, 1);
    ob_sub(r, r, &one);
}

static void ob_load(ob *r, const uint8_t *p, int nb)
{
    int i;
    ob_zero(r);
    if (!p)
        return;
    for (i = 0; i < nb; i++)
        r->v[i >> 2] |= (uint32_t)p[i] << (8 * (i & 3));
    r->n = (nb + 3) / 4;
    ob_fix(r);
}

static void ob_store(const ob *a, uint8_t *p, int nb)
{
    int i;
    for (i = 0; i < nb; i++)
        p[i] = (uint8_t)(a->v[i >> 2] >> (8 * (i & 3)));
}

/* floor division q = a / b, rem = a % b (b != 0), restoring, bit by bit */
static void ob_divmod(ob *q, ob *rem, const ob *a, const ob *b)
{
    ob r, qq;
    int i, L = ob_bitlen(a);
    ob_zero(&r);
    ob_zero(&qq);
    for (i = L - 1; i >= 0; i--) {
        ob_shl(&r, &r, 1);
        if (ob_bit(a, i))
            ob_setbit(&r, 0);
        if (ob_cmp(&r, b) >= 0) {
            ob_sub(&r, &r, b);
            ob_setbit(&qq, i);
        }
    }
    *q = qq;
    *rem = r;
}

/* floor(sqrt(a)) by the digit-by-digit (binary restoring) method */
static void ob_isqrt(ob *root, const ob *a)
{
    ob rem, res, bit, t;
    int L = ob_bitlen(a), k;
    ob_zero(&res);
    rem = *a;
    if (L == 0) { ob_zero(root); return; }
    k = (L - 1) & ~1;                       /* highest even bit <= L-1 */
    ob_zero(&bit);
    ob_setbit(&bit, k);
    while (!ob_is_zero(&bit)) {
        ob_add(&t, &res, &bit);
        if (ob_cmp(&rem, &t) >= 0) {
            ob_sub(&rem, &rem, &t);
            ob_shr(&res, &res, 1);
            ob_add(&res, &res, &bit);
        } else {
            ob_shr(&res, &res, 1);
        }
        ob_shr(&bit, &bit, 2);
    }
    *root = res;
}

/* ---- encodings (softfloat.c:18-82) ----------------------------------- */

static void set_field(ob *r, int lo, int nb, uint32_t val)
{
    int i;
    for (i = 0; i < nb; i++)
        if ((val >> i) & 1u)
            ob_setbit(r, lo + i);
}

static void enc_zero(const fmt_t *f, int sign, ob *o)
{
    ob_zero(o);
    if (sign)
        ob_setbit(o, f->width - 1);
}

static void enc_inf(const fmt_t *f, int sign, ob *o)
{
    ob_zero(o);
    set_field(o, f->man_w, f->exp_w, f->exp_mask);
    if (sign)
        ob_setbit(o, f->width - 1);
}

/* the one NaN arithmetic emits: sign 0, exponent all ones, quiet bit set */
static void enc_qnan(const fmt_t *f, ob *o)
{
    ob_zero(o);
    set_field(o, f->man_w, f->exp_w, f->exp_mask);
    ob_setbit(o, f->man_w - 1);
}

static void enc_max_normal(const fmt_t *f, int sign, ob *o)
{
    int i;
    ob_zero(o);
    for (i = 0; i < f->man_w; i++)
        ob_setbit(o, i);
    set_field(o, f->man_w, f->exp_w, f->exp_mask - 1u);
    if (sign)
        ob_setbit(o, f->width - 1);
}

static void enc_one(const fmt_t *f, ob *o)
{
    ob_zero(o);
    set_field(o, f->man_w, f->exp_w, (uint32_t)f->bias);
}

/* ---- unpack (softfloat.c:85-116) ------------------------------------ */

enum { K_ZERO, K_SUB, K_NORM, K_INF, K_NAN };

typedef struct {
    int kind, sign, signaling;
    ob m;               /* value = (-1)^sign * m * 2^e */
    int e;
} unp;

static void unpack(const fmt_t *f, const ob *x, unp *u)
{
    uint32_t ef = ob_extract(x, f->man_w, f->exp_w);
    u->sign = ob_bit(x, f->width - 1);
    u->signaling = 0;
    u->e = 0;
    u->m = *x;
    ob_mask(&u->m, f->man_w);
    if (ef == f->exp_mask) {
        if (ob_is_zero(&u->m)) {
            u->kind = K_INF;
        } else {
            u->kind = K_NAN;
            u->signaling = !ob_bit(x, f->man_w - 1);
        }
        ob_zero(&u->m);
        return;
    }
    if (ef == 0) {
        if (ob_is_zero(&u->m)) {
            u->kind = K_ZERO;
            return;
        }
        u->kind = K_SUB;
        u->e = f->emin - f->man_w;
        return;
    }
    u->kind = K_NORM;
    ob_setbit(&u->m, f->man_w);
    u->e = (int)ef - f->bias - f->man_w;
}

/* ---- rounding (softfloat.c:120-261) --------------------------------- */

/* rnd 5 is 9.5's roundTiesTowardZero, an internal direction of the
 * augmented operations only (augmented.c; golden softfloat RND_RTTZ):
 * nearest, ties toward the smaller magnitude, overflow to infinity. */
static int round_up(int rnd, int sign, int guard, int sticky, int lsb)
{
    switch (rnd) {
    case 0: return guard && (sticky || lsb);           /* RNE */
    case 4: return guard;                              /* RMM */
    case 1: return 0;                                  /* RTZ */
    case 2: return sign && (guard || sticky);          /* RDN */
    case 5: return guard && sticky;                    /* RTTZ */
    default: return !sign && (guard || sticky);        /* RUP */
    }
}

static int overflow_to_inf(int rnd, int sign)
{
    if (rnd == 1) return 0;
    if (rnd == 2) return sign;
    if (rnd == 3) return !sign;
    return 1;
}

/* (m + eps) * 2^e rounded to a multiple of 2^q (softfloat.c:158-186) */
static int round_at(const ob *m, int e, int q, int sign, int rnd, int sticky,
                    ob *kept, int *inexact)
{
    int sh = q - e;
    *inexact = 0;
    if (sh <= 0) {
        if (sticky)
            return 1;
        return ob_shl(kept, m, -sh);
    }
    ob_shr(kept, m, sh);
    if (!ob_low_nonzero(m, sh) && !sticky)
        return 0;
    {
        int g = ob_bit(m, sh - 1);
        int s = ob_low_nonzero(m, sh - 1) || sticky;
        int l = ob_bit(kept, 0);
        if (round_up(rnd, sign, g, s, l) && ob_inc(kept))
            return 1;
    }
    *inexact = 1;
    return 0;
}

/* softfloat.c:192-261: tininess after rounding, underflow only when tiny
 * and inexact, overflow to infinity or max-normal by mode. */
static int round_pack(const fmt_t *f, int sign, const ob *m, int e,
                      int sticky, int rnd, ob *out, uint32_t *flags)
{
    int p = f->prec, L = ob_bitlen(m), e_norm, q_unb, q, e_res, tiny;
    int inexact = 0, dummy = 0;
    ob ku, k;
    uint32_t fl = 0;

    if (L == 0 || (sticky && L <= p))
        return 1;
    e_norm = e + L - 1;
    q_unb = e_norm - (p - 1);
    if (round_at(m, e, q_unb, sign, rnd, sticky, &ku, &dummy))
        return 1;
    tiny = (q_unb + ob_bitlen(&ku) - 1) < f->emin;

    q = (e_norm > f->emin ? e_norm : f->emin) - (p - 1);
    if (round_at(m, e, q, sign, rnd, sticky, &k, &inexact))
        return 1;
    if (inexact)
        fl |= 16u;
    if (ob_is_zero(&k)) {
        enc_zero(f, sign, out);
        *flags = fl | 8u;
        return 0;
    }
    e_res = q + ob_bitlen(&k) - 1;
    if (e_res > f->emax) {
        if (overflow_to_inf(rnd, sign))
            enc_inf(f, sign, out);
        else
            enc_max_normal(f, sign, out);
        *flags = fl | 4u | 16u;
        return 0;
    }
    if (tiny && inexact)
        fl |= 8u;
    if (e_res < f->emin) {                      /* subnormal */
        *out = k;
        if (sign)
            ob_setbit(out, f->width - 1);
        *flags = fl;
        return 0;
    }
    if (ob_bitlen(&k) == p + 1)
        ob_shr(&k, &k, 1);                      /* carried out */
    ob_clearbit(&k, f->man_w);
    *out = k;
    set_field(out, f->man_w, f->exp_w, (uint32_t)(e_res + f->bias));
    if (sign)
        ob_setbit(out, f->width - 1);
    *flags = fl;
    return 0;
}

/* ---- FMA with bounded alignment (softfloat.c:263-428) --------------- */

static void nan_result(const fmt_t *f, const unp *a, const unp *b,
                       const unp *c, ob *out, uint32_t *flags)
{
    int inv = (a && a->kind == K_NAN && a->signaling) ||
              (b && b->kind == K_NAN && b->signaling) ||
              (c && c->kind == K_NAN && c->signaling);
    enc_qnan(f, out);
    *flags = inv ? 1u : 0u;
}

static int fma_core(const fmt_t *f, const ob *xa, const ob *xb, const ob *xc,
                    int rnd, ob *out, uint32_t *flags)
{
    unp ua, ub, uc;
    ob mp, tp, tc, t;
    int sp, ep, Lp, Lc, VEp, VEc, FAR, e0;

    unpack(f, xa, &ua);
    unpack(f, xb, &ub);
    unpack(f, xc, &uc);
    *flags = 0;

    if (ua.kind == K_NAN || ub.kind == K_NAN || uc.kind == K_NAN) {
        nan_result(f, &ua, &ub, &uc, out, flags);
        return 0;
    }
    sp = ua.sign ^ ub.sign;
    if (ua.kind == K_INF || ub.kind == K_INF) {
        if (ua.kind == K_ZERO || ub.kind == K_ZERO) {
            enc_qnan(f, out);                   /* inf * 0 */
            *flags = 1u;
            return 0;
        }
        if (uc.kind == K_INF && uc.sign != sp) {
            enc_qnan(f, out);                   /* inf - inf */
            *flags = 1u;
            return 0;
        }
        enc_inf(f, sp, out);
        return 0;
    }
    if (uc.kind == K_INF) {
        enc_inf(f, uc.sign, out);
        return 0;
    }
    if (ua.kind == K_ZERO || ub.kind == K_ZERO) {
        if (uc.kind == K_ZERO) {
            int rs = (uc.sign == sp) ? uc.sign : (rnd == 2);
            enc_zero(f, rs, out);
            return 0;
        }
        *out = *xc;                             /* 0*b + c is c, exactly */
        return 0;
    }
    if (ob_mul(&mp, &ua.m, &ub.m))
        return 1;
    ep = ua.e + ub.e;
    if (uc.kind == K_ZERO)
        return round_pack(f, sp, &mp, ep, 0, rnd, out, flags);

    Lp = ob_bitlen(&mp);
    Lc = ob_bitlen(&uc.m);
    VEp = ep + Lp - 1;
    VEc = uc.e + Lc - 1;
    FAR = 2 * f->prec + 4;
    if (VEp - VEc > FAR || VEc - VEp > FAR) {
        /* the smaller term is only a sticky below the larger one */
        const ob *bm;
        int be, bs, os, L, k;
        ob m;
        if (VEp > VEc) { bm = &mp;   be = ep;   bs = sp;      os = uc.sign; }
        else           { bm = &uc.m; be = uc.e; bs = uc.sign; os = sp; }
        L = ob_bitlen(bm);
        k = f->prec + 2 - L;
        if (k < 2)
            k = 2;
        if (ob_shl(&m, bm, k))
            return 1;
        if (os != bs)
            ob_dec(&m);
        return round_pack(f, bs, &m, be - k, 1, rnd, out, flags);
    }
    e0 = ep < uc.e ? ep : uc.e;
    if (ob_shl(&tp, &mp, ep - e0) || ob_shl(&tc, &uc.m, uc.e - e0))
        return 1;
    if (sp == uc.sign) {
        if (ob_add(&t, &tp, &tc))
            return 1;
        return round_pack(f, sp, &t, e0, 0, rnd, out, flags);
    }
    {
        int c = ob_cmp(&tp, &tc);
        if (c == 0) {
            enc_zero(f, rnd == 2, out);          /* exact cancellation */
            return 0;
        }
        if (c > 0) {
            ob_sub(&t, &tp, &tc);
            return round_pack(f, sp, &t, e0, 0, rnd, out, flags);
        }
        ob_sub(&t, &tc, &tp);
        return round_pack(f, uc.sign, &t, e0, 0, rnd, out, flags);
    }
}

/* operand steering (softfloat.c:438-468) */
static int arith(const fmt_t *f, int op, const ob *a, const ob *b,
                 const ob *c, int rnd, ob *out, uint32_t *flags)
{
    ob sb, sc;
    switch (op) {
    case 0:
        return fma_core(f, a, b, c, rnd, out, flags);
    case 1:                                     /* ADD: a*1 + c */
        enc_one(f, &sb);
        return fma_core(f, a, &sb, c, rnd, out, flags);
    case 2:                                     /* SUB: a*1 + (-c) */
        enc_one(f, &sb);
        sc = *c;
        if (ob_bit(&sc, f->width - 1))
            ob_clearbit(&sc, f->width - 1);
        else
            ob_setbit(&sc, f->width - 1);
        return fma_core(f, a, &sb, &sc, rnd, out, flags);
    default:                                    /* MUL: a*b + (+-0) */
        enc_zero(f, ob_bit(a, f->width - 1) ^ ob_bit(b, f->width - 1), &sc);
        return fma_core(f, a, b, &sc, rnd, out, flags);
    }
}

/* ---- quiet and integer operations (softfloat.c:470-609) ------------- */

static void magnitude(const fmt_t *f, const ob *x, ob *r)
{
    *r = *x;
    ob_clearbit(r, f->width - 1);
}

static int numeric_lt(const fmt_t *f, const ob *a, const ob *b)
{
    ob ma, mb;
    int sa = ob_bit(a, f->width - 1), sb = ob_bit(b, f->width - 1);
    magnitude(f, a, &ma);
    magnitude(f, b, &mb);
    if (ob_is_zero(&ma) && ob_is_zero(&mb))
        return 0;
    if (sa != sb)
        return sa;
    return sa ? (ob_cmp(&ma, &mb) > 0) : (ob_cmp(&ma, &mb) < 0);
}

static int is_nan(const fmt_t *f, const ob *x, int *sig)
{
    ob fr;
    if (ob_extract(x, f->man_w, f->exp_w) != f->exp_mask)
        return 0;
    fr = *x;
    ob_mask(&fr, f->man_w);
    if (ob_is_zero(&fr))
        return 0;
    *sig = !ob_bit(x, f->man_w - 1);
    return 1;
}

static void minmax(const fmt_t *f, const ob *a, const ob *b, int want_max,
                   int number, ob *out, uint32_t *flags)
{
    int sa = 0, sb = 0, an = is_nan(f, a, &sa), bn = is_nan(f, b, &sb);
    ob ma, mb;
    *flags = ((an && sa) || (bn && sb)) ? 1u : 0u;
    if (an || bn) {
        if (!number || (an && bn))
            enc_qnan(f, out);
        else
            *out = an ? *b : *a;
        return;
    }
    magnitude(f, a, &ma);
    magnitude(f, b, &mb);
    if (ob_is_zero(&ma) && ob_is_zero(&mb)) {
        int za = ob_bit(a, f->width - 1), zb = ob_bit(b, f->width - 1);
        if (za == zb)
            *out = *a;
        else
            *out = want_max ? (za ? *b : *a) : (za ? *a : *b);
        return;
    }
    {
        int lt = numeric_lt(f, a, b);
        if (want_max)
            *out = lt ? *b : *a;
        else
            *out = lt ? *a : *b;
    }
}

static void compare(const fmt_t *f, const ob *a, const ob *b, int op,
                    ob *out, uint32_t *flags)
{
    int sa = 0, sb = 0, an = is_nan(f, a, &sa), bn = is_nan(f, b, &sb);
    int lt, gt, eq, truth;
    *flags = ((an && sa) || (bn && sb)) ? 1u : 0u;
    if (an || bn) {
        enc_zero(f, 0, out);
        return;
    }
    lt = numeric_lt(f, a, b);
    gt = numeric_lt(f, b, a);
    eq = !lt && !gt;
    truth = op == 12 ? lt : op == 13 ? (lt || eq) : eq;
    if (truth)
        enc_one(f, out);
    else
        enc_zero(f, 0, out);
}

static int integer_op(const fmt_t *f, int op, const ob *a, const ob *b, ob *out)
{
    int i, sh;
    ob t;
    switch (op) {
    case 16: case 17: case 18:
        ob_zero(&t);
        for (i = 0; i < OBL; i++)
            t.v[i] = op == 16 ? (a->v[i] & b->v[i])
                   : op == 17 ? (a->v[i] | b->v[i]) : (a->v[i] ^ b->v[i]);
        t.n = OBL;
        ob_fix(&t);
        *out = t;
        return 0;
    case 19:
        if (ob_add(out, a, b))
            return 1;
        ob_mask(out, f->width);
        return 0;
    case 20:
        t = *a;
        ob_setbit(&t, f->width);
        ob_sub(out, &t, b);
        ob_mask(out, f->width);
        return 0;
    case 21:
        sh = (int)(ob_extract(b, 0, 32) & (uint32_t)(f->width - 1));
        if (ob_shl(out, a, sh))
            return 1;
        ob_mask(out, f->width);
        return 0;
    case 22:
        sh = (int)(ob_extract(b, 0, 32) & (uint32_t)(f->width - 1));
        ob_shr(out, a, sh);
        return 0;
    case 23:
        if (ob_cmp(a, b) < 0)
            enc_one(f, out);
        else
            enc_zero(f, 0, out);
        return 0;
    case 30: {
        uint32_t pa = ob_extract(a, 0, 32), pb = ob_extract(b, 0, 32);
        ob_u32(out, (uint32_t)((uint64_t)pa * pb));
        return 0;
    }
    default:
        return 1;
    }
}

/* ---- divide/sqrt seeds (softfloat.c:611-735) ------------------------ */

static uint32_t recip_entry(uint32_t i)
{
    uint32_t num = 1u << 28, den = 1024u + (i << 1) + 1u;
    uint32_t q = num / den, r = num % den;
    if (2u * r > den || (2u * r == den && (q & 1u)))
        q++;
    return q;
}

static uint32_t rsqrt_entry(uint32_t j)
{
    uint32_t odd = j >> 9, i = j & 511u;
    uint64_t m2 = (uint64_t)(1024u + (i << 1) + 1u) << odd;
    uint64_t t = (1ull << 44) / m2, q = 0, bit;
    for (bit = 1ull << 17; bit; bit >>= 1)
        if ((q | bit) * (q | bit) <= t)
            q |= bit;
    while ((q + 1) * (q + 1) * m2 <= (1ull << 44))
        q++;
    if ((2 * q + 1) * (2 * q + 1) * m2 < (1ull << 46))
        q++;
    return (uint32_t)q;
}

static void seed_pack(const fmt_t *f, int sign, uint32_t r, int e, ob *out)
{
    ob m;
    uint32_t fl = 0;
    ob_u32(&m, r);
    (void)round_pack(f, sign, &m, e, 0, 0, out, &fl);
}

static void recip_seed(const fmt_t *f, const ob *x, ob *out)
{
    int sign = ob_bit(x, f->width - 1), E, e_out;
    uint32_t ef = ob_extract(x, f->man_w, f->exp_w);
    ob fr = *x;
    ob_mask(&fr, f->man_w);
    if (ef == f->exp_mask) {
        if (!ob_is_zero(&fr)) enc_qnan(f, out);
        else enc_zero(f, sign, out);
        return;
    }
    if (ef == 0) { enc_inf(f, sign, out); return; }
    E = (int)ef - f->bias;
    e_out = -E - 18;
    if (e_out + 17 > f->emax) { enc_inf(f, sign, out); return; }
    seed_pack(f, sign, recip_entry(ob_extract(x, f->man_w - 9, 9)), e_out, out);
}

static void rsqrt_seed(const fmt_t *f, const ob *x, ob *out)
{
    int sign = ob_bit(x, f->width - 1), E, odd, e_out;
    uint32_t ef = ob_extract(x, f->man_w, f->exp_w);
    ob fr = *x;
    ob_mask(&fr, f->man_w);
    if (ef == f->exp_mask && !ob_is_zero(&fr)) { enc_qnan(f, out); return; }
    if (ef == 0) { enc_inf(f, sign, out); return; }
    if (sign) { enc_qnan(f, out); return; }
    if (ef == f->exp_mask) { enc_zero(f, 0, out); return; }
    E = (int)ef - f->bias;
    odd = E & 1;
    e_out = -((E - odd) / 2) - 17;
    seed_pack(f, 0, rsqrt_entry(((uint32_t)odd << 9) |
                                ob_extract(x, f->man_w - 9, 9)), e_out, out);
}

/* ---- dispatch (softfloat.c:939-1009) -------------------------------- */

static int compute(const fmt_t *f, int op, int rnd, const ob *a, const ob *b,
                   const ob *c, ob *out, uint32_t *flags)
{
    *flags = 0;
    switch (op) {
    case 0: case 1: case 2: case 3:
        return arith(f, op, a, b, c, rnd, out, flags);
    case 4:
        magnitude(f, a, out);
        return 0;
    case 5:
        *out = *a;
        if (ob_bit(a, f->width - 1)) ob_clearbit(out, f->width - 1);
        else ob_setbit(out, f->width - 1);
        return 0;
    case 6:
        magnitude(f, a, out);
        if (ob_bit(b, f->width - 1))
            ob_setbit(out, f->width - 1);
        return 0;
    case 7:  minmax(f, a, b, 0, 0, out, flags); return 0;
    case 8:  minmax(f, a, b, 1, 0, out, flags); return 0;
    case 9:  minmax(f, a, b, 0, 1, out, flags); return 0;
    case 10: minmax(f, a, b, 1, 1, out, flags); return 0;
    case 11: {
        ob mc;
        magnitude(f, c, &mc);
        *out = ob_is_zero(&mc) ? *b : *a;
        return 0;
    }
    case 12: case 13: case 14:
        compare(f, a, b, op, out, flags);
        return 0;
    case 16: case 17: case 18: case 19: case 20: case 21: case 22: case 23:
    case 30:
        return integer_op(f, op, a, b, out);
    case 26:
        recip_seed(f, a, out);
        return 0;
    case 27:
        rsqrt_seed(f, a, out);
        return 0;
    default:
        /* unassigned (and the reductions, which cft_run refuses before
         * reaching here): the canonical quiet NaN and invalid */
        enc_qnan(f, out);
        *flags = 1u;
        return 0;
    }
}

/* ---- the contract's div and sqrt (softfloat.py:424-505) ------------- */

static void fold_sticky(ob *q, int rem_nonzero)
{
    ob_shl(q, q, 1);
    if (rem_nonzero)
        ob_setbit(q, 0);
}

static int div_core(const fmt_t *f, int rnd, const ob *xa, const ob *xb,
                    ob *out, uint32_t *flags)
{
    unp ua, ub;
    int sq, k, e;
    ob num, q, rem;
    unpack(f, xa, &ua);
    unpack(f, xb, &ub);
    *flags = 0;
    if (ua.kind == K_NAN || ub.kind == K_NAN) {
        nan_result(f, &ua, &ub, 0, out, flags);
        return 0;
    }
    sq = ua.sign ^ ub.sign;
    if (ua.kind == K_INF) {
        if (ub.kind == K_INF) { enc_qnan(f, out); *flags = 1u; return 0; }
        enc_inf(f, sq, out);
        return 0;
    }
    if (ub.kind == K_INF) { enc_zero(f, sq, out); return 0; }
    if (ub.kind == K_ZERO) {
        if (ua.kind == K_ZERO) { enc_qnan(f, out); *flags = 1u; return 0; }
        enc_inf(f, sq, out);
        *flags = 2u;
        return 0;
    }
    if (ua.kind == K_ZERO) { enc_zero(f, sq, out); return 0; }
    k = (f->prec + 3) + ob_bitlen(&ub.m) - ob_bitlen(&ua.m) + 1;
    if (k < 0)
        k = 0;
    if (ob_shl(&num, &ua.m, k))
        return 1;
    ob_divmod(&q, &rem, &num, &ub.m);
    if (ob_bitlen(&q) < f->prec + 3)
        return 1;
    fold_sticky(&q, !ob_is_zero(&rem));
    e = (ua.e - ub.e) - k - 1;
    return round_pack(f, sq, &q, e, 0, rnd, out, flags);
}

static int sqrt_core(const fmt_t *f, int rnd, const ob *xa, ob *out,
                     uint32_t *flags)
{
    unp ua;
    int t, e;
    ob m, r, r2;
    unpack(f, xa, &ua);
    *flags = 0;
    if (ua.kind == K_NAN) {
        nan_result(f, &ua, 0, 0, out, flags);
        return 0;
    }
    if (ua.kind == K_ZERO) { *out = *xa; return 0; }
    if (ua.sign) { enc_qnan(f, out); *flags = 1u; return 0; }
    if (ua.kind == K_INF) { *out = *xa; return 0; }
    e = ua.e;
    t = 2 * (f->prec + 3) - ob_bitlen(&ua.m);
    if (t < 0)
        t = 0;
    t += (t ^ e) & 1;                            /* keep e - t even */
    if (ob_shl(&m, &ua.m, t))
        return 1;
    e -= t;
    ob_isqrt(&r, &m);
    if (ob_bitlen(&r) < f->prec + 3)
        return 1;
    if (ob_mul(&r2, &r, &r))
        return 1;
    fold_sticky(&r, ob_cmp(&r2, &m) != 0);
    /* e is even here; e/2 is exact, floor equals truncation */
    return round_pack(f, 0, &r, e / 2 - 1, 0, rnd, out, flags);
}

/* ---- exported entry points ------------------------------------------ */

static int bad_fmt(int fmt) { return fmt < 0 || fmt > 3; }

int sfp_compute(int fmt, int op, int rnd, const uint8_t *a, const uint8_t *b,
                const uint8_t *c, uint8_t *d, uint32_t *flags)
{
    const fmt_t *f;
    ob A, B, C, O;
    int nb, st;
    if (bad_fmt(fmt))
        return 1;
    f = &FMTS[fmt];
    nb = f->width / 8;
    ob_load(&A, a, nb);
    ob_load(&B, b, nb);
    ob_load(&C, c, nb);
    ob_zero(&O);
    st = compute(f, op, rnd, &A, &B, &C, &O, flags);
    if (!st)
        ob_store(&O, d, nb);
    return st;
}

int sfp_div(int fmt, int rnd, const uint8_t *a, const uint8_t *b, uint8_t *d,
            uint32_t *flags)
{
    const fmt_t *f;
    ob A, B, O;
    int nb, st;
    if (bad_fmt(fmt))
        return 1;
    f = &FMTS[fmt];
    nb = f->width / 8;
    ob_load(&A, a, nb);
    ob_load(&B, b, nb);
    ob_zero(&O);
    st = div_core(f, rnd, &A, &B, &O, flags);
    if (!st)
        ob_store(&O, d, nb);
    return st;
}

int sfp_sqrt(int fmt, int rnd, const uint8_t *a, uint8_t *d, uint32_t *flags)
{
    const fmt_t *f;
    ob A, O;
    int nb, st;
    if (bad_fmt(fmt))
        return 1;
    f = &FMTS[fmt];
    nb = f->width / 8;
    ob_load(&A, a, nb);
    ob_zero(&O);
    st = sqrt_core(f, rnd, &A, &O, flags);
    if (!st)
        ob_store(&O, d, nb);
    return st;
}

int sfp_run(int kind, int fmt, int op, int rnd, const void *a, const void *b,
            const void *c, void *d, size_t n, uint32_t scalar_mask,
            uint8_t *lane_flags, uint32_t *acc)
{
    const uint8_t *pa = (const uint8_t *)a, *pb = (const uint8_t *)b;
    const uint8_t *pc = (const uint8_t *)c;
    uint8_t *pd = (uint8_t *)d;
    size_t esz, i, sa, sb, sc;
    uint32_t all = 0;
    uint8_t tmp[32];
    if (bad_fmt(fmt))
        return 1;
    esz = (size_t)FMTS[fmt].width / 8;
    sa = (scalar_mask & 1u) ? 0 : esz;
    sb = (scalar_mask & 2u) ? 0 : esz;
    sc = (scalar_mask & 4u) ? 0 : esz;
    for (i = 0; i < n; i++) {
        uint32_t fl = 0;
        int st;
        const uint8_t *ea = pa ? pa + i * sa : NULL;
        const uint8_t *eb = pb ? pb + i * sb : NULL;
        const uint8_t *ec = pc ? pc + i * sc : NULL;
        if (kind == 1)
            st = sfp_div(fmt, rnd, ea, eb, tmp, &fl);
        else if (kind == 2)
            st = sfp_sqrt(fmt, rnd, ea, tmp, &fl);
        else
            st = sfp_compute(fmt, op, rnd, ea, eb, ec, tmp, &fl);
        if (st)
            return 1;
        memcpy(pd + i * esz, tmp, esz);       /* load before store: d may alias */
        if (lane_flags)
            lane_flags[i] = (uint8_t)fl;
        all |= fl;
    }
    if (acc)
        *acc = all;
    return 0;
}

/* ---- reductions ---------------------------------------------------------
 *
 * The fixed tree (host/src/softfloat.c:850-937): T(lo, hi) is +0 for an
 * empty range, the leaf for one element (the element itself for SUM; the
 * rounded product for DOT), else add(T(lo, mid), T(mid, hi)) with mid = lo
 * + k/2, k the smallest power of two >= hi - lo - so the left child is the
 * largest power of two strictly inside the range. The add is ADD with the
 * left subtree in a and the right in c. Flags OR over every node.
 *
 * The compositions (host/src/device.c:2880-3066): SUMSQ is DOT(a, a) and
 * SUMABS is SUM over the magnitudes; when either's result is a NaN and an
 * element is an infinity, the result is +inf and the flags are INVALID iff
 * an element is a signalling NaN (IEEE 754-2019 9.4), replacing the tree's.
 * MAXALL halves with the elementwise MAX (op 8): pairs (x[i], x[i + m/2]),
 * an odd last element carried; n == 1 returns a[0] verbatim. n == 0 gives
 * +0 (MAXALL: -inf) and no flags (device.c:2812-2832). The segmented form
 * is the same per slice, flags ORed (device.c:3201-3216). */
static int red_tree(int fmt, int op, int rnd, const uint8_t *a, const uint8_t *b, size_t lo,
                    size_t hi, uint8_t *out, uint32_t *flags)
{
    const size_t esz = (size_t)FMTS[fmt].width / 8;
    uint8_t left[32], right[32], zero[32];
    uint32_t lf = 0, rf = 0, af = 0;
    size_t m, k, mid;
    *flags = 0;
    memset(zero, 0, sizeof zero);
    if (hi == lo) {
        memset(out, 0, esz);
        return 0;
    }
    if (hi - lo == 1) {
        if (op == 25)
            return sfp_compute(fmt, 3, rnd, a + lo * esz, b + lo * esz, zero, out, flags);
        memcpy(out, a + lo * esz, esz);
        return 0;
    }
    m = hi - lo;
    k = 1;
    while (k < m)
        k <<= 1;
    mid = lo + (k >> 1);
    if (red_tree(fmt, op, rnd, a, b, lo, mid, left, &lf))
        return 1;
    if (red_tree(fmt, op, rnd, a, b, mid, hi, right, &rf))
        return 1;
    if (sfp_compute(fmt, 1, rnd, left, zero, right, out, &af))
        return 1;
    *flags = lf | rf | af;
    return 0;
}

static int is_nan_bytes(const fmt_t *f, const uint8_t *p)
{
    ob v;
    ob_load(&v, p, f->width / 8);
    if (ob_extract(&v, f->man_w, f->exp_w) != f->exp_mask)
        return 0;
    ob_mask(&v, f->man_w);
    return !ob_is_zero(&v);
}

/* 9.4's infinity rule over a[0..n): 1 when it applies (device.c:2678-2703). */
static int inf_override(const fmt_t *f, const uint8_t *a, size_t n, uint8_t *out,
                        uint32_t *flags)
{
    const int nb = f->width / 8;
    int saw_inf = 0, saw_snan = 0;
    size_t i;
    for (i = 0; i < n; i++) {
        ob v, frac;
        ob_load(&v, a + i * nb, nb);
        if (ob_extract(&v, f->man_w, f->exp_w) != f->exp_mask)
            continue;
        frac = v;
        ob_mask(&frac, f->man_w);
        if (ob_is_zero(&frac))
            saw_inf = 1;
        else if (!ob_bit(&v, f->man_w - 1))
            saw_snan = 1;
    }
    if (!saw_inf)
        return 0;
    {
        ob o;
        enc_inf(f, 0, &o);
        ob_store(&o, out, nb);
    }
    *flags = saw_snan ? 1u : 0u;          /* INVALID */
    return 1;
}

int sfp_reduce(int fmt, int op, int rnd, const void *a, const void *b, void *d, size_t n,
               uint32_t *flags)
{
    const fmt_t *f;
    size_t esz;
    uint8_t *pd = (uint8_t *)d;
    const uint8_t *pa = (const uint8_t *)a, *pb = (const uint8_t *)b;
    uint32_t fl = 0;
    if (bad_fmt(fmt) || !d)
        return 1;
    f = &FMTS[fmt];
    esz = (size_t)f->width / 8;
    *flags = 0;
    if (n == 0) {
        ob z;
        if (op == 31)
            enc_inf(f, 1, &z);
        else
            ob_zero(&z);
        ob_store(&z, pd, (int)esz);
        return 0;
    }
    if (op == 31) {
        uint8_t *buf = (uint8_t *)malloc((n + 1) * esz);
        size_t m = n, i;
        if (!buf)
            return 1;
        memcpy(buf, pa, n * esz);
        while (m > 1) {
            const size_t h = m / 2;
            const int odd = (m & 1u) != 0;
            for (i = 0; i < h; i++) {
                uint8_t t[32];
                uint32_t pf = 0;
                if (sfp_compute(fmt, 8, rnd, buf + i * esz, buf + (i + h) * esz, NULL, t, &pf)) {
                    free(buf);
                    return 1;
                }
                fl |= pf;
                memcpy(buf + i * esz, t, esz);     /* i < h: reads of later pairs untouched */
            }
            if (odd)
                memmove(buf + h * esz, buf + 2 * h * esz, esz);
            m = h + (size_t)odd;
        }
        memcpy(pd, buf, esz);
        free(buf);
        *flags = fl;
        return 0;
    }
    if (op == 28 || op == 29) {
        int st;
        if (op == 28) {
            st = red_tree(fmt, 25, rnd, pa, pa, 0, n, pd, &fl);
        } else {
            uint8_t *tmp = (uint8_t *)malloc(n * esz);
            size_t i;
            if (!tmp)
                return 1;
            for (i = 0; i < n; i++) {
                uint32_t af = 0;
                if (sfp_compute(fmt, 4, rnd, pa + i * esz, NULL, NULL, tmp + i * esz, &af)) {
                    free(tmp);
                    return 1;
                }
                fl |= af;
            }
            {
                uint32_t sf = 0;
                st = red_tree(fmt, 24, rnd, tmp, NULL, 0, n, pd, &sf);
                fl |= sf;
            }
            free(tmp);
        }
        if (st)
            return 1;
        if (is_nan_bytes(f, pd)) {
            uint32_t of = 0;
            if (inf_override(f, pa, n, pd, &of))
                fl = of;
        }
        *flags = fl;
        return 0;
    }
    if (op != 24 && op != 25)
        return 1;
    if (red_tree(fmt, op, rnd, pa, pb, 0, n, pd, &fl))
        return 1;
    *flags = fl;
    return 0;
}

int sfp_reduce_seg(int fmt, int op, int rnd, const void *a, const void *b, void *d, size_t n,
                   size_t seg, uint32_t *flags)
{
    const size_t esz = bad_fmt(fmt) ? 0 : (size_t)FMTS[fmt].width / 8;
    size_t s;
    uint32_t all = 0;
    if (!esz || !seg || n % seg)
        return 1;
    for (s = 0; s < n / seg; s++) {
        uint32_t fl = 0;
        if (sfp_reduce(fmt, op, rnd, (const uint8_t *)a + s * seg * esz,
                       b ? (const uint8_t *)b + s * seg * esz : NULL, (uint8_t *)d + s * esz,
                       seg, &fl))
            return 1;
        all |= fl;
    }
    *flags = all;
    return 0;
}


/* ---- the augmented operations, IEEE 754-2019 9.5 --------------------------
 *
 * (python/cft_golden/augmented.py defines them; host/src/augmented.c is its
 * C port.) r is x op y rounded with roundTiesTowardZero, e the exact
 * residual x op y - r, representable for addition whenever r is finite;
 * for multiplication a residual with digits below the smallest quantum is
 * delivered rounded the same way, with UNDERFLOW and INEXACT. Flags: an
 * overflowing r gives (inf, inf, OVERFLOW|INEXACT); otherwise UNDERFLOW iff
 * the residual is non-zero and below 2^emin; nothing else. An exactly zero
 * residual takes r's sign. NaN inputs give the canonical quiet NaN twice,
 * INVALID iff one is signalling; inf - inf and inf * 0 give it with
 * INVALID. Addition aligns exactly only when the value exponents are
 * within p + 1 (augmented.c's FAR bound): farther apart, r is the larger
 * operand and e the smaller, exactly. fn: 0 add, 1 sub, 2 mul. */
static int aug_pair(const fmt_t *f, int sign_t, const ob *t, int e0, int is_mul, ob *r,
                    ob *e, uint32_t *flags)
{
    uint32_t rf = 0, ef = 0;
    unp ur;
    ob rm, A, B, mag;
    int re, q, sign_e, tiny;
    if (round_pack(f, sign_t, t, e0, 0, 5, r, &rf))
        return 1;
    if (rf & 4u) {
        enc_inf(f, sign_t, r);
        *e = *r;
        *flags = 4u | 16u;
        return 0;
    }
    unpack(f, r, &ur);
    if (ur.kind == K_ZERO) {
        ob_zero(&rm);
        re = e0;
    } else {
        rm = ur.m;
        re = ur.e;
    }
    q = e0 < re ? e0 : re;
    if (ob_shl(&A, t, e0 - q) || ob_shl(&B, &rm, re - q))
        return 1;
    if (sign_t == ur.sign || ur.kind == K_ZERO) {
        if (ob_cmp(&A, &B) >= 0) {
            ob_sub(&mag, &A, &B);
            sign_e = sign_t;
        } else {
            ob_sub(&mag, &B, &A);
            sign_e = !sign_t;
        }
    } else {
        if (ob_add(&mag, &A, &B))
            return 1;
        sign_e = sign_t;
    }
    if (ob_is_zero(&mag)) {
        enc_zero(f, ur.sign, e);
        *flags = 0;
        return 0;
    }
    tiny = (q + ob_bitlen(&mag) - 1) < f->emin;
    if (round_pack(f, sign_e, &mag, q, 0, 5, e, &ef))
        return 1;
    if (!is_mul) {
        if (ef & 16u)
            return 1;                         /* representable by 9.5; never */
        *flags = tiny ? 8u : 0u;
        return 0;
    }
    *flags = (ef & 16u) ? (8u | 16u) : (tiny ? 8u : 0u);
    return 0;
}

int sfp_aug(int fmt, int fn, const uint8_t *x, const uint8_t *y, uint8_t *r, uint8_t *e,
            uint32_t *flags)
{
    const fmt_t *f;
    ob X, Y, R, E;
    unp ua, ub;
    int nb;
    if (bad_fmt(fmt) || fn < 0 || fn > 2)
        return 1;
    f = &FMTS[fmt];
    nb = f->width / 8;
    ob_load(&X, x, nb);
    ob_load(&Y, y, nb);
    if (fn == 1) {                               /* x - y is x + (-y) */
        if (ob_bit(&Y, f->width - 1))
            ob_clearbit(&Y, f->width - 1);
        else
            ob_setbit(&Y, f->width - 1);
    }
    unpack(f, &X, &ua);
    unpack(f, &Y, &ub);
    *flags = 0;
    if (ua.kind == K_NAN || ub.kind == K_NAN) {
        enc_qnan(f, &R);
        E = R;
        *flags = ((ua.kind == K_NAN && ua.signaling) || (ub.kind == K_NAN && ub.signaling)) ? 1u : 0u;
    } else if (fn == 2) {
        const int sp = ua.sign ^ ub.sign;
        if ((ua.kind == K_INF && ub.kind == K_ZERO) || (ua.kind == K_ZERO && ub.kind == K_INF)) {
            enc_qnan(f, &R);
            E = R;
            *flags = 1u;
        } else if (ua.kind == K_INF || ub.kind == K_INF) {
            enc_inf(f, sp, &R);
            E = R;
        } else if (ua.kind == K_ZERO || ub.kind == K_ZERO) {
            enc_zero(f, sp, &R);
            E = R;
        } else {
            ob t;
            if (ob_mul(&t, &ua.m, &ub.m) || aug_pair(f, sp, &t, ua.e + ub.e, 1, &R, &E, flags))
                return 1;
        }
    } else if (ua.kind == K_INF && ub.kind == K_INF && ua.sign != ub.sign) {
        enc_qnan(f, &R);
        E = R;
        *flags = 1u;
    } else if (ua.kind == K_INF || ub.kind == K_INF) {
        enc_inf(f, ua.kind == K_INF ? ua.sign : ub.sign, &R);
        E = R;
    } else if (ua.kind == K_ZERO && ub.kind == K_ZERO) {
        enc_zero(f, ua.sign == ub.sign ? ua.sign : 0, &R);
        E = R;
    } else if (ua.kind == K_ZERO || ub.kind == K_ZERO) {
        R = ua.kind == K_ZERO ? Y : X;
        enc_zero(f, ob_bit(&R, f->width - 1), &E);
    } else {
        const int vx = ua.e + ob_bitlen(&ua.m) - 1, vy = ub.e + ob_bitlen(&ub.m) - 1;
        const int gap = vx > vy ? vx - vy : vy - vx;
        if (gap >= f->prec + 2) {
            /* FAR: the larger operand is r, the smaller e, exactly */
            const int xbig = vx > vy;
            R = xbig ? X : Y;
            E = xbig ? Y : X;
            *flags = ((xbig ? vy : vx) < f->emin) ? 8u : 0u;
        } else {
            const int e0 = ua.e < ub.e ? ua.e : ub.e;
            ob A, B, t;
            int st;
            if (ob_shl(&A, &ua.m, ua.e - e0) || ob_shl(&B, &ub.m, ub.e - e0))
                return 1;
            if (ua.sign == ub.sign) {
                if (ob_add(&t, &A, &B))
                    return 1;
                st = ua.sign;
            } else if (ob_cmp(&A, &B) >= 0) {
                ob_sub(&t, &A, &B);
                st = ua.sign;
            } else {
                ob_sub(&t, &B, &A);
                st = ub.sign;
            }
            if (ob_is_zero(&t)) {
                enc_zero(f, 0, &R);               /* exact cancellation */
                E = R;
            } else if (aug_pair(f, st, &t, e0, 0, &R, &E, flags)) {
                return 1;
            }
        }
    }
    ob_store(&R, r, nb);
    ob_store(&E, e, nb);
    return 0;
}
