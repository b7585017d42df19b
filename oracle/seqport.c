/* seqport.c - the oracle's sequencer executor (test infrastructure only).
 *
 * A restatement of the reference's per-lane program semantics
 * (host/src/seq_exec.h:175-923, host/src/program.c:1823-2040) for an image
 * a loader has already accepted. It runs one lane at a time: the
 * reference's own argument (host/src/program.c:11-31) is that lane blocks
 * are a partitioning the result cannot see, because inactive lanes write
 * nothing and the early exit only skips iterations in which no lane is
 * active.
 *
 * augmentedAddition (control codes 10 and 11) runs through sfport.c's
 * sfp_aug, the restatement of 9.5 the elementwise checks pin.
 */
#include "sfport.h"

#include <stdlib.h>
#include <string.h>

#define NREG 32
#define MAX_DEPTH 4

static uint32_t le32(const uint8_t *p)
{
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
           ((uint32_t)p[3] << 24);
}

/* the instruction word's fields (seq_exec.h:175-200) */
typedef struct {
    int op, rd, ra, rb, rc, rnd, ka, kb, kc, kx, ctrl;
    uint32_t imm;
} insn_t;

static void decode(uint64_t w, insn_t *d)
{
    d->op = (int)(w & 0xFF);
    d->rd = (int)((w >> 8) & 0xF);
    d->ra = (int)((w >> 12) & 0xF);
    d->rb = (int)((w >> 16) & 0xF);
    d->rc = (int)((w >> 20) & 0xF);
    d->rnd = (int)((w >> 24) & 0x7);
    d->ka = (int)((w >> 27) & 1);
    d->kb = (int)((w >> 28) & 1);
    d->kc = (int)((w >> 29) & 1);
    d->kx = (int)((w >> 30) & 1);
    d->ctrl = (int)((w >> 31) & 1);
    d->imm = (uint32_t)(w >> 32);
    /* the five-bit register numbers: imm[24..27] are rd, ra, rb, rc's
     * fifth bits (seq_exec.h:90-96) */
    d->rd |= (int)((d->imm >> 24) & 1) << 4;
    if (!d->ka || d->ctrl) d->ra |= (int)((d->imm >> 25) & 1) << 4;
    if (!d->kb || d->ctrl) d->rb |= (int)((d->imm >> 26) & 1) << 4;
    if (!d->kc || d->ctrl) d->rc |= (int)((d->imm >> 27) & 1) << 4;
}

/* an operand's source: a register, or a constant index (seq_exec.h:232-246) */
static int source(const insn_t *d, int which, int *is_const)
{
    const int kf[3] = { d->ka, d->kb, d->kc };
    const int reg[3] = { d->ra, d->rb, d->rc };
    *is_const = kf[which];
    if (!kf[which])
        return reg[which];
    if (d->kx)
        return (int)((d->imm >> (8 * which)) & 0xFFu) |
               (int)(((d->imm >> (28 + which)) & 1u) << 8);
    return reg[which] & 0xF;
}

typedef struct {
    int fmt;
    size_t esz;
    uint32_t n_insns, n_consts, maxdep, flags, n_sin, n_sout;
    const uint8_t *consts;          /* n_consts * esz bytes */
    uint64_t *insns;
    uint32_t depth, log2d, used;
    int scratch_active;
} prog_t;

static void st_zero(uint8_t *p, size_t esz) { memset(p, 0, esz); }

static int bitlen_bytes(const uint8_t *p, size_t esz)
{
    int i, b;
    for (i = (int)esz - 1; i >= 0; i--)
        if (p[i]) {
            for (b = 7; b >= 0; b--)
                if ((p[i] >> b) & 1)
                    return i * 8 + b + 1;
        }
    return 0;
}

static uint32_t low_bits(const uint8_t *p, size_t esz, int nb)
{
    uint32_t r = 0;
    int i;
    for (i = 0; i < 4 && (size_t)i < esz; i++)
        r |= (uint32_t)p[i] << (8 * i);
    if (nb < 32)
        r &= (1u << nb) - 1u;
    return r;
}

static int find_endrep(const prog_t *P, uint32_t pc)
{
    int depth = 0;
    uint32_t j;
    for (j = pc; j < P->n_insns; j++) {
        insn_t d;
        decode(P->insns[j], &d);
        if (!d.ctrl)
            continue;
        if (d.op == 1)
            depth++;
        else if (d.op == 2 && --depth == 0)
            return (int)j;
    }
    return (int)P->n_insns;
}

/* One lane, seq_run_block with a block of one (seq_exec.h:412-685). */
static int run_lane(const prog_t *P, const uint8_t *konst, uint8_t *regs,
                    uint8_t *scratch, uint8_t *dep, uint32_t *count,
                    int keep, uint8_t *lflag, uint32_t *flags,
                    uint32_t *status)
{
    const size_t esz = P->esz;
    struct { uint32_t body, left; } stk[MAX_DEPTH];
    int sp = 0, qd = 0, active = keep;
    uint32_t pc = 0;
    const int width = (int)esz * 8;

    while (pc < P->n_insns) {
        insn_t d;
        decode(P->insns[pc], &d);
        if (!d.ctrl) {
            int ka, kb, kc, ia, ib, ic;
            uint8_t out[32];
            uint32_t fl = 0;
            ia = source(&d, 0, &ka);
            ib = source(&d, 1, &kb);
            ic = source(&d, 2, &kc);
            if (active) {
                const uint8_t *pa = ka ? konst + ia * esz : regs + ia * esz;
                const uint8_t *pb = kb ? konst + ib * esz : regs + ib * esz;
                const uint8_t *pc_ = kc ? konst + ic * esz : regs + ic * esz;
                if (sfp_compute(P->fmt, d.op, d.rnd, pa, pb, pc_, out, &fl))
                    return 1;
                memcpy(regs + d.rd * esz, out, esz);
                if (!qd) {
                    *flags |= fl;
                    *lflag |= (uint8_t)fl;
                }
            }
            pc++;
            continue;
        }
        switch (d.op) {
        case 0:                                 /* HALT */
            return 0;
        case 1:                                 /* REPEAT */
            if (d.imm == 0 || !active) {
                pc = (uint32_t)find_endrep(P, pc) + 1;
                break;
            }
            stk[sp].body = pc + 1;
            stk[sp].left = d.imm;
            sp++;
            pc++;
            break;
        case 2:                                 /* ENDREP */
            stk[sp - 1].left--;
            if (stk[sp - 1].left > 0 && active) {
                pc = stk[sp - 1].body;
            } else {
                sp--;
                pc++;
            }
            break;
        case 3:                                 /* DEPOSIT */
            if (active) {
                if (*count >= P->maxdep) {
                    *status |= 1u << 4;
                    *lflag |= 1u << 5;
                } else {
                    memcpy(dep + (size_t)(*count) * esz, regs + d.ra * esz, esz);
                    (*count)++;
                }
            }
            pc++;
            break;
        case 4:                                 /* SETACT: narrows only */
            if (active) {
                uint8_t m[32];
                memcpy(m, regs + d.ra * esz, esz);
                m[esz - 1] &= 0x7F;
                active = bitlen_bytes(m, esz) != 0;
            }
            pc++;
            break;
        case 5:                                 /* ACTALL */
            active = keep;
            pc++;
            break;
        case 6: case 7: {                       /* STL, LDL */
            uint32_t slot = d.imm & 0x00FFFFFFu;
            if (active) {
                if (!scratch || slot >= P->depth)
                    return 1;
                if (d.op == 6)
                    memcpy(scratch + slot * esz, regs + d.ra * esz, esz);
                else
                    memcpy(regs + d.rd * esz, scratch + slot * esz, esz);
            }
            pc++;
            break;
        }
        case 8: case 9: {                       /* STX, LDX */
            int strict = (P->flags & 4u) != 0;
            int step = (int)(d.imm & 0xFFFu);
            if (step & 0x800)
                step -= 0x1000;
            if (d.op == 9 && d.rd == d.rb)
                step = 0;                       /* the load wins */
            if (active) {
                const uint8_t *ix = regs + d.rb * esz;
                if (strict && bitlen_bytes(ix, esz) > (int)P->log2d) {
                    *status |= 1u << 5;
                    *lflag |= 1u << 6;
                    if (d.op == 9)
                        st_zero(regs + d.rd * esz, esz);
                } else {
                    uint32_t slot = low_bits(ix, esz, (int)P->log2d) &
                                    (P->depth - 1u);
                    if (!scratch)
                        return 1;
                    if (d.op == 8)
                        memcpy(scratch + slot * esz, regs + d.ra * esz, esz);
                    else
                        memcpy(regs + d.rd * esz, scratch + slot * esz, esz);
                }
                if (step) {
                    /* rb := rb +/- |step| modulo 2^width, by IADD/ISUB */
                    uint8_t mag[32], out[32];
                    uint32_t fl = 0, s = (uint32_t)(step < 0 ? -step : step);
                    memset(mag, 0, sizeof mag);
                    mag[0] = (uint8_t)s;
                    mag[1] = (uint8_t)(s >> 8);
                    if (sfp_compute(P->fmt, step > 0 ? 19 : 20, 0,
                                    regs + d.rb * esz, mag, NULL, out, &fl))
                        return 1;
                    memcpy(regs + d.rb * esz, out, esz);
                }
            }
            pc++;
            (void)width;
            break;
        }
        case 10: case 11:                       /* AUGADD, AUGERR */
            /* 9.5's augmentedAddition(ra, rb): r or e to rd, flags as an
             * ALU instruction's (seq_exec.h:337-371) */
            if (active) {
                uint8_t r[32], e[32];
                uint32_t fl = 0;
                if (sfp_aug(P->fmt, 0, regs + d.ra * esz, regs + d.rb * esz, r, e, &fl))
                    return 1;
                memcpy(regs + d.rd * esz, d.op == 11 ? e : r, esz);
                if (!qd) {
                    *flags |= fl;
                    *lflag |= (uint8_t)fl;
                }
            }
            pc++;
            break;
        case 12:                                /* QUIET */
            qd++;
            pc++;
            break;
        case 13:                                /* ENDQUIET */
            qd--;
            pc++;
            break;
        case 14:                                /* RAISE */
            if (active) {
                uint32_t low = low_bits(regs + d.ra * esz, esz, 8);
                if (!qd) {
                    *flags |= low & 0x1Fu;
                    *lflag |= (uint8_t)(low & 0x1Fu);
                }
                if ((low >> 7) & 1u) {
                    *status |= 1u << 6;
                    *lflag |= 1u << 7;
                }
            }
            pc++;
            break;
        default:
            return 1;
        }
    }
    return 0;
}

static void load_in(uint8_t *dst, const uint8_t *src, const uint32_t *idx,
                    size_t e, size_t esz)
{
    if (!idx) {
        memcpy(dst, src + e * esz, esz);
        return;
    }
    if (idx[e] == 0xFFFFFFFFu) {
        memset(dst, 0, esz);
        return;
    }
    memcpy(dst, src + (size_t)idx[e] * esz, esz);
}

int sfp_seq_run(const void *image, size_t bytes, sfp_seq_args *A)
{
    const uint8_t *p = (const uint8_t *)image;
    prog_t P;
    uint32_t pc, reach = 0;
    size_t i, kbytes;
    uint8_t *regs, *scratch = NULL;
    int rc = 0;
    static const int widths[4] = { 4, 8, 16, 32 };

    if (!p || bytes < 32 || le32(p) != 0x50544643u)
        return 2;
    memset(&P, 0, sizeof P);
    P.n_insns = le32(p + 8);
    P.n_consts = le32(p + 12);
    P.maxdep = le32(p + 16);
    P.fmt = (int)le32(p + 20);
    P.flags = le32(p + 24);
    if (P.fmt < 0 || P.fmt > 3)
        return 2;
    P.esz = (size_t)widths[P.fmt];
    if (P.flags & 2u) {
        P.n_sin = le32(p + 28) & 0xFFFFu;
        P.n_sout = le32(p + 28) >> 16;
    }
    kbytes = (P.flags & 1u) ? 0 : (size_t)P.n_consts * P.esz;
    if (bytes != 32 + kbytes + (size_t)P.n_insns * 8)
        return 2;
    P.consts = (P.flags & 1u) ? (const uint8_t *)A->bank : p + 32;
    P.insns = (uint64_t *)malloc((P.n_insns ? P.n_insns : 1) * sizeof(uint64_t));
    if (!P.insns)
        return 2;
    for (pc = 0; pc < P.n_insns; pc++)
        P.insns[pc] = (uint64_t)le32(p + 32 + kbytes + pc * 8) |
                      ((uint64_t)le32(p + 32 + kbytes + pc * 8 + 4) << 32);

    /* the scratch footprint (program.c:1102-1135) */
    P.depth = A->depth ? A->depth : 256u;
    while ((1u << P.log2d) < P.depth)
        P.log2d++;
    {
        int indexed = 0, touched = 0;
        for (pc = 0; pc < P.n_insns; pc++) {
            insn_t d;
            decode(P.insns[pc], &d);
            if (!d.ctrl)
                continue;
            if (d.op == 6 || d.op == 7) {
                uint32_t slot = d.imm & 0x00FFFFFFu;
                touched = 1;
                if (slot + 1u > P.used)
                    P.used = slot + 1u;
            } else if (d.op == 8 || d.op == 9) {
                touched = indexed = 1;
            }
        }
        if (indexed)
            P.used = P.depth;
        P.scratch_active = touched || (P.flags & 2u);
    }
    if (P.scratch_active) {
        reach = P.used;
        if (P.n_sin > reach) reach = P.n_sin;
        if (P.n_sout > reach) reach = P.n_sout;
        if (reach > P.depth) reach = P.depth;
        scratch = (uint8_t *)calloc(P.depth, P.esz);
    }
    regs = (uint8_t *)calloc(NREG, P.esz);
    if (!regs || (P.scratch_active && !scratch)) {
        free(regs); free(scratch); free(P.insns);
        return 2;
    }

    A->flags_out = 0;
    A->status_out = 0;
    for (i = 0; i < A->n && !rc; i++) {
        const uint8_t *msk = A->lane_mask;
        int keep = !msk || ((msk[i >> 3] >> (i & 7)) & 1);
        uint32_t count = 0;
        uint8_t lf = 0;
        uint8_t *dep = A->deposits ? (uint8_t *)A->deposits + i * P.maxdep * P.esz
                                   : NULL;
        uint32_t s;
        if (!keep)
            continue;               /* a masked lane writes nothing at all */
        if (dep)
            memset(dep, 0, (size_t)P.maxdep * P.esz);
        memset(regs, 0, NREG * P.esz);
        load_in(regs, (const uint8_t *)A->a, A->idx_a, i, P.esz);
        if (A->b)
            load_in(regs + P.esz, (const uint8_t *)A->b, A->idx_b, i, P.esz);
        if (A->c)
            load_in(regs + 2 * P.esz, (const uint8_t *)A->c, A->idx_c, i, P.esz);
        if (scratch) {
            memset(scratch, 0, (size_t)reach * P.esz);
            for (s = 0; A->scratch_in && s < P.n_sin; s++)
                load_in(scratch + s * P.esz, (const uint8_t *)A->scratch_in,
                        A->idx_scratch_in, i * P.n_sin + s, P.esz);
        }
        rc = run_lane(&P, P.consts, regs, scratch, dep, &count, keep, &lf,
                      &A->flags_out, &A->status_out);
        if (A->counts)
            A->counts[i] = count;
        if (A->lane_flags)
            A->lane_flags[i] = lf;
        if (A->scratch_out && P.n_sout)
            for (s = 0; s < P.n_sout; s++)
                memcpy((uint8_t *)A->scratch_out + (i * P.n_sout + s) * P.esz,
                       scratch + s * P.esz, P.esz);
    }
    free(regs);
    free(scratch);
    free(P.insns);
    return rc;
}
