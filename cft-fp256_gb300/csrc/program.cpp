// program.cpp - the sequencer's host side: the .cftp image loader and
// validator, the run-argument rules, the run driver and the digests.
//
// Accept/refuse behaviour follows the reference's cft_program_load
// (host/src/program.c:1283-1580) rule for rule and in its order, with the
// same status codes; the sentences are this library's own. This device
// publishes every sequencer feature the reference's software backend does,
// augmented addition (control codes 10 and 11) included.
#include <cstring>
#include <new>
#include <vector>

#include "../../include/cft_gb300.h"
#include "api_core.h"
#include "bundle.h"
#include "sha256.h"

using namespace cftg;

namespace {

constexpr uint32_t MAGIC = 0x50544643u;              // "CFTP"
constexpr uint32_t FLAGS_KNOWN = CFT_PROG_FLAG_BANK_EXT | CFT_PROG_FLAG_SCRATCH_IO |
                                 CFT_PROG_FLAG_SCRATCH_STRICT;
constexpr uint32_t MAX_DEPOSITS = 1u << 20;
constexpr uint32_t ADDR_CONSTS = 512u;
constexpr uint64_t MAX_ISSUE = (uint64_t)1 << 40;
constexpr uint64_t COUNT_CAP = (uint64_t)1 << 62;

// control codes (reference seq_exec.h:67-74)
enum { HALT = 0, REPEAT, ENDREP, DEPOSIT, SETACT, ACTALL, STL, LDL, STX, LDX, AUGADD, AUGERR,
       QUIET, ENDQUIET, RAISE, NCTRL };

uint32_t rd32(const uint8_t *p)
{
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

struct Dec {
    int op, rd, ra, rb, rc, rnd, ka, kb, kc, kx, ctrl;
    int hd, ha, hb, hc, k9a, k9b, k9c;
    uint32_t imm;
};

Dec decode(uint64_t w)
{
    Dec d;
    d.op = (int)(w & 0xFF);
    d.rd = (int)((w >> 8) & 0xF);
    d.ra = (int)((w >> 12) & 0xF);
    d.rb = (int)((w >> 16) & 0xF);
    d.rc = (int)((w >> 20) & 0xF);
    d.rnd = (int)((w >> 24) & 7);
    d.ka = (int)((w >> 27) & 1);
    d.kb = (int)((w >> 28) & 1);
    d.kc = (int)((w >> 29) & 1);
    d.kx = (int)((w >> 30) & 1);
    d.ctrl = (int)((w >> 31) & 1);
    d.imm = (uint32_t)(w >> 32);
    d.hd = (int)((d.imm >> 24) & 1);
    d.ha = (int)((d.imm >> 25) & 1);
    d.hb = (int)((d.imm >> 26) & 1);
    d.hc = (int)((d.imm >> 27) & 1);
    d.k9a = (int)((d.imm >> 28) & 1);
    d.k9b = (int)((d.imm >> 29) & 1);
    d.k9c = (int)((d.imm >> 30) & 1);
    return d;
}

int reg(int lo, int hi) { return lo | (hi << 4); }

// which operand fields, and which bits of imm, each control code reads
// (reference program.c:520-560); a set field it does not read is refused
struct CtrlRow { const char *name; unsigned regs; uint32_t imm; };
constexpr unsigned F_RD = 1, F_RA = 2, F_RB = 4;
constexpr uint32_t HI_RD = 1u << 24, HI_RA = 1u << 25, HI_RB = 1u << 26;
constexpr uint32_t SLOT = 0x00FFFFFFu, STEP = 0x00000FFFu;
const CtrlRow CTRL[NCTRL] = {
    {"HALT", 0, 0},
    {"REPEAT", 0, 0xFFFFFFFFu},
    {"ENDREP", 0, 0},
    {"DEPOSIT", F_RA, HI_RA},
    {"SETACT", F_RA, HI_RA},
    {"ACTALL", 0, 0},
    {"STL", F_RA, SLOT | HI_RA},
    {"LDL", F_RD, SLOT | HI_RD},
    {"STX", F_RA | F_RB, HI_RA | HI_RB | STEP},
    {"LDX", F_RD | F_RB, HI_RD | HI_RB | STEP},
    {"AUGADD", F_RD | F_RA | F_RB, HI_RD | HI_RA | HI_RB},
    {"AUGERR", F_RD | F_RA | F_RB, HI_RD | HI_RA | HI_RB},
    {"QUIET", 0, 0},
    {"ENDQUIET", 0, 0},
    {"RAISE", F_RA, HI_RA},
};

}  // namespace

struct cft_program {
    cft_device *dev = nullptr;
    SeqProgram P;
    std::vector<uint64_t> insns;
    std::vector<uint8_t> image;
    std::vector<int32_t> endrep;
    uint64_t *d_insns = nullptr;
    int32_t *d_endrep = nullptr;
    void *d_consts = nullptr;          // the image's constants (not BANK_EXT)
    DevMem bank;                       // a run's bank (BANK_EXT)
    std::mutex sched_mu;               // schedules for G threads a lane, by G
    std::map<int, cftg::DevBundles> sched;
    std::map<int, bool> unschedulable;
};

namespace {

// An ALU instruction's operand rules (reference program.c:223-313).
cft_status check_operands(const Dec &d, uint32_t pc, uint32_t n_consts)
{
    const char *nm = cft_op_name((cft_op)d.op);
    if (d.kx && !(d.ka || d.kb || d.kc)) {
        set_error("instruction %u (%s): kx is set and no operand names a constant", pc, nm);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (d.imm & 0x80000000u) {
        set_error("instruction %u (%s): imm[31] is reserved and set", pc, nm);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (!d.kx && (d.imm & SLOT)) {
        set_error("instruction %u (%s): without kx imm[23:0] must be zero", pc, nm);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (!d.kx && (d.imm & 0x70000000u)) {
        set_error("instruction %u (%s): without kx the ninth index bits imm[30:28] must be zero",
                  pc, nm);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const int kf[3] = {d.ka, d.kb, d.kc}, hi[3] = {d.ha, d.hb, d.hc}, k9[3] = {d.k9a, d.k9b, d.k9c};
    const int rg[3] = {d.ra, d.rb, d.rc};
    for (int w = 0; w < 3; w++)
        if (kf[w] && hi[w]) {
            set_error("instruction %u (%s): operand %c names a constant, so its register high "
                      "bit must be zero",
                      pc, nm, 'a' + w);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    for (int w = 0; w < 3; w++) {
        const uint32_t byte = (d.imm >> (8 * w)) & 0xFFu;
        uint32_t idx;
        if (d.kx && kf[w]) {
            idx = byte | ((uint32_t)k9[w] << 8);
            if (rg[w]) {
                set_error("instruction %u (%s): operand %c names constant %u through imm under kx, "
                          "so its register field must be zero",
                          pc, nm, 'a' + w, idx);
                return CFT_ERR_INVALID_ARGUMENT;
            }
        } else if (d.kx) {
            if (byte) {
                set_error("instruction %u (%s): operand %c names a register under kx, so its byte "
                          "of imm must be zero",
                          pc, nm, 'a' + w);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            if (k9[w]) {
                set_error("instruction %u (%s): operand %c names a register, so its ninth index "
                          "bit must be zero",
                          pc, nm, 'a' + w);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            continue;
        } else if (kf[w]) {
            idx = (uint32_t)rg[w];
        } else {
            continue;
        }
        if (idx >= n_consts) {
            set_error("instruction %u (%s): operand %c names constant %u and the header declares "
                      "%u",
                      pc, nm, 'a' + w, idx, n_consts);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    }
    return CFT_OK;
}

cft_status ctrl_fields(const Dec &d, uint32_t pc)
{
    const CtrlRow &row = CTRL[d.op];
    const int regs[4] = {d.rd, d.ra, d.rb, d.rc};
    static const char *const rn[4] = {"rd", "ra", "rb", "rc"};
    for (int f = 0; f < 4; f++)
        if (regs[f] && !(row.regs & (1u << f))) {
            set_error("instruction %u is %s, which does not read %s; it must be zero", pc,
                      row.name, rn[f]);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    if (d.rnd) {
        set_error("instruction %u is %s, which reads no rounding attribute; rnd must be zero", pc,
                  row.name);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const int fl[4] = {d.ka, d.kb, d.kc, d.kx};
    for (int f = 0; f < 4; f++)
        if (fl[f]) {
            set_error("instruction %u is %s, which reads no constant; ka/kb/kc/kx must be clear",
                      pc, row.name);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    if (d.imm & ~row.imm) {
        set_error("instruction %u is %s, which reads only imm & 0x%08x; imm = 0x%08x", pc,
                  row.name, row.imm, d.imm);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    return CFT_OK;
}

uint64_t cadd(uint64_t a, uint64_t b)
{
    const uint64_t s = a + b;
    return s > COUNT_CAP ? COUNT_CAP : s;
}

uint64_t cmul(uint64_t a, uint64_t b)
{
    if (a && b > COUNT_CAP / a) return COUNT_CAP;
    return a * b;
}

// The instruction stream's rules (reference program.c:601-800), in order.
cft_status validate(const std::vector<uint64_t> &ins, uint32_t n_consts, uint32_t max_scratch)
{
    int depth = 0, qdepth = 0, top = 0, nb = 0;
    uint64_t mult[5] = {1, 0, 0, 0, 0};
    uint64_t worst = 0;
    int bkind[8];
    uint32_t bpc[8];
    const uint32_t n = (uint32_t)ins.size();
    for (uint32_t pc = 0; pc < n; pc++) {
        const Dec d = decode(ins[pc]);
        worst = cadd(worst, mult[top]);
        if (!d.ctrl) {
            cft_status st = check_operands(d, pc, n_consts);
            if (st != CFT_OK) return st;
            if (d.rnd > 4) {
                set_error("instruction %u (%s): rounding attribute %d is reserved", pc,
                          cft_op_name((cft_op)d.op), d.rnd);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            continue;
        }
        if (d.op >= NCTRL) {
            set_error("instruction %u is control code %d; the control codes are 0 to %d", pc,
                      d.op, NCTRL - 1);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        cft_status st = ctrl_fields(d, pc);
        if (st != CFT_OK) return st;
        if ((d.op == STL || d.op == LDL) && max_scratch && (d.imm & SLOT) >= max_scratch) {
            set_error("this program's scratch slot is %u; this device's is %u (scratch slots a "
                      "lane, indexed from 0) - cft_caps.max_scratch",
                      d.imm & SLOT, max_scratch - 1u);
            return CFT_ERR_UNSUPPORTED;
        }
        if (d.op == REPEAT) {
            if (d.imm == 0) {
                set_error("instruction %u is REPEAT 0, which is not a loop", pc);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            if (depth >= 4) {
                set_error("instruction %u is a REPEAT inside %d open loops; loops nest 4 deep", pc,
                          depth);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            depth++;
            top++;
            mult[top] = cmul(mult[top - 1], d.imm);
            bkind[nb] = REPEAT;
            bpc[nb++] = pc;
        } else if (d.op == ENDREP) {
            if (depth == 0) {
                set_error("instruction %u is an ENDREP with no REPEAT open", pc);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            if (bkind[nb - 1] != REPEAT) {
                set_error("instruction %u closes a loop while the quiet region opened at %u is "
                          "open",
                          pc, bpc[nb - 1]);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            nb--;
            depth--;
            top--;
        } else if (d.op == QUIET) {
            if (qdepth >= 4) {
                set_error("instruction %u is a QUIET inside %d open regions; regions nest 4 deep",
                          pc, qdepth);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            qdepth++;
            bkind[nb] = QUIET;
            bpc[nb++] = pc;
        } else if (d.op == ENDQUIET) {
            if (qdepth == 0) {
                set_error("instruction %u is an ENDQUIET with no region open", pc);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            if (bkind[nb - 1] != QUIET) {
                set_error("instruction %u closes a region around the loop opened at %u", pc,
                          bpc[nb - 1]);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            nb--;
            qdepth--;
        } else if ((d.op == ACTALL || d.op == HALT) && depth > 0) {
            set_error("instruction %u is %s inside a loop, which would make the early exit "
                      "observable",
                      pc, CTRL[d.op].name);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        if (d.op == HALT && qdepth > 0) {
            set_error("instruction %u is HALT inside the quiet region opened at %u", pc,
                      bpc[nb - 1]);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        if (worst > MAX_ISSUE) {
            set_error("instruction %u takes the worst-case issue count to %s%llu, past 2^40", pc,
                      worst >= COUNT_CAP ? "at least " : "", (unsigned long long)worst);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    }
    if (depth != 0) {
        set_error("the program ends inside %d open loop(s)", depth);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (qdepth != 0) {
        set_error("the program ends inside %d open quiet region(s)", qdepth);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (worst > MAX_ISSUE) {
        set_error("the program's worst-case issue count is %s%llu, past 2^40",
                  worst >= COUNT_CAP ? "at least " : "", (unsigned long long)worst);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    return CFT_OK;
}

// What only a device can refuse of the instructions (reference
// program.c:925-1080): nothing here - this device publishes every feature
// the software backend does.
cft_status against_device(const std::vector<uint64_t> &)
{
    return CFT_OK;
}

// The whole of cft_program_load's decision over an image, with no device
// state touched. Fills `out` on success.
cft_status check_image(const uint8_t *p, size_t bytes, uint32_t max_scratch, cft_program *out)
{
    if (bytes < 32) {
        set_error("this image is %lu bytes, shorter than the 32-byte header", (unsigned long)bytes);
        return CFT_ERR_ARTIFACT;
    }
    const uint32_t magic = rd32(p), ver = rd32(p + 4), n_insns = rd32(p + 8),
                   n_consts = rd32(p + 12), maxdep = rd32(p + 16), prec = rd32(p + 20),
                   flags = rd32(p + 24), scr_io = rd32(p + 28);
    if (magic != MAGIC) {
        set_error("this image's magic is 0x%08x, not \"CFTP\"", magic);
        return CFT_ERR_ARTIFACT;
    }
    if (ver != 1u) {
        set_error("this image is program-image version %u; this library reads version 1", ver);
        return CFT_ERR_ARTIFACT;
    }
    if (flags & ~FLAGS_KNOWN) {
        set_error("this image's header flags 0x%08x carry bits this library does not know "
                  "(known mask 0x%08x)",
                  flags, FLAGS_KNOWN);
        return CFT_ERR_ARTIFACT;
    }
    if (!(flags & CFT_PROG_FLAG_SCRATCH_IO) && scr_io) {
        set_error("header word 7 (scratch_io) is 0x%08x without SCRATCH_IO; it must be zero",
                  scr_io);
        return CFT_ERR_ARTIFACT;
    }
    if (prec > 3) {
        set_error("this image's precision code is %u; the ladder is 0..3", prec);
        return CFT_ERR_ARTIFACT;
    }
    const size_t esz = esz_of((int)prec);
    const uint32_t n_stored = (flags & CFT_PROG_FLAG_BANK_EXT) ? 0u : n_consts;
    const uint64_t want = 32u + (uint64_t)n_stored * esz + (uint64_t)n_insns * 8u;
    if ((uint64_t)bytes != want) {
        set_error("this image is %llu bytes and its header describes %llu",
                  (unsigned long long)bytes, (unsigned long long)want);
        return CFT_ERR_ARTIFACT;
    }
    if (maxdep > MAX_DEPOSITS) {
        set_error("this program's max_deposits is %u; this device's is %u (deposit slots a lane) "
                  "- cft_caps.max_deposits",
                  maxdep, MAX_DEPOSITS);
        return CFT_ERR_UNSUPPORTED;
    }
    if (n_consts > ADDR_CONSTS) {
        set_error("this image declares %u constants and an instruction addresses at most %u",
                  n_consts, ADDR_CONSTS);
        return CFT_ERR_UNSUPPORTED;
    }
    uint32_t n_sin = 0, n_sout = 0;
    if (flags & CFT_PROG_FLAG_SCRATCH_IO) {
        n_sin = scr_io & 0xFFFFu;
        n_sout = scr_io >> 16;
        if (n_sin > max_scratch || n_sout > max_scratch) {
            set_error("this program's scratch block is %u in / %u out; this device's depth is %u "
                      "(scratch slots a lane) - cft_caps.max_scratch",
                      n_sin, n_sout, max_scratch);
            return CFT_ERR_UNSUPPORTED;
        }
    }
    std::vector<uint64_t> ins(n_insns);
    const size_t kbytes = (size_t)n_stored * esz;
    for (uint32_t i = 0; i < n_insns; i++)
        ins[i] = (uint64_t)rd32(p + 32 + kbytes + 8 * (size_t)i) |
                 ((uint64_t)rd32(p + 32 + kbytes + 8 * (size_t)i + 4) << 32);
    cft_status st = validate(ins, n_consts, max_scratch);
    if (st != CFT_OK) return st;
    st = against_device(ins);
    if (st != CFT_OK) return st;
    if (!out) return CFT_OK;

    // footprint (reference program.c:1102-1135) and the executor's tables
    SeqProgram &P = out->P;
    P.fmt = (int)prec;
    P.n_insns = n_insns;
    P.n_consts = n_consts;
    P.max_deposits = maxdep;
    P.flags = flags;
    P.n_scratch_in = n_sin;
    P.n_scratch_out = n_sout;
    P.scratch_depth = max_scratch;
    P.scratch_log2 = 0;
    while ((1u << P.scratch_log2) < max_scratch) P.scratch_log2++;
    uint32_t used = 0, hireg = 0;
    bool indexed = false, touched = false;
    out->endrep.assign(n_insns, 0);
    std::vector<uint32_t> open;
    for (uint32_t pc = 0; pc < n_insns; pc++) {
        const Dec d = decode(ins[pc]);
        auto seen = [&](int r) { if ((uint32_t)r + 1 > hireg) hireg = (uint32_t)r + 1; };
        if (d.ctrl) {
            if (d.op == STL || d.op == LDL) {
                touched = true;
                if ((d.imm & SLOT) + 1u > used) used = (d.imm & SLOT) + 1u;
            } else if (d.op == STX || d.op == LDX) {
                touched = indexed = true;
            }
            if (d.op == REPEAT) open.push_back(pc);
            if (d.op == ENDREP) {
                out->endrep[open.back()] = (int32_t)pc;
                open.pop_back();
            }
            const unsigned rr = CTRL[d.op].regs;
            if (rr & F_RD) seen(reg(d.rd, d.hd));
            if (rr & F_RA) seen(reg(d.ra, d.ha));
            if (rr & F_RB) seen(reg(d.rb, d.hb));
        } else {
            seen(reg(d.rd, d.hd));
            if (!d.ka) seen(reg(d.ra, d.ha));
            if (!d.kb) seen(reg(d.rb, d.hb));
            if (!d.kc) seen(reg(d.rc, d.hc));
        }
    }
    P.scratch_used = indexed ? max_scratch : used;
    P.scratch_active = (touched || (flags & CFT_PROG_FLAG_SCRATCH_IO)) ? 1 : 0;
    uint32_t reach = 0;
    if (P.scratch_active) {
        reach = P.scratch_used;
        if (n_sin > reach) reach = n_sin;
        if (n_sout > reach) reach = n_sout;
        if (reach > max_scratch) reach = max_scratch;
    }
    P.reach = reach;
    P.nregs = hireg < 3 ? 3 : hireg;
    out->insns = std::move(ins);
    out->image.assign(p, p + bytes);
    return CFT_OK;
}

cft_status bank_rule(const cft_program *pr, const void *bank, size_t bank_bytes, const char *who)
{
    const SeqProgram &P = pr->P;
    if (!(P.flags & CFT_PROG_FLAG_BANK_EXT)) {
        if (bank || bank_bytes) {
            set_error("%s was given a %lu-byte bank and this program carries its own constants",
                      who, (unsigned long)bank_bytes);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        return CFT_OK;
    }
    const size_t want = (size_t)P.n_consts * esz_of(P.fmt);
    if (bank_bytes != want) {
        set_error("%s was given a %lu-byte bank and this program's bank is %lu bytes", who,
                  (unsigned long)bank_bytes, (unsigned long)want);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (want && !bank) {
        set_error("%s: this program's constants arrive with the run and the bank is NULL", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    return CFT_OK;
}

}  // namespace

// The loaded program as the executor reads it, and the handle it was
// loaded on (for entry points outside this file that launch it).
const SeqProgram *cftg::program_seq(const cft_program *pr, cft_device **dev)
{
    if (!pr) return nullptr;
    if (dev) *dev = pr->dev;
    return &pr->P;
}

extern "C" cft_status cftg_program_check(const void *image, size_t bytes, uint32_t max_scratch)
{
    clear_error();
    if (!image) {
        set_error("cftg_program_check: image is NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    return check_image(static_cast<const uint8_t *>(image), bytes, max_scratch ? max_scratch : 256u,
                       nullptr);
}

extern "C" cft_status cft_program_load(cft_device *dev, const void *image, size_t bytes,
                                       cft_program **out)
{
    clear_error();
    if (!dev || !image || !out) {
        set_error("cft_program_load was given a NULL %s", !dev ? "device" : !image ? "image" : "out");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    // a resident buffer holding the image is read from its current bytes
    size_t off = 0;
    cft_buffer *ib = find_buffer(dev, image, bytes, &off);
    if (ib && ib->state == B_DIRTY) {
        cft_status st = cft_buffer_from_device(ib);
        if (st != CFT_OK) return st;
    }
    cft_program *pr = new (std::nothrow) cft_program();
    if (!pr) return CFT_ERR_OUT_OF_MEMORY;
    cft_status st = check_image(static_cast<const uint8_t *>(image), bytes, dev->max_scratch, pr);
    if (st != CFT_OK) {
        delete pr;
        return st;
    }
    pr->dev = dev;
    cudaSetDevice(dev->ordinal);
    const size_t esz = esz_of(pr->P.fmt);
    const size_t ni = pr->insns.size() ? pr->insns.size() : 1;
    bool ok = cudaMalloc(&pr->d_insns, ni * 8) == cudaSuccess &&
              cudaMalloc(&pr->d_endrep, ni * 4) == cudaSuccess;
    if (ok && !pr->insns.empty()) {
        ok = cudaMemcpy(pr->d_insns, pr->insns.data(), pr->insns.size() * 8,
                        cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy(pr->d_endrep, pr->endrep.data(), pr->endrep.size() * 4,
                        cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (ok && !(pr->P.flags & CFT_PROG_FLAG_BANK_EXT) && pr->P.n_consts) {
        ok = cudaMalloc(&pr->d_consts, pr->P.n_consts * esz) == cudaSuccess &&
             cudaMemcpy(pr->d_consts, pr->image.data() + 32, pr->P.n_consts * esz,
                        cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        cft_program_free(pr);
        set_error("cft_program_load: could not place the program on the device");
        return CFT_ERR_OUT_OF_MEMORY;
    }
    pr->P.d_insns = pr->d_insns;
    pr->P.d_endrep = pr->d_endrep;
    pr->P.d_consts = pr->d_consts;
    *out = pr;
    return CFT_OK;
}

cft_status cftg::program_insns(const void *image, size_t bytes, std::vector<uint64_t> &insns,
                               uint32_t *reach)
{
    cft_program tmp;
    cft_status st = check_image(static_cast<const uint8_t *>(image), bytes, 256u, &tmp);
    if (st != CFT_OK) return st;
    insns = tmp.insns;
    *reach = tmp.P.reach;
    return CFT_OK;
}

const DevBundles *cftg::program_bundles(cft_program *pr, int G)
{
    std::lock_guard<std::mutex> g(pr->sched_mu);
    auto it = pr->sched.find(G);
    if (it != pr->sched.end()) return &it->second;
    if (pr->unschedulable.count(G)) return nullptr;
    BundleSchedule s;
    if (!build_bundles(pr->insns, pr->P.reach, G, s) || !s.nb) {
        pr->unschedulable[G] = true;
        return nullptr;
    }
    DevBundles d;
    d.G = G;
    d.nb = s.nb;
    d.nloc = s.nloc;
    d.weighted = s.weighted;
    d.ops_weighted = s.ops_weighted;
    void *o = nullptr, *c = nullptr, *a = nullptr, *m = nullptr;
    cudaSetDevice(pr->dev->ordinal);
    bool ok = cudaMalloc(&o, s.ops.size() * 8) == cudaSuccess && cudaMalloc(&c, s.nb * 4) == cudaSuccess &&
              cudaMalloc(&a, s.nb * 4) == cudaSuccess && cudaMalloc(&m, s.nb * 4) == cudaSuccess &&
              cudaMemcpy(o, s.ops.data(), s.ops.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(c, s.ctl.data(), s.nb * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(a, s.arg.data(), s.nb * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(m, s.match.data(), s.nb * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        for (void *p : {o, c, a, m})
            if (p) cudaFree(p);
        return nullptr;
    }
    d.ops = static_cast<const uint64_t *>(o);
    d.ctl = static_cast<const uint32_t *>(c);
    d.arg = static_cast<const uint32_t *>(a);
    d.match = static_cast<const int32_t *>(m);
    return &(pr->sched[G] = d);
}

extern "C" void cft_program_free(cft_program *pr)
{
    if (!pr) return;
    for (auto &kv : pr->sched)
        for (const void *p : {(const void *)kv.second.ops, (const void *)kv.second.ctl,
                              (const void *)kv.second.arg, (const void *)kv.second.match})
            cudaFree(const_cast<void *>(p));
    if (pr->d_insns) cudaFree(pr->d_insns);
    if (pr->d_endrep) cudaFree(pr->d_endrep);
    if (pr->d_consts) cudaFree(pr->d_consts);
    pr->bank.release();
    delete pr;
}

extern "C" cft_status cft_program_get_info(cft_program *pr, cft_program_info *out)
{
    clear_error();
    if (!pr || !out) return CFT_ERR_INVALID_ARGUMENT;
    cft_program_info i;
    memset(&i, 0, sizeof i);
    i.format = (cft_format)pr->P.fmt;
    i.max_deposits = pr->P.max_deposits;
    i.n_insns = pr->P.n_insns;
    i.n_consts = pr->P.n_consts;
    i.flags = pr->P.flags;
    i.n_scratch_in = pr->P.n_scratch_in;
    i.n_scratch_out = pr->P.n_scratch_out;
    i.scratch_used = pr->P.scratch_used;
    size_t give = out->struct_size;
    if (give > sizeof i) give = sizeof i;
    if (give < sizeof(size_t)) return CFT_ERR_INVALID_ARGUMENT;
    i.struct_size = give;
    memcpy(out, &i, give);
    return CFT_OK;
}

// ---- runs ---------------------------------------------------------------------------------

namespace {

// The run-argument rules (reference program.c:1651-1822, 2050-2260).
cft_status check_run(cft_program *pr, const cft_run_args &A, const char *who)
{
    const SeqProgram &P = pr->P;
    const size_t esz = esz_of(P.fmt);
    if (A.n != 0) {
        if (!A.a) {
            set_error("%s: stream a is NULL - it initialises r0 in every lane", who);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        if (!A.deposits && P.max_deposits) {
            set_error("%s: deposits is NULL for a program with max_deposits = %u", who,
                      P.max_deposits);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        const size_t per = esz * (P.max_deposits ? P.max_deposits : 1u);
        if (A.n > ((size_t)-1) / per) {
            set_error("%s: n = %llu lanes is more than this library can size", who,
                      (unsigned long long)A.n);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    }
    cft_status st = bank_rule(pr, A.bank, A.bank_bytes, who);
    if (st != CFT_OK) return st;
    // the scratch blocks
    struct { const void *buf; size_t bytes; uint32_t slots; const char *name; } side[2] = {
        {A.scratch_in, A.scratch_in_bytes, P.n_scratch_in, "in"},
        {A.scratch_out, A.scratch_out_bytes, P.n_scratch_out, "out"}};
    if (!(P.flags & CFT_PROG_FLAG_SCRATCH_IO)) {
        for (auto &s : side)
            if (s.buf || s.bytes) {
                set_error("%s was given a scratch-%s block and this program declares no scratch "
                          "I/O",
                          who, s.name);
                return CFT_ERR_INVALID_ARGUMENT;
            }
    } else {
        for (int w = 0; w < 2; w++) {
            size_t want = (side[w].slots && A.n) ? A.n * side[w].slots * esz : 0;
            if (w == 0 && A.idx_scratch_in) want = A.idx_scratch_src * esz;
            if (side[w].bytes != want) {
                set_error("%s was given a %lu-byte scratch-%s block and this program's is %lu "
                          "bytes",
                          who, (unsigned long)side[w].bytes, side[w].name, (unsigned long)want);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            if (want && !side[w].buf) {
                set_error("%s: the scratch-%s block is NULL", who, side[w].name);
                return CFT_ERR_INVALID_ARGUMENT;
            }
        }
    }
    // index tables, mask and lane flags
    const uint32_t *idx[3] = {A.idx_a, A.idx_b, A.idx_c};
    const size_t src[3] = {A.idx_a_src, A.idx_b_src, A.idx_c_src};
    const void *strm[3] = {A.a, A.b, A.c};
    for (int r = 0; r < 3; r++) {
        if (!idx[r]) {
            if (src[r]) {
                set_error("%s: idx_%c_src is set with no table", who, 'a' + r);
                return CFT_ERR_INVALID_ARGUMENT;
            }
            continue;
        }
        if (!strm[r]) {
            set_error("%s: idx_%c indexes stream %c, which is NULL", who, 'a' + r, 'a' + r);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        if (!src[r]) {
            set_error("%s: idx_%c is set and idx_%c_src is zero", who, 'a' + r, 'a' + r);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    }
    if (!A.idx_scratch_in && A.idx_scratch_src) {
        set_error("%s: idx_scratch_src is set with no idx_scratch_in", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (A.idx_scratch_in) {
        if (P.n_scratch_in == 0) {
            set_error("%s: idx_scratch_in is set and the program declares no scratch input", who);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        if (!A.scratch_in) {
            set_error("%s: idx_scratch_in indexes scratch_in, which is NULL", who);
            return CFT_ERR_INVALID_ARGUMENT;
        }
        if (!A.idx_scratch_src) {
            set_error("%s: idx_scratch_in is set and idx_scratch_src is zero", who);
            return CFT_ERR_INVALID_ARGUMENT;
        }
    }
    if (!A.lane_mask && A.lane_mask_bytes) {
        set_error("%s: lane_mask_bytes = %lu with no lane_mask", who,
                  (unsigned long)A.lane_mask_bytes);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (A.lane_mask && A.lane_mask_bytes != (A.n + 7) / 8) {
        set_error("%s: lane_mask_bytes is %lu and a mask over %lu lanes is %lu bytes", who,
                  (unsigned long)A.lane_mask_bytes, (unsigned long)A.n,
                  (unsigned long)((A.n + 7) / 8));
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (!A.lane_flags && A.lane_flags_bytes) {
        set_error("%s: lane_flags_bytes = %lu with no lane_flags", who,
                  (unsigned long)A.lane_flags_bytes);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (A.lane_flags && A.lane_flags_bytes != A.n) {
        set_error("%s: lane_flags_bytes is %lu and %lu lanes take %lu bytes", who,
                  (unsigned long)A.lane_flags_bytes, (unsigned long)A.n, (unsigned long)A.n);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    for (int r = 0; r < 3; r++) {
        if (!idx[r]) continue;
        for (size_t i = 0; i < A.n; i++)
            if (idx[r][i] != CFT_IDX_NONE && (size_t)idx[r][i] >= src[r]) {
                set_error("%s: idx_%c[%lu] = %u is at or past the %lu elements of stream %c", who,
                          'a' + r, (unsigned long)i, idx[r][i], (unsigned long)src[r], 'a' + r);
                return CFT_ERR_INVALID_ARGUMENT;
            }
    }
    if (A.idx_scratch_in) {
        const size_t entries = A.n * (size_t)P.n_scratch_in;
        for (size_t e = 0; e < entries; e++)
            if (A.idx_scratch_in[e] != CFT_IDX_NONE &&
                (size_t)A.idx_scratch_in[e] >= A.idx_scratch_src) {
                set_error("%s: idx_scratch_in[%lu] = %u is at or past the %lu elements of the pool",
                          who, (unsigned long)e, A.idx_scratch_in[e],
                          (unsigned long)A.idx_scratch_src);
                return CFT_ERR_INVALID_ARGUMENT;
            }
    }
    return CFT_OK;
}

// A caller's buffer on the device for the run: a resident buffer's copy
// (made current) or a staging allocation, uploaded when `upload`.
struct Bound {
    void *dptr = nullptr;
    cft_buffer *buf = nullptr;
    DevMem own;
    ~Bound() { own.release(); }
};

cft_status bind(cft_device *dev, const void *host, size_t bytes, bool upload, Bound &b,
                cudaStream_t s, const char *who)
{
    if (!host || !bytes) return CFT_OK;
    size_t off = 0;
    b.buf = find_buffer(dev, host, bytes, &off);
    if (b.buf) {
        if (b.buf->state == B_LOST) {
            set_error("%s: a resident buffer of this run is LOST; publish it first", who);
            return CFT_ERR_INTERNAL;
        }
        if (b.buf->state == B_STALE) {
            cudaError_t e = cudaMemcpyAsync(b.buf->dptr, b.buf->host, b.buf->bytes,
                                            cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) return poison(dev, who, e);
            b.buf->state = B_FRESH;
            b.buf->staged_binds++;
        } else {
            b.buf->resident_binds++;
        }
        b.dptr = (uint8_t *)b.buf->dptr + off;
        return CFT_OK;
    }
    if (b.own.ensure(bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("%s: could not allocate %lu bytes of device memory", who, (unsigned long)bytes);
        return CFT_ERR_OUT_OF_MEMORY;
    }
    b.dptr = b.own.p;
    if (upload) {
        cudaError_t e = cudaMemcpyAsync(b.dptr, host, bytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return poison(dev, who, e);
    }
    return CFT_OK;
}

cft_status run_program(cft_program *pr, const cft_run_args &A, const char *who)
{
    cft_device *dev = pr->dev;
    SeqProgram P = pr->P;
    const size_t n = A.n, esz = esz_of(P.fmt);
    cudaSetDevice(dev->ordinal);
    cudaStream_t s = dev->s[0];
    const bool masked = A.lane_mask != nullptr;
    Bound ba, bb, bc, bia, bib, bic, bsi, bisi, bso, bdep, bcnt, bmask, blf;
    cft_status st;
    const size_t na = A.idx_a ? A.idx_a_src : n, nb = A.idx_b ? A.idx_b_src : n,
                 nc = A.idx_c ? A.idx_c_src : n;
    if ((st = bind(dev, A.a, na * esz, true, ba, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.b, nb * esz, true, bb, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.c, nc * esz, true, bc, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.idx_a, n * 4, true, bia, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.idx_b, n * 4, true, bib, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.idx_c, n * 4, true, bic, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.scratch_in, A.scratch_in_bytes, true, bsi, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.idx_scratch_in, A.idx_scratch_in ? n * P.n_scratch_in * 4 : 0, true,
                   bisi, s, who)) != CFT_OK)
        return st;
    if ((st = bind(dev, A.lane_mask, A.lane_mask_bytes, true, bmask, s, who)) != CFT_OK) return st;
    // outputs: with a mask, masked lanes keep the caller's bytes, so the
    // caller's buffer is the starting point
    const size_t dep_bytes = n * (size_t)P.max_deposits * esz;
    if ((st = bind(dev, A.deposits, dep_bytes, masked, bdep, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.counts, A.counts ? n * 4 : 0, masked, bcnt, s, who)) != CFT_OK) return st;
    if ((st = bind(dev, A.scratch_out, A.scratch_out_bytes, masked, bso, s, who)) != CFT_OK)
        return st;
    if ((st = bind(dev, A.lane_flags, A.lane_flags_bytes, masked, blf, s, who)) != CFT_OK) return st;
    if (bdep.dptr && !masked) {
        cudaError_t e = cudaMemsetAsync(bdep.dptr, 0, dep_bytes, s);
        if (e != cudaSuccess) return poison(dev, who, e);
    }
    // the constant bank of a BANK_EXT program
    if (P.flags & CFT_PROG_FLAG_BANK_EXT) {
        const size_t kb = (size_t)P.n_consts * esz;
        if (kb) {
            if (pr->bank.ensure(kb) != cudaSuccess) {
                cudaGetLastError();
                return CFT_ERR_OUT_OF_MEMORY;
            }
            size_t off = 0;
            cft_buffer *kbuf = find_buffer(dev, A.bank, kb, &off);
            if (kbuf && kbuf->state == B_DIRTY) {
                cudaError_t e = cudaMemcpyAsync(pr->bank.p, (uint8_t *)kbuf->dptr + off, kb,
                                                cudaMemcpyDeviceToDevice, s);
                if (e != cudaSuccess) return poison(dev, who, e);
            } else {
                cudaError_t e = cudaMemcpyAsync(pr->bank.p, A.bank, kb, cudaMemcpyHostToDevice, s);
                if (e != cudaSuccess) return poison(dev, who, e);
            }
            P.d_consts = pr->bank.p;
        }
    }
    // scratch for the lanes: reach slots each
    DevMem scratch;
    if (P.reach) {
        if (scratch.ensure(n * (size_t)P.reach * esz) != cudaSuccess) {
            cudaGetLastError();
            set_error("%s: could not allocate %lu bytes of lane scratch", who,
                      (unsigned long)(n * (size_t)P.reach * esz));
            return CFT_ERR_OUT_OF_MEMORY;
        }
    }
    cudaMemsetAsync(dev->d_word, 0, 3 * sizeof(uint32_t), s);
    SeqLaunch L;
    L.P = P;
    L.n = n;
    L.a = ba.dptr;
    L.b = bb.dptr;
    L.c = bc.dptr;
    L.ia = (const uint32_t *)bia.dptr;
    L.ib = (const uint32_t *)bib.dptr;
    L.ic = (const uint32_t *)bic.dptr;
    L.isi = (const uint32_t *)bisi.dptr;
    L.scratch_in = bsi.dptr;
    L.scratch_out = bso.dptr;
    L.deposits = bdep.dptr;
    L.counts = (uint32_t *)bcnt.dptr;
    L.lane_mask = (const uint8_t *)bmask.dptr;
    L.lane_flags = (uint8_t *)blf.dptr;
    L.scratch = scratch.p;
    L.word = dev->d_word;
    cudaError_t e = launch_seq(L, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dev->h_word, dev->d_word, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    // outputs home (non-resident ones)
    struct { Bound *b; void *host; size_t bytes; } outs[4] = {
        {&bdep, A.deposits, dep_bytes}, {&bcnt, A.counts, A.counts ? n * 4 : 0},
        {&bso, A.scratch_out, A.scratch_out_bytes}, {&blf, A.lane_flags, A.lane_flags_bytes}};
    for (auto &o : outs) {
        if (e != cudaSuccess) break;
        if (!o.host || !o.bytes || o.b->buf) continue;
        e = cudaMemcpyAsync(o.host, o.b->dptr, o.bytes, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    scratch.release();
    if (e != cudaSuccess) {
        for (auto &o : outs)
            if (o.b->buf) o.b->buf->state = B_LOST;
        return poison(dev, who, e);
    }
    for (auto &o : outs)
        if (o.b->buf) o.b->buf->state = B_DIRTY;
    if (dev->h_word[2]) {
        set_error("%s: the GPU executor reported invariant failure 0x%x - a defect in this "
                  "library, not in the call",
                  who, dev->h_word[2]);
        return CFT_ERR_INTERNAL;
    }
    flags_emit(dev, dev->h_word[0] & CFT_FLAGS_ALL, A.flags_out);
    if (A.bus_out) *A.bus_out = dev->h_word[1];
    return CFT_OK;
}

}  // namespace

extern "C" cft_status cft_program_run_ex(cft_program *pr, const cft_run_args *args)
{
    clear_error();
    if (!pr || !args) {
        set_error("cft_program_run_ex: %s is NULL", pr ? "args" : "prog");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (args->struct_size != sizeof(cft_run_args)) {
        set_error("cft_program_run_ex was given a %lu-byte cft_run_args and this library's is %lu "
                  "bytes",
                  (unsigned long)args->struct_size, (unsigned long)sizeof(cft_run_args));
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cft_run_args A = *args;
    if (A.bus_out) *A.bus_out = 0;
    cft_status st = check_run(pr, A, "cft_program_run_ex");
    if (st != CFT_OK) return st;
    if (pr->dev->poisoned) {
        set_error("cft_program_run_ex: this handle failed earlier; close it and open it again");
        return CFT_ERR_INTERNAL;
    }
    if (A.n == 0) {
        flags_emit(pr->dev, 0, A.flags_out);
        return CFT_OK;
    }
    if (!A.bank_bytes) A.bank = nullptr;
    return run_program(pr, A, "cft_program_run_ex");
}

static void args_init(cft_run_args *A, const void *a, const void *b, const void *c, void *dep,
                      uint32_t *counts, size_t n, uint32_t *flags, uint32_t *bus)
{
    memset(A, 0, sizeof *A);
    A->struct_size = sizeof *A;
    A->a = a;
    A->b = b;
    A->c = c;
    A->n = n;
    A->deposits = dep;
    A->counts = counts;
    A->flags_out = flags;
    A->bus_out = bus;
}

extern "C" cft_status cft_program_run(cft_program *pr, const void *a, const void *b, const void *c,
                                      void *deposits, uint32_t *counts, size_t n, uint32_t *flags,
                                      uint32_t *bus)
{
    clear_error();
    if (bus) *bus = 0;
    if (!pr) return CFT_ERR_INVALID_ARGUMENT;
    if (pr->P.flags & CFT_PROG_FLAG_BANK_EXT) {
        set_error("this program's constants arrive with each run (BANK_EXT); call "
                  "cft_program_run_bank");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    if (pr->P.flags & CFT_PROG_FLAG_SCRATCH_IO) {
        set_error("this program declares scratch I/O; call cft_program_run_ex");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cft_run_args A;
    args_init(&A, a, b, c, deposits, counts, n, flags, bus);
    return cft_program_run_ex(pr, &A);
}

extern "C" cft_status cft_program_run_bank(cft_program *pr, const void *bank, size_t bank_bytes,
                                           const void *a, const void *b, const void *c,
                                           void *deposits, uint32_t *counts, size_t n,
                                           uint32_t *flags_out, uint32_t *bus_out)
{
    clear_error();
    if (bus_out) *bus_out = 0;
    if (!pr) return CFT_ERR_INVALID_ARGUMENT;
    cft_status st = bank_rule(pr, bank, bank_bytes, "cft_program_run_bank");
    if (st != CFT_OK) return st;
    if (pr->P.flags & CFT_PROG_FLAG_SCRATCH_IO) {
        set_error("this program declares scratch I/O; call cft_program_run_ex");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    cft_run_args A;
    args_init(&A, a, b, c, deposits, counts, n, flags_out, bus_out);
    A.bank = bank;
    A.bank_bytes = bank_bytes;
    return cft_program_run_ex(pr, &A);
}

extern "C" cft_status cft_program_digest(cft_program *pr, const void *bank, size_t bank_bytes,
                                         uint8_t out[32])
{
    clear_error();
    if (!pr || !out) return CFT_ERR_INVALID_ARGUMENT;
    cft_status st = bank_rule(pr, bank, bank_bytes, "cft_program_digest");
    if (st != CFT_OK) return st;
    Sha256 h;
    h.init();
    h.update(pr->image.data(), pr->image.size());
    if (bank_bytes) h.update(bank, bank_bytes);
    h.final(out);
    return CFT_OK;
}

extern "C" cft_status cft_sha256(const void *data, size_t bytes, uint8_t out[32])
{
    clear_error();
    if (!out || (!data && bytes)) return CFT_ERR_INVALID_ARGUMENT;
    Sha256 h;
    h.init();
    if (bytes) h.update(data, bytes);
    h.final(out);
    return CFT_OK;
}
