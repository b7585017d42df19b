// asm.cpp - the `.cfta` text form: assembler, disassembler and header
// report, and the ODE banks, as C++ behind the C ABI (cftg_asm_*,
// cftg_ode_bank, cftg_program_load_source in include/cft_gb300.h), so that
// a serving client can submit program SOURCE.
//
// The text form and the image are the reference's (docs/PROGRAMS.md,
// docs/SEQUENCER.md); python/cft_golden/asm.py defines both and
// host/tools/cft-asm.c is its C tool. Output here is held byte for byte to
// asm.py: the same image for every source it assembles, a refusal for every
// source it refuses, the same disassembly and the same `-i` report.
//
//  * characters (asm.py:950-1060): UTF-8; a line ends at LF (a CR just
//    before it belongs to the end); the other line breaks, NUL and Ctrl-Z
//    are refused anywhere; before a line's first `;` only printable ASCII,
//    spaces and tabs;
//  * a line is split at runs of white space and commas; `;` starts a
//    comment; names are case-insensitive; numbers read as Python's int()
//    reads them (decimal with one sign and at most 4,300 digits, or 0x hex,
//    single underscores between digits);
//  * directives .format .deposits .bank .const .reg .slot .scratch
//    (asm.py:1190-1440); ALU lines name the operand fields the opcode reads
//    or all three; control lines the fifteen control codes
//    (asm.py:1442-1580);
//  * the image is validated with the loader's rules before it is written
//    (asm.py:620-850): reserved fields, constant indices, loop and quiet
//    nesting, the 2^40 worst-case instruction bound, static slots inside
//    the declared depth.
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "api_core.h"
#include "chars.h"
#include "sha256.h"

namespace cftg {
namespace asmb {

// ---- the image --------------------------------------------------------------

enum : uint32_t { MAGIC = 0x50544643u, VERSION = 1u, HEADER_BYTES = 32u };
enum : uint32_t { F_BANK_EXT = 1u, F_SCRATCH_IO = 2u, F_SCRATCH_STRICT = 4u, F_KNOWN = 7u };
enum { NREG = 32, REG_FIELD = 16, KADDR_PLAIN = 16, KADDR_KX = 512, MAX_LOOP = 4, MAX_QUIET = 4 };
static const int64_t MAX_WORST = (int64_t)1 << 40;
static const int64_t MAX_DEPOSITS = (int64_t)1 << 20;
static const int64_t SCRATCH_D_DEFAULT = 256, SCRATCH_D_MAX = (int64_t)1 << 24;
static const uint32_t SLOT_MASK = 0x00FFFFFFu, SCRATCH_IO_MAX = 0xFFFFu, IMM_RESERVED = 0x80000000u;
static const uint32_t STEP_MASK = 0xFFFu;

enum Ctrl {
    C_HALT = 0, C_REPEAT, C_ENDREP, C_DEPOSIT, C_SETACT, C_ACTALL, C_STL, C_LDL, C_STX, C_LDX,
    C_AUGADD, C_AUGERR, C_QUIET, C_ENDQUIET, C_RAISE, C_COUNT
};
static const char *const CTRL_NAME[C_COUNT] = {"halt", "repeat", "endrep", "deposit", "setact",
                                               "actall", "stl", "ldl", "stx", "ldx", "augadd",
                                               "augerr", "quiet", "endquiet", "raise"};
// Register fields each control code reads (bit 0 rd, 1 ra, 2 rb, 3 rc) and
// whether imm[23:0] is a scratch slot; everything else must be zero.
static const uint8_t CTRL_REGS[C_COUNT] = {0, 0, 0, 2, 2, 0, 2, 1, 6, 5, 7, 7, 0, 0, 2};
static const bool CTRL_SLOT[C_COUNT] = {false, false, false, false, false, false, true, true,
                                        false, false, false, false, false, false, false};

// Operand fields each ALU opcode reads (bit 0 ra, 1 rb, 2 rc); 0 for an
// opcode the sequencer's ALU does not name (reductions, unassigned codes).
static uint8_t alu_fields(int op)
{
    switch (op) {
    case 0: case 11: return 7;                 // fma, select
    case 1: case 2: return 5;                  // add, sub read a and c
    case 4: case 5: case 26: case 27: return 1;
    case 3: case 6: case 7: case 8: case 9: case 10: case 12: case 13: case 14:
    case 16: case 17: case 18: case 19: case 20: case 21: case 22: case 23: case 30: return 3;
    default: return 0;
    }
}

static const char *const RND_NAME[5] = {"rne", "rtz", "rdn", "rup", "rmm"};
static const char *const FMT_NAME[4] = {"fp32", "fp64", "fp128", "fp256"};

struct Image {
    int fmt = -1;
    std::vector<uint64_t> insns;
    std::vector<chars::Enc> consts;             // n_consts entries; placeholders under BANK_EXT
    int64_t max_deposits = 0;
    uint32_t flags = 0;
    int64_t scratch_depth = SCRATCH_D_DEFAULT;
    uint32_t scratch_io = 0;
};

struct D {                                      // a decoded instruction word
    int op, rnd;
    bool ka, kb, kc, kx, ctrl;
    uint32_t imm;
    int lo[4], hi[4];                           // rd, ra, rb, rc
    int reg(int f) const { return lo[f] | (hi[f] << 4); }
};

static D decode(uint64_t w)
{
    D d;
    d.imm = (uint32_t)(w >> 32);
    d.op = (int)(w & 0xFF);
    d.rnd = (int)((w >> 24) & 7);
    d.ka = (w >> 27) & 1;
    d.kb = (w >> 28) & 1;
    d.kc = (w >> 29) & 1;
    d.kx = (w >> 30) & 1;
    d.ctrl = (w >> 31) & 1;
    for (int f = 0; f < 4; f++) {
        d.lo[f] = (int)((w >> (8 + 4 * f)) & 0xF);
        d.hi[f] = (int)((d.imm >> (24 + f)) & 1);
    }
    return d;
}

// The three sources of an ALU word as (index, is_const), a/b/c order.
static void sources(const D &d, int idx[3], bool isk[3])
{
    const bool k[3] = {d.ka, d.kb, d.kc};
    for (int s = 0; s < 3; s++) {
        isk[s] = k[s];
        if (k[s]) {
            idx[s] = d.kx ? (int)(((d.imm >> (8 * s)) & 0xFF) | (((d.imm >> (28 + s)) & 1) << 8))
                          : d.lo[1 + s];
        } else {
            idx[s] = d.reg(1 + s);
        }
    }
}

static int step_of(const D &d)
{
    if (!d.ctrl || (d.op != C_STX && d.op != C_LDX)) return 0;
    const int s = (int)(d.imm & STEP_MASK);
    return (s & 0x800) ? s - 4096 : s;
}

static std::string strf(const char *fmt, ...) __attribute__((format(printf, 1, 2)));
static std::string strf(const char *fmt, ...)
{
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    return b;
}

static bool check_alu(const Image &im, size_t pc, const D &d, std::string *why)
{
    if (d.rnd > 4) return *why = strf("[%zu] rnd=%d is reserved", pc, d.rnd), false;
    if (d.imm & IMM_RESERVED) return *why = strf("[%zu] imm[31] is reserved and must be zero", pc), false;
    if (d.kx && !(d.ka || d.kb || d.kc))
        return *why = strf("[%zu] kx is set and no operand names a constant", pc), false;
    const bool k[3] = {d.ka, d.kb, d.kc};
    static const char *const key[3] = {"ra", "rb", "rc"};
    for (int s = 0; s < 3; s++) {
        const uint32_t byte = (d.imm >> (8 * s)) & 0xFF, ninth = (d.imm >> (28 + s)) & 1;
        if (ninth && !(d.kx && k[s]))
            return *why = strf("[%zu] imm[%d] (the ninth bit of %s's constant index) is not read "
                               "and must be zero", pc, 28 + s, key[s]), false;
        if (!k[s]) {
            if (d.kx && byte)
                return *why = strf("[%zu] %s names a register, so its byte of imm must be zero", pc,
                                   key[s]), false;
            continue;
        }
        if (d.hi[1 + s])
            return *why = strf("[%zu] %s names a constant, so its register high bit must be zero",
                               pc, key[s]), false;
        uint32_t idx;
        if (d.kx) {
            if (d.lo[1 + s])
                return *why = strf("[%zu] %s names a constant through imm under kx, so the %s field "
                                   "must be zero", pc, key[s], key[s]), false;
            idx = byte | (ninth << 8);
        } else {
            idx = (uint32_t)d.lo[1 + s];
        }
        if (idx >= im.consts.size())
            return *why = strf("[%zu] %s names constant %u but the bank holds %zu", pc, key[s], idx,
                               im.consts.size()), false;
    }
    if (!d.kx && (d.imm & 0x00FFFFFFu))
        return *why = strf("[%zu] an ALU instruction without kx has no immediate below imm[24]",
                           pc), false;
    return true;
}

static bool check_ctrl(const Image &im, size_t pc, const D &d, std::string *why)
{
    if (d.op >= C_COUNT) return *why = strf("[%zu] unknown control code %d", pc, d.op), false;
    const char *name = CTRL_NAME[d.op];
    const uint8_t regs = CTRL_REGS[d.op];
    static const char *const fld[4] = {"rd", "ra", "rb", "rc"};
    for (int f = 0; f < 4; f++)
        if (!(regs >> f & 1) && d.lo[f])
            return *why = strf("[%zu] %s does not read %s, so it must be zero", pc, name, fld[f]), false;
    if (d.rnd || d.ka || d.kb || d.kc || d.kx)
        return *why = strf("[%zu] %s reads no rounding attribute and no constant flag", pc, name), false;
    if (d.op != C_REPEAT) {
        uint32_t allowed = CTRL_SLOT[d.op] ? SLOT_MASK : 0u;
        if (d.op == C_STX || d.op == C_LDX) allowed |= STEP_MASK;
        for (int f = 0; f < 4; f++)
            if (regs >> f & 1) allowed |= 1u << (24 + f);
        if (d.imm & ~allowed)
            return *why = strf("[%zu] %s does not read imm beyond its operands, and imm is 0x%08x",
                               pc, name, d.imm), false;
    }
    if (CTRL_SLOT[d.op] && (int64_t)(d.imm & SLOT_MASK) >= im.scratch_depth)
        return *why = strf("[%zu] %s names scratch slot %u and the program declares a scratch of "
                           "%lld slots (.scratch N)", pc, name, d.imm & SLOT_MASK,
                           (long long)im.scratch_depth), false;
    return true;
}

static bool validate(const Image &im, std::string *why)
{
    if (im.max_deposits < 0 || im.max_deposits > MAX_DEPOSITS)
        return *why = strf("max_deposits=%lld, cap %lld", (long long)im.max_deposits,
                           (long long)MAX_DEPOSITS), false;
    if (im.flags & ~F_KNOWN)
        return *why = strf("header flags 0x%08x: only BANK_EXT, SCRATCH_IO and SCRATCH_STRICT are "
                           "defined", im.flags), false;
    if (im.consts.size() > (size_t)KADDR_KX)
        return *why = strf("%zu constants; the bank addresses at most %d", im.consts.size(),
                           KADDR_KX), false;
    const int64_t sd = im.scratch_depth;
    if (sd < 1 || sd > SCRATCH_D_MAX || (sd & (sd - 1)))
        return *why = strf("a scratch depth is a power of two in 1..%lld", (long long)SCRATCH_D_MAX),
               false;
    if (!(im.flags & F_SCRATCH_IO) && im.scratch_io)
        return *why = strf("header word 7 is 0x%08x with SCRATCH_IO clear", im.scratch_io), false;
    if ((int64_t)(im.scratch_io & 0xFFFF) > sd || (int64_t)(im.scratch_io >> 16) > sd)
        return *why = strf(".scratch in/out is more than the %lld slots the program declares",
                           (long long)sd), false;
    int depth = 0, qdepth = 0;
    std::vector<std::pair<int, size_t>> brackets;       // (code, pc)
    std::vector<int64_t> mult{1};
    int64_t worst = 0;
    const int64_t CAP = (int64_t)1 << 62;
    for (size_t pc = 0; pc < im.insns.size(); pc++) {
        const D d = decode(im.insns[pc]);
        worst = (int64_t)std::min<__int128>(CAP, (__int128)worst + mult.back());
        if (!d.ctrl) {
            if (!check_alu(im, pc, d, why)) return false;
            continue;
        }
        if (!check_ctrl(im, pc, d, why)) return false;
        switch (d.op) {
        case C_REPEAT:
            if (d.imm == 0) return *why = strf("[%zu] repeat 0 is not a loop; omit it", pc), false;
            if (++depth > MAX_LOOP) return *why = strf("[%zu] loops nest deeper than %d", pc, MAX_LOOP), false;
            {
                const __int128 m = (__int128)mult.back() * d.imm;
                mult.push_back(m > CAP ? CAP : (int64_t)m);
            }
            brackets.push_back({C_REPEAT, pc});
            break;
        case C_ENDREP:
            if (--depth < 0) return *why = strf("[%zu] endrep without repeat", pc), false;
            if (brackets.back().first != C_REPEAT)
                return *why = strf("[%zu] endrep closes its loop while the quiet region opened at "
                                   "[%zu] is open", pc, brackets.back().second), false;
            brackets.pop_back();
            mult.pop_back();
            break;
        case C_QUIET:
            if (++qdepth > MAX_QUIET)
                return *why = strf("[%zu] quiet regions nest deeper than %d", pc, MAX_QUIET), false;
            brackets.push_back({C_QUIET, pc});
            break;
        case C_ENDQUIET:
            if (qdepth == 0) return *why = strf("[%zu] endquiet with no quiet region open", pc), false;
            if (brackets.back().first != C_QUIET)
                return *why = strf("[%zu] endquiet inside the loop opened at [%zu], around a region "
                                   "opened outside it", pc, brackets.back().second), false;
            qdepth--;
            brackets.pop_back();
            break;
        case C_ACTALL:
            if (depth > 0) return *why = strf("[%zu] actall inside a loop", pc), false;
            break;
        case C_HALT:
            if (depth > 0) return *why = strf("[%zu] halt inside a loop", pc), false;
            break;
        default: break;
        }
        if (d.op == C_HALT && qdepth)
            return *why = strf("[%zu] halt inside the quiet region opened at [%zu]", pc,
                               brackets.back().second), false;
        if (worst > MAX_WORST)
            return *why = strf("[%zu] worst-case instruction count exceeds 2^40", pc), false;
    }
    if (depth) return *why = strf("%d loop(s) left open at the end", depth), false;
    if (qdepth)
        return *why = strf("%d quiet region(s) left open at the end, the innermost opened at [%zu]",
                           qdepth, brackets.back().second), false;
    if (worst > MAX_WORST) return *why = "worst-case instruction count exceeds 2^40", false;
    return true;
}

static size_t esz(int fmt) { return (size_t)4 << fmt; }

static void put32(std::vector<uint8_t> &o, uint32_t v)
{
    for (int i = 0; i < 4; i++) o.push_back((uint8_t)(v >> (8 * i)));
}

static std::vector<uint8_t> to_bytes(const Image &im)
{
    std::vector<uint8_t> o;
    put32(o, MAGIC);
    put32(o, VERSION);
    put32(o, (uint32_t)im.insns.size());
    put32(o, (uint32_t)im.consts.size());
    put32(o, (uint32_t)im.max_deposits);
    put32(o, (uint32_t)im.fmt);
    put32(o, im.flags);
    put32(o, im.scratch_io);
    if (!(im.flags & F_BANK_EXT))
        for (const auto &k : im.consts) {
            const uint8_t *b = reinterpret_cast<const uint8_t *>(k.w);
            o.insert(o.end(), b, b + esz(im.fmt));
        }
    for (uint64_t w : im.insns)
        for (int i = 0; i < 8; i++) o.push_back((uint8_t)(w >> (8 * i)));
    return o;
}

static uint32_t rd32(const uint8_t *p) { return p[0] | p[1] << 8 | p[2] << 16 | (uint32_t)p[3] << 24; }

// The depth a readback assumes: the smallest power of two, at least 256,
// covering every static slot and both scratch-I/O counts (asm.py:466-490).
static int64_t infer_depth(const Image &im)
{
    int64_t need = 1;
    for (uint64_t w : im.insns) {
        const D d = decode(w);
        if (d.ctrl && (d.op == C_STL || d.op == C_LDL)) need = std::max<int64_t>(need, (d.imm & SLOT_MASK) + 1);
    }
    if (im.flags & F_SCRATCH_IO)
        need = std::max<int64_t>(need, std::max(im.scratch_io & 0xFFFF, im.scratch_io >> 16));
    int64_t depth = SCRATCH_D_DEFAULT;
    while (depth < need) depth *= 2;
    return depth;
}

static bool from_bytes(const uint8_t *p, size_t n, Image *im, std::string *why)
{
    if (n < HEADER_BYTES) return *why = "shorter than a header", false;
    const uint32_t magic = rd32(p), ver = rd32(p + 4), n_insns = rd32(p + 8), n_consts = rd32(p + 12),
                   maxdep = rd32(p + 16), prec = rd32(p + 20), flags = rd32(p + 24),
                   sio = rd32(p + 28);
    if (magic != MAGIC) return *why = strf("bad magic 0x%08x, expected 0x%08x", magic, MAGIC), false;
    if (ver != VERSION) return *why = strf("program version %u, this loader speaks %u", ver, VERSION), false;
    if (flags & ~F_KNOWN) return *why = strf("header flags 0x%08x carry reserved bits", flags), false;
    if (!(flags & F_SCRATCH_IO) && sio)
        return *why = "reserved header word 7 must be zero unless flags.SCRATCH_IO says it is scratch_io", false;
    if (prec > 3) return *why = strf("precision code %u is not on the ladder", prec), false;
    const size_t carried = (flags & F_BANK_EXT) ? 0 : n_consts;
    const uint64_t want = HEADER_BYTES + (uint64_t)carried * esz((int)prec) + (uint64_t)n_insns * 8;
    if ((uint64_t)n != want)
        return *why = strf("%zu bytes, header describes %llu", n, (unsigned long long)want), false;
    im->fmt = (int)prec;
    im->max_deposits = maxdep;
    im->flags = flags;
    im->scratch_io = sio;
    im->consts.assign(n_consts, chars::Enc());
    size_t off = HEADER_BYTES;
    for (size_t i = 0; i < carried; i++, off += esz((int)prec))
        memcpy(im->consts[i].w, p + off, esz((int)prec));
    im->insns.resize(n_insns);
    for (size_t i = 0; i < n_insns; i++, off += 8) {
        uint64_t w = 0;
        for (int b = 0; b < 8; b++) w |= (uint64_t)p[off + b] << (8 * b);
        im->insns[i] = w;
    }
    im->scratch_depth = infer_depth(*im);
    return validate(*im, why);
}

// ---- the text form's characters ---------------------------------------------

static const char *line_break_name(uint32_t cp)
{
    switch (cp) {
    case 0x0d: return "a carriage return (0x0d) that is not part of a CRLF line end";
    case 0x0b: return "a vertical tab (0x0b)";
    case 0x0c: return "a form feed (0x0c)";
    case 0x1c: return "a file separator (0x1c)";
    case 0x1d: return "a group separator (0x1d)";
    case 0x1e: return "a record separator (0x1e)";
    case 0x85: return "a next line (U+0085)";
    case 0x2028: return "a line separator (U+2028)";
    case 0x2029: return "a paragraph separator (U+2029)";
    default: return nullptr;
    }
}

// Strict UTF-8 (no overlong forms, no surrogates, at most U+10FFFF): the
// code points, or false with the offset of the first bad byte.
static bool utf8_decode(const std::string &s, std::vector<uint32_t> *cps, size_t *bad)
{
    size_t i = 0;
    while (i < s.size()) {
        const uint8_t c = (uint8_t)s[i];
        uint32_t cp;
        int len;
        if (c < 0x80) { cp = c; len = 1; }
        else if (c >= 0xC2 && c <= 0xDF) { cp = c & 0x1F; len = 2; }
        else if (c >= 0xE0 && c <= 0xEF) { cp = c & 0x0F; len = 3; }
        else if (c >= 0xF0 && c <= 0xF4) { cp = c & 0x07; len = 4; }
        else { *bad = i; return false; }
        if (i + (size_t)len > s.size()) { *bad = i; return false; }
        for (int k = 1; k < len; k++) {
            const uint8_t t = (uint8_t)s[i + (size_t)k];
            if ((t & 0xC0) != 0x80) { *bad = i; return false; }
            cp = (cp << 6) | (t & 0x3F);
        }
        if ((len == 3 && (cp < 0x800 || (cp >= 0xD800 && cp <= 0xDFFF))) ||
            (len == 4 && (cp < 0x10000 || cp > 0x10FFFF))) {
            *bad = i;
            return false;
        }
        cps->push_back(cp);
        i += (size_t)len;
    }
    return true;
}

// ---- numbers as int() reads them ----------------------------------------------

// A parsed number, saturated to +-2^62: every bound it is compared with is
// far inside that.
struct Num {
    int64_t v;
};

static const int64_t SAT = (int64_t)1 << 62;
static const size_t MAX_DECIMAL_DIGITS = 4300;

static bool hexd(char c) { return (c >= '0' && c <= '9') || (c >= 'a' && c <= 'f'); }
static int hexv(char c) { return c <= '9' ? c - '0' : c - 'a' + 10; }

// digit ("_"? digit)* over [from, s.size()), digits by pred; value saturated.
static bool digits_us(const std::string &s, size_t from, bool hex, int64_t *v, size_t *ndig)
{
    if (from >= s.size()) return false;
    int64_t acc = 0;
    size_t nd = 0;
    bool prev_digit = false;
    for (size_t i = from; i < s.size(); i++) {
        const char c = s[i];
        if (c == '_') {
            if (!prev_digit || i + 1 >= s.size()) return false;
            prev_digit = false;
            continue;
        }
        if (!(hex ? hexd(c) : (c >= '0' && c <= '9'))) return false;
        prev_digit = true;
        nd++;
        const int d = hex ? hexv(c) : c - '0';
        if (acc < SAT) acc = std::min<int64_t>(SAT, acc * (hex ? 16 : 10) + d);
    }
    if (!prev_digit) return false;
    *v = acc;
    *ndig = nd;
    return true;
}

static std::string lower(std::string s)
{
    for (auto &c : s)
        if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
    return s;
}

static bool is_ident(const std::string &t)
{
    if (t.empty()) return false;
    auto a = [](char c) { return (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || c == '_'; };
    if (!a(t[0])) return false;
    for (char c : t)
        if (!a(c) && !(c >= '0' && c <= '9')) return false;
    return true;
}

// ^r(\d+)$, case-insensitive: the digits, or empty.
static std::string regname_digits(const std::string &t)
{
    if (t.size() < 2 || (t[0] != 'r' && t[0] != 'R')) return "";
    for (size_t i = 1; i < t.size(); i++)
        if (t[i] < '0' || t[i] > '9') return "";
    return t.substr(1);
}

// ---- the assembler --------------------------------------------------------------

struct Asm {
    std::string source;
    size_t lineno = 0;
    std::string err;
    Image im;
    bool have_fmt = false, have_dep = false, have_depth = false, have_in = false, have_out = false;
    int64_t n_in = 0, n_out = 0;
    std::vector<std::pair<std::string, int>> const_index;       // lower name -> index
    std::vector<std::pair<std::string, int>> reg_names;
    std::vector<std::pair<std::string, int64_t>> slot_names;

    bool fail(const std::string &m)
    {
        err = source + ":" + std::to_string(lineno) + ": " + m;
        return false;
    }
    template <class V> static bool find(const std::vector<std::pair<std::string, V>> &t, const std::string &k, V *v)
    {
        for (const auto &e : t)
            if (e.first == k) {
                if (v) *v = e.second;
                return true;
            }
        return false;
    }
    bool defined(const std::string &low)
    {
        return find<int>(const_index, low, nullptr) || find<int>(reg_names, low, nullptr) ||
               find<int64_t>(slot_names, low, nullptr);
    }

    // A decimal of at most 4,300 digits.
    bool decimal(const std::string &tok, const std::string &digs, const char *what, int64_t *v)
    {
        if (digs.size() > MAX_DECIMAL_DIGITS)
            return fail(strf("%s: '%.40s...' has %zu digits, and a decimal number has at most %zu",
                             what, tok.c_str(), digs.size(), MAX_DECIMAL_DIGITS));
        size_t nd;
        digits_us(digs, 0, false, v, &nd);
        return true;
    }

    // A number as int() reads one: 0x hex, or a decimal with one sign.
    bool uint(const std::string &tok, const char *what, int64_t *v)
    {
        const std::string t = lower(tok);
        size_t nd;
        if (t.size() >= 2 && t[0] == '0' && t[1] == 'x') {
            const size_t from = (t.size() > 2 && t[2] == '_') ? 3 : 2;
            if (digits_us(t, from, true, v, &nd)) return true;
        } else {
            const size_t from = (!t.empty() && (t[0] == '+' || t[0] == '-')) ? 1 : 0;
            if (digits_us(t, from, false, v, &nd)) {
                if (nd > MAX_DECIMAL_DIGITS)
                    return fail(strf("%s: a decimal number has at most %zu digits and this one has %zu",
                                     what, MAX_DECIMAL_DIGITS, nd));
                if (t[0] == '-') *v = -*v;
                return true;
            }
        }
        return fail(strf("%s: '%s' is not a number", what, tok.c_str()));
    }

    bool reg(const std::string &tok, int *r)
    {
        const std::string low = lower(tok);
        if (find<int>(reg_names, low, r)) return true;
        const std::string digs = regname_digits(tok);
        if (digs.empty()) {
            if (find<int>(const_index, low, nullptr))
                return fail(tok + " is a constant, and this operand must be a register");
            if (find<int64_t>(slot_names, low, nullptr))
                return fail(tok + " is a scratch slot, and this operand must be a register");
            return fail("'" + tok + "' is not a register");
        }
        int64_t n;
        if (!decimal(tok, digs, "a register", &n)) return false;
        if (n < 0 || n >= NREG) return fail(strf("r%lld is outside r0..r%d", (long long)n, NREG - 1));
        *r = (int)n;
        return true;
    }

    bool slot(const std::string &tok, int64_t *s)
    {
        const std::string low = lower(tok);
        if (find<int64_t>(slot_names, low, s)) return true;
        if (is_ident(tok)) {
            const bool isreg = find<int>(reg_names, low, nullptr) || !regname_digits(tok).empty();
            const bool isk = find<int>(const_index, low, nullptr);
            if (isreg || isk)
                return fail(tok + (isreg ? " is a register" : " is a constant") +
                            ", and a static slot is a number or a `.slot` name - the indexed form "
                            "is `stx` and `ldx`");
            return fail("'" + tok + "' is not a slot");
        }
        return uint(tok, "a scratch slot", s);
    }

    bool step(const std::string &tok, int64_t *v)
    {
        const bool signed_ = !tok.empty() && (tok[0] == '+' || tok[0] == '-');
        const std::string body = signed_ ? tok.substr(1) : tok;
        if (!body.empty() && (body[0] == '+' || body[0] == '-'))
            return fail("'" + tok + "' carries two signs; a post-step is one optional sign and a number");
        if (!regname_digits(body).empty() || find<int>(reg_names, lower(body), nullptr))
            return fail(tok + " is a register, and a post-step is a signed number");
        if (!uint(body, "a post-step", v)) return false;
        if (tok[0] == '-') *v = -*v;
        if (*v < -2048 || *v > 2047)
            return fail(strf("step %lld outside -2048..2047: a post-step is a signed 12-bit field",
                             (long long)*v));
        return true;
    }

    bool operand(const std::string &tok, int *v, bool *isk)
    {
        if (find<int>(const_index, lower(tok), v)) {
            *isk = true;
            return true;
        }
        *isk = false;
        return reg(tok, v);
    }

    bool name_ok(const std::string &name)
    {
        if (!is_ident(name)) return fail("'" + name + "' is not a name");
        if (defined(lower(name))) return fail(name + " is already defined");
        if (!regname_digits(name).empty()) return fail(name + " would shadow a register");
        return true;
    }

    // -- directives -----------------------------------------------------------

    bool do_format(const std::vector<std::string> &a)
    {
        if (have_fmt) return fail(".format appears twice");
        if (!im.insns.empty() || !im.consts.empty() || have_dep) return fail(".format must come first");
        if (a.size() != 1) return fail(".format takes one name");
        const std::string n = lower(a[0]);
        for (int f = 0; f < 4; f++)
            if (n == FMT_NAME[f]) {
                im.fmt = f;
                have_fmt = true;
                return true;
            }
        return fail("'" + a[0] + "' is not fp32, fp64, fp128 or fp256");
    }

    bool do_deposits(const std::vector<std::string> &a)
    {
        if (a.size() != 1) return fail(".deposits takes one number");
        if (!uint(a[0], ".deposits", &im.max_deposits)) return false;
        have_dep = true;
        return true;
    }

    bool do_bank(const std::vector<std::string> &a)
    {
        if (a.size() != 1 || lower(a[0]) != "external") return fail(".bank takes the word `external`");
        if (!im.consts.empty())
            return fail(".bank external must precede the .const lines it turns into declarations");
        im.flags |= F_BANK_EXT;
        return true;
    }

    bool do_scratch(const std::vector<std::string> &a)
    {
        if (!im.insns.empty()) return fail(".scratch must come before the instructions");
        if (a.size() == 1 && lower(a[0]) == "strict") {
            if (im.flags & F_SCRATCH_STRICT) return fail(".scratch strict appears twice");
            im.flags |= F_SCRATCH_STRICT;
            return true;
        }
        if (a.size() == 1) {
            if (have_depth) return fail(".scratch N appears twice");
            int64_t v;
            if (!uint(a[0], ".scratch", &v)) return false;
            if (v < 1 || v > SCRATCH_D_MAX || (v & (v - 1)))
                return fail(strf(".scratch takes a power of two in 1..%lld", (long long)SCRATCH_D_MAX));
            im.scratch_depth = v;
            have_depth = true;
            return true;
        }
        const std::string which = a.size() == 2 ? lower(a[0]) : "";
        if (which != "in" && which != "out")
            return fail(".scratch takes a depth, `strict`, or `in N`, or `out M`");
        int64_t v;
        if (!uint(a[1], which == "in" ? ".scratch in" : ".scratch out", &v)) return false;
        if (v < 0) return fail(".scratch " + which + " is a sixteen-bit count, and it is below zero");
        if (v > SCRATCH_IO_MAX) return fail(".scratch " + which + " is a sixteen-bit count, at most 65535");
        if (which == "in") {
            if (have_in) return fail(".scratch in appears twice");
            n_in = v;
            have_in = true;
        } else {
            if (have_out) return fail(".scratch out appears twice");
            n_out = v;
            have_out = true;
        }
        im.flags |= F_SCRATCH_IO;
        return true;
    }

    bool do_slot(const std::vector<std::string> &a)
    {
        if (a.size() != 3 || a[1] != "=") return fail(".slot takes NAME = N");
        if (!name_ok(a[0])) return false;
        int64_t v;
        if (!uint(a[2], ".slot", &v)) return false;
        if (v > (int64_t)SLOT_MASK) return fail("a static slot is imm[23:0], so at most 16777215");
        slot_names.push_back({lower(a[0]), v});
        return true;
    }

    bool do_reg(const std::vector<std::string> &a)
    {
        if (a.size() != 3 || a[1] != "=") return fail(".reg takes NAME = rN");
        if (!name_ok(a[0])) return false;
        const std::string digs = regname_digits(a[2]);
        if (digs.empty()) return fail("'" + a[2] + "' is not r0..r31");
        int64_t n;
        if (!decimal(a[2], digs, "a register", &n)) return false;
        if (n < 0 || n >= NREG) return fail(strf("r%lld is outside r0..r%d", (long long)n, NREG - 1));
        reg_names.push_back({lower(a[0]), (int)n});
        return true;
    }

    // int(text, 16) as Python reads it: sign? ("0x" "_"?)? hexdigit ("_"? hexdigit)*.
    static bool py_int16(const std::string &s, bool *neg, chars::Nat *v)
    {
        std::string t = lower(s);
        while (!t.empty() && t[0] == ' ') t.erase(0, 1);          // int() strips white space
        while (!t.empty() && t.back() == ' ') t.pop_back();
        size_t i = 0;
        *neg = false;
        if (i < t.size() && (t[i] == '+' || t[i] == '-')) *neg = t[i++] == '-';
        if (i + 1 < t.size() && t[i] == '0' && t[i + 1] == 'x') {
            i += 2;
            if (i < t.size() && t[i] == '_') i++;
        }
        std::string digs;
        bool prev = false;
        for (; i < t.size(); i++) {
            if (t[i] == '_') {
                if (!prev || i + 1 >= t.size()) return false;
                prev = false;
                continue;
            }
            if (!hexd(t[i])) return false;
            digs += t[i];
            prev = true;
        }
        if (!prev) return false;
        v->w.assign(digs.size() / 8 + 1, 0u);
        for (size_t k = 0; k < digs.size(); k++) {
            const size_t pos = digs.size() - 1 - k;
            v->w[pos / 8] |= (uint32_t)hexv(digs[k]) << (4 * (pos % 8));
        }
        v->trim();
        return true;
    }

    bool literal(const std::string &text, chars::Enc *out)
    {
        if (!have_fmt) return fail(".format must come before any constant");
        const std::string &t = text;
        const bool sgn = !t.empty() && (t[0] == '+' || t[0] == '-');
        const std::string body = sgn ? t.substr(1) : t;
        std::string why;
        uint32_t fl;
        if (body.size() >= 2 && lower(body.substr(0, 2)) == "0x") {
            if (lower(body).find('p') != std::string::npos) {
                if (!chars::from_hex(im.fmt, t, 0, out, &fl, &why))
                    return fail("'" + text + "' is not a hexadecimal-significand sequence this format "
                                "can read (" + why + ")");
                return true;
            }
            if (sgn)
                return fail("a raw 0x encoding carries its own sign bit; write the whole word, or use "
                            "the 5.12.3 form with a binary exponent");
            bool neg;
            chars::Nat v;
            if (!py_int16(body.substr(2), &neg, &v)) return fail("'" + text + "' is not a hexadecimal encoding");
            if (neg && !v.zero()) return fail("'" + text + "' is a negative encoding, which does not fit the format");
            if (v.bits() > chars::geo(im.fmt).width)
                return fail(text + " is wider than " + FMT_NAME[im.fmt]);
            *out = chars::Enc();
            for (size_t i = 0; i < v.w.size(); i++) out->w[i] = v.w[i];
            return true;
        }
        if (!chars::from_decimal(im.fmt, t, 0, out, &fl, &why))
            return fail("'" + text + "' is not a number this format can read (" + why + ")");
        return true;
    }

    bool do_const(const std::vector<std::string> &a)
    {
        const bool ext = im.flags & F_BANK_EXT;
        const bool bare = a.size() == 1 && ext;
        if (!bare && (a.size() < 3 || a[1] != "="))
            return fail(std::string(".const takes NAME = value") +
                        (ext ? ", or NAME alone under .bank external" : ""));
        if (!name_ok(a[0])) return false;
        chars::Enc bits;
        if (!bare) {
            std::string text = a[2];
            for (size_t i = 3; i < a.size(); i++) text += " " + a[i];
            if (!literal(text, &bits)) return false;
            if (ext) bits = chars::Enc();               // declared, not carried
        }
        if (im.consts.size() >= (size_t)KADDR_KX) return fail("the bank addresses at most 512 constants");
        const_index.push_back({lower(a[0]), (int)im.consts.size()});
        im.consts.push_back(bits);
        return true;
    }

    // -- instructions ----------------------------------------------------------

    static uint64_t ctrl_word(int code, int rd, int ra, int rb, uint32_t imm)
    {
        const int f[4] = {rd, ra, rb, 0};
        uint64_t w = (uint64_t)code | (1ull << 31);
        for (int k = 0; k < 4; k++) {
            w |= (uint64_t)(f[k] & 0xF) << (8 + 4 * k);
            if (f[k] >> 4) imm |= 1u << (24 + k);
        }
        return w | ((uint64_t)imm << 32);
    }

    bool do_ctrl(int code, const std::vector<std::string> &a)
    {
        const char *name = CTRL_NAME[code];
        if (code == C_REPEAT) {
            if (a.size() != 1) return fail("repeat takes a trip count");
            int64_t trip;
            if (!uint(a[0], "repeat", &trip)) return false;
            if (trip == 0) return fail("repeat 0 is not a loop; omit it");
            if (trip >= ((int64_t)1 << 32)) return fail("a trip count is a 32-bit immediate");
            if (trip < 1) return fail("repeat trip count must be 1..2^32-1");
            im.insns.push_back(((uint64_t)C_REPEAT | (1ull << 31)) | ((uint64_t)trip << 32));
            return true;
        }
        if (code == C_DEPOSIT || code == C_SETACT || code == C_RAISE) {
            if (a.size() != 1) return fail(std::string(name) + " takes one register");
            int r;
            if (!reg(a[0], &r)) return false;
            im.insns.push_back(ctrl_word(code, 0, r, 0, 0));
            return true;
        }
        if (code == C_STL || code == C_LDL) {
            if (a.size() != 2) return fail(std::string(name) + " takes a register and a slot");
            int r;
            int64_t s;
            if (!reg(a[0], &r) || !slot(a[1], &s)) return false;
            if (s > (int64_t)SLOT_MASK) return fail("a static slot is imm[23:0], so at most 16777215");
            if (s < 0) return fail(strf("scratch slot %lld does not fit imm[23:0]", (long long)s));
            im.insns.push_back(code == C_STL ? ctrl_word(code, 0, r, 0, (uint32_t)s)
                                             : ctrl_word(code, r, 0, 0, (uint32_t)s));
            return true;
        }
        if (code == C_STX || code == C_LDX) {
            if (a.size() != 2 && a.size() != 3)
                return fail(std::string(name) + " takes two registers - the value and the index - "
                            "and an optional signed post-step");
            int r0, r1;
            int64_t st = 0;
            if (!reg(a[0], &r0) || !reg(a[1], &r1)) return false;
            if (a.size() == 3 && !step(a[2], &st)) return false;
            const uint32_t imm = (uint32_t)st & STEP_MASK;
            im.insns.push_back(code == C_STX ? ctrl_word(code, 0, r0, r1, imm)
                                             : ctrl_word(code, r0, 0, r1, imm));
            return true;
        }
        if (code == C_AUGADD || code == C_AUGERR) {
            if (a.size() != 3)
                return fail(std::string(name) + " takes three registers - the destination and the two addends");
            int rd, ra, rb;
            if (!reg(a[0], &rd) || !reg(a[1], &ra) || !reg(a[2], &rb)) return false;
            im.insns.push_back(ctrl_word(code, rd, ra, rb, 0));
            return true;
        }
        if (!a.empty()) return fail(std::string(name) + " takes no operands");
        im.insns.push_back(ctrl_word(code, 0, 0, 0, 0));
        return true;
    }

    bool do_alu(const std::string &mnem, const std::vector<std::string> &a)
    {
        std::vector<std::string> parts;
        size_t start = 0;
        for (size_t i = 0; i <= mnem.size(); i++)
            if (i == mnem.size() || mnem[i] == '.') {
                parts.push_back(mnem.substr(start, i - start));
                start = i + 1;
            }
        const std::string name = parts[0];
        for (int c = 0; c < C_COUNT; c++)
            if (name == CTRL_NAME[c]) {
                bool attr = false;
                for (size_t i = 1; i < parts.size(); i++) attr |= parts[i] != "kx";
                return fail(name + " is a control instruction and takes no suffix" +
                            ((c == C_AUGADD || c == C_AUGERR) && attr
                                 ? " - 754-2019 9.5 fixes its rounding (roundTiesTowardZero), so no "
                                   "attribute can be written"
                                 : ""));
            }
        int rnd = 0;
        bool force_kx = false;
        for (size_t i = 1; i < parts.size(); i++) {
            if (parts[i] == "kx") {
                force_kx = true;
                continue;
            }
            int r = -1;
            for (int k = 0; k < 5; k++)
                if (parts[i] == RND_NAME[k]) r = k;
            if (r < 0) return fail("'" + parts[i] + "' is not rne, rtz, rdn, rup, rmm or kx");
            rnd = r;
        }
        int op = -1;
        uint8_t fields = 7;
        bool explicit_only = false;
        if (name.size() > 2 && name.compare(0, 2, "op") == 0 &&
            name.find_first_not_of("0123456789", 2) == std::string::npos) {
            int64_t v;
            if (!decimal(name, name.substr(2), "an opcode", &v)) return false;
            if (v > 255) return fail(strf("op%lld does not fit the opcode byte", (long long)v));
            op = (int)v;
            explicit_only = true;
        } else {
            for (int o = 0; o < 32; o++)
                if (alu_fields(o) && name == cft_op_name((cft_op)o)) op = o;
            if (op < 0) return fail("'" + name + "' is not an opcode this ISA has");
            fields = alu_fields(op);
        }
        if (a.empty()) return fail(name + " takes a destination");
        int rd;
        if (!reg(a[0], &rd)) return false;
        const size_t nrest = a.size() - 1;
        const int nf = __builtin_popcount(fields);
        int order[3], no = 0;
        if (nrest == 3) {
            order[0] = 0, order[1] = 1, order[2] = 2, no = 3;
        } else if (!explicit_only && (int)nrest == nf) {
            for (int s = 0; s < 3; s++)
                if (fields >> s & 1) order[no++] = s;
        } else {
            std::string fl;
            static const char *const fn[3] = {"ra", "rb", "rc"};
            for (int s = 0; s < 3; s++)
                if (fields >> s & 1) fl += std::string(fl.empty() ? "" : ", ") + fn[s];
            return fail(strf("%s reads %d operand(s) (%s); write that many, or all three in ra, rb, rc "
                             "order - %zu given", name.c_str(), nf, fl.c_str(), nrest));
        }
        int val[3] = {0, 0, 0};
        bool isk[3] = {false, false, false};
        for (int k = 0; k < no; k++)
            if (!operand(a[1 + (size_t)k], &val[order[k]], &isk[order[k]])) return false;
        if (force_kx && !(isk[0] || isk[1] || isk[2]))
            return fail("`.kx` on an instruction whose operands are all registers selects nothing, "
                        "and the loader refuses it - it is a second spelling of the plain form");
        bool kx = force_kx;
        for (int s = 0; s < 3; s++) kx |= isk[s] && val[s] >= KADDR_PLAIN;
        uint32_t imm = 0;
        uint64_t w = (uint64_t)op | ((uint64_t)rnd << 24) | ((uint64_t)isk[0] << 27) |
                     ((uint64_t)isk[1] << 28) | ((uint64_t)isk[2] << 29) | ((uint64_t)kx << 30);
        w |= (uint64_t)(rd & 0xF) << 8;
        if (rd >> 4) imm |= 1u << 24;
        for (int s = 0; s < 3; s++) {
            if (isk[s] && kx) {
                imm |= (uint32_t)(val[s] & 0xFF) << (8 * s);
                imm |= (uint32_t)(val[s] >> 8) << (28 + s);
                continue;
            }
            w |= (uint64_t)(val[s] & 0xF) << (12 + 4 * s);
            if (val[s] >> 4) imm |= 1u << (25 + s);      // a register's fifth bit (constants < 16 here)
        }
        im.insns.push_back(w | ((uint64_t)imm << 32));
        return true;
    }

    // -- the pass ----------------------------------------------------------------

    bool lines(const std::string &text, std::vector<std::string> *out)
    {
        std::vector<uint32_t> cps;
        size_t bad;
        if (!utf8_decode(text, &cps, &bad)) {
            size_t line = 1;
            for (size_t i = 0; i < bad; i++) line += text[i] == '\n';
            err = source + ":" + std::to_string(line) +
                  strf(": the source is not UTF-8 (byte 0x%02x)", (unsigned)(uint8_t)text[bad]);
            return false;
        }
        // split the code points at LF
        std::vector<std::vector<uint32_t>> segs(1);
        for (uint32_t cp : cps) {
            if (cp == '\n') segs.emplace_back();
            else segs.back().push_back(cp);
        }
        const bool ended = !cps.empty() && cps.back() == '\n';
        if (ended) segs.pop_back();
        if (cps.empty()) segs.clear();
        for (size_t i = 0; i < segs.size(); i++) {
            lineno = i + 1;
            auto &seg = segs[i];
            if ((ended || i + 1 < segs.size()) && !seg.empty() && seg.back() == '\r') seg.pop_back();
            bool comment = false;
            std::string s;
            for (uint32_t cp : seg) {
                if (const char *nm = line_break_name(cp))
                    return fail(std::string(nm) + ": a line ends at a line feed, or a carriage return "
                                "and a line feed, and at no other character, so a source holds none "
                                "of the others anywhere");
                if (cp == 0x00 || cp == 0x1a)
                    return fail(std::string(cp ? "a Ctrl-Z (0x1a)" : "a NUL (0x00)") +
                                ": a source holds none anywhere, in a comment or out of one");
                if (comment) continue;
                if (cp == ';') {
                    comment = true;
                    continue;
                }
                if (!(cp == '\t' || (cp >= 0x20 && cp <= 0x7E)))
                    return fail((cp < 0x20 || cp == 0x7F ? strf("the control character 0x%02x", cp)
                                                         : strf("the character U+%04X", cp)) +
                                " outside a comment, where a line holds only printable ASCII, "
                                "spaces and tabs");
                s += (char)cp;
            }
            out->push_back(s);                            // the line before its comment
        }
        lineno = 0;
        return true;
    }

    bool run(const std::string &text)
    {
        std::vector<std::string> ls;
        if (!lines(text, &ls)) return false;
        for (size_t li = 0; li < ls.size(); li++) {
            lineno = li + 1;
            std::vector<std::string> toks;
            std::string cur;
            for (char c : ls[li]) {
                if (c == ' ' || c == '\t' || c == ',') {
                    if (!cur.empty()) toks.push_back(cur), cur.clear();
                } else {
                    cur += c;
                }
            }
            if (!cur.empty()) toks.push_back(cur);
            if (toks.empty()) continue;
            const std::string &head = toks[0];
            const std::vector<std::string> args(toks.begin() + 1, toks.end());
            if (head[0] == '.') {
                const std::string d = lower(head);
                bool ok;
                if (d == ".format") ok = do_format(args);
                else if (d == ".deposits") ok = do_deposits(args);
                else if (d == ".bank") ok = do_bank(args);
                else if (d == ".const") ok = do_const(args);
                else if (d == ".reg") ok = do_reg(args);
                else if (d == ".slot") ok = do_slot(args);
                else if (d == ".scratch") ok = do_scratch(args);
                else ok = fail("'" + head + "' is not a directive");
                if (!ok) return false;
                continue;
            }
            if (!have_fmt) return fail(".format must come first");
            const std::string low = lower(head);
            int code = -1;
            for (int c = 0; c < C_COUNT; c++)
                if (low == CTRL_NAME[c]) code = c;
            if (!(code >= 0 ? do_ctrl(code, args) : do_alu(low, args))) return false;
        }
        lineno = 0;
        if (!have_fmt) return fail(".format is required");
        if (!have_dep) return fail(".deposits is required");
        im.scratch_io = (uint32_t)(n_in & 0xFFFF) | ((uint32_t)(n_out & 0xFFFF) << 16);
        std::string why;
        if (!validate(im, &why)) {
            err = source + ": " + why;
            return false;
        }
        return true;
    }
};

// ---- the disassembler and the header report -------------------------------------

static std::string hexword(const chars::Enc &k, int fmt)
{
    std::string s;
    for (int i = (int)esz(fmt) / 4 - 1; i >= 0; i--) s += strf("%08x", k.w[i]);
    return s;
}

static std::string disassemble(const Image &im)
{
    std::string o;
    auto line = [&](const std::string &s) { o += s + "\n"; };
    line(strf(".format   %s", FMT_NAME[im.fmt]));
    line(strf(".deposits %lld", (long long)im.max_deposits));
    if (im.scratch_depth != SCRATCH_D_DEFAULT) line(strf(".scratch  %lld", (long long)im.scratch_depth));
    if (im.flags & F_SCRATCH_STRICT) line(".scratch  strict");
    if (im.flags & F_SCRATCH_IO) {
        line(strf(".scratch  in %u", im.scratch_io & 0xFFFF));
        line(strf(".scratch  out %u", im.scratch_io >> 16));
    }
    const bool ext = im.flags & F_BANK_EXT;
    if (ext) line(".bank     external");
    for (size_t i = 0; i < im.consts.size(); i++) {
        if (ext) line(strf(".const    k%zu", i));
        else line(strf(".const    k%zu = 0x", i) + hexword(im.consts[i], im.fmt));
    }
    if (!im.consts.empty() || ext) line("");
    auto opnd = [](int idx, bool k) { return k ? strf("k%d", idx) : strf("r%d", idx); };
    int indent = 0;
    for (uint64_t w : im.insns) {
        const D d = decode(w);
        if (d.ctrl) {
            const char *name = CTRL_NAME[d.op];
            if (d.op == C_ENDREP || d.op == C_ENDQUIET) indent--;
            const std::string pad((size_t)(2 * std::max(indent, 0)), ' ');
            switch (d.op) {
            case C_REPEAT: line(pad + strf("%s %u", name, d.imm)); indent++; break;
            case C_QUIET: line(pad + name); indent++; break;
            case C_DEPOSIT: case C_SETACT: case C_RAISE: line(pad + strf("%s r%d", name, d.reg(1))); break;
            case C_STL: line(pad + strf("%s r%d, %u", name, d.reg(1), d.imm & SLOT_MASK)); break;
            case C_LDL: line(pad + strf("%s r%d, %u", name, d.reg(0), d.imm & SLOT_MASK)); break;
            case C_STX: case C_LDX: {
                const int st = step_of(d);
                line(pad + strf("%s r%d, r%d", name, d.op == C_STX ? d.reg(1) : d.reg(0), d.reg(2)) +
                     (st ? strf(", %+d", st) : ""));
                break;
            }
            case C_AUGADD: case C_AUGERR:
                line(pad + strf("%s r%d, r%d, r%d", name, d.reg(0), d.reg(1), d.reg(2)));
                break;
            default: line(pad + name); break;
            }
            continue;
        }
        const std::string pad((size_t)(2 * std::max(indent, 0)), ' ');
        const uint8_t fields = alu_fields(d.op);
        std::string name = fields ? cft_op_name((cft_op)d.op) : strf("op%d", d.op);
        if (d.rnd != 0) name += std::string(".") + RND_NAME[d.rnd];
        int idx[3];
        bool isk[3];
        sources(d, idx, isk);
        if (d.kx) {
            bool big = false;
            for (int s = 0; s < 3; s++) big |= isk[s] && idx[s] >= KADDR_PLAIN;
            if (!big) name += ".kx";
        }
        bool shortf = fields != 0;
        for (int s = 0; s < 3 && shortf; s++)
            if (!(fields >> s & 1) && (idx[s] != 0 || isk[s])) shortf = false;
        std::string args;
        for (int s = 0; s < 3; s++)
            if (!shortf || (fields >> s & 1)) args += std::string(args.empty() ? "" : ", ") + opnd(idx[s], isk[s]);
        line(pad + strf("%s r%d, ", name.c_str(), d.reg(0)) + args);
    }
    return o;
}

static std::string info(const Image &im, const std::vector<uint8_t> &data)
{
    // the feature names, in CAPS bit order then CAPS2's
    bool f_kx = false, f_r32 = false, f_kx9 = false, f_imul = false, f_scr = false, f_aug = false,
         f_step = false, f_fc = false;
    int64_t top = -1;
    bool indexed = false;
    for (uint64_t w : im.insns) {
        const D d = decode(w);
        if (d.ctrl) {
            for (int f = 0; f < 4; f++)
                if ((CTRL_REGS[d.op] >> f & 1) && d.reg(f) >= REG_FIELD) f_r32 = true;
            if (d.op >= C_STL && d.op <= C_LDX) f_scr = true;
            if (d.op == C_AUGADD || d.op == C_AUGERR) f_aug = true;
            if (step_of(d)) f_step = true;
            if (d.op == C_QUIET || d.op == C_ENDQUIET || d.op == C_RAISE) f_fc = true;
            if (d.op == C_STL || d.op == C_LDL) top = std::max<int64_t>(top, d.imm & SLOT_MASK);
            if (d.op == C_STX || d.op == C_LDX) indexed = true;
            continue;
        }
        if (d.kx) {
            f_kx = true;
            int idx[3];
            bool isk[3];
            sources(d, idx, isk);
            for (int s = 0; s < 3; s++)
                if (isk[s] && idx[s] >= 256) f_kx9 = true;
        }
        if (d.op == 30) f_imul = true;
        for (int f = 0; f < 4; f++)
            if (d.hi[f]) f_r32 = true;
    }
    const bool ext = im.flags & F_BANK_EXT, sio = im.flags & F_SCRATCH_IO;
    std::string feats;
    auto add = [&](bool on, const char *n) {
        if (on) feats += std::string(feats.empty() ? "" : " ") + n;
    };
    add(f_kx, "kx");
    add(f_r32, "REGS32");
    add(ext, "BANK_PTR");
    add(f_kx9, "KX9");
    add(f_imul, "IMUL");
    add(f_scr, "SCRATCH");
    add(sio, "SCRATCH_IO");
    add(f_aug, "AUGADD");
    add(f_step, "SCRATCH_STEP");
    add(f_fc, "FLAG_CONTROL");
    std::string scratch;
    if (top < 0 && !indexed) scratch = "-";
    else {
        if (top >= 0) scratch = strf("highest static slot %lld, ", (long long)top);
        scratch += indexed ? "indexed" : "not indexed";
    }
    std::string names;
    if (ext) names += "BANK_EXT";
    if (sio) names += std::string(names.empty() ? "" : " ") + "SCRATCH_IO";
    uint8_t dig[32];
    Sha256 h;
    h.init();
    h.update(data.data(), data.size());
    h.final(dig);
    std::string hex;
    for (uint8_t b : dig) hex += strf("%02x", b);
    std::string o;
    o += strf("format        %s\n", FMT_NAME[im.fmt]);
    o += strf("instructions  %zu\n", im.insns.size());
    o += strf("constants     %zu", im.consts.size()) + (ext ? "  (external: supplied per run)" : "") + "\n";
    o += strf("deposits      %lld\n", (long long)im.max_deposits);
    o += "scratch       " + scratch + "\n";
    o += "scratch-io    " + (sio ? strf("in %u, out %u", im.scratch_io & 0xFFFF, im.scratch_io >> 16) : std::string("-")) + "\n";
    o += strf("flags         0x%08x", im.flags) + (names.empty() ? "" : "  " + names) + "\n";
    o += strf("bytes         %zu\n", data.size());
    o += "features      " + (feats.empty() ? std::string("-") : feats) + "\n";
    o += "sha256        " + hex + "\n";
    return o;
}

// ---- the ODE banks ------------------------------------------------------------------

// The default bank of one of the reference's ODE segment programs for step
// h (programs/gen_odes.py:156-197): exact values rounded once from their
// decimals, H2 = H * 0.5 and MH = -H exactly, H6 = RN(H / 6), BETA = RN(8/3).
static bool ode_bank(const std::string &system, int fmt, const std::string &h_text,
                     std::vector<chars::Enc> *out, std::string *why)
{
    using namespace chars;
    auto dec = [&](const char *t) {
        Enc x;
        uint32_t fl;
        std::string w;
        from_decimal(fmt, t, 0, &x, &fl, &w);
        return x;
    };
    auto quotient = [&](const Enc &a, const Enc &b) {
        int sa, sb;
        Nat ma, mb;
        int64_t ea, eb;
        decode_finite(fmt, a, &sa, &ma, &ea);
        decode_finite(fmt, b, &sb, &mb, &eb);
        if (ea >= eb) shl(ma, ea - eb);
        else shl(mb, eb - ea);
        uint32_t fl;
        return round_rational(fmt, sa ^ sb, ma, mb, 0, &fl);
    };
    auto product = [&](const Enc &a, const Enc &b) {
        int sa, sb;
        Nat ma, mb;
        int64_t ea, eb;
        decode_finite(fmt, a, &sa, &ma, &ea);
        decode_finite(fmt, b, &sb, &mb, &eb);
        uint32_t fl;
        return round_pack(fmt, sa ^ sb, mul(ma, mb), ea + eb, 0, &fl);
    };
    Enc h;
    uint32_t fl;
    if (!from_decimal(fmt, h_text, 0, &h, &fl, why)) return false;
    {
        int s;
        Nat m;
        int64_t e;
        if (!decode_finite(fmt, h, &s, &m, &e)) {
            *why = "the step must be a finite non-zero value in the format";
            return false;
        }
    }
    const Enc two = dec("2"), h2 = product(h, dec("0.5")), h6 = quotient(h, dec("6"));
    Enc mh = h;
    mh.w[(geo(fmt).width - 1) / 32] ^= 1u << ((geo(fmt).width - 1) & 31);
    out->clear();
    if (system == "lorenz63-rk4") {
        *out = {h, h2, h6, two, dec("10"), dec("28"), quotient(dec("8"), dec("3"))};
    } else if (system == "lorenz96-rk4") {
        *out = {h, h2, h6, two, dec("8")};
    } else if (system == "henonheiles-lf") {
        *out = {h, h2, mh, dec("1"), two};
    } else {
        *why = "unknown system '" + system + "' (lorenz63-rk4, lorenz96-rk4, henonheiles-lf)";
        return false;
    }
    return true;
}

}  // namespace asmb
}  // namespace cftg

// ---- the C ABI --------------------------------------------------------------------------

using namespace cftg;

static char *dup_text(const std::string &s)
{
    char *p = static_cast<char *>(malloc(s.size() + 1));
    if (p) memcpy(p, s.c_str(), s.size() + 1);
    return p;
}

extern "C" CFT_API cft_status cftg_asm_assemble(const char *text, size_t len, const char *source,
                                                void **image, size_t *image_bytes)
{
    clear_error();
    if (!image || !image_bytes || (!text && len)) {
        set_error("cftg_asm_assemble: text, image and image_bytes must not be NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *image = nullptr;
    *image_bytes = 0;
    asmb::Asm A;
    A.source = source ? source : "<text>";
    if (!A.run(std::string(text ? text : "", len))) {
        set_error("%s", A.err.c_str());
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const std::vector<uint8_t> b = asmb::to_bytes(A.im);
    void *p = malloc(b.size());
    if (!p) {
        set_error("cftg_asm_assemble: out of host memory");
        return CFT_ERR_OUT_OF_MEMORY;
    }
    memcpy(p, b.data(), b.size());
    *image = p;
    *image_bytes = b.size();
    return CFT_OK;
}

static cft_status read_image(const void *image, size_t bytes, asmb::Image *im, const char *who)
{
    if (!image && bytes) {
        set_error("%s: image is NULL", who);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    std::string why;
    if (!asmb::from_bytes(static_cast<const uint8_t *>(image), bytes, im, &why)) {
        set_error("%s: %s", who, why.c_str());
        return CFT_ERR_INVALID_ARGUMENT;
    }
    return CFT_OK;
}

extern "C" CFT_API cft_status cftg_asm_disassemble(const void *image, size_t bytes, char **text)
{
    clear_error();
    if (!text) {
        set_error("cftg_asm_disassemble: text is NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *text = nullptr;
    asmb::Image im;
    const cft_status st = read_image(image, bytes, &im, "cftg_asm_disassemble");
    if (st != CFT_OK) return st;
    *text = dup_text(asmb::disassemble(im));
    return *text ? CFT_OK : CFT_ERR_OUT_OF_MEMORY;
}

extern "C" CFT_API cft_status cftg_asm_info(const void *image, size_t bytes, char **text)
{
    clear_error();
    if (!text) {
        set_error("cftg_asm_info: text is NULL");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    *text = nullptr;
    asmb::Image im;
    const cft_status st = read_image(image, bytes, &im, "cftg_asm_info");
    if (st != CFT_OK) return st;
    const uint8_t *p = static_cast<const uint8_t *>(image);
    *text = dup_text(asmb::info(im, std::vector<uint8_t>(p, p + bytes)));
    return *text ? CFT_OK : CFT_ERR_OUT_OF_MEMORY;
}

extern "C" CFT_API void cftg_asm_free(void *p) { free(p); }

extern "C" CFT_API cft_status cftg_ode_bank(const char *system, cft_format fmt, const char *h,
                                            void *bank, size_t cap, size_t *bytes)
{
    clear_error();
    if (bytes) *bytes = 0;
    if (!system || !h || (cap && !bank) || (int)fmt < 0 || (int)fmt > 3) {
        set_error("cftg_ode_bank: system and h must not be NULL, fmt is 0..3, and bank may be NULL "
                  "only with cap 0");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    std::vector<chars::Enc> vals;
    std::string why;
    if (!asmb::ode_bank(system, (int)fmt, h, &vals, &why)) {
        set_error("cftg_ode_bank: %s", why.c_str());
        return CFT_ERR_INVALID_ARGUMENT;
    }
    const size_t e = esz_of((int)fmt), need = vals.size() * e;
    if (bytes) *bytes = need;
    if (!bank && cap == 0) return CFT_OK;                        // a size query
    if (cap < need) {
        set_error("cftg_ode_bank: the bank needs %zu bytes and cap is %zu", need, cap);
        return CFT_ERR_INVALID_ARGUMENT;
    }
    for (size_t i = 0; i < vals.size(); i++) memcpy(static_cast<uint8_t *>(bank) + i * e, vals[i].w, e);
    return CFT_OK;
}

extern "C" CFT_API cft_status cftg_program_load_source(cft_device *dev, const char *text, size_t len,
                                                       const char *source, cft_program **out)
{
    void *img = nullptr;
    size_t n = 0;
    cft_status st = cftg_asm_assemble(text, len, source, &img, &n);
    if (st != CFT_OK) return st;
    st = cft_program_load(dev, img, n, out);
    free(img);
    return st;
}
