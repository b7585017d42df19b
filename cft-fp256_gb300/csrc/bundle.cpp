// bundle.cpp - a lane's program spread over G threads.
//
// A trajectory launch holds few lanes, each running a long chain of
// operations; one thread a lane leaves most of the GPU idle and every
// operation's latency exposed. Inside a straight-line stretch of a program,
// though, many operations are independent (the components of an ODE's
// right-hand side, the stages' updates). This file schedules each stretch
// into bundles of at most G operations that may run at the same time, so
// that G threads serve one lane: in a bundle every thread reads its
// operands, then (after a warp barrier) every thread writes its result.
//
// Semantics are kept exactly: an operation reads the value its program
// order gives it (it is placed after every earlier writer of what it reads,
// after every earlier writer of what it writes, and not before any earlier
// reader of what it writes - the read-then-write bundle step makes that
// last case safe within one bundle). Flags are ORed, so their order does
// not matter. Only programs whose control is REPEAT/ENDREP/HALT and whose
// memory accesses are LDL/STL at fixed slots are scheduled (no deposits,
// lane-mask changes, indexed scratch, quiet regions or raises: those carry
// an order of their own); the others run one thread a lane.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/cft_gb300.h"
#include "api_core.h"
#include "bundle.h"

namespace cftg {

namespace {

enum { C_HALT = 0, C_REPEAT = 1, C_ENDREP = 2, C_STL = 6, C_LDL = 7 };
constexpr uint32_t SLOT_MASK = 0x00FFFFFFu;

int regof(int lo, uint32_t imm, int which) { return lo | (int)(((imm >> (24 + which)) & 1u) << 4); }

struct Access {
    int reads[3];
    int nreads = 0;
    int write = -1;            // resource written: register r, or 32 + slot
};

// What an instruction reads and writes, resources numbered registers 0..31
// and scratch slots 32.. .
Access access_of(uint64_t w)
{
    Access a;
    const int op = (int)(w & 0xFF);
    const bool ctrl = ((w >> 31) & 1) != 0;
    const uint32_t imm = (uint32_t)(w >> 32);
    const int rd = (int)((w >> 8) & 0xF), ra = (int)((w >> 12) & 0xF), rb = (int)((w >> 16) & 0xF),
              rc = (int)((w >> 20) & 0xF);
    if (ctrl) {
        const int slot = 32 + (int)(imm & SLOT_MASK);
        if (op == C_LDL) {
            a.reads[a.nreads++] = slot;
            a.write = regof(rd, imm, 0);
        } else {                                   // STL
            a.reads[a.nreads++] = regof(ra, imm, 1);
            a.write = slot;
        }
        return a;
    }
    const unsigned need = op_operands(op);
    const int ks[3] = {(int)((w >> 27) & 1), (int)((w >> 28) & 1), (int)((w >> 29) & 1)};
    const int rs[3] = {ra, rb, rc};
    for (int k = 0; k < 3; k++)
        if (((need >> k) & 1u) && !ks[k]) a.reads[a.nreads++] = regof(rs[k], imm, 1 + k);
    a.write = regof(rd, imm, 0);
    return a;
}

// A micro-operation of a stretch before scheduling: its word (the layout
// of BundleSchedule::ops), the locations it reads and the one it writes.
struct UOp { uint64_t word; int reads[3]; int nreads; int write; };

constexpr uint64_t U_MOVE = 1ull << 14, U_NEG_C = 1ull << 15;
constexpr int OP_NEG = 5;

int ufield(uint64_t w, int shift) { return (int)((w >> shift) & 0xFFFu); }

uint64_t uset(uint64_t w, int shift, int loc)
{
    return (w & ~(0xFFFull << shift)) | ((uint64_t)(loc & 0xFFF) << shift);
}

// The locations a micro-operation reads, from its word.
void reads_of(UOp &u)
{
    u.nreads = 0;
    if (u.word & U_MOVE) {
        u.reads[u.nreads++] = ufield(u.word, 28);
        return;
    }
    const unsigned need = op_operands((int)(u.word & 0xFF));
    for (int k = 0; k < 3; k++)
        if (((need >> k) & 1u) && !((u.word >> (11 + k)) & 1u)) u.reads[u.nreads++] = ufield(u.word, 28 + 12 * k);
}

// Two rewrites of a stretch's micro-operations that shorten its schedule's
// dependence chains and leave every location's value where and when the
// plain program would have it:
//  1. A NEG (a sign flip: exact, no flags, NaN payloads kept) read as a
//     later operation's operand c is folded into that read: the operation
//     reads the NEG's own operand with bit U_NEG_C, and flips the sign bit
//     itself. The operation no longer waits for the NEG; a NEG whose value
//     nothing reads any more is dropped.
//  2. The value a stretch leaves in a register or slot is written there by
//     its producer instead of by a MOVE at the stretch's end, when nothing
//     after the producer (in program order) reads that location's value
//     from before the stretch; the list scheduler then keeps the producer
//     at or after the earlier readers of that old value (a bundle reads all
//     its operands before any result is written).
void rewrite_stretch(std::vector<UOp> &list, std::vector<char> &dead, int arch, int nloc)
{
    const size_t n = list.size();
    std::vector<int> prod(nloc, -1);
    for (size_t i = 0; i < n; i++)
        if (list[i].write >= arch) prod[list[i].write] = (int)i;     // temps: written once
    // 1. NEG folded into operand c
    for (size_t i = 0; i < n; i++) {
        UOp &u = list[i];
        const uint64_t w = u.word;
        if ((w & (U_MOVE | U_NEG_C)) || !((op_operands((int)(w & 0xFF)) >> 2) & 1u) || ((w >> 13) & 1u))
            continue;
        const int v = ufield(w, 52);
        if (v < arch || prod[v] < 0) continue;
        const uint64_t nw = list[prod[v]].word;
        if ((nw & U_MOVE) || (int)(nw & 0xFF) != OP_NEG) continue;
        u.word = uset(w, 52, ufield(nw, 28)) | (((nw >> 11) & 1ull) << 13) | U_NEG_C;
        reads_of(u);
    }
    std::vector<int> readers(nloc, 0);
    for (size_t i = 0; i < n; i++)
        for (int k = 0; k < list[i].nreads; k++) readers[list[i].reads[k]]++;
    for (size_t i = 0; i < n; i++) {
        const uint64_t w = list[i].word;
        if (!(w & U_MOVE) && (int)(w & 0xFF) == OP_NEG && list[i].write >= arch && !readers[list[i].write]) {
            dead[i] = 1;
            for (int k = 0; k < list[i].nreads; k++) readers[list[i].reads[k]]--;
        }
    }
    // 2. the stretch's end MOVEs folded into their values' producers
    std::vector<int> into(nloc, -1);                   // temp -> the location it now writes
    for (size_t m = 0; m < n; m++) {
        UOp &mv = list[m];
        if (dead[m] || !(mv.word & U_MOVE) || mv.write >= arch) continue;
        const int loc = mv.write, v = ufield(mv.word, 28);
        if (v < arch) continue;
        if (into[v] >= 0) {                            // already lives in another home
            mv.word = uset(mv.word, 28, into[v]);
            reads_of(mv);
            continue;
        }
        const int p = prod[v];
        if (p < 0 || dead[p]) continue;
        bool later_read = false;
        for (size_t j = (size_t)p + 1; j < n && !later_read; j++) {
            if (dead[j] || j == m) continue;
            for (int k = 0; k < list[j].nreads; k++)
                if (list[j].reads[k] == loc) later_read = true;
        }
        if (later_read) continue;
        list[p].word = uset(list[p].word, 16, loc);
        list[p].write = loc;
        for (size_t j = (size_t)p + 1; j < n; j++) {
            if (dead[j]) continue;
            UOp &u = list[j];
            bool hit = false;
            for (int k = 0; k < 3; k++) {
                const int sh = 28 + 12 * k;
                const bool isloc = (u.word & U_MOVE) ? k == 0 : !((u.word >> (11 + k)) & 1u);
                if (isloc && ufield(u.word, sh) == v) {
                    u.word = uset(u.word, sh, loc);
                    hit = true;
                }
            }
            if (hit) reads_of(u);
        }
        into[v] = loc;
        dead[m] = 1;
    }
}

}  // namespace

// Schedule `insns` for G threads a lane. False when the program has an
// instruction outside the scheduled set or needs more locations than a
// micro-operation can name.
//
// Within each straight-line stretch every value written gets a location of
// its own (renaming), so only true dependences order the operations:
// registers are locations 0..31, scratch slots 32..32+reach-1, and the
// stretch's values 32+reach onward. LDL and STL become renames (no work)
// once the value they move has a location of its own; a read of a slot's or
// register's value from before the stretch is first copied (MOVE). At the
// end of the stretch every register and slot written in it is moved back to
// its own location, so each stretch starts and ends with the program's
// registers and slots where the plain interpreter keeps them.
bool build_bundles(const std::vector<uint64_t> &insns, uint32_t reach, int G, BundleSchedule &s)
{
    s = BundleSchedule();
    s.G = G;
    const int arch = 32 + (int)reach;               // registers, then slots
    std::vector<uint32_t> open;
    std::vector<uint32_t> region;
    double weight = 1.0;
    std::vector<double> wstack;
    int temps_max = 0;
    bool too_big = false;

    auto uop = [](int op, int rnd, bool move, int dest, const int src[3], const bool kst[3]) {
        uint64_t w = (uint64_t)(op & 0xFF) | ((uint64_t)(rnd & 7) << 8) |
                     ((uint64_t)kst[0] << 11) | ((uint64_t)kst[1] << 12) | ((uint64_t)kst[2] << 13) |
                     ((uint64_t)move << 14) | ((uint64_t)dest << 16) | ((uint64_t)src[0] << 28) |
                     ((uint64_t)src[1] << 40) | ((uint64_t)src[2] << 52);
        return w;
    };

    auto flush = [&]() {
        if (region.empty()) return;
        std::vector<int> map(arch);
        for (int i = 0; i < arch; i++) map[i] = i;
        std::vector<char> dirty(arch, 0);
        std::vector<UOp> list;
        int next = arch;
        auto fresh = [&]() { return next++; };
        auto own = [&](int loc) {                    // loc's value in a location of its own
            if (map[loc] >= arch) return map[loc];
            const int t = fresh();
            const int src[3] = {map[loc], 0, 0};
            const bool k[3] = {false, false, false};
            list.push_back(UOp{uop(0, 0, true, t, src, k), {map[loc]}, 1, t});
            map[loc] = t;
            return t;
        };
        for (uint32_t pc : region) {
            const uint64_t w = insns[pc];
            const int op = (int)(w & 0xFF);
            const uint32_t imm = (uint32_t)(w >> 32);
            if ((w >> 31) & 1) {
                const int slot = 32 + (int)(imm & SLOT_MASK);
                if (op == C_LDL) {
                    const int rd = regof((int)((w >> 8) & 0xF), imm, 0);
                    map[rd] = own(slot);
                    dirty[rd] = 1;
                } else {
                    const int ra = regof((int)((w >> 12) & 0xF), imm, 1);
                    map[slot] = own(ra);
                    dirty[slot] = 1;
                }
                continue;
            }
            const Access a = access_of(w);
            const unsigned need = op_operands(op);
            int src[3] = {0, 0, 0};
            bool kst[3] = {false, false, false};
            UOp u;
            u.nreads = 0;
            const int rs[3] = {(int)((w >> 12) & 0xF), (int)((w >> 16) & 0xF), (int)((w >> 20) & 0xF)};
            for (int k = 0; k < 3; k++) {
                if (!((need >> k) & 1u)) continue;
                if ((w >> (27 + k)) & 1) {
                    kst[k] = true;
                    src[k] = ((w >> 30) & 1) ? (int)(((imm >> (8 * k)) & 0xFFu) | (((imm >> (28 + k)) & 1u) << 8))
                                             : rs[k];
                } else {
                    src[k] = map[regof(rs[k], imm, 1 + k)];
                    u.reads[u.nreads++] = src[k];
                }
            }
            const int t = fresh();
            u.write = t;
            u.word = uop(op, (int)((w >> 24) & 7), false, t, src, kst);
            list.push_back(u);
            map[a.write] = t;
            dirty[a.write] = 1;
        }
        for (int loc = 0; loc < arch; loc++) {
            if (!dirty[loc] || map[loc] == loc) continue;
            const int src[3] = {map[loc], 0, 0};
            const bool k[3] = {false, false, false};
            list.push_back(UOp{uop(0, 0, true, loc, src, k), {map[loc]}, 1, loc});
        }
        temps_max = std::max(temps_max, next - arch);
        if (next > 4095) too_big = true;
        std::vector<char> dead(list.size(), 0);
        rewrite_stretch(list, dead, arch, next);
        // list scheduling over locations: after every earlier writer of what
        // an operation reads or writes, not before an earlier reader of what
        // it writes
        const size_t b0 = s.ctl.size();
        std::vector<int> count, last_write(next, -1), max_read(next, -1);
        for (size_t li = 0; li < list.size(); li++) {
            if (dead[li]) continue;
            const UOp &u = list[li];
            int earliest = 0;
            for (int k = 0; k < u.nreads; k++) earliest = std::max(earliest, last_write[u.reads[k]] + 1);
            earliest = std::max(earliest, last_write[u.write] + 1);
            earliest = std::max(earliest, max_read[u.write]);
            int b = earliest;
            while (b < (int)count.size() && count[b] >= G) b++;
            if (b >= (int)count.size()) count.resize(b + 1, 0);
            const size_t at = b0 + (size_t)b;
            if (at >= s.ctl.size()) {
                const size_t grow = at + 1 - s.ctl.size();
                s.ctl.insert(s.ctl.end(), grow, BUNDLE_OPS);
                s.arg.insert(s.arg.end(), grow, 0u);
                s.match.insert(s.match.end(), grow, -1);
                s.ops.insert(s.ops.end(), grow * (size_t)G, BUNDLE_NOP);
            }
            s.ops[at * G + count[b]] = u.word;
            count[b]++;
            for (int k = 0; k < u.nreads; k++) max_read[u.reads[k]] = std::max(max_read[u.reads[k]], b);
            last_write[u.write] = b;
        }
        s.weighted += weight * (double)count.size();
        s.ops_weighted += weight * (double)region.size();
        region.clear();
    };
    auto control = [&](uint32_t kind, uint32_t arg) {
        flush();
        s.ctl.push_back(kind);
        s.arg.push_back(arg);
        s.match.push_back(-1);
        s.ops.insert(s.ops.end(), (size_t)G, BUNDLE_NOP);
        s.weighted += weight;
        s.ops_weighted += weight;
        return (uint32_t)(s.ctl.size() - 1);
    };

    for (uint32_t pc = 0; pc < insns.size(); pc++) {
        const uint64_t w = insns[pc];
        const int op = (int)(w & 0xFF);
        if (!((w >> 31) & 1)) {                    // ALU
            region.push_back(pc);
            continue;
        }
        const uint32_t imm = (uint32_t)(w >> 32);
        switch (op) {
        case C_LDL:
        case C_STL:
            if ((imm & SLOT_MASK) >= reach) return false;
            region.push_back(pc);
            break;
        case C_REPEAT: {
            const uint32_t b = control(BUNDLE_REPEAT, imm);
            open.push_back(b);
            wstack.push_back(weight);
            weight *= (double)(imm ? imm : 1u);
            break;
        }
        case C_ENDREP: {
            if (open.empty()) return false;
            flush();
            const uint32_t r = open.back();
            open.pop_back();
            const uint32_t b = control(BUNDLE_ENDREP, 0);      // runs once a pass
            weight = wstack.back();
            wstack.pop_back();
            s.match[b] = (int32_t)r;
            s.match[r] = (int32_t)b;
            break;
        }
        case C_HALT:
            control(BUNDLE_HALT, 0);
            break;
        default:
            return false;
        }
    }
    flush();
    if (!open.empty() || too_big) return false;
    s.nb = (uint32_t)s.ctl.size();
    s.nloc = (uint32_t)(arch + temps_max);
    return true;
}

}  // namespace cftg

// The schedule as arrays, for inspection and for the checks that replay it
// on the host: ops (nb x G words, NOP = all ones), ctl (kind per bundle),
// arg (REPEAT counts) and match (REPEAT <-> ENDREP). Returns
// CFT_ERR_UNSUPPORTED for a program outside the scheduled set, and the
// bundle count in *nb (arrays filled only when cap >= *nb).
extern "C" cft_status cftg_program_schedule(const void *image, size_t bytes, uint32_t G,
                                            uint64_t *ops, uint32_t *ctl, uint32_t *arg,
                                            int32_t *match, size_t cap, size_t *nb)
{
    using namespace cftg;
    clear_error();
    if (!image || !nb || G < 1 || G > 32 || (G & (G - 1))) {
        set_error("cftg_program_schedule: needs an image, nb and G a power of two in 1..32");
        return CFT_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint64_t> insns;
    uint32_t reach = 0;
    cft_status st = program_insns(image, bytes, insns, &reach);
    if (st != CFT_OK) return st;
    BundleSchedule s;
    if (!build_bundles(insns, reach, (int)G, s)) {
        set_error("cftg_program_schedule: the program has control outside REPEAT/ENDREP/HALT "
                  "and LDL/STL");
        return CFT_ERR_UNSUPPORTED;
    }
    *nb = s.nb;
    if (cap >= s.nb && ops && ctl && arg && match) {
        memcpy(ops, s.ops.data(), s.ops.size() * 8);
        memcpy(ctl, s.ctl.data(), s.ctl.size() * 4);
        memcpy(arg, s.arg.data(), s.arg.size() * 4);
        memcpy(match, s.match.data(), s.match.size() * 4);
    }
    return CFT_OK;
}

namespace cftg {

// Choose the threads a lane for a trajectory launch of n lanes: the G whose
// schedule steps through the fewest bundles a run, weighed by how many warps
// then share a scheduler (152 SMs x 4) and by how many lanes share a warp,
// with a bundle counted a quarter dearer than one instruction of the plain
// interpreter (two warp barriers, operands read from shared memory). G = 1
// keeps the plain interpreter.
//  * Sharing a scheduler: with the lanes' run counts (runs_desc, longest
//    first as the launch places them), the warps' lengths summed over the
//    longest one's - the warps that are still running, on average, while
//    the longest lane runs - over the schedulers; without them, all the
//    warps over the schedulers.
//  * Sharing a warp: a warp's lanes take their own branches through each
//    operation and the warp runs them all, a bundle costing 4 % more for
//    each lane past the first (measured on Lorenz-63's configuration at
//    binary256: 16 threads a lane ran its 4,096 lanes in 1.34 s, 8 threads
//    a lane in 1.45 s, at the same 13 bundles a step). Counted for the
//    launches that give their run counts (cftg_traj_create); the serving
//    loop's batches, which share the GPU with element batches, keep the
//    plain count (there more threads a lane lengthened program requests'
//    latency: p50 33 -> 39 ms).
// Binary128/256 programs may also take the cooperative arithmetic
// (coop.cuh): W threads a micro-operation, so G threads hold G/W of them a
// bundle, a bundle counted at COOP_BUNDLE instead; only when
// CFTG_LANE_COOP=1 asks for it (see below). CFTG_LANE_THREADS forces G.
void plan_lanes(cft_program *prog, size_t n, TrajLaunch &L, const uint32_t *runs_desc)
{
    constexpr double PLAIN_BUNDLE = 1.25, COOP_BUNDLE = 0.8, LANE_DIVERGENCE = 0.04;
    L.G = 1;
    L.K = 1;
    L.nb = 0;
    if (!prog || !n) return;
    const char *env = getenv("CFTG_LANE_THREADS");
    const int forced = env ? atoi(env) : 0;
    const char *cenv = getenv("CFTG_LANE_COOP");
    const int coop_mode = cenv ? atoi(cenv) : 0;
    const double slots = (double)sm_count() * 4.0;
    auto contention = [&](int G) {
        double warps;
        if (runs_desc && runs_desc[0]) {
            // warp w holds lanes [w*LPB, w*LPB + LPB), the longest of them first
            const size_t lpb = (size_t)(32 / G > 0 ? 32 / G : 1);
            double sum = 0;
            for (size_t w = 0; w * lpb < n; w++) sum += (double)runs_desc[w * lpb];
            warps = sum / (double)runs_desc[0];
        } else {
            warps = std::ceil((double)n * G / 32.0);
        }
        return warps > slots ? warps / slots : 1.0;
    };
    const DevBundles *one = program_bundles(prog, 1);
    if (!one) return;                                  // not schedulable: plain interpreter
    const int W = (int)(esz_of(L.P.fmt) / 4);
    double best = one->ops_weighted * contention(1);
    int bestG = 1, bestK = 1;
    // a forced G takes its first candidate, and the cooperative one instead
    // only when it is estimated cheaper (or forced too)
    // the block's shared memory (seq.cu go_traj_g): the lanes' locations and
    // the constants as further locations (whose indices must fit the
    // micro-operation's 12-bit fields), the cooperative scratch, the schedule
    auto consider = [&](int G, int K, double cost) {
        const DevBundles *d = program_bundles(prog, G / K);
        if (!d || d->nloc + L.P.n_consts > 4096u) return;
        size_t bytes = (size_t)(d->nloc + L.P.n_consts) * (size_t)(W * (32 / G) + (W >= 4 ? 4 : W)) * 4;
        if (K > 1) bytes += (size_t)(32 / W) * (size_t)(9 * W) * 4;
        bytes = (bytes + 7) / 8 * 8 + (size_t)(d->nb + 1) * (size_t)(G / K) * 8 + (size_t)(d->nb + 1) * 12;
        if (bytes > (200u << 10)) return;
        const double est = d->weighted * cost * contention(G) *
                           (runs_desc ? 1.0 + LANE_DIVERGENCE * (double)(32 / G - 1) : 1.0);
        if ((forced && bestG != G) || est < best) {
            best = est;
            bestG = G;
            bestK = K;
        }
    };
    for (int G = 2; G <= 32; G *= 2) {
        if (forced && G != forced) continue;
        if (coop_mode != 1 || W < 4) consider(G, 1, PLAIN_BUNDLE);
        if (coop_mode == 1 && W >= 4 && G >= W) consider(G, W, COOP_BUNDLE);
    }
    if (bestG == 1) return;
    const DevBundles *d = program_bundles(prog, bestG / bestK);
    L.G = bestG;
    L.K = bestK;
    L.nb = d->nb;
    L.nloc = d->nloc;
    L.b_ops = d->ops;
    L.b_ctl = d->ctl;
    L.b_arg = d->arg;
    L.b_match = d->match;
}

}  // namespace cftg
