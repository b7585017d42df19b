// seq.cu - the sequencer on the GPU: one thread a lane, a warp a block of
// lanes, every control decision taken per warp.
//
// The program model is the reference's (host/src/seq_exec.h:412-923). Its
// executor runs lanes in blocks and lets REPEAT/ENDREP skip a loop only
// when no lane of the block is active; the reference argues that the
// block size is invisible in the results (host/src/program.c:11-31): an
// inactive lane writes, deposits and raises nothing, and ACTALL and HALT
// are refused inside loops. Here the block is the warp. Control flow is
// therefore warp-uniform (decided with __any_sync), every lane of a warp
// decodes the same instruction from a broadcast load, and only the
// arithmetic itself - one element of the opcode per active lane - runs
// per thread.
//
// A lane's 32 registers live in shared memory, structure-of-words
// (word w of register r of lane t at [(r*W + w)*T + t]), so a warp's
// accesses to one register hit 32 consecutive banks. Only the registers
// the program names are allocated. Scratch slots live in global memory in
// the same structure-of-words layout across the launch's lanes.
#include "aug.cuh"
#include "cftg_internal.h"
#include "coop.cuh"
#include "simple_ops.cuh"

namespace cftg {

namespace {

constexpr uint32_t NONE = 0xFFFFFFFFu;

struct Insn {
    int op, rd, ra, rb, rc, rnd, ka, kb, kc, kx, ctrl;
    uint32_t imm;
};

// instruction word fields (reference seq_exec.h:175-200)
SFD Insn decode(uint64_t w)
{
    Insn d;
    d.op = (int)(w & 0xFF);
    d.rd = (int)((w >> 8) & 0xF);
    d.ra = (int)((w >> 12) & 0xF);
    d.rb = (int)((w >> 16) & 0xF);
    d.rc = (int)((w >> 20) & 0xF);
    d.rnd = (int)((w >> 24) & 0x7);
    d.ka = (int)((w >> 27) & 1);
    d.kb = (int)((w >> 28) & 1);
    d.kc = (int)((w >> 29) & 1);
    d.kx = (int)((w >> 30) & 1);
    d.ctrl = (int)((w >> 31) & 1);
    d.imm = (uint32_t)(w >> 32);
    return d;
}

SFD int reg5(int lo, uint32_t imm, int which) { return lo | (int)(((imm >> (24 + which)) & 1u) << 4); }

// operand `which` (0 a, 1 b, 2 c): register number or constant index
// (reference seq_exec.h:232-246)
SFD int source(const Insn &d, int which, bool &is_const)
{
    const int kf = which == 0 ? d.ka : which == 1 ? d.kb : d.kc;
    const int reg = which == 0 ? d.ra : which == 1 ? d.rb : d.rc;
    is_const = kf != 0;
    if (!kf) return reg5(reg, d.imm, 1 + which);
    if (d.kx) return (int)((d.imm >> (8 * which)) & 0xFFu) | (int)(((d.imm >> (28 + which)) & 1u) << 8);
    return reg;
}

template <int W>
struct Lane {
    uint32_t *sm;       // this block's register file
    int T, t;           // lanes in the block, this lane's index
    SFD uint32_t &at(int r, int w) const { return sm[(r * W + w) * T + t]; }
    SFD void get(int r, uint32_t (&x)[W]) const
    {
#pragma unroll
        for (int w = 0; w < W; w++) x[w] = at(r, w);
    }
    SFD void put(int r, const uint32_t (&x)[W]) const
    {
#pragma unroll
        for (int w = 0; w < W; w++) at(r, w) = x[w];
    }
};

template <int W>
SFD void load_elem_g(const void *base, size_t j, uint32_t (&x)[W])
{
    const uint32_t *p = static_cast<const uint32_t *>(base) + j * W;
#pragma unroll
    for (int w = 0; w < W; w++) x[w] = p[w];
}

template <int W>
SFD void load_in(const void *src, const uint32_t *idx, size_t e, uint32_t (&x)[W])
{
    if (idx) {
        const uint32_t t = idx[e];
        if (t == NONE) {
            sfw::zero(x);
            return;
        }
        load_elem_g<W>(src, t, x);
        return;
    }
    load_elem_g<W>(src, e, x);
}

}  // namespace

// A lane's scratch slots: structure-of-words across the launch's lanes.
template <int W>
struct Scratch {
    uint32_t *base;       // NULL for a program without scratch
    size_t nl, local;     // lanes in the launch, this lane's index among them
    SFD uint32_t &at(uint32_t slot, int w) const { return base[((size_t)slot * W + w) * nl + local]; }
};

// What one pass of the interpreter leaves for its lane.
struct LaneRun {
    uint32_t count = 0, flags = 0, status = 0, err = 0;
    uint8_t lflag = 0;
};

// One run of the program for this lane (reference seq_exec.h:412-685):
// control decided per warp, arithmetic per active lane. `active` starts as
// the lane's keep bit; `dep` is the deposit buffer (AoS) or NULL. UNIFIED
// runs FMA/ADD/SUB/MUL through one FMA code path (arith_rt): more work for
// ADD and MUL, a quarter of the code, which is what a launch of few, long
// lanes (latency-bound, one warp a scheduler) wants.
template <int FMT, bool UNIFIED = false>
SFD void interpret(const SeqProgram &P, const Lane<sf::Fmt<FMT>::W> &R,
                   const Scratch<sf::Fmt<FMT>::W> &sc, uint32_t *dep, size_t lane, bool keep,
                   bool active, LaneRun &o)
{
    constexpr int W = sf::Fmt<FMT>::W;
    const uint32_t log2d = P.scratch_log2;
    uint32_t x[W];
    uint32_t &count = o.count, &flags = o.flags, &status = o.status, &err = o.err;
    uint8_t &lflag = o.lflag;
    uint32_t body[4], left[4];
    int sp = 0, qd = 0;
    uint32_t pc = 0;
    const uint32_t *kons = static_cast<const uint32_t *>(P.d_consts);

    while (pc < P.n_insns) {
        const Insn d = decode(__ldg(P.d_insns + pc));
        if (!d.ctrl) {
            if (active) {
                bool ka, kb, kc;
                const int ia = source(d, 0, ka), ib = source(d, 1, kb), ic = source(d, 2, kc);
                uint32_t va[W], vb[W], vc[W], o[W], fl = 0u;
                if (ka) { for (int w = 0; w < W; w++) va[w] = __ldg(kons + ia * W + w); } else R.get(ia, va);
                if (kb) { for (int w = 0; w < W; w++) vb[w] = __ldg(kons + ib * W + w); } else R.get(ib, vb);
                if (kc) { for (int w = 0; w < W; w++) vc[w] = __ldg(kons + ic * W + w); } else R.get(ic, vc);
                if (UNIFIED && d.op <= 3) {
                    sf::arith_rt<FMT>(d.op, va, vb, vc, d.rnd, o, fl);
                } else {
                    switch (d.op) {
                    case 0: sf::arith<FMT, sf::OP_FMA>(va, vb, vc, d.rnd, o, fl); break;
                    case 1: sf::arith<FMT, sf::OP_ADD>(va, vb, vc, d.rnd, o, fl); break;
                    case 2: sf::arith<FMT, sf::OP_SUB>(va, vb, vc, d.rnd, o, fl); break;
                    case 3: sf::arith<FMT, sf::OP_MUL>(va, vb, vc, d.rnd, o, fl); break;
                    default: sf::simple<FMT>(d.op, va, vb, vc, o, fl); break;
                    }
                }
                R.put(reg5(d.rd, d.imm, 0), o);
                if (!qd) {
                    flags |= fl;
                    lflag |= (uint8_t)fl;
                }
            }
            pc++;
            continue;
        }
        switch (d.op) {
        case 0:                                              // HALT
            pc = P.n_insns;
            break;
        case 1: {                                            // REPEAT
            const bool any = __any_sync(0xFFFFFFFFu, active);
            if (d.imm == 0u || !any) {
                pc = (uint32_t)P.d_endrep[pc] + 1u;
                break;
            }
            if (sp >= 4) { err |= 1u; pc = P.n_insns; break; }
            body[sp] = pc + 1;
            left[sp] = d.imm;
            sp++;
            pc++;
            break;
        }
        case 2: {                                            // ENDREP
            const bool any = __any_sync(0xFFFFFFFFu, active);
            if (sp <= 0) { err |= 2u; pc = P.n_insns; break; }
            left[sp - 1]--;
            if (left[sp - 1] > 0u && any) {
                pc = body[sp - 1];
            } else {
                sp--;
                pc++;
            }
            break;
        }
        case 3:                                              // DEPOSIT
            if (active) {
                if (count >= P.max_deposits) {
                    status |= 1u << 4;
                    lflag |= 1u << 5;
                } else {
                    R.get(reg5(d.ra, d.imm, 1), x);
                    uint32_t *p = dep + (lane * (size_t)P.max_deposits + count) * W;
#pragma unroll
                    for (int w = 0; w < W; w++) p[w] = x[w];
                    count++;
                }
            }
            pc++;
            break;
        case 4:                                              // SETACT: narrows only
            if (active) {
                R.get(reg5(d.ra, d.imm, 1), x);
                x[W - 1] &= 0x7FFFFFFFu;
                active = !sfw::is_zero(x);
            }
            pc++;
            break;
        case 5:                                              // ACTALL
            active = keep;
            pc++;
            break;
        case 6: case 7: {                                    // STL, LDL
            const uint32_t slot = d.imm & 0x00FFFFFFu;
            if (active) {
                if (!sc.base || slot >= P.reach) {
                    err |= 4u;
                } else if (d.op == 6) {
                    R.get(reg5(d.ra, d.imm, 1), x);
#pragma unroll
                    for (int w = 0; w < W; w++) sc.at(slot, w) = x[w];
                } else {
#pragma unroll
                    for (int w = 0; w < W; w++) x[w] = sc.at(slot, w);
                    R.put(reg5(d.rd, d.imm, 0), x);
                }
            }
            pc++;
            break;
        }
        case 8: case 9: {                                    // STX, LDX
            const int rb = reg5(d.rb, d.imm, 2), rd = reg5(d.rd, d.imm, 0);
            int step = (int)(d.imm & 0xFFFu);
            if (step & 0x800) step -= 0x1000;
            if (d.op == 9 && rd == rb) step = 0;             // the loaded value wins
            if (active) {
                uint32_t ix[W];
                R.get(rb, ix);
                const bool strict = (P.flags & 4u) != 0u;
                if (strict && sfw::bitlen(ix) > (int)log2d) {
                    status |= 1u << 5;
                    lflag |= 1u << 6;
                    if (d.op == 9) {
                        sfw::zero(x);
                        R.put(rd, x);
                    }
                } else {
                    const uint32_t slot = (log2d >= 32 ? ix[0] : (ix[0] & ((1u << log2d) - 1u))) &
                                          (P.scratch_depth - 1u);
                    if (!sc.base || slot >= P.reach) {
                        err |= 8u;
                    } else if (d.op == 8) {
                        R.get(reg5(d.ra, d.imm, 1), x);
#pragma unroll
                        for (int w = 0; w < W; w++) sc.at(slot, w) = x[w];
                    } else {
#pragma unroll
                        for (int w = 0; w < W; w++) x[w] = sc.at(slot, w);
                        R.put(rd, x);
                    }
                }
                if (step) {
                    // rb := rb +/- |step| modulo 2^width (IADD / ISUB)
                    R.get(rb, ix);
                    uint32_t m[W];
                    sfw::zero(m);
                    m[0] = (uint32_t)(step < 0 ? -step : step);
                    if (step > 0) sfw::add(ix, ix, m);
                    else sfw::sub(ix, ix, m);
                    R.put(rb, ix);
                }
            }
            pc++;
            break;
        }
        case 10: case 11:                                    // AUGADD, AUGERR
            // 9.5's augmentedAddition(ra, rb): r (AUGADD) or e (AUGERR) to
            // rd, both operands read before rd is written (reference
            // seq_exec.h:337-371); flags as an ALU instruction's
            if (active) {
                uint32_t xa[W], xb[W], vr[W], ve[W], fl = 0u;
                R.get(reg5(d.ra, d.imm, 1), xa);
                R.get(reg5(d.rb, d.imm, 2), xb);
                sf::augmented<FMT>(sf::AUG_ADD, xa, xb, vr, ve, fl);
                R.put(reg5(d.rd, d.imm, 0), d.op == 11 ? ve : vr);
                if (!qd) {
                    flags |= fl;
                    lflag |= (uint8_t)fl;
                }
            }
            pc++;
            break;
        case 12:                                             // QUIET
            qd++;
            pc++;
            break;
        case 13:                                             // ENDQUIET
            qd--;
            pc++;
            break;
        case 14:                                             // RAISE
            if (active) {
                R.get(reg5(d.ra, d.imm, 1), x);
                const uint32_t low = x[0] & 0xFFu;
                if (!qd) {
                    flags |= low & 0x1Fu;
                    lflag |= (uint8_t)(low & 0x1Fu);
                }
                if (low & 0x80u) {
                    status |= 1u << 6;
                    lflag |= 1u << 7;
                }
            }
            pc++;
            break;
        default:                                             // refused at load
            err |= 16u;
            pc = P.n_insns;
            break;
        }
    }

}

template <int FMT>
__global__ void k_seq(const SeqLaunch L, size_t lane0, size_t nl)
{
    constexpr int W = sf::Fmt<FMT>::W;
    extern __shared__ uint32_t smem[];
    const SeqProgram &P = L.P;
    const int T = blockDim.x, t = threadIdx.x;
    const size_t local = (size_t)blockIdx.x * T + t;
    const size_t lane = lane0 + local;
    const bool have = local < nl;
    const int nregs = (int)P.nregs;
    Lane<W> R{smem, T, t};

    bool keep = have;
    if (have && L.lane_mask) keep = (L.lane_mask[lane >> 3] >> (lane & 7)) & 1u;
    bool active = keep;

    // registers +0, then r0..r2 from the streams (reference seq_exec.h:810-860)
    for (int r = 0; r < nregs; r++) {
#pragma unroll
        for (int w = 0; w < W; w++) R.at(r, w) = 0u;
    }
    uint32_t x[W];
    if (keep) {
        if (nregs > 0) { load_in<W>(L.a, L.ia, lane, x); R.put(0, x); }
        if (nregs > 1 && L.b) { load_in<W>(L.b, L.ib, lane, x); R.put(1, x); }
        if (nregs > 2 && L.c) { load_in<W>(L.c, L.ic, lane, x); R.put(2, x); }
    }
    // scratch: +0 to its reach, then the first n_scratch_in slots preloaded
    uint32_t *scr = static_cast<uint32_t *>(L.scratch);
    const Scratch<W> scv{scr, nl, local};
    auto sc = [&](uint32_t slot, int w) -> uint32_t & { return scv.at(slot, w); };
    if (keep && scr) {
        for (uint32_t s = 0; s < P.reach; s++) {
#pragma unroll
            for (int w = 0; w < W; w++) sc(s, w) = 0u;
        }
        if (L.scratch_in) {
            for (uint32_t s = 0; s < P.n_scratch_in; s++) {
                load_in<W>(L.scratch_in, L.isi, lane * P.n_scratch_in + s, x);
#pragma unroll
                for (int w = 0; w < W; w++) sc(s, w) = x[w];
            }
        }
    }
    uint32_t *dep = static_cast<uint32_t *>(L.deposits);
    if (keep && dep && L.lane_mask) {
        // with a mask the buffer holds the caller's bytes; this lane's are
        // the run's, and start at +0
        for (size_t k = 0; k < (size_t)P.max_deposits * W; k++)
            dep[lane * (size_t)P.max_deposits * W + k] = 0u;
    }
    __syncwarp();

    LaneRun o;
    interpret<FMT>(P, R, Scratch<W>{scr, nl, local}, dep, lane, keep, active, o);
    uint32_t flags = o.flags, status = o.status, err = o.err;
    const uint32_t count = o.count;
    const uint8_t lflag = o.lflag;

    // outputs of the lanes the caller has (reference seq_exec.h:880-923)
    if (keep) {
        if (L.counts) L.counts[lane] = count;
        if (L.lane_flags) L.lane_flags[lane] = lflag;
        if (L.scratch_out && scr) {
            uint32_t *so = static_cast<uint32_t *>(L.scratch_out);
            for (uint32_t s = 0; s < P.n_scratch_out; s++) {
#pragma unroll
                for (int w = 0; w < W; w++) so[(lane * P.n_scratch_out + s) * W + w] = sc(s, w);
            }
        }
    }
    flags = __reduce_or_sync(0xFFFFFFFFu, flags);
    status = __reduce_or_sync(0xFFFFFFFFu, status);
    err = __reduce_or_sync(0xFFFFFFFFu, err);
    if ((t & 31) == 0) {
        if (flags) atomicOr(L.word + 0, flags);
        if (status) atomicOr(L.word + 1, status);
        if (err) atomicOr(L.word + 2, err);
    }
}

// A lane of an early-completing launch (TrajLaunch::req_of) has finished:
// one thread a lane, after the lane's final block is written and fenced.
SFD void lane_finished(const TrajLaunch &L, size_t lane, uint32_t lflags, uint32_t lstatus)
{
    const uint32_t r = L.req_of[lane];
    if (lflags) atomicOr(L.req_acc + 2 * (size_t)r, lflags);
    if (lstatus) atomicOr(L.req_acc + 2 * (size_t)r + 1, lstatus);
    __threadfence();
    if (atomicSub(L.req_left + r, 1u) == 1u) {                // the request's last lane
        __threadfence();
        const uint32_t f = atomicOr(L.req_acc + 2 * (size_t)r, 0u);
        const uint32_t st = atomicOr(L.req_acc + 2 * (size_t)r + 1, 0u);
        volatile uint32_t *d = L.req_done + 4 * (size_t)r;
        d[0] = f;
        d[1] = st;
        __threadfence_system();
        d[2] = 1u;
    }
}

// The block of `slots` elements a finished lane leaves, in its request's
// host output (TrajLaunch::req_out), or NULL.
template <int W>
SFD uint32_t *lane_out(const TrajLaunch &L, size_t lane, uint32_t slots)
{
    if (!L.req_out) return nullptr;
    const uint32_t r = L.req_of[lane];
    uint32_t *o = static_cast<uint32_t *>(L.req_out[r]);
    return o ? o + (size_t)(lane - L.req_lane0[r]) * slots * W : nullptr;
}

// Trajectories: each lane runs the program `segments[lane]` times, the
// scratch-out block of one run feeding the scratch-in block of the next
// (n_scratch_in == n_scratch_out), every run a complete program run as
// cft_program_run_ex defines it (registers +0, r0..r2 from the streams,
// scratch past the carried block +0). Lanes are visited in `order` (the host
// sorts them by segment count, longest first, so a warp's lanes finish
// together); a lane whose segments are done is inactive for the rest of its
// warp's runs. Every `snap_every` runs the carried block is copied to the
// lane's snapshot list. Flags, STATUS and the lane byte are ORed over runs
// (STATUS also per lane when lane_status is given). A NULL a stream reads +0.
// EARLY: the launch completes requests as their lanes finish
// (TrajLaunch::req_of); a separate instantiation, since the code for it
// costs the plain launches a few per cent even when it does not run.
template <int FMT, bool EARLY>
__global__ void k_traj(const TrajLaunch L, bool scratch_shared)
{
    constexpr int W = sf::Fmt<FMT>::W;
    extern __shared__ uint32_t smem[];
    const SeqProgram &P = L.P;
    const int T = blockDim.x, t = threadIdx.x;
    const size_t local = (size_t)blockIdx.x * T + t;
    const bool have = local < L.n;
    const size_t lane = have ? (L.order ? L.order[local] : local) : 0;
    const uint32_t segs = have ? L.segments[lane] : 0u;
    const int nregs = (int)P.nregs;
    const uint32_t slots = P.n_scratch_out;
    Lane<W> R{smem, T, t};
    // the scratch block in shared memory behind the registers when it fits
    // (a trajectory's state lives there for the whole launch), else global
    const Scratch<W> sc = scratch_shared
        ? Scratch<W>{smem + (size_t)(nregs > 0 ? nregs : 1) * W * T, (size_t)T, (size_t)t}
        : Scratch<W>{static_cast<uint32_t *>(L.scratch), L.n, local};
    uint32_t *state = static_cast<uint32_t *>(L.state);
    uint32_t *snaps = static_cast<uint32_t *>(L.snaps);
    uint32_t x[W];
    if (have && sc.base) {
        for (uint32_t s = 0; s < slots; s++) {
#pragma unroll
            for (int w = 0; w < W; w++) sc.at(s, w) = state[(lane * slots + s) * W + w];
        }
    }
    uint32_t flags = 0, status = 0, err = 0;
    uint8_t lflag = 0;
    for (uint32_t seg = 0;; seg++) {
        const bool mine = have && seg < segs;
        if (!__any_sync(0xFFFFFFFFu, mine)) break;
        for (int r = 0; r < nregs; r++) {
#pragma unroll
            for (int w = 0; w < W; w++) R.at(r, w) = 0u;
        }
        if (mine) {
            if (nregs > 0 && L.a) { load_in<W>(L.a, nullptr, lane, x); R.put(0, x); }
            if (nregs > 1 && L.b) { load_in<W>(L.b, nullptr, lane, x); R.put(1, x); }
            if (nregs > 2 && L.c) { load_in<W>(L.c, nullptr, lane, x); R.put(2, x); }
            if (sc.base) {
                for (uint32_t s = slots; s < P.reach; s++) {
#pragma unroll
                    for (int w = 0; w < W; w++) sc.at(s, w) = 0u;
                }
            }
        }
        __syncwarp();
        LaneRun o;
        interpret<FMT, true>(P, R, sc, nullptr, lane, mine, mine, o);
        flags |= o.flags;
        status |= o.status;
        err |= o.err;
        lflag |= o.lflag;
        if (mine && snaps && L.snap_every && (seg + 1) % L.snap_every == 0) {
            const uint32_t k = (seg + 1) / L.snap_every - 1;
            if (k < L.max_snaps) {
                for (uint32_t s = 0; s < slots; s++) {
#pragma unroll
                    for (int w = 0; w < W; w++)
                        snaps[((lane * L.max_snaps + k) * slots + s) * W + w] = sc.at(s, w);
                }
            }
        }
        if (EARLY && mine && seg + 1 == segs) {               // this lane is done
            uint32_t *ho = lane_out<W>(L, lane, slots);
            for (uint32_t s = 0; s < slots; s++) {
#pragma unroll
                for (int w = 0; w < W; w++) {
                    const uint32_t v = sc.base ? sc.at(s, w) : state[(lane * slots + s) * W + w];
                    state[(lane * slots + s) * W + w] = v;
                    if (ho) ho[s * W + w] = v;
                }
            }
            if (L.lane_flags) L.lane_flags[lane] = lflag;
            if (L.lane_status) L.lane_status[lane] = status;
            __threadfence_system();
            lane_finished(L, lane, lflag & 0x1Fu, status);
        }
    }
    if (have) {
        if (sc.base) {
            for (uint32_t s = 0; s < slots; s++) {
#pragma unroll
                for (int w = 0; w < W; w++) state[(lane * slots + s) * W + w] = sc.at(s, w);
            }
        }
        if (L.lane_flags) L.lane_flags[lane] = lflag;
        if (L.lane_status) L.lane_status[lane] = status;
    }
    flags = __reduce_or_sync(0xFFFFFFFFu, flags);
    status = __reduce_or_sync(0xFFFFFFFFu, status);
    err = __reduce_or_sync(0xFFFFFFFFu, err);
    if ((t & 31) == 0) {
        if (flags) atomicOr(L.word + 0, flags);
        if (status) atomicOr(L.word + 1, status);
        if (err) atomicOr(L.word + 2, err);
    }
}

// The words between one location and the next in a trajectory block's
// shared memory (k_traj_g): LPB lanes of W words, then a pad of one vector
// (16 bytes from binary128 up, the element below) so that one lane's
// different locations start in different banks.
template <int W>
__host__ __device__ constexpr int traj_g_stride(int lpb) { return W * lpb + (W >= 4 ? 4 : W); }

// A location's W words as one or two vector loads or stores (the stride
// keeps every location 16-byte aligned from binary128 up, 8-byte at
// binary64).
template <int W>
SFD void load_loc(const uint32_t *p, uint32_t (&x)[W])
{
    if constexpr (W >= 4) {
#pragma unroll
        for (int h = 0; h < W / 4; h++) {
            const uint4 v = reinterpret_cast<const uint4 *>(p)[h];
            x[4 * h] = v.x; x[4 * h + 1] = v.y; x[4 * h + 2] = v.z; x[4 * h + 3] = v.w;
        }
    } else if constexpr (W == 2) {
        const uint2 v = *reinterpret_cast<const uint2 *>(p);
        x[0] = v.x; x[1] = v.y;
    } else {
        x[0] = p[0];
    }
}

template <int W>
SFD void store_loc(uint32_t *p, const uint32_t (&x)[W])
{
    if constexpr (W >= 4) {
#pragma unroll
        for (int h = 0; h < W / 4; h++)
            reinterpret_cast<uint4 *>(p)[h] = make_uint4(x[4 * h], x[4 * h + 1], x[4 * h + 2], x[4 * h + 3]);
    } else if constexpr (W == 2) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(x[0], x[1]);
    } else {
        p[0] = x[0];
    }
}

// Trajectories with G threads a lane through the bundle schedule
// (bundle.cpp). A block is one warp holding 32/G lanes; the G threads
// [li*G, li*G + G) serve lane li. A lane's locations (registers 0..31,
// scratch slots 32.., renamed values after them, then the constant bank)
// live in shared memory, location p of lane li at [p*RS + li*W] with RS a
// location's LPB lanes plus a pad (traj_g_stride), so that an operand is
// one or two vector loads and the group's threads, touching different
// locations, hit different banks. Each bundle: every thread reads its
// micro-operation's operands and computes, the warp meets, every thread
// writes its result, the warp meets again; the next bundle's control word
// and micro-operation are read while this one computes. Only
// programs without deposits, lane-mask changes, indexed scratch, quiet
// regions or raises are scheduled, so the lane byte holds the IEEE flags
// alone and STATUS stays 0.
//
// COOP (binary128/256): each micro-operation is computed by a group of W
// threads (coop.cuh), thread j of it writing word j of the result; a lane's
// G threads then hold G/W micro-operations a bundle, and the group's scratch
// sits in shared memory at word coop_at.
template <int FMT, bool EARLY, bool COOP>
__global__ void __launch_bounds__(32) k_traj_g(const TrajLaunch L, uint32_t staged,
                                               uint32_t coop_at)
{
    constexpr int W = sf::Fmt<FMT>::W;
    constexpr int K = COOP ? W : 1;                  // threads a micro-operation
    extern __shared__ __align__(16) uint32_t smem[];
    const SeqProgram &P = L.P;
    const int G = L.G, LPB = 32 / G, S = G / K;      // S: micro-operations a bundle
    const int t = threadIdx.x, g = t & (G - 1), li = t / G;
    const int slot = g / K, jw = g & (K - 1);
    const size_t local = (size_t)blockIdx.x * LPB + li;
    const bool have = local < L.n;
    const size_t lane = have ? (L.order ? L.order[local] : local) : 0;
    const uint32_t segs = have ? L.segments[lane] : 0u;
    const int nregs = P.nregs > 0 ? (int)P.nregs : 1;
    const uint32_t slots = P.n_scratch_out, reach = P.reach;
    // location p of lane li: W consecutive words at p * RS + li * W, so an
    // operand is one or two vector loads; the pad after each location's LPB
    // lanes puts the same lane's different locations in different banks
    const int RS = traj_g_stride<W>(LPB);
    auto LOC = [&](uint32_t p, int w) -> uint32_t & { return smem[p * RS + li * W + w]; };
    uint32_t *state = static_cast<uint32_t *>(L.state);
    uint32_t *snaps = static_cast<uint32_t *>(L.snaps);
    // The schedule into shared memory at word `staged`, and the constant
    // bank as locations kloc .. kloc + n_consts - 1 of every lane of the
    // block (the launch checks that they fit and that the indices stay
    // within the micro-operation's 12-bit fields): operands are then all
    // read the one way, and the schedule with shared-memory loads.
    const uint32_t kloc = L.nloc;
    const uint64_t *b_ops;
    const uint32_t *b_ctl, *b_arg;
    const int32_t *b_match;
    {
        // one more bundle past the end, a HALT of no-operations, so that the
        // loop may read the next bundle's words ahead of time
        const uint32_t nb = L.nb, nops = nb * (uint32_t)S, nb1 = nb + 1;
        uint64_t *so = reinterpret_cast<uint64_t *>(smem + staged);
        uint32_t *sw = reinterpret_cast<uint32_t *>(so + nops + S);
        for (uint32_t i = nops + t; i < nops + S; i += 32) so[i] = ~0ull;
        if (t == 0) {
            sw[nb] = 3u;                               // HALT
            sw[nb1 + nb] = 0u;
            sw[2 * nb1 + nb] = 0u;
        }
        for (uint32_t i = t; i < nops; i += 32) {
            uint64_t u = L.b_ops[i];
            if (u != ~0ull) {
                // operand fields a (bits 28-39), b (40-51), c (52-63), read
                // from the bank when bits 11, 12, 13 are set
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    if ((u >> (11 + k)) & 1u) {
                        const int at = 28 + 12 * k;
                        const uint64_t idx = ((u >> at) & 0xFFFu) + kloc;
                        u = (u & ~(0xFFFull << at) & ~(1ull << (11 + k))) | (idx << at);
                    }
                }
            }
            so[i] = u;
        }
        for (uint32_t i = t; i < nb; i += 32) {
            sw[i] = L.b_ctl[i];
            sw[nb1 + i] = L.b_arg[i];
            sw[2 * nb1 + i] = (uint32_t)L.b_match[i];
        }
        const uint32_t *kons = static_cast<const uint32_t *>(P.d_consts);
        if (kons) {
            const uint32_t per = (uint32_t)(W * LPB);
            for (uint32_t i = t; i < P.n_consts * per; i += 32) {
                const uint32_t k = i / per, r = i - k * per, w = r / (uint32_t)LPB, l = r - w * LPB;
                smem[(kloc + k) * RS + l * W + w] = kons[k * W + w];
            }
        }
        __syncwarp();
        b_ops = so;
        b_ctl = sw;
        b_arg = sw + nb1;
        b_match = reinterpret_cast<const int32_t *>(sw + 2 * nb1);
    }
    // the cooperative groups' scratch (coop.cuh), zeroed once
    [[maybe_unused]] uint32_t *sb = nullptr;
    [[maybe_unused]] coop::Group grp;
    if constexpr (COOP) {
        constexpr int SW = coop::scratch_words<W>();
        coop::zero_scratch(smem + coop_at, (32 / W) * SW, t);
        sb = smem + coop_at + (t / W) * SW;
        grp = coop::group_of<W>(t);
        __syncwarp();
    }
    if (have) {
        for (uint32_t sl = g; sl < slots; sl += G) {
#pragma unroll
            for (int w = 0; w < W; w++) LOC(32 + sl, w) = state[(lane * slots + sl) * W + w];
        }
    }
    uint32_t flags = 0, err = 0;
    uint32_t x[W];
    for (uint32_t seg = 0;; seg++) {
        const bool mine = have && seg < segs;
        if (!__any_sync(0xFFFFFFFFu, mine)) break;
        __syncwarp();
        for (int r = g; r < nregs; r += G) {
#pragma unroll
            for (int w = 0; w < W; w++) LOC(r, w) = 0u;
        }
        if (mine) {
            for (uint32_t sl = slots + g; sl < reach; sl += G) {
#pragma unroll
                for (int w = 0; w < W; w++) LOC(32 + sl, w) = 0u;
            }
        }
        __syncwarp();
        if (mine && g == 0) {
            if (nregs > 0 && L.a) { load_in<W>(L.a, nullptr, lane, x); for (int w = 0; w < W; w++) LOC(0, w) = x[w]; }
            if (nregs > 1 && L.b) { load_in<W>(L.b, nullptr, lane, x); for (int w = 0; w < W; w++) LOC(1, w) = x[w]; }
            if (nregs > 2 && L.c) { load_in<W>(L.c, nullptr, lane, x); for (int w = 0; w < W; w++) LOC(2, w) = x[w]; }
        }
        __syncwarp();
        uint32_t body[4], left[4];
        int sp = 0;
        uint32_t b = 0;
        // this bundle's control word and micro-operation; an operation
        // bundle reads the next bundle's while it computes
        uint32_t kind = b_ctl[0];
        uint64_t u = b_ops[slot];
        while (b < L.nb) {
            if (kind == 0u) {                              // micro-operations
                const uint32_t kind_next = b_ctl[b + 1];
                const uint64_t u_next = b_ops[(size_t)(b + 1) * S + slot];
                uint32_t res[W];
                int dest = -1;
                // COOP: the operands of this group's FMA/ADD/SUB/MUL, which
                // every lane of the warp then computes at once
                [[maybe_unused]] uint32_t ca[K > 1 ? W : 1], cb[K > 1 ? W : 1], cc[K > 1 ? W : 1];
                [[maybe_unused]] int cop = 0, crnd = 0;
                [[maybe_unused]] bool carith = false;
                if constexpr (COOP) {
#pragma unroll
                    for (int w = 0; w < W; w++) ca[w] = cb[w] = cc[w] = 0u;
                }
                if (mine && u != ~0ull) {
                    const uint32_t ia = (uint32_t)(u >> 28) & 0xFFFu;
                    if ((u >> 14) & 1u) {                  // MOVE
                        if constexpr (COOP) res[0] = LOC(ia, jw);
                        else load_loc<W>(&LOC(ia, 0), res);
                    } else {
                        const uint32_t ib = (uint32_t)(u >> 40) & 0xFFFu, ic = (uint32_t)(u >> 52) & 0xFFFu;
                        const int op = (int)(u & 0xFFu), rnd = (int)((u >> 8) & 7u);
                        uint32_t va[W], vb[W], vc[W], fl = 0u;
                        load_loc<W>(&LOC(ia, 0), va);              // constants are locations too
                        load_loc<W>(&LOC(ib, 0), vb);
                        load_loc<W>(&LOC(ic, 0), vc);
                        if ((u >> 15) & 1u) vc[W - 1] ^= 0x80000000u;    // a NEG folded into c
                        if constexpr (COOP) {
                            if (op <= 3) {
                                carith = true;
                                cop = op;
                                crnd = rnd;
#pragma unroll
                                for (int w = 0; w < W; w++) {
                                    ca[w] = va[w];
                                    cb[w] = vb[w];
                                    cc[w] = vc[w];
                                }
                            } else {
                                uint32_t full[W];
                                sf::simple<FMT>(op, va, vb, vc, full, fl);
                                uint32_t r = 0u;
#pragma unroll
                                for (int w = 0; w < W; w++) r = w == jw ? full[w] : r;
                                res[0] = r;
                                flags |= fl;
                            }
                        } else {
                            // latency form: this warp's lanes wait on each result
                            if (op <= 3) sf::arith_rt<FMT, true>(op, va, vb, vc, rnd, res, fl);
                            else sf::simple<FMT>(op, va, vb, vc, res, fl);
                            flags |= fl;
                        }
                    }
                    dest = (int)((u >> 16) & 0xFFFu);
                }
                if constexpr (COOP) {
                    // the warp's groups together (coop.cuh); where a group does
                    // not take its element, the one-thread code (the same in
                    // every thread of the group), word jw kept
                    uint32_t r, fl = 0u;
                    const bool ok = coop::arith_group<FMT>(grp, cop, ca, cb, cc, crnd, sb, r, fl);
                    if (carith) {
                        if (!ok) {
                            uint32_t full[W];
                            sf::arith_rt<FMT, true>(cop, ca, cb, cc, crnd, full, fl);
                            r = 0u;
#pragma unroll
                            for (int w = 0; w < W; w++) r = w == jw ? full[w] : r;
                        }
                        res[0] = r;
                        flags |= fl;
                    }
                }
                __syncwarp();
                if (dest >= 0) {
                    if constexpr (COOP) LOC((uint32_t)dest, jw) = res[0];
                    else store_loc<W>(&LOC((uint32_t)dest, 0), res);
                }
                __syncwarp();
                b++;
                kind = kind_next;
                u = u_next;
                continue;
            } else if (kind == 1u) {                       // REPEAT
                const bool any = __any_sync(0xFFFFFFFFu, mine);
                const uint32_t imm = b_arg[b];
                if (imm == 0u || !any) {
                    b = (uint32_t)b_match[b] + 1u;
                } else if (sp >= 4) {
                    err |= 1u;
                    break;
                } else {
                    body[sp] = b + 1;
                    left[sp] = imm;
                    sp++;
                    b++;
                }
            } else if (kind == 2u) {                       // ENDREP
                const bool any = __any_sync(0xFFFFFFFFu, mine);
                if (sp <= 0) {
                    err |= 2u;
                    break;
                }
                left[sp - 1]--;
                if (left[sp - 1] > 0u && any) {
                    b = body[sp - 1];
                } else {
                    sp--;
                    b++;
                }
            } else {                                       // HALT
                break;
            }
            kind = b_ctl[b];
            u = b_ops[(size_t)b * S + slot];
        }
        __syncwarp();
        if (mine && snaps && L.snap_every && (seg + 1) % L.snap_every == 0) {
            const uint32_t k = (seg + 1) / L.snap_every - 1;
            if (k < L.max_snaps) {
                for (uint32_t sl = g; sl < slots; sl += G) {
#pragma unroll
                    for (int w = 0; w < W; w++)
                        snaps[((lane * L.max_snaps + k) * slots + sl) * W + w] = LOC(32 + sl, w);
                }
            }
        }
        const bool last = EARLY && mine && seg + 1 == segs;        // this lane is done
        if (EARLY && __any_sync(0xFFFFFFFFu, last)) {
            uint32_t lf = flags;
            for (int o = 1; o < G; o <<= 1) lf |= __shfl_xor_sync(0xFFFFFFFFu, lf, o);
            if (last) {
                uint32_t *ho = lane_out<W>(L, lane, slots);
                for (uint32_t sl = g; sl < slots; sl += G) {
#pragma unroll
                    for (int w = 0; w < W; w++) {
                        const uint32_t v = LOC(32 + sl, w);
                        state[(lane * slots + sl) * W + w] = v;
                        if (ho) ho[sl * W + w] = v;
                    }
                }
                __threadfence_system();
            }
            __syncwarp();
            if (last && g == 0) {
                if (L.lane_flags) L.lane_flags[lane] = (uint8_t)(lf & 0x1Fu);
                if (L.lane_status) L.lane_status[lane] = 0u;
                lane_finished(L, lane, lf & 0x1Fu, 0u);
            }
        }
    }
    __syncwarp();
    if (have) {
        for (uint32_t sl = g; sl < slots; sl += G) {
#pragma unroll
            for (int w = 0; w < W; w++) state[(lane * slots + sl) * W + w] = LOC(32 + sl, w);
        }
    }
    uint32_t lf = flags;                                   // the lane's G threads
    for (int o = 1; o < G; o <<= 1) lf |= __shfl_xor_sync(0xFFFFFFFFu, lf, o);
    if (have && g == 0) {
        if (L.lane_flags) L.lane_flags[lane] = (uint8_t)(lf & 0x1Fu);
        if (L.lane_status) L.lane_status[lane] = 0u;
    }
    flags = __reduce_or_sync(0xFFFFFFFFu, flags);
    err = __reduce_or_sync(0xFFFFFFFFu, err);
    if (t == 0) {
        if (flags) atomicOr(L.word + 0, flags);
        if (err) atomicOr(L.word + 2, err);
    }
}

// A kernel's dynamic shared-memory ceiling and L1/shared split are set once
// a device, to the device's opt-in maximum: changing a function's attributes
// between launches can wait for the function's running launches, which in a
// serving loop are trajectories of a quarter second.
template <typename K>
static cudaError_t smem_ceiling_once(K kernel, unsigned &done_mask)
{
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned bit = 1u << (dev & 31);
    if (done_mask & bit) return cudaSuccess;
    int optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) done_mask |= bit;
    return e;
}

// The shared memory a trajectory block asks for so that an SM holds no more
// of this launch's blocks than L.sm_regs registers allow (TrajLaunch).
template <typename K>
static size_t capped_smem(K kernel, const TrajLaunch &L, int threads, size_t smem)
{
    if (!L.sm_regs || !L.sm_smem) return smem;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) {
        cudaGetLastError();
        return smem;
    }
    int dev = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    // registers are allocated a warp at a time, in units of 256
    const size_t warp_regs = ((size_t)fa.numRegs * 32 + 255) / 256 * 256;
    const size_t block_regs = warp_regs * (size_t)((threads + 31) / 32);
    size_t k = L.sm_regs / block_regs;
    if (k < 1) k = 1;
    const long each = (long)(L.sm_smem / k) - reserved - (long)fa.sharedSizeBytes;
    return each > (long)smem ? (size_t)each / 1024 * 1024 : smem;
}

template <int FMT>
static int seq_threads(const SeqProgram &P, size_t *smem)
{
    constexpr int W = sf::Fmt<FMT>::W;
    const int nregs = (int)P.nregs;
    const size_t per_lane = (size_t)(nregs > 0 ? nregs : 1) * W * 4;
    int T = (int)((64u << 10) / per_lane);
    T = (T / 32) * 32;
    if (T > 256) T = 256;
    if (T < 32) T = 32;
    *smem = per_lane * T;
    return T;
}

// A trajectory launch usually holds few lanes (thousands), each running
// long: blocks are made just large enough that the lanes spread over every
// SM, so that each warp has a scheduler to itself as far as there are SMs.
template <int FMT>
static cudaError_t go_traj(const TrajLaunch &L, cudaStream_t s)
{
    constexpr int W = sf::Fmt<FMT>::W;
    size_t smem = 0;
    int T = seq_threads<FMT>(L.P, &smem);
    const size_t sms = (size_t)sm_count();
    const size_t spread = ((L.n + sms - 1) / sms + 31) / 32 * 32;
    const size_t regs = (size_t)(L.P.nregs > 0 ? L.P.nregs : 1) * W * 4;
    if (spread < (size_t)T) {
        T = (int)spread;
        smem = regs * T;
    }
    const size_t scr = (size_t)L.P.reach * W * 4;
    const bool shared = L.P.reach > 0 && (regs + scr) * T <= (160u << 10);
    if (shared) smem += scr * T;
    const size_t blocks = (L.n + T - 1) / T;
    if (L.req_of) {
        smem = capped_smem(k_traj<FMT, true>, L, T, smem);
        static unsigned done = 0;
        cudaError_t e = smem_ceiling_once(k_traj<FMT, true>, done);
        if (e != cudaSuccess) return e;
        k_traj<FMT, true><<<(unsigned)blocks, T, smem, s>>>(L, shared);
    } else {
        smem = capped_smem(k_traj<FMT, false>, L, T, smem);
        static unsigned done = 0;
        cudaError_t e = smem_ceiling_once(k_traj<FMT, false>, done);
        if (e != cudaSuccess) return e;
        k_traj<FMT, false><<<(unsigned)blocks, T, smem, s>>>(L, shared);
    }
    return cudaGetLastError();
}

template <int FMT, bool COOP>
static cudaError_t go_traj_g(const TrajLaunch &L, cudaStream_t s)
{
    constexpr int W = sf::Fmt<FMT>::W;
    const int LPB = 32 / L.G, S = L.G / (COOP ? W : 1);
    // a lane's locations and the constants as further locations, the
    // cooperative groups' scratch, then the schedule, 8-byte aligned
    // (traj_g_smem, which the planner checked against its limits)
    size_t need = (size_t)(L.nloc + L.P.n_consts) * (size_t)traj_g_stride<W>(LPB) * 4;
    uint32_t coop_at = 0;
    if (COOP) {
        coop_at = (uint32_t)(need / 4);
        need += (size_t)(32 / W) * coop::scratch_words<W>() * 4;
    }
    const size_t at = (need + 7) / 8 * 8;
    const uint32_t staged = (uint32_t)(at / 4);
    need = at + (size_t)(L.nb + 1) * S * 8 + (size_t)(L.nb + 1) * 12;   // and a sentinel bundle
    const size_t blocks = (L.n + LPB - 1) / LPB;
    if (L.req_of) {
        const size_t smem = capped_smem(k_traj_g<FMT, true, COOP>, L, 32, need);
        static unsigned done = 0;
        cudaError_t e = smem_ceiling_once(k_traj_g<FMT, true, COOP>, done);
        if (e != cudaSuccess) return e;
        k_traj_g<FMT, true, COOP><<<(unsigned)blocks, 32, smem, s>>>(L, staged, coop_at);
    } else {
        const size_t smem = capped_smem(k_traj_g<FMT, false, COOP>, L, 32, need);
        static unsigned done = 0;
        cudaError_t e = smem_ceiling_once(k_traj_g<FMT, false, COOP>, done);
        if (e != cudaSuccess) return e;
        k_traj_g<FMT, false, COOP><<<(unsigned)blocks, 32, smem, s>>>(L, staged, coop_at);
    }
    return cudaGetLastError();
}

cudaError_t launch_traj(const TrajLaunch &L, cudaStream_t s)
{
    if (L.n == 0) return cudaSuccess;
    if (L.G > 1 && L.nb) {
        switch (L.P.fmt) {
        case 0: return go_traj_g<0, false>(L, s);
        case 1: return go_traj_g<1, false>(L, s);
        case 2: return L.K > 1 ? go_traj_g<2, true>(L, s) : go_traj_g<2, false>(L, s);
        default: return L.K > 1 ? go_traj_g<3, true>(L, s) : go_traj_g<3, false>(L, s);
        }
    }
    switch (L.P.fmt) {
    case 0: return go_traj<0>(L, s);
    case 1: return go_traj<1>(L, s);
    case 2: return go_traj<2>(L, s);
    default: return go_traj<3>(L, s);
    }
}

template <int FMT>
static cudaError_t go_seq(const SeqLaunch &L, cudaStream_t s)
{
    constexpr int W = sf::Fmt<FMT>::W;
    const int nregs = (int)L.P.nregs;
    const size_t per_lane = (size_t)(nregs > 0 ? nregs : 1) * W * 4;
    int T = (int)((64u << 10) / per_lane);
    T = (T / 32) * 32;
    if (T > 256) T = 256;
    if (T < 32) T = 32;
    const size_t smem = per_lane * T;
    static unsigned done = 0;
    cudaError_t e = smem_ceiling_once(k_seq<FMT>, done);
    if (e != cudaSuccess) return e;
    const size_t blocks = (L.n + T - 1) / T;
    k_seq<FMT><<<(unsigned)blocks, T, smem, s>>>(L, 0, L.n);
    return cudaGetLastError();
}

cudaError_t launch_seq(const SeqLaunch &L, cudaStream_t s)
{
    if (L.n == 0) return cudaSuccess;
    switch (L.P.fmt) {
    case 0: return go_seq<0>(L, s);
    case 1: return go_seq<1>(L, s);
    case 2: return go_seq<2>(L, s);
    default: return go_seq<3>(L, s);
    }
}

}  // namespace cftg
