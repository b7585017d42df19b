// bundle.h - a lane's program spread over G threads (bundle.cpp): the
// schedule's host form and its device copy.
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/cft.h"

namespace cftg {

enum : uint32_t { BUNDLE_OPS = 0, BUNDLE_REPEAT = 1, BUNDLE_ENDREP = 2, BUNDLE_HALT = 3 };
constexpr uint64_t BUNDLE_NOP = ~0ull;       // control code 255: never a real instruction

// A bundle slot holds a micro-operation over locations (registers 0..31,
// scratch slots 32.., then values renamed within a stretch):
//   bits 0-7 opcode, 8-10 rounding, 11-13 operand a/b/c is a constant index,
//   14 MOVE (dest = a), 15 operand c read with its sign bit flipped (a NEG
//   folded into the read), 16-27 dest, 28-39 a, 40-51 b, 52-63 c.
struct BundleSchedule {
    int G = 1;
    uint32_t nb = 0;
    uint32_t nloc = 0;              // locations a lane needs
    std::vector<uint64_t> ops;      // nb x G micro-operations, BUNDLE_NOP where empty
    std::vector<uint32_t> ctl;      // per bundle: BUNDLE_*
    std::vector<uint32_t> arg;      // REPEAT: the count
    std::vector<int32_t> match;     // REPEAT <-> its ENDREP
    double weighted = 0;            // bundles one run steps through (REPEAT counts applied)
    double ops_weighted = 0;        // the same for one thread a lane (instructions)
};

bool build_bundles(const std::vector<uint64_t> &insns, uint32_t reach, int G, BundleSchedule &s);

// An image's instruction words and scratch reach, after cft_program_load's
// checks (program.cpp).
cft_status program_insns(const void *image, size_t bytes, std::vector<uint64_t> &insns,
                         uint32_t *reach);

// A loaded program's schedule for G threads a lane on its device, built and
// uploaded on first use and kept with the program; null when the program
// is outside the scheduled set.
struct DevBundles {
    int G = 1;
    uint32_t nb = 0, nloc = 0;
    double weighted = 0, ops_weighted = 0;
    const uint64_t *ops = nullptr;
    const uint32_t *ctl = nullptr, *arg = nullptr;
    const int32_t *match = nullptr;
};

}  // namespace cftg

struct cft_program;
namespace cftg {
struct TrajLaunch;
const DevBundles *program_bundles(cft_program *pr, int G);
// Sets L.G and the schedule for a launch of n lanes (G = 1: plain).
// runs_desc (optional): the lanes' run counts, longest first, in the
// order the launch places lanes (traj.cpp), for the estimate of how many
// warps share a scheduler over the longest lane's life.
void plan_lanes(cft_program *prog, size_t n, TrajLaunch &L, const uint32_t *runs_desc = nullptr);
}
