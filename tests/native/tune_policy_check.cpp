// CPU check of the 3D sweep autotuner's policy (pfast_gb300/csrc/tune_policy.h): which
// (schedule, tile shape) candidates a phase may use under each option, the untuned default,
// and the fastest pick once every allowed candidate has been timed.  Prints "ok <case>" per
// passing case and "FAIL <case>" otherwise; exits non-zero on a failure.
#include <cstdio>

#include "tune_policy.h"

using namespace pfast;

static int failures = 0;
static void check(bool c, const char* what) {
    std::printf("%s %s\n", c ? "ok" : "FAIL", what);
    if (!c) ++failures;
}

int main() {
    const bool both[2] = {true, true}, none[2] = {false, false}, first[2] = {true, false};
    // allowed sets: bits 2*schedule + shape
    check(tune_allowed(0, 0, both) == 0x3fu, "automatic: all six candidates");
    check(tune_allowed(0, 0, none) == 0x03u, "automatic, grid too large for the dataflow kernel: per diagonal");
    check(tune_allowed(0, 0, first) == 0x17u, "automatic, only 4x8x32 fits: its dataflow and hybrid");
    check(tune_allowed(1, 0, both) == 0x03u, "per diagonal forced: both shapes");
    check(tune_allowed(2, 0, both) == 0x0cu, "dataflow forced: both shapes");
    check(tune_allowed(3, 2, both) == 0x20u, "hybrid and 8x4x32 forced");
    check(tune_allowed(2, 1, none) == 0x01u, "dataflow forced on a grid that does not fit: per diagonal, 4x8x32");
    check(tune_allowed(3, 2, none) == 0x02u, "hybrid forced on a grid that does not fit: per diagonal, 8x4x32");

    // untuned defaults (152 SMs)
    check(tune_pick(nullptr, 0x3fu, 256, 152) == 0, "untuned, 256 sources: per diagonal 4x8x32");
    check(tune_pick(nullptr, 0x3fu, 304, 152) == 2, "untuned, two sources per SM: dataflow 4x8x32");
    check(tune_pick(nullptr, 0x03u, 1000, 152) == 0, "untuned, no dataflow allowed: per diagonal");
    check(tune_pick(nullptr, 0x20u, 1, 152) == 5, "untuned, one candidate allowed: that one");

    // tuned
    TuneEntry e;
    const double ms[6] = {600, 650, 560, 600, 540, 580};
    for (int c = 0; c < 6; ++c) { e.ms[c] = 2 * ms[c]; e.n[c] = 2; }
    check(tune_pick(&e, 0x3fu, 256, 152) == 4, "tuned: the fastest (hybrid 4x8x32)");
    check(tune_pick(&e, 0x0cu, 256, 152) == 2, "tuned, dataflow forced: the faster shape");
    check(tune_pick(&e, 0x03u, 256, 152) == 0, "tuned, per diagonal forced: 4x8x32");
    e.ms[1] = 3 * 500; e.n[1] = 3;   // means, not sums
    check(tune_pick(&e, 0x03u, 256, 152) == 1, "tuned: compared by mean phase time");
    TuneEntry part;
    part.ms[0] = 100; part.n[0] = 1;   // only one candidate timed
    check(tune_pick(&part, 0x3fu, 400, 152) == 2, "partly tuned: the untuned default");
    check(tune_pick(&part, 0x01u, 400, 152) == 0, "partly tuned, the timed one is the only one allowed");
    TuneEntry tie;
    for (int c = 0; c < 6; ++c) { tie.ms[c] = 100; tie.n[c] = 1; }
    check(tune_pick(&tie, 0x3cu, 1, 152) == 2, "equal times: the lowest index");

    std::printf("%d failures\n", failures);
    return failures ? 1 : 0;
}
