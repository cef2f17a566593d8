// tune_policy.h -- the 3D sweep autotuner's choice of (schedule, tile shape) for one phase
// (host code; the CPU check tests/native/tune_policy_check.cpp compiles it with g++).
//
// Candidates c = 2 * schedule + shape: schedule 0 one launch per tile diagonal, 1 dataflow
// (one launch per phase), 2 hybrid (first outer iteration per diagonal, then dataflow); shape
// 0 = 4x8x32 tiles, 1 = 8x4x32.  pfast_survey3d_autotune records each candidate's phase times
// per (device, sweep kind, grid, active instances); a phase then takes the fastest allowed one.
#pragma once

namespace pfast {

constexpr int kTuneCandidates = 6;

struct TuneEntry {
    double ms[kTuneCandidates] = {};   // summed phase times
    int n[kTuneCandidates] = {};       // phases timed
};

// The candidates a phase may use: schedule_opt and shape_opt as pfast_options (0 automatic,
// else schedule 1..3 / shape 1..2); dataflow_fits[s]: the grid's tiles of shape s fit the
// dataflow kernel's shared memory.  Dataflow or hybrid asked for on a grid that does not fit:
// per diagonal.
inline unsigned tune_allowed(int schedule_opt, int shape_opt, const bool dataflow_fits[2]) {
    unsigned allowed = 0;
    for (int shape = 0; shape < 2; ++shape) {
        if (shape_opt != 0 && shape_opt - 1 != shape) continue;
        if (schedule_opt == 0 || schedule_opt == 1) allowed |= 1u << shape;
        if ((schedule_opt == 0 || schedule_opt == 2) && dataflow_fits[shape]) allowed |= 4u << shape;
        if ((schedule_opt == 0 || schedule_opt == 3) && dataflow_fits[shape]) allowed |= 16u << shape;
    }
    if (!allowed) allowed = shape_opt == 0 ? 1u : 1u << (shape_opt - 1);
    return allowed;
}

// The candidate of a phase: once every allowed candidate has been timed (e non-null), the one
// with the smallest mean phase time (the first of equal ones); before that, the dataflow kernel
// with 4x8x32 tiles from two active instances per SM, else one launch per tile diagonal
// (falling back to the lowest allowed candidate).
inline int tune_pick(const TuneEntry* e, unsigned allowed, int nact, int sms) {
    if (e) {
        int best = -1;
        bool all = true;
        for (int c = 0; c < kTuneCandidates; ++c) {
            if (!(allowed >> c & 1)) continue;
            if (e->n[c] == 0) { all = false; break; }
            if (best < 0 || e->ms[c] / e->n[c] < e->ms[best] / e->n[best]) best = c;
        }
        if (all && best >= 0) return best;
    }
    const int first = nact >= 2 * sms && (allowed & 0xcu) ? 2 : 0;
    for (int c = first; c < kTuneCandidates; ++c)
        if (allowed >> c & 1) return c;
    for (int c = 0; c < kTuneCandidates; ++c)
        if (allowed >> c & 1) return c;
    return 0;
}

}  // namespace pfast
