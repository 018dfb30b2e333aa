// Autotuner of the pipelined FP32 push's launch shape (host side).
//
// The shape (device.cuh PushShape) decides how a 1024-slot tile is split
// into work: tiles of at most `item_cells` cells are cut into work items of
// `item` particles that warps claim one at a time, sparser tiles are pushed
// slot by slot; `per_sm` persistent blocks run on each SM. The best split
// depends on the particles per cell and on how uneven they are, so it is
// measured on the simulation itself: after a particle upload the next steps
// run outside the step graph, each under one candidate shape, with the push
// kernel bracketed by CUDA events. The search is by coordinates, one phase
// per parameter, the incumbent re-measured in every phase (the particles
// drift between steps) and every candidate timed kReps times, round robin,
// keeping its fastest time. A challenger replaces the incumbent only when it
// is faster by more than kMargin. Every trial is an ordinary step of the
// simulation: only the launch shape differs, not the result of a particle.
#pragma once

#include <algorithm>
#include <limits>
#include <vector>

#include "device.cuh"

namespace ipg {

class PushTuner {
public:
    static constexpr int kReps = 2;          // timed trials per candidate and phase
    static constexpr int kWarm = 1;          // untimed steps first (module load, first-touch)
    static constexpr float kMargin = 0.01f;  // relative gain a challenger needs

    // Starts a tuning pass from the default shape (per_sm: the resident
    // maximum); `max_per_sm` bounds the blocks-per-SM candidates.
    void start(int max_per_sm) {
        max_per_sm_ = std::max(1, max_per_sm);
        best_ = kDefaultPushShape;
        best_.per_sm = max_per_sm_;
        best_ms_ = 0.f;
        phase_ = 0;
        trials_ = 0;
        warm_ = kWarm;
        running_ = true;
        tuned_ = false;
        begin_phase();
    }
    // Takes a shape tuned before (the same workload): no trials.
    void adopt(const PushShape& s, float ms) {
        best_ = s;
        best_ms_ = ms;
        trials_ = 0;
        running_ = false;
        tuned_ = true;
    }
    // Fixes a shape: no tuning.
    void fix(const PushShape& s) {
        best_ = s;
        best_ms_ = 0.f;
        running_ = false;
        tuned_ = false;
    }
    bool running() const { return running_; }
    bool tuned() const { return tuned_; }
    int trials() const { return trials_; }
    float best_ms() const { return best_ms_; }
    // The shape steps use (the incumbent while tuning).
    const PushShape& shape() const { return best_; }
    // The shape of the next step (a trial while running).
    PushShape next() const {
        if (!running_ || warm_ > 0) return best_;
        return cand_[trial_ % cand_.size()];
    }
    // The push time of the step that just ran under next().
    void record(float ms) {
        if (!running_) return;
        if (warm_ > 0) {
            --warm_;
            return;
        }
        const size_t i = (size_t)trial_ % cand_.size();
        ms_[i] = std::min(ms_[i], ms);
        ++trials_;
        if (++trial_ < (int)cand_.size() * kReps) return;
        // phase done: candidate 0 is the incumbent
        size_t win = 0;
        for (size_t c = 1; c < cand_.size(); ++c)
            if (ms_[c] < ms_[win] * (1.f - kMargin)) win = c;
        best_ = cand_[win];
        best_ms_ = ms_[win];
        ++phase_;
        begin_phase();
    }

private:
    // Candidates of the current phase (incumbent first); past the last
    // phase, the pass ends.
    void begin_phase() {
        for (;;) {
            cand_.assign(1, best_);
            if (phase_ == 0) {  // particles per work item
                for (int item : {128, 512, 1024}) add(best_, &PushShape::item, item);
            } else if (phase_ == 1) {  // densest tile pushed slot by slot
                for (int cells : {16, 8, 0}) add(best_, &PushShape::item_cells, cells);
            } else if (phase_ == 2) {  // persistent blocks per SM
                for (int b = 1; b < max_per_sm_; ++b) add(best_, &PushShape::per_sm, b);
            } else {
                running_ = false;
                tuned_ = true;
                return;
            }
            if (cand_.size() > 1) break;
            ++phase_;  // nothing to compare in this phase
        }
        ms_.assign(cand_.size(), std::numeric_limits<float>::infinity());
        trial_ = 0;
    }
    void add(PushShape s, int32_t PushShape::*field, int value) {
        if (s.*field == value) return;
        s.*field = value;
        cand_.push_back(s);
    }

    PushShape best_ = kDefaultPushShape;
    float best_ms_ = 0.f;
    std::vector<PushShape> cand_;
    std::vector<float> ms_;
    int max_per_sm_ = 1;
    int phase_ = 0, trial_ = 0, trials_ = 0, warm_ = 0;
    bool running_ = false, tuned_ = false;
};

}  // namespace ipg
