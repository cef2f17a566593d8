// serve_policy.h -- admission policy of the request server (pure C++, no CUDA).
//
// Requests wait in arrival order.  A request needs `fixed` bytes of device memory plus
// `per_src` bytes for every source it solves at once; it may run with any batch of 1 ..
// nsrc sources, so it can be admitted into a small allowance and still finish (in more
// batches).  When a slot is free the policy admits the oldest request that fits, with the
// largest batch its allowance allows; the allowance is the free budget when nothing else
// waits, else an equal share of the budget per slot, so one large request does not starve
// the rest.  A younger request may overtake a waiting older one only `max_bypass` times;
// after that the older one blocks admission until it fits (no starvation).
#pragma once

#include <algorithm>
#include <cstddef>
#include <deque>

namespace pfast {
namespace serve {

struct Need {
    long long ticket = 0;
    size_t fixed = 0;    // bytes independent of the batch (model-sized buffers, outputs)
    size_t per_src = 0;  // bytes per source solved at once
    int nsrc = 1;        // sources of the request (largest useful batch)
    int bypassed = 0;    // admissions that overtook this request
};

struct Decision {
    long long ticket = -1;   // -1: admit nothing now
    int batch = 0;
    size_t bytes = 0;
};

class Policy {
public:
    Policy(size_t budget, int slots, int max_bypass = 8)
        : budget_(budget), slots_(std::max(1, slots)), max_bypass_(max_bypass) {}

    void enqueue(const Need& n) { queue_.push_back(n); }
    size_t used() const { return used_; }
    size_t budget() const { return budget_; }
    int running() const { return running_; }
    size_t waiting() const { return queue_.size(); }

    // Memory that could ever be given to one request (a request needing more is rejected).
    bool feasible(const Need& n) const { return n.fixed + n.per_src <= budget_; }

    // Pick the next request to start, if a slot is free and one fits.
    Decision next() {
        Decision d;
        if (running_ >= slots_ || queue_.empty()) return d;
        const size_t free_b = budget_ - used_;
        const size_t share = std::max(budget_ / (size_t)slots_, (size_t)1);
        for (size_t i = 0; i < queue_.size(); ++i) {
            Need& n = queue_[i];
            const bool others_wait = queue_.size() > 1 || running_ > 0;
            const size_t allow = others_wait ? std::min(free_b, std::max(share, n.fixed + n.per_src)) : free_b;
            if (n.fixed + n.per_src <= allow) {
                const size_t room = allow - n.fixed;
                const int batch = (int)std::min<size_t>((size_t)std::max(1, n.nsrc), room / std::max<size_t>(1, n.per_src));
                d.ticket = n.ticket;
                d.batch = std::max(1, batch);
                d.bytes = n.fixed + (size_t)d.batch * n.per_src;
                for (size_t k = 0; k < i; ++k) queue_[k].bypassed += 1;
                queue_.erase(queue_.begin() + (long)i);
                used_ += d.bytes;
                running_ += 1;
                return d;
            }
            if (n.bypassed >= max_bypass_) break;   // the oldest overtaken too often: wait for it
        }
        return d;
    }

    // A started request finished and returned its memory.
    void finish(size_t bytes) {
        used_ -= std::min(used_, bytes);
        running_ = std::max(0, running_ - 1);
    }

    // Memory held outside requests (resident models and surveys); may be negative to release.
    bool reserve(size_t bytes) {
        if (used_ + bytes > budget_) return false;
        used_ += bytes;
        return true;
    }
    void release(size_t bytes) { used_ -= std::min(used_, bytes); }

private:
    size_t budget_;
    int slots_;
    int max_bypass_;
    size_t used_ = 0;
    int running_ = 0;
    std::deque<Need> queue_;
};

}  // namespace serve
}  // namespace pfast
