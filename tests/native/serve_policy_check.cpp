// Exercises the request server's admission policy (pfast_gb300/csrc/serve_policy.h) on the
// CPU: prints one line per scenario, checked by tests/test_serve_policy.py.
#include <cstdio>
#include "serve_policy.h"

using pfast::serve::Need;
using pfast::serve::Policy;

static Need need(long long t, size_t fixed, size_t per_src, int nsrc) {
    Need n;
    n.ticket = t;
    n.fixed = fixed;
    n.per_src = per_src;
    n.nsrc = nsrc;
    return n;
}

int main() {
    {   // alone: the whole budget, largest batch that fits
        Policy p(1000, 4);
        p.enqueue(need(1, 100, 50, 100));
        auto d = p.next();
        std::printf("alone %lld %d %zu %zu\n", d.ticket, d.batch, d.bytes, p.used());
    }
    {   // FIFO with shares: two waiting requests split the budget by slots
        Policy p(1000, 2);
        p.enqueue(need(1, 100, 50, 100));
        p.enqueue(need(2, 100, 50, 100));
        auto a = p.next();
        auto b = p.next();
        auto c = p.next();   // no free slot
        std::printf("shares %lld %d %lld %d %lld %zu\n", a.ticket, a.batch, b.ticket, b.batch, c.ticket, p.used());
    }
    {   // a big head that does not fit is overtaken by a small one, at most max_bypass times
        Policy p(1000, 8, 2);
        p.enqueue(need(1, 100, 100, 1));      // 200 bytes, runs
        auto first = p.next();
        p.enqueue(need(2, 900, 10, 1));       // needs 910: does not fit beside ticket 1
        p.enqueue(need(3, 10, 10, 1));
        p.enqueue(need(4, 10, 10, 1));
        p.enqueue(need(5, 10, 10, 1));
        auto a = p.next();   // 3 overtakes 2
        auto b = p.next();   // 4 overtakes 2
        auto c = p.next();   // 2 was overtaken twice: blocks; 5 waits
        p.finish(first.bytes);
        p.finish(a.bytes);
        p.finish(b.bytes);
        auto e = p.next();   // now 2 fits
        auto f = p.next();   // then 5, beside 2 (910 + 20 <= 1000)
        std::printf("bypass %lld %lld %lld %lld %lld %lld\n", first.ticket, a.ticket, b.ticket, c.ticket, e.ticket,
                    f.ticket);
    }
    {   // resident reservations count against the budget; feasibility
        Policy p(1000, 2);
        bool r1 = p.reserve(600);
        bool r2 = p.reserve(600);
        p.enqueue(need(1, 100, 100, 10));
        auto d = p.next();
        Need big = need(9, 2000, 1, 1);
        std::printf("reserve %d %d %lld %d %zu %d\n", (int)r1, (int)r2, d.ticket, d.batch, p.used(),
                    (int)p.feasible(big));
    }
    return 0;
}
