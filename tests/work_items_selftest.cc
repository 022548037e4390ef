// work_items_selftest.cc -- the material phase's work items
// (lg::build_material_items, lg_problem.cc) on the reference's region draws.
// A mesh whose repeated counts all reach T = 3/8 resident keeps one item per
// element in region visit order, each with its region's repetitions.  Any
// other mesh gets repetition items: every element has exactly one writer,
// its shares add up to its region's repetitions, no share exceeds
// R = max(1, ceil(total / (4 resident))), the shares come largest first, and
// the count stays within what the handle reserves (numElem + 4 x resident).
// Prints one line per case and the number of failed checks; exits 1 if any.
#include <algorithm>
#include <cstdio>
#include <map>
#include <vector>

#include "lg_problem.h"

static int g_bad = 0;
static void check(bool ok, const char *what, int nx)
{
    if (!ok) {
        if (g_bad < 20) std::printf("  FAILED %s (s=%d)\n", what, nx);
        ++g_bad;
    }
}

int main()
{
    const long long resident = 152LL * 1024;
    const int cases[][4] = {{4, 4, 1, 30}, {8, 11, 1, 1}, {16, 16, 2, 4}, {20, 11, 1, 12},
                            {30, 11, 1, 1}, {30, 16, 2, 4}, {48, 11, 1, 1}, {64, 11, 1, 1},
                            {64, 16, 2, 4}, {96, 11, 1, 1}, {1, 1, 1, 1}};
    for (const auto &c : cases) {
        const int nx = c[0];
        const lg::Problem p = lg::build_sedov_scalars(nx, c[1], c[2], c[3], 3.0, 1.0);
        std::vector<int> item_elem, item_rep;
        const bool split = lg::build_material_items(p, resident, item_elem, item_rep);
        check(item_elem.size() == item_rep.size(), "array lengths", nx);
        check((long long)item_elem.size() <= p.numElem + 4 * resident, "capacity", nx);
        std::map<int, long long> count;
        std::vector<int> region_of(p.numElem, -1);
        long long total = 0;
        for (int r = 0; r < p.numReg; ++r) {
            const int rr = lg::region_rep(r, p.numReg, p.cost);
            count[rr] += (long long)p.regElemlist[r].size();
            total += (long long)rr * p.regElemlist[r].size();
            for (int e : p.regElemlist[r]) region_of[e] = r;
        }
        bool want_split = false;
        for (const auto &kv : count)
            if (kv.first >= 2 && kv.second > 0 && kv.second < 3 * resident / 8) want_split = true;
        check(split == want_split, "split exactly when a repeated count is small", nx);
        if (!split) {
            check((int)item_elem.size() == p.numElem, "one item per element", nx);
            size_t i = 0;
            for (const int r : lg::region_visit_order(p.numReg, p.cost))
                for (int e : p.regElemlist[r]) {
                    check(item_elem[i] == e, "region order", nx);
                    check(item_rep[i] == lg::region_rep(r, p.numReg, p.cost),
                          "the region's repetitions", nx);
                    ++i;
                }
        } else {
            const long long R = std::max<long long>(1, (total + 4 * resident - 1) / (4 * resident));
            std::vector<int> reps(p.numElem, 0), nwriter(p.numElem, 0);
            int prev = 1 << 30;
            for (size_t i = 0; i < item_elem.size(); ++i) {
                const int e = item_elem[i], r = item_rep[i];
                check(e >= 0 && e < p.numElem, "element in range", nx);
                check(r != 0, "an item has repetitions", nx);
                const int share = r > 0 ? r : -r;
                check(share <= R, "share at most R", nx);
                check(share <= prev, "largest shares first", nx);
                prev = share;
                if (e >= 0 && e < p.numElem) {
                    reps[e] += share;
                    nwriter[e] += r > 0;
                }
            }
            for (int e = 0; e < p.numElem; ++e) {
                check(nwriter[e] == 1, "exactly one writer", nx);
                check(region_of[e] >= 0 &&
                          reps[e] == lg::region_rep(region_of[e], p.numReg, p.cost),
                      "shares add up to the region's repetitions", nx);
            }
        }
        std::printf("s=%d r=%d b=%d c=%d: %d elements, %zu items, %s\n", nx, c[1], c[2], c[3],
                    p.numElem, item_elem.size(), split ? "split" : "one per element");
    }
    std::printf("failed checks %d\n", g_bad);
    return g_bad != 0;
}
