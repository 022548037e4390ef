// work_items_selftest.cc -- the material kernel's work items
// (lg::build_work_items, lg_problem.cc) on the reference's region draws:
// every element has exactly one writer item, the shares of its items add up
// to its region's EOS repetition count, an element's items never straddle a
// block of 128, the count stays within what the handle reserves
// (numElem + 2 x resident), the slots of the shared-item path
// (lg::build_item_slots) list each block's distinct elements once with every
// item pointing at its element's slot, and a mesh whose repeated counts all reach
// T = 3/8 resident keeps one item per element in the plain region order.  Prints one line per case
// and the number of failed checks; exits 1 if any.
#include <cstdio>
#include <map>
#include <set>
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
                            {64, 16, 2, 4}, {96, 11, 1, 1}};
    for (const auto &c : cases) {
        const int nx = c[0];
        const lg::Problem p = lg::build_sedov_scalars(nx, c[1], c[2], c[3], 3.0, 1.0);
        std::vector<int> item_elem, item_rep;
        const int writers = lg::build_work_items(p, resident, 128, item_elem, item_rep);
        check(writers == p.numElem, "one writer per element", nx);
        check(item_elem.size() == item_rep.size(), "array lengths", nx);
        check((long long)item_elem.size() <= p.numElem + 2 * resident, "capacity", nx);
        std::vector<int> region_of(p.numElem, -1), reps(p.numElem, 0), nwriter(p.numElem, 0);
        for (int r = 0; r < p.numReg; ++r)
            for (int e : p.regElemlist[r]) region_of[e] = r;
        std::map<int, std::set<size_t>> blocks;
        size_t pad = 0;
        for (size_t i = 0; i < item_elem.size(); ++i) {
            const int e = item_elem[i], r = item_rep[i];
            if (e < 0) {
                check(r == 0, "padding has no repetitions", nx);
                ++pad;
                continue;
            }
            check(r != 0, "an item has repetitions", nx);
            reps[e] += r > 0 ? r : -r;
            nwriter[e] += r > 0;
            blocks[e].insert(i / 128);
        }
        for (int e = 0; e < p.numElem; ++e) {
            check(nwriter[e] == 1, "exactly one writer", nx);
            check(region_of[e] >= 0 &&
                      reps[e] == lg::region_rep(region_of[e], p.numReg, p.cost),
                  "shares add up to the region's repetitions", nx);
        }
        for (const auto &b : blocks) check(b.second.size() == 1, "items within one block", nx);
        // slots of the shared-item path: per block its distinct elements in
        // order, every item pointing at its own element's slot
        std::vector<int> slot_elem, item_slot;
        lg::build_item_slots(item_elem, 128, slot_elem, item_slot);
        check(slot_elem.size() == (item_elem.size() + 127) / 128 * 128, "slot array covers blocks",
              nx);
        check(item_slot.size() == item_elem.size(), "one slot per item", nx);
        std::vector<int> slotted(p.numElem, 0);
        for (size_t b = 0; b * 128 < item_elem.size(); ++b) {
            bool ended = false;
            for (int j = 0; j < 128; ++j) {
                const int e = slot_elem[b * 128 + j];
                if (e < 0) {
                    ended = true;
                    continue;
                }
                check(!ended, "slots are dense", nx);
                check(e < p.numElem, "slot element in range", nx);
                slotted[e]++;
            }
        }
        for (int e = 0; e < p.numElem; ++e) check(slotted[e] == 1, "each element in one slot", nx);
        for (size_t i = 0; i < item_elem.size(); ++i) {
            if (item_elem[i] < 0) {
                check(item_slot[i] == -1, "padding has no slot", nx);
                continue;
            }
            check(item_slot[i] >= 0 && item_slot[i] < 128 &&
                      slot_elem[(i / 128) * 128 + item_slot[i]] == item_elem[i],
                  "item slot names its element", nx);
        }
        // a mesh where every repeated count has at least T elements keeps one
        // item per element, in plain region order
        std::map<int, long long> count;
        for (int r = 0; r < p.numReg; ++r)
            count[lg::region_rep(r, p.numReg, p.cost)] += (long long)p.regElemlist[r].size();
        bool unsplit = true;
        for (const auto &kv : count)
            if (kv.first > 1 && kv.second > 0 && kv.second < 3 * resident / 8) unsplit = false;
        if (unsplit) {
            check((int)item_elem.size() == p.numElem, "one item per element on a large mesh", nx);
            size_t i = 0;
            for (const int r : lg::region_visit_order(p.numReg, p.cost))
                for (int e : p.regElemlist[r]) check(item_elem[i++] == e, "region order", nx);
        }
        std::printf("s=%d r=%d b=%d c=%d: %d elements, %zu items, %zu padding\n", nx, c[1], c[2],
                    c[3], p.numElem, item_elem.size(), pad);
    }
    std::printf("failed checks %d\n", g_bad);
    return g_bad != 0;
}
