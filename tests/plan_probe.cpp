// C entry point over the fused schedule's work planner (fdtd_gb300/csrc/planner.cpp) for the CPU
// tests: compiled with the planner into a small host-only library by tests/test_planner.py.
#include <cstring>
#include <vector>

#include "planner.h"

// counts: 2 + kPlanShellLists entries (interior, the shell lists, then the CPML items); items: all
// of them in that order (when not NULL, at most cap). cpml: plan CPML items where the grid allows.
// Returns the interior chunk length.
extern "C" int plan_probe(const int* grid9, const int* design_box, int cpml, int* counts, int* items, long long cap) {
    const fdtd::PlanGrid g{grid9[0], grid9[1], grid9[2], grid9[3], grid9[4], grid9[5], grid9[6], grid9[7], grid9[8]};
    fdtd::FusedPlan plan;
    const int kc = fdtd::plan_chunk(g);
    fdtd::plan_fused(g, kc, design_box, plan, cpml != 0);
    std::vector<const std::vector<fdtd::PlanItem>*> lists = {&plan.interior};
    for (const auto& s : plan.shell) lists.push_back(&s);
    lists.push_back(&plan.cpml);
    long long n = 0;
    for (size_t q = 0; q < lists.size(); ++q) {
        counts[q] = (int)lists[q]->size();
        for (const fdtd::PlanItem& it : *lists[q]) {
            if (items && n < cap) std::memcpy(items + 4 * n, &it, sizeof(it));
            ++n;
        }
    }
    return kc;
}
