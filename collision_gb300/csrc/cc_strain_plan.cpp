// Strain-limiting schedule of one scene; see cc_strain_plan.h.
#include "cc_strain_plan.h"

#include <algorithm>
#include <functional>
#include <queue>
#include <utility>

namespace ccg {

void append_strain_schedule(const std::vector<StrainEdge>& edges, int v0, int nv, std::vector<StrainEdge>& all_edges,
                            std::vector<int4>& hdr, std::vector<int2>& load, std::vector<int2>& wb, SceneDev& sd,
                            int caps[3]) {
    const int kAhead = kStrainAhead;
    const int m = (int)edges.size();
    std::vector<int> lvl((size_t)m), last((size_t)nv, 0);
    int nlevels = 0;
    for (int i = 0; i < m; ++i) {
        int a = edges[i].p0 - v0, b = edges[i].p1 - v0;
        int l = 1 + std::max(last[a], last[b]);
        lvl[i] = l;
        last[a] = last[b] = l;
        nlevels = std::max(nlevels, l);
    }
    std::vector<int> level_off((size_t)nlevels + 1, 0);
    for (int i = 0; i < m; ++i) level_off[lvl[i]]++;
    for (int l = 1; l <= nlevels; ++l) level_off[l] += level_off[l - 1];
    // level_off[l] = edges of levels <= l = start of (0-based) level l
    std::vector<StrainEdge> sorted((size_t)m);
    {
        std::vector<int> cur(level_off.begin(), level_off.end());
        for (int i = 0; i < m; ++i) sorted[cur[lvl[i] - 1]++] = edges[i];
    }
    std::vector<int> first((size_t)nv, -1), lastl((size_t)nv, -1);
    for (int l = 0; l < nlevels; ++l)
        for (int i = level_off[l]; i < level_off[l + 1]; ++i)
            for (int p : {sorted[i].p0 - v0, sorted[i].p1 - v0}) {
                if (first[p] < 0) first[p] = l;
                lastl[p] = l;
            }
    std::vector<std::pair<int, int>> order;  // (copy-in level, local point)
    for (int p = 0; p < nv; ++p)
        if (first[p] >= 0) order.push_back({std::max(0, first[p] - kAhead), p});
    std::sort(order.begin(), order.end());
    std::vector<int> slot((size_t)nv, -1);
    std::priority_queue<std::pair<int, int>, std::vector<std::pair<int, int>>, std::greater<>> busy;  // (end, slot)
    std::priority_queue<int, std::vector<int>, std::greater<>> freeq;
    int nslots = 0;
    for (auto& lp : order) {
        while (!busy.empty() && busy.top().first < lp.first) {
            freeq.push(busy.top().second);
            busy.pop();
        }
        int sl;
        if (!freeq.empty()) {
            sl = freeq.top();
            freeq.pop();
        } else {
            sl = nslots++;
        }
        slot[lp.second] = sl;
        busy.push({lastl[lp.second] + 2, sl});
    }
    for (auto& ed : sorted) {
        ed.s0 = slot[ed.p0 - v0];
        ed.s1 = slot[ed.p1 - v0];
    }
    std::vector<int> load_off((size_t)nlevels + 1, 0), wb_off((size_t)nlevels + 2, 0);
    for (auto& lp : order) load_off[lp.first + 1]++;
    for (int p = 0; p < nv; ++p)
        if (first[p] >= 0) wb_off[lastl[p] + 2]++;  // written back at level last + 1
    for (int l = 0; l < nlevels; ++l) load_off[l + 1] += load_off[l];
    for (int l = 0; l <= nlevels; ++l) wb_off[l + 1] += wb_off[l];
    const int ebase = (int)all_edges.size(), lbase = (int)load.size(), wbase = (int)wb.size();
    load.resize(load.size() + order.size());
    wb.resize(wb.size() + order.size());
    {
        std::vector<int> lc(load_off.begin(), load_off.end()), wc(wb_off.begin(), wb_off.end());
        for (auto& lp : order) load[lbase + lc[lp.first]++] = int2{v0 + lp.second, slot[lp.second]};
        for (int p = 0; p < nv; ++p)
            if (first[p] >= 0) wb[wbase + wc[lastl[p] + 1]++] = int2{v0 + p, slot[p]};
    }
    sd.strain_hdr0 = (int)(hdr.size() / 2);
    sd.strain_levels = nlevels;
    sd.strain_slots = nslots;
    caps[0] = caps[1] = caps[2] = 0;  // most edges, copy-ins, write-backs of one level
    for (int l = 0; l < nlevels; ++l) {
        caps[0] = std::max(caps[0], level_off[l + 1] - level_off[l]);
        caps[1] = std::max(caps[1], load_off[l + 1] - load_off[l]);
        caps[2] = std::max(caps[2], wb_off[l + 1] - wb_off[l]);
    }
    for (int l = 0; l < nlevels; ++l) {
        hdr.push_back(int4{ebase + level_off[l], ebase + level_off[l + 1], lbase + load_off[l], lbase + load_off[l + 1]});
        hdr.push_back(int4{wbase + wb_off[l], wbase + wb_off[l + 1], 0, 0});
    }
    sd.wb_final0 = wbase + wb_off[nlevels];
    sd.wb_final1 = wbase + wb_off[nlevels + 1];
    all_edges.insert(all_edges.end(), sorted.begin(), sorted.end());
}

}  // namespace ccg
