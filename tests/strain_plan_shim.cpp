// Test shim: the strain schedule builder (collision_gb300/csrc/cc_strain_plan.cpp)
// behind one C function, so that the CPU tests can check its levels, slots,
// copy-ins and write-backs without a GPU.
#include <cstring>

#include "cc_strain_plan.h"

// Edges (p0[i], p1[i]) of one scene whose points are [v0, v0 + nv). Writes
// the sorted edges (p0, p1, s0, s1: 4 ints each), the level headers (8 ints
// per level), the copy-in and write-back lists (2 ints per entry) and info =
// {levels, slots, wb_final0, wb_final1, cap edges, cap copy-ins, cap
// write-backs, copy-ins, write-backs}. Returns -1 when a buffer is too small.
extern "C" int strain_plan(const int* p0, const int* p1, int m, int v0, int nv, int* edges_out, int* hdr_out,
                           int hdr_cap, int* load_out, int* wb_out, int list_cap, int* info) {
    std::vector<ccg::StrainEdge> edges((size_t)m);
    for (int i = 0; i < m; ++i) edges[(size_t)i] = ccg::StrainEdge{p0[i], p1[i], 1.0, -1, -1};
    std::vector<ccg::StrainEdge> all;
    std::vector<int4> hdr;
    std::vector<int2> load, wb;
    ccg::SceneDev sd;
    std::memset(&sd, 0, sizeof(sd));
    int caps[3];
    ccg::append_strain_schedule(edges, v0, nv, all, hdr, load, wb, sd, caps);
    if ((int)hdr.size() > hdr_cap || (int)load.size() > list_cap || (int)wb.size() > list_cap) return -1;
    for (size_t i = 0; i < all.size(); ++i) {
        edges_out[4 * i] = all[i].p0;
        edges_out[4 * i + 1] = all[i].p1;
        edges_out[4 * i + 2] = all[i].s0;
        edges_out[4 * i + 3] = all[i].s1;
    }
    for (size_t i = 0; i < hdr.size(); ++i) {
        hdr_out[4 * i] = hdr[i].x;
        hdr_out[4 * i + 1] = hdr[i].y;
        hdr_out[4 * i + 2] = hdr[i].z;
        hdr_out[4 * i + 3] = hdr[i].w;
    }
    for (size_t i = 0; i < load.size(); ++i) {
        load_out[2 * i] = load[i].x;
        load_out[2 * i + 1] = load[i].y;
    }
    for (size_t i = 0; i < wb.size(); ++i) {
        wb_out[2 * i] = wb[i].x;
        wb_out[2 * i + 1] = wb[i].y;
    }
    const int vals[9] = {sd.strain_levels, sd.strain_slots, sd.wb_final0, sd.wb_final1, caps[0], caps[1], caps[2],
                         (int)load.size(), (int)wb.size()};
    std::memcpy(info, vals, sizeof(vals));
    return 0;
}
